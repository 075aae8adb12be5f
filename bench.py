"""Benchmark: point inversions/s on one GB300 (mixed precision vs plain FP64).

Workload (default "large"): one bicubic rational B-spline surface, 64x64 control net, clamped
non-uniform knots (interior gaps U[0.5,1.5]), z = 0.1 N(0,1) smoothed by a 5-point stencil,
w ~ U[0.5,2]; 2^20 inversion queries P = S(u,v) + |N(0,1e-2)| n(u,v).  Seeded synthetic data.

A step = one nurbs_invert launch over the whole query batch with the queries resident in HBM
(`value`).  `e2e` repeats it through nurbs_invert_host with pinned host buffers: the
host->device copy of the queries and the device->host copy of uv/status/residual are inside
each timed step.  L2 is flushed (a 512 MB write) before every timed step.

On one GPU the same line also carries sub-records of the other workloads, each with its own
clock samples: "batched" (4096 uneven surfaces, one persistent launch from a CUDA graph, mixed vs
FP64, oracle parity sample), "quintic" (degree 5, 256x256 net, 2^24 queries, per-query parameter
error against the oracle), "eval_large" (2^26 evaluations of S..Svv, FP64 and FP32, with their
rooflines), "project" (nurbs_project of 2^20 points near and far from the 64x64 surface, mixed and
FP64, oracle parity sample), "quadtree" (nurbs_invert_quadtree of 2^20 points on that surface, no
tree build), "pcurve" (nurbs_pcurve of 2^20 samples of closed curves on that surface) and
"serving" (continuous batching over a pool of 10^4 surfaces: peak
throughput, p50/p99 at half of peak, FP64 server at the top rate).  --headline-only leaves them
out.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload ...]

Under torchrun (N > 1) every rank inverts its own batch of the same size (weak scaling, no
data-path collective); rank 0 prints the JSON line with the max time over ranks.
"""
from __future__ import annotations

import argparse
import importlib.util
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG_DIR = os.path.join(ROOT, "gpu-nurbs_gb300")
sys.path.insert(0, ROOT)

METRIC = "point inversions/s at <=1e-9 param err, mixed vs plain FP64; serve p50/p99 ms"


def load_pkg():
    if "gpu_nurbs_gb300" in sys.modules:
        return sys.modules["gpu_nurbs_gb300"]
    spec = importlib.util.spec_from_file_location("gpu_nurbs_gb300", os.path.join(PKG_DIR, "__init__.py"),
                                                  submodule_search_locations=[PKG_DIR])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["gpu_nurbs_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={gpu_index}", f"--query-gpu={self.FIELDS}",
                                       "--format=csv,noheader,nounits", "-lms", "100"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        rows = [l.split(",") for l in open(self.f.name).read().strip().splitlines() if l.strip()]
        os.unlink(self.f.name)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
                for k, nm in enumerate(names):
                    if r[5 + k].strip() == "Active":
                        reasons.add(nm)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# DRAM bytes (read + write) per launch of the dominant kernel, from one ncu capture each of the
# same kernel on the same workload, per unit of work so that they scale to the launch size:
# traffic grows with the number of queries or points.
TRAFFIC_PER_UNIT = {
    "large": (38.02e6 + 27.69e6) / (1 << 20),   # mixed k_invert, bytes per query (2^20-query capture)
    "eval-large": (69.05e6 + 542.67e6) / (1 << 22),  # FP64 k_eval S..Svv, bytes per point (2^22 points)
}


def workload_label(name, n):
    """The workload a bench line is about (the same string for this library and the reference arm)."""
    return {"large": f"large: bicubic 64x64 net, 2^{int(np.log2(n))} queries, offsets |N(0,1e-2)|",
            "small": f"small: bicubic 8x8 net, {n} queries, offsets N(0,1e-3)",
            "quintic": f"quintic: degree 5x5 256x256 net, 2^{int(np.log2(n))} queries, offsets N(0,1e-3)"}[name]


def mean_step_ms_over_ranks(ts, world, device):
    """Per-step time of the slowest rank: each rank's total over its timed steps, the maximum
    taken over ranks (an all-reduce of one number; nothing else crosses ranks), divided by the
    step count."""
    tot = sum(ts)
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([tot], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        tot = float(t.item())
    return tot / len(ts)


def event_timer(torch, flush):
    """Times fn over `steps` steps with CUDA events on the current stream; L2 is flushed (a
    512 MB write) before each step."""
    stream = torch.cuda.current_stream()

    def timed(fn, steps):
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        for k in range(steps):
            flush.fill_(float(k))
            evs[k][0].record(stream)
            fn()
            evs[k][1].record(stream)
        torch.cuda.synchronize()
        return [e0.elapsed_time(e1) for e0, e1 in evs]
    return timed


def host_cores():
    return len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()


def oracle_parity_sample(surf, P, g_uv, g_st, g_res, res_abs=1e-14):
    """Checks a GPU inversion on a bounded sample against the oracle (the CPU-baseline leg's
    own results), with the oracle's answers at FP32 resolution deciding which queries are
    UNSTABLE; adds the parameter error of the matching queries (max, p99).  Returns the parity
    record and the oracle's wall time for the plain inversion of the sample."""
    import oracle as O
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from parity import classify_inversion
    cores = host_cores()
    o = O.OracleSurface(surf)
    o.tree()
    t0 = time.perf_counter()
    ouv, ost, ores, _ = o.invert(P, threads=cores)
    dt = time.perf_counter() - t0
    c = classify_inversion(g_uv, g_st, g_res, ouv, ost, ores, P, res_abs=res_abs,
                           perturbed=o.stability_set(P, threads=cores))
    return {k: v for k, v in c.items() if k != "fail_idx"}, dt


def merge_parity(tot, c):
    for k, v in c.items():
        if k.startswith("max_"):
            tot[k] = max(tot.get(k, 0.0), v)
        elif k.startswith("p99_"):
            tot.setdefault(k + "_per_surface", []).append(v)
        else:
            tot[k] = tot.get(k, 0) + v
    return tot


def make_workload(gn, torch, name, n, seed):
    from gpu_nurbs_gb300 import synth
    if name == "large":
        surf, kind = synth.surface_large(), "large"
    elif name == "small":
        surf, kind = synth.surface_small(), "small"
    elif name == "quintic":
        surf, kind = synth.surface_quintic(), "small"
    else:
        raise SystemExit(f"unknown workload {name}")
    s = gn.Surface(surf)
    uv, off = synth.query_params(n, seed, kind)
    E = s.eval(torch.as_tensor(uv, device="cuda"), gn.S | gn.SU | gn.SV).cpu().numpy()
    P = synth.form_queries(E[0:3].T, E[3:6].T, E[6:9].T, off)
    return surf, s, uv, P


def fp64_peak_tflops(torch):
    """FP64 FMA throughput of this GPU, measured with the library-independent probe kernel
    shipped in the package (independent FMA chains; 2 flops per FMA)."""
    gn = load_pkg()
    import ctypes as C
    L = gn.lib()
    if not hasattr(L, "nurbs_probe_fp_peak"):
        return None, None
    f = L.nurbs_probe_fp_peak
    f.restype = C.c_int
    f.argtypes = [C.c_int, C.POINTER(C.c_double), C.c_void_p]
    out = C.c_double()
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    best64 = best32 = 0.0
    for _ in range(3):
        if f(64, C.byref(out), st) == 0:
            best64 = max(best64, out.value)
        if f(32, C.byref(out), st) == 0:
            best32 = max(best32, out.value)
    return best64 or None, best32 or None


def run_ours(a):
    import torch
    import torch.distributed as dist
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    gn = load_pkg()
    n = a.queries or ((1 << 24) if a.workload == "quintic" else (1 << 20))
    surf, s, uv_true, P = make_workload(gn, torch, a.workload, n, 1000 + rank)
    Pd = torch.as_tensor(P, device="cuda")
    uv = torch.empty((n, 2), dtype=torch.float64, device="cuda")
    st = torch.empty(n, dtype=torch.int32, device="cuda")
    res = torch.empty(n, dtype=torch.float64, device="cuda")
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    timed = event_timer(torch, flush)

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()

    inv_mixed = lambda: s.invert(Pd, gn.PREC_MIXED, out=(uv, st, res))
    inv_fp64 = lambda: s.invert(Pd, gn.PREC_FP64, out=(uv, st, res))
    # pinned host buffers for the end-to-end leg
    Ph = torch.from_numpy(P).pin_memory().numpy()
    huv = torch.empty((n, 2), dtype=torch.float64).pin_memory().numpy()
    hst = torch.empty(n, dtype=torch.int32).pin_memory().numpy()
    hres = torch.empty(n, dtype=torch.float64).pin_memory().numpy()
    inv_host = lambda: s.invert_host(Ph, gn.PREC_MIXED, out=(huv, hst, hres))

    for _ in range(a.warmup):
        inv_mixed()
        inv_fp64()
    torch.cuda.synchronize()
    # accuracy of this run's mixed results against the generating parameters
    inv_mixed()
    g_uv, g_st, res_mixed = uv.cpu().numpy(), st.cpu().numpy(), res.cpu().numpy()
    found = g_st == 0
    err = np.abs(g_uv - uv_true).max(1)
    acc = {"found_frac": float(found.mean()),
           "uv_err_vs_truth_p50": float(np.median(err[found])) if found.any() else None,
           "uv_err_vs_truth_p99": float(np.percentile(err[found], 99)) if found.any() else None,
           "frac_found_within_1e9_of_truth": float((err[found] <= 1e-9).mean()) if found.any() else None}

    clocks = Clocks(local)
    barrier()
    t_mixed = timed(inv_mixed, a.steps)
    barrier()
    t_fp64 = timed(inv_fp64, max(3, a.steps // 4))
    barrier()
    clk = clocks.stop()
    # e2e through the C-ABI with host buffers
    for _ in range(2):
        inv_host()
    barrier()
    t_e2e = []
    for k in range(a.steps):
        flush.fill_(float(k))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        inv_host()
        t_e2e.append((time.perf_counter() - t0) * 1e3)
    barrier()

    agg = lambda ts: mean_step_ms_over_ranks(ts, world, "cuda")

    ms_mixed, ms_fp64, ms_e2e = agg(t_mixed), agg(t_fp64), agg(t_e2e)
    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return
    peak64, peak32 = fp64_peak_tflops(torch)
    k1 = surf["p"] + 1
    k2 = surf["q"] + 1
    # nominal algorithmic work per query (p=q=3: ~2.6 kflop): (1+I) evaluations of S,Su,Sv
    # plus I 2x2 solves, I = 6 iterations
    I = 6
    flop_q = (1 + I) * 2 * (4 * k1 * k2 * 2 + 4 * k1 * 3) + I * 30
    qps = n * world / (ms_mixed / 1e3)
    achieved = flop_q * n / (ms_mixed / 1e3) / 1e12
    line = {
        "metric": METRIC,
        "value": qps,
        "unit": "inversions/s",
        "n_gpus": world,
        "steps": a.steps,
        "warmup": a.warmup,
        "ms_per_step": ms_mixed,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "fp32+fp64 (mixed)",
        "data": "synthetic (seeded)",
        "config": {"workload": workload_label(a.workload, n),
                   "queries_per_step": n, "precision": "mixed", "l2": "flushed (512 MB write) before each step",
                   "parallelism": f"replicas x{world}"},
        "fp64_value": n * world / (ms_fp64 / 1e3),
        "fp64_ms_per_step": ms_fp64,
        "mixed_vs_fp64": ms_fp64 / ms_mixed,
        "accuracy": acc,
        "e2e": {"value": n * world / (ms_e2e / 1e3), "unit": "inversions/s", "h2d_bytes_per_step": n * 24,
                "d2h_bytes_per_step": n * (16 + 4 + 8), "ms_per_step": ms_e2e,
                "step_ms": [round(t, 3) for t in t_e2e]},
        "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak64, "unit": "TFLOP/s",
                     "frac": (achieved / peak64) if peak64 else None,
                     "traffic": TRAFFIC_PER_UNIT[a.workload] * n if a.workload in TRAFFIC_PER_UNIT else None,
                     "traffic_unit": "bytes per launch",
                     "peak_source": "FP64 FMA probe kernel run in this process",
                     "fp32_peak": peak32, "flop_per_query_nominal": flop_q},
        "clocks": clk,
        "gpu_launches": a.steps,
    }
    work = work_counts(gn, s, Pd)
    if work:
        # the FP32 pipe with the work the kernel actually did: FP32 seed iterations x flops each
        fi = flop_iter32(surf["p"], surf["q"])
        f32 = work["seed_iterations"] * fi
        line["roofline"]["fp32_actual"] = {
            "fp32_iterations_per_query": work["seed_iterations"] / n,
            "final_fp64_polishes_per_query": work["final_polishes"] / n,
            "flop_per_fp32_iteration": fi,
            "achieved": f32 / (ms_mixed / 1e3) / 1e12, "peak": peak32, "unit": "TFLOP/s",
            "frac": f32 / (ms_mixed / 1e3) / 1e12 / peak32 if peak32 else None}
    if not a.no_cpu:
        line["cpu_baseline"], line["parity_sample"] = cpu_baseline(surf, P, a.cpu_sample, g_uv, g_st, res_mixed)
    if world == 1 and not a.headline_only and a.workload == "large":
        for name, fn in (("batched", batched_record), ("quintic", quintic_record), ("eval_large", eval_record),
                         ("project", project_record), ("quadtree", quadtree_record), ("pcurve", pcurve_record),
                         ("serving", serving_record)):
            t0 = time.perf_counter()
            try:
                line[name] = fn(a, compact=True)
            except Exception as e:  # a failed sub-record is reported, the headline stands
                line[name] = {"error": f"{type(e).__name__}: {e}"}
            line[name]["wall_s"] = round(time.perf_counter() - t0, 1)
            print(f"[bench] {name} {line[name]['wall_s']} s", file=sys.stderr, flush=True)
    print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


def flop_iter32(p, q):
    """Algorithmic flops of one FP32 seed iteration: S..Svv (the evaluation count of the
    measurement section: 2 [4 k1 k2 n_v + 4 k1 n_out] with n_v = 3, n_out = 6), the quotient rule
    (~12 per output component) and the 2x2 Newton solve (~30)."""
    k1, k2 = p + 1, q + 1
    return 2 * (4 * k1 * k2 * 3 + 4 * k1 * 6) + 12 * 18 + 30


def work_counts(gn, s, Pd):
    """Seed iterations of one mixed inversion of Pd, counted by the library's counting variant
    of the kernel (untimed)."""
    try:
        return s.count_work(Pd, gn.PREC_MIXED)
    except (AttributeError, gn.NurbsError):
        return None


def batched_record(a, compact=False):
    """Batched uneven workload: 4096 surfaces (p,q in {2,3,5}, nets 4..48), per-surface query
    counts log-uniform in 16..65536, queries S(u,v) + N(0,1e-3) n; one persistent launch per
    step, replayed from a CUDA graph, launch configuration picked by the pool's autotuner."""
    import torch
    gn = load_pkg()
    from gpu_nurbs_gb300 import synth
    t_start = time.perf_counter()
    steps = 6 if compact else a.steps

    def phase(msg):
        print(f"[batched] {time.perf_counter() - t_start:8.2f}s {msg}", file=sys.stderr, flush=True)

    surfs, nq = synth.batched_surfaces(a.surfaces)
    phase("surfaces generated")
    t0 = time.perf_counter()
    budget = int(sum(gn.surface_bytes(sf) for sf in surfs) * 1.05) + (512 << 20)
    pool = gn.Pool(budget, max_surfaces=len(surfs))
    ids = pool.add(surfs)
    torch.cuda.synchronize()
    t_upload = time.perf_counter() - t0
    phase(f"pool filled ({t_upload:.2f}s)")
    offsets = np.concatenate([[0], np.cumsum(nq)]).astype(np.int64)
    n = int(offsets[-1])
    batch = gn.Batch(ids, offsets)
    r = synth.Rng(synth.SEED_BASE + 2 + 1000)
    uv_true = np.stack([r.uniform(n), r.uniform(n)], 1)
    off = torch.as_tensor(r.normal(n, 1e-3), device="cuda")
    E = pool.eval(batch, torch.as_tensor(uv_true, device="cuda"), gn.S | gn.SU | gn.SV)
    nrm = torch.linalg.cross(E[3:6].T, E[6:9].T, dim=1)
    nrm = nrm / nrm.norm(dim=1, keepdim=True)
    Pd = (E[0:3].T + off[:, None] * nrm).contiguous()
    del E, nrm
    torch.cuda.synchronize()
    phase(f"{n} queries formed")
    out = (torch.empty((n, 2), dtype=torch.float64, device="cuda"), torch.empty(n, dtype=torch.int32, device="cuda"),
           torch.empty(n, dtype=torch.float64, device="cuda"))
    cache = os.path.join(os.path.expanduser("~"), ".cache", "gpu_nurbs_gb300", "autotune.txt")
    os.makedirs(os.path.dirname(cache), exist_ok=True)
    tile, ctas, tune_ms = pool.autotune(batch, Pd, out, gn.PREC_MIXED, max_queries=a.tune_queries, cache_path=cache)
    phase(f"autotuned: tile {tile}, ctas/SM {ctas}, {tune_ms:.2f} ms")
    g_mixed = pool.graph(batch, Pd, out, gn.PREC_MIXED)
    g_fp64 = pool.graph(batch, Pd, out, gn.PREC_FP64)
    phase("graphs captured")
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    timed = event_timer(torch, flush)

    for _ in range(3 if compact else max(3, a.warmup)):
        g_mixed.launch()
    torch.cuda.synchronize()
    phase("mixed warm-up done")
    # end to end (pinned host queries in, results out, every step) right after the device-timed
    # steps, before the long FP64 steps heat the GPU
    Ph = Pd.cpu().pin_memory()
    hout = [torch.empty(x.shape, dtype=x.dtype).pin_memory() for x in out]
    clocks = Clocks(0)
    t_mixed = timed(g_mixed.launch, steps)
    phase("mixed timed")
    t_e2e, parts = [], []
    for k in range(1 + max(3, steps // 2)):   # the first pass (untimed) maps the pinned buffers
        flush.fill_(float(k))
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ev[0].record(stream)
        Pd.copy_(Ph, non_blocking=True)
        ev[1].record(stream)
        g_mixed.launch()
        ev[2].record(stream)
        for h, d in zip(hout, out):
            h.copy_(d, non_blocking=True)
        ev[3].record(stream)
        torch.cuda.synchronize()
        if k > 0:
            t_e2e.append((time.perf_counter() - t0) * 1e3)
            parts.append([round(ev[i].elapsed_time(ev[i + 1]), 2) for i in range(3)])
    phase("e2e timed")
    g_fp64.launch()
    torch.cuda.synchronize()
    phase("fp64 warm-up done")
    t_fp64 = timed(g_fp64.launch, max(2, steps // 8))
    phase("fp64 timed")
    clk = clocks.stop()
    g_mixed.launch()
    torch.cuda.synchronize()
    g_uv, g_st, g_res = (x.cpu().numpy() for x in out)
    phase("results copied")
    ms_mixed = sum(t_mixed) / len(t_mixed)
    ms_fp64 = sum(t_fp64) / len(t_fp64)
    ms_e2e = sum(t_e2e) / len(t_e2e)
    found = g_st == 0
    err = np.abs(g_uv - uv_true).max(1)
    rec = {
        "metric": METRIC, "value": n / (ms_mixed / 1e3), "unit": "inversions/s", "n_gpus": 1, "steps": steps,
        "warmup": 3, "ms_per_step": ms_mixed, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32+fp64 (mixed)", "data": "synthetic (seeded)",
        "config": {"workload": f"batched: {len(surfs)} surfaces, p,q in {{2,3,5}}, nets 4..48, {n} queries "
                               "(log-uniform 16..65536 per surface), offsets N(0,1e-3)",
                   "queries_per_step": n, "precision": "mixed", "launch": "one persistent kernel per step, CUDA graph",
                   "autotuned": {"tile_queries": tile, "ctas_per_sm": ctas, "tune_ms": tune_ms},
                   "l2": "flushed (512 MB write) before each step", "parallelism": "replicas x1"},
        "fp64_value": n / (ms_fp64 / 1e3), "fp64_ms_per_step": ms_fp64, "mixed_vs_fp64": ms_fp64 / ms_mixed,
        "upload_convert_s": t_upload,
        "accuracy": {"found_frac": float(found.mean()),
                     "frac_found_within_1e9_of_truth": float((err[found] <= 1e-9).mean()) if found.any() else None},
        "e2e": {"value": n / (ms_e2e / 1e3), "unit": "inversions/s", "h2d_bytes_per_step": n * 24,
                "d2h_bytes_per_step": n * 28, "ms_per_step": ms_e2e,
                "step_ms": [round(t, 3) for t in t_e2e], "h2d_kernel_d2h_ms": parts},
        "clocks": clk, "gpu_launches": steps,
    }
    if not a.no_cpu:
        # oracle on the first surfaces' queries (a bounded sample), checking this run's results
        P_h = Ph.numpy()
        tot, dt, done, k = dict(), 0.0, 0, 0
        while done < a.cpu_sample and k < len(surfs):
            sl = slice(int(offsets[k]), int(min(offsets[k + 1], offsets[k] + a.cpu_sample - done)))
            c, t = oracle_parity_sample(surfs[k], P_h[sl], g_uv[sl], g_st[sl], g_res[sl])
            merge_parity(tot, c)
            dt += t
            done += sl.stop - sl.start
            k += 1
        tot["p99_uv_err_same_max_over_surfaces"] = max(tot.pop("p99_uv_err_same_per_surface", [0.0]))
        rec["cpu_baseline"] = {"value": done / dt, "unit": "inversions/s", "cores": host_cores(), "kind": "port",
                               "sample": f"{done} queries of the first {k} surfaces, the oracle's inversion"}
        rec["parity_sample"] = tot
    if compact:
        keep = ("value", "unit", "ms_per_step", "fp64_value", "mixed_vs_fp64", "e2e", "config", "clocks",
                "parity_sample", "accuracy", "steps")
        rec = {k: rec[k] for k in keep if k in rec}
        rec["e2e"] = {k: rec["e2e"][k] for k in ("value", "ms_per_step", "h2d_bytes_per_step", "d2h_bytes_per_step")}
    return rec


def run_batched(a):
    print(json.dumps(batched_record(a)))


def quintic_record(a, compact=False):
    """Degree-5 256x256 surface, 2^24 queries S(u,v) + N(0,1e-3) n: mixed and FP64 inversions/s,
    and the per-query parameter error against the oracle (max, p99) on a bounded sample."""
    import torch
    gn = load_pkg()
    n = 1 << 24
    steps = 5 if compact else a.steps
    surf, s, uv_true, P = make_workload(gn, torch, "quintic", n, 1000)
    Pd = torch.as_tensor(P, device="cuda")
    out = (torch.empty((n, 2), dtype=torch.float64, device="cuda"), torch.empty(n, dtype=torch.int32, device="cuda"),
           torch.empty(n, dtype=torch.float64, device="cuda"))
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    timed = event_timer(torch, flush)
    inv_mixed = lambda: s.invert(Pd, gn.PREC_MIXED, out=out)
    inv_fp64 = lambda: s.invert(Pd, gn.PREC_FP64, out=out)
    for _ in range(3):
        inv_mixed()
    inv_fp64()
    torch.cuda.synchronize()
    clocks = Clocks(0)
    t_mixed = timed(inv_mixed, steps)
    t_fp64 = timed(inv_fp64, 2)
    clk = clocks.stop()
    inv_mixed()
    g_uv, g_st, g_res = (x.cpu().numpy() for x in out)
    ms_mixed, ms_fp64 = sum(t_mixed) / len(t_mixed), sum(t_fp64) / len(t_fp64)
    rec = {"value": n / (ms_mixed / 1e3), "unit": "inversions/s", "ms_per_step": ms_mixed, "steps": steps,
           "fp64_value": n / (ms_fp64 / 1e3), "fp64_ms_per_step": ms_fp64, "mixed_vs_fp64": ms_fp64 / ms_mixed,
           "config": {"workload": workload_label("quintic", n), "l2": "flushed (512 MB write) before each step"},
           "clocks": clk}
    if not a.no_cpu:
        m = min(a.cpu_sample // 2, n)
        import oracle as O
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        from parity import eval_errors
        # residuals can differ by as much as the two FP64 evaluations of S do at degree 5
        ev = s.eval(torch.as_tensor(uv_true[:m], device="cuda"), gn.S).cpu().numpy()
        res_abs = max(1e-14, 4 * eval_errors(ev, O.OracleSurface(surf).eval(uv_true[:m], 1))[0])
        c, dt = oracle_parity_sample(surf, P[:m], g_uv[:m], g_st[:m], g_res[:m], res_abs=res_abs)
        rec["parity_sample"] = c
        rec["cpu_baseline"] = {"value": m / dt, "unit": "inversions/s", "cores": host_cores(), "kind": "port",
                               "sample": f"{m} queries of the workload, the oracle's inversion"}
    return rec


def projection_queries(surf, s, gn, torch, n, seed):
    """Projection workload: 80 % of the points off the surface along its normal by up to +-10 %
    of the control net's extent, 20 % anywhere in a box six extents wide around it."""
    r = np.random.default_rng(seed)
    nf = n // 5
    uv = r.random((n - nf, 2))
    E = s.eval(torch.as_tensor(uv, device="cuda"), gn.S | gn.SU | gn.SV).cpu().numpy()
    N = np.cross(E[3:6].T, E[6:9].T)
    N /= np.linalg.norm(N, axis=1)[:, None]
    cps = np.asarray(surf["cps"]).reshape(-1, 3)
    ext = np.ptp(cps, 0).max()
    near = E[0:3].T + N * ((r.random(n - nf) - 0.5) * 0.2 * ext)[:, None]
    far = cps.mean(0) + (r.random((nf, 3)) - 0.5) * 6 * ext
    return np.ascontiguousarray(np.concatenate([near, far]))


def project_record(a, compact=False):
    """Point projection (nurbs_project, mixed and FP64) on the 64x64 bicubic surface: 2^20 points,
    80 % within 10 % of the extent of the surface, 20 % far from it; projections/s, with parity of
    the mixed results and the oracle's CPU time on a bounded sample."""
    import torch
    gn = load_pkg()
    from gpu_nurbs_gb300 import synth
    n = (1 << 20) if compact or not a.queries else a.queries
    steps = 5 if compact else a.steps
    surf = synth.surface_large()
    s = gn.Surface(surf)
    P = projection_queries(surf, s, gn, torch, n, 2024)
    Pd = torch.as_tensor(P, device="cuda")
    out = (torch.empty((n, 2), dtype=torch.float64, device="cuda"), torch.empty(n, dtype=torch.int32, device="cuda"),
           torch.empty(n, dtype=torch.float64, device="cuda"))
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    timed = event_timer(torch, flush)
    run = lambda: s.project(Pd, gn.PREC_MIXED, out=out)
    run64 = lambda: s.project(Pd, gn.PREC_FP64, out=out)
    for _ in range(3):
        run()
    run64()
    torch.cuda.synchronize()
    clocks = Clocks(0)
    t = timed(run, steps)
    t64 = timed(run64, max(2, steps // 2))
    clk = clocks.stop()
    run()
    g_uv, g_st, g_res = (x.cpu().numpy() for x in out)
    ms, ms64 = sum(t) / len(t), sum(t64) / len(t64)
    rec = {"value": n / (ms / 1e3), "unit": "projections/s", "ms_per_step": ms, "steps": steps, "dtype": "f32+f64",
           "fp64_value": n / (ms64 / 1e3), "fp64_ms_per_step": ms64, "mixed_vs_fp64": ms64 / ms,
           "config": {"workload": f"project-64x64-bicubic-{n} points (80 % within 10 % of the extent, 20 % far)",
                      "l2": "flushed (512 MB write) before each step"},
           "found_frac": float(np.mean(g_st <= 1)), "clocks": clk}
    if not a.no_cpu:
        import oracle as O
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        from parity import project_parity
        m = min(a.cpu_sample // 2, n)
        idx = np.linspace(0, n - 1, m).astype(np.int64)  # near and far points both
        o = O.OracleSurface(surf)
        o.cones()
        t0 = time.perf_counter()
        o.project(P[idx], threads=host_cores())
        dt = time.perf_counter() - t0
        c = project_parity(o, P[idx], g_uv[idx], g_st[idx], g_res[idx])
        rec["parity_sample"] = {k: v for k, v in c.items() if k != "fail_idx"}
        rec["cpu_baseline"] = {"value": m / dt, "unit": "projections/s", "cores": host_cores(), "kind": "port",
                               "sample": f"{m} points of the workload, evenly spaced, the oracle's projection"}
    return rec


def quadtree_record(a, compact=False):
    """Adaptive quadtree inversion (nurbs_invert_quadtree, mixed and FP64; the reference's first
    inversion with max_edge 1e-4 as its driver calls it) of 2^20 points on the 64x64 bicubic
    surface; no tree build.  Inversions/s, parity of the mixed results with the oracle on a
    bounded sample and its CPU time."""
    import torch
    gn = load_pkg()
    from gpu_nurbs_gb300 import synth
    n = (1 << 20) if compact or not a.queries else a.queries
    max_edge = 1e-4
    steps = 5 if compact else a.steps
    surf = synth.surface_large()
    s = gn.Surface(surf)
    uv0 = np.random.default_rng(99).random((n, 2))
    P = np.ascontiguousarray(s.eval(torch.as_tensor(uv0, device="cuda"), gn.S).cpu().numpy().T)
    Pd = torch.as_tensor(P, device="cuda")
    out = (torch.empty((n, 2), dtype=torch.float64, device="cuda"), torch.empty(n, dtype=torch.int32, device="cuda"),
           torch.empty(n, dtype=torch.float64, device="cuda"))
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    timed = event_timer(torch, flush)
    run = lambda: s.invert_quadtree(Pd, max_edge, gn.PREC_MIXED, out=out)
    run64 = lambda: s.invert_quadtree(Pd, max_edge, gn.PREC_FP64, out=out)
    for _ in range(3):
        run()
    run64()
    torch.cuda.synchronize()
    clocks = Clocks(0)
    t = timed(run, steps)
    t64 = timed(run64, max(2, steps // 2))
    clk = clocks.stop()
    run()
    g_uv, g_st, g_res = (x.cpu().numpy() for x in out)
    ms, ms64 = sum(t) / len(t), sum(t64) / len(t64)
    rec = {"value": n / (ms / 1e3), "unit": "inversions/s", "ms_per_step": ms, "steps": steps, "dtype": "f32+f64",
           "fp64_value": n / (ms64 / 1e3), "fp64_ms_per_step": ms64, "mixed_vs_fp64": ms64 / ms,
           "config": {"workload": f"quadtree-64x64-bicubic-{n} on-surface points, max_edge 1e-4",
                      "l2": "flushed (512 MB write) before each step"},
           "found_frac": float(np.mean(g_st <= 1)), "max_uv_err": float(np.abs(g_uv - uv0)[g_st <= 1].max()),
           "clocks": clk}
    if not a.no_cpu:
        import oracle as O
        m = min(a.cpu_sample, n)
        o = O.OracleSurface(surf)
        t0 = time.perf_counter()
        ouv, ost, ores, _ = o.invert_quadtree(P[:m], max_edge, threads=host_cores())
        dt = time.perf_counter() - t0
        f = ost <= 1
        rec["parity_sample"] = {"n": m, "status_equal": int(np.sum(g_st[:m] == ost)),
                                "max_uv_diff": float(np.abs(g_uv[:m][f] - ouv[f]).max()) if f.any() else 0.0}
        rec["cpu_baseline"] = {"value": m / dt, "unit": "inversions/s", "cores": host_cores(), "kind": "port",
                               "sample": f"first {m} points of the workload, the oracle's quadtree inversion"}
    return rec


def pcurve_record(a, compact=False):
    """p-curves (nurbs_pcurve, mixed and FP64): 2^20 ordered samples of closed curves on the 64x64
    bicubic surface (256 loops of 4096 samples, radii and centres seeded), each sample 1e-3 off the
    surface along its normal.  Samples/s, parity with the oracle's p-curve on a bounded sample
    (status, flags, parameters to 1e-9) and its CPU time."""
    import torch
    gn = load_pkg()
    from gpu_nurbs_gb300 import synth
    n_loops, per = (256, 4096) if compact or not a.queries else (max(1, a.queries // 4096), 4096)
    n = n_loops * per
    steps = 5 if compact else a.steps
    surf = synth.surface_large()
    s = gn.Surface(surf)
    r = np.random.default_rng(77)
    t = np.linspace(0.0, 1.0, per)
    cu, cv = 0.25 + 0.5 * r.random(n_loops), 0.25 + 0.5 * r.random(n_loops)
    ru, rv = 0.05 + 0.15 * r.random(n_loops), 0.05 + 0.15 * r.random(n_loops)
    uv = np.stack([(cu[:, None] + ru[:, None] * np.cos(2 * np.pi * t)).ravel(),
                   (cv[:, None] + rv[:, None] * np.sin(2 * np.pi * t)).ravel()], 1)
    E = s.eval(torch.as_tensor(uv, device="cuda"), gn.S | gn.SU | gn.SV).cpu().numpy()
    N = np.cross(E[3:6].T, E[6:9].T)
    N /= np.linalg.norm(N, axis=1)[:, None]
    C = np.ascontiguousarray(E[0:3].T + 1e-3 * N)
    Cd = torch.as_tensor(C, device="cuda")
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    timed = event_timer(torch, flush)
    run = lambda: s.pcurve(Cd, gn.PREC_MIXED)
    run64 = lambda: s.pcurve(Cd, gn.PREC_FP64)
    for _ in range(3):
        run()
    run64()
    torch.cuda.synchronize()
    clocks = Clocks(0)
    tm = timed(run, steps)
    t64 = timed(run64, max(2, steps // 2))
    clk = clocks.stop()
    g_uv, g_st, g_res, g_fl = (x.cpu().numpy() for x in run())
    ms, ms64 = sum(tm) / len(tm), sum(t64) / len(t64)
    rec = {"value": n / (ms / 1e3), "unit": "samples/s", "ms_per_step": ms, "steps": steps, "dtype": "f32+f64",
           "fp64_value": n / (ms64 / 1e3), "fp64_ms_per_step": ms64, "mixed_vs_fp64": ms64 / ms,
           "config": {"workload": f"pcurve-64x64-bicubic: {n_loops} closed loops x {per} samples, 1e-3 off the surface",
                      "l2": "flushed (512 MB write) before each step"},
           "found_frac": float(np.mean(g_st <= 1)), "flagged_frac": float(np.mean(g_fl != 0)),
           "max_uv_err_vs_curve": float(np.abs(g_uv - uv)[g_st == 0].max()), "clocks": clk}
    if not a.no_cpu:
        import oracle as O
        m = min(a.cpu_sample // per, n_loops) * per
        o = O.OracleSurface(surf)
        t0 = time.perf_counter()
        ouv, ost, ores, ofl = o.pcurve(C[:m], threads=host_cores())
        dt = time.perf_counter() - t0
        f = (ost <= 1) & (g_st[:m] <= 1)
        rec["parity_sample"] = {"n": m, "status_equal": int(np.sum(g_st[:m] == ost)),
                                "flags_equal": int(np.sum(g_fl[:m] == ofl)),
                                "max_uv_diff": float(np.abs(g_uv[:m][f] - ouv[f]).max()) if f.any() else 0.0}
        rec["cpu_baseline"] = {"value": m / dt, "unit": "samples/s", "cores": host_cores(), "kind": "port",
                               "sample": f"the first {m // per} loops of the workload, the oracle's p-curve"}
    return rec


def run_pcurve(a):
    print(json.dumps(pcurve_record(a)))


def run_quadtree(a):
    print(json.dumps(quadtree_record(a)))


def run_project(a):
    print(json.dumps(project_record(a)))


def measured_hbm_gbs():
    """HBM copy bandwidth of the GB300s (the measured-peaks file), else the fallback."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured copy bandwidth of this pool's GB300"
    except (OSError, ValueError, KeyError):
        return 6800.0, "fallback 6.8 TB/s"


def eval_record(a, compact=False, which="eval-large"):
    """Batched evaluation throughput: 'eval-small' = 2^20 (u,v) on the 8x8 bicubic surface with
    S, Su, Sv; 'eval-large' = 2^26 (u,v) on the 64x64 bicubic surface with S..Svv.  FP64 and FP32."""
    import torch
    gn = load_pkg()
    from gpu_nurbs_gb300 import synth
    small = which == "eval-small"
    surf = synth.surface_small() if small else synth.surface_large()
    mask = 7 if small else 63
    n = ((1 << 20) if small else (1 << 26)) if compact or not a.queries else a.queries
    steps = 8 if compact else a.steps
    s = gn.Surface(surf)
    r = synth.Rng(synth.SEED_BASE + 77)
    uv = torch.as_tensor(np.stack([r.uniform(n), r.uniform(n)], 1), device="cuda")
    uv32 = uv.float()
    nb = bin(mask).count("1")
    out = torch.empty((3 * nb, n), dtype=torch.float64, device="cuda")
    out32 = torch.empty((3 * nb, n), dtype=torch.float32, device="cuda")
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    timed = event_timer(torch, flush)
    L = gn.lib()

    def ev64():
        gn.check(L.nurbs_eval(s.h, uv.data_ptr(), n, mask, out.data_ptr(), gn.PREC_FP64, gn._stream()), "eval")

    def ev32():
        gn.check(L.nurbs_eval_f32(s.h, uv32.data_ptr(), n, mask, out32.data_ptr(), gn._stream()), "eval")

    # the same count of points on a row-major parameter grid (a tessellation: the 32 points of a
    # warp lie in one or two spans, so the coefficient gathers are broadcasts)
    side = int(round(n ** 0.5))
    g = (torch.arange(side, device="cuda", dtype=torch.float32) + 0.5) / side
    uvg = torch.stack([g.repeat_interleave(side), g.repeat(side)], 1).contiguous()
    ng = side * side

    def ev32g():
        gn.check(L.nurbs_eval_f32(s.h, uvg.data_ptr(), ng, mask, out32.data_ptr(), gn._stream()), "eval")

    # third order (Suuu..Svvv) and the normal with its second derivatives, FP64, on a quarter of
    # the points (their outputs share the FP64 output buffer)
    n3 = n // 4

    def ev3():
        gn.check(L.nurbs_eval(s.h, uv.data_ptr(), n3, 0x3C0, out.data_ptr(), gn.PREC_FP64, gn._stream()), "eval")

    def evn():
        gn.check(L.nurbs_eval_normal(s.h, uv.data_ptr(), n3, 0x39, out.data_ptr(), gn._stream()), "eval")

    for _ in range(3):
        ev64()
        ev32()
        ev32g()
    torch.cuda.synchronize()
    clocks = Clocks(0)
    t64 = timed(ev64, steps)
    t32 = timed(ev32, steps)
    t32g = timed(ev32g, steps)
    t3 = timed(ev3, steps) if nb >= 4 else [float("nan")]
    tn = timed(evn, steps) if nb >= 4 else [float("nan")]
    clk = clocks.stop()
    ms64, ms32 = sum(t64) / len(t64), sum(t32) / len(t32)
    ms32g = sum(t32g) / len(t32g)
    peak64, peak32 = fp64_peak_tflops(torch)
    hbm, hbm_src = measured_hbm_gbs()
    k1, k2 = surf["p"] + 1, surf["q"] + 1
    nv_, nout = (2, 3) if small else (3, 6)
    flop = 2 * (4 * k1 * k2 * nv_ + 4 * k1 * nout)       # algorithmic flops per point
    bytes64, bytes32 = 16 + 24 * nout, 8 + 12 * nout
    ach64 = flop * n / (ms64 / 1e3) / 1e12
    gbs32 = bytes32 * n / (ms32 / 1e3) / 1e9
    return {
        "metric": "evaluations/s (FP64, " + ("S,Su,Sv" if small else "S..Svv") + ")", "value": n / (ms64 / 1e3),
        "unit": "points/s", "n_gpus": 1, "steps": steps, "warmup": 3, "ms_per_step": ms64,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp64", "data": "synthetic (seeded)",
        "config": {"workload": which, "points_per_step": n, "outputs": "SoA",
                   "l2": "flushed (512 MB write) before each step"},
        "fp32_value": n / (ms32 / 1e3), "fp32_ms_per_step": ms32,
        "roofline": {"bound": "fp64", "achieved": ach64, "peak": peak64, "unit": "TFLOP/s",
                     "frac": ach64 / peak64 if peak64 else None,
                     "traffic": TRAFFIC_PER_UNIT[which] * n if which in TRAFFIC_PER_UNIT else None,
                     "traffic_unit": "bytes per launch",
                     "flop_per_point": flop, "bytes_per_point_fp64": bytes64, "bytes_per_point_fp32": bytes32,
                     "hbm_achieved_gbs": bytes64 * n / (ms64 / 1e3) / 1e9,
                     "fp32": {"bound": "hbm", "achieved": gbs32, "peak": hbm, "unit": "GB/s",
                              "frac": gbs32 / hbm if hbm else None, "peak_source": hbm_src,
                              "note": "random (u,v): bound by the L1 wavefronts of per-lane span gathers"},
                     "fp64_third_order": {"points_per_step": n3, "value": n3 / (sum(t3) / len(t3) / 1e3),
                                          "outputs": "Suuu, Suuv, Suvv, Svvv"},
                     "fp64_normals": {"points_per_step": n3, "value": n3 / (sum(tn) / len(tn) / 1e3),
                                      "outputs": "N, Nuu, Nuv, Nvv"},
                     "fp32_grid": {"points_per_step": ng, "value": ng / (ms32g / 1e3), "ms_per_step": ms32g,
                                   "bound": "hbm", "achieved": bytes32 * ng / (ms32g / 1e3) / 1e9, "peak": hbm,
                                   "unit": "GB/s", "frac": bytes32 * ng / (ms32g / 1e3) / 1e9 / hbm if hbm else None,
                                   "uv": "row-major parameter grid (tessellation order)"},
                     "fp32_achieved_tflops": flop * n / (ms32 / 1e3) / 1e12, "fp32_peak": peak32},
        "clocks": clk, "gpu_launches": 5 * steps,
    }


def run_eval(a):
    print(json.dumps(eval_record(a, which=a.workload)))


def serving_record(a, compact=False):
    """Serving: a pool of 10^4 surfaces (generated as the batched workload) under a 20 GB budget;
    Poisson request arrivals swept over rates; each request targets a surface drawn Zipf(1.1)
    with 1..4096 queries (log-uniform), 10% of requests upload a new surface.  Requests are
    replayed by the library's native load generator against the continuous-batching server;
    latency counts from the scheduled arrival.  The headline is p99 at half of the peak rate."""
    import torch
    gn = load_pkg()
    from gpu_nurbs_gb300 import synth
    t_start = time.perf_counter()
    serve_seconds = min(a.serve_seconds, 0.5) if compact else a.serve_seconds
    rates = [1e4, 1e5, 3e5, 1e6] if compact else [float(x) for x in a.rates.split(",")]

    def phase(msg):
        print(f"[serving] {time.perf_counter() - t_start:8.2f}s {msg}", file=sys.stderr, flush=True)

    npool = a.surfaces if a.surfaces != 4096 else 10000
    surfs, _ = synth.batched_surfaces(npool, seed=synth.SEED_BASE + 4)
    pool = gn.Pool(20 << 30, max_surfaces=npool + 200000)
    ids = pool.add(surfs)
    pool.set_config(a.serve_chunk, 4)
    phase(f"pool of {npool} surfaces, {pool.info().used_bytes / 2**30:.2f} GiB")
    r = synth.Rng(synth.SEED_BASE + 4 + 1)
    # Zipf(1.1) over the pool (ranks shuffled so popularity is not tied to generation order)
    ranks = np.arange(1, npool + 1, dtype=np.float64)
    pz = ranks ** -1.1
    pz /= pz.sum()
    perm = r.g.permutation(npool)
    upload_bank = synth.batched_surfaces(2000, seed=synth.SEED_BASE + 4 + 2)[0]

    def trace(rate, nreq):
        kind = (r.uniform(nreq) < a.upload_frac).astype(np.int32)
        sizes = np.where(kind == 0, np.exp(r.uniform(nreq, 0.0, np.log(4096.0))).astype(np.int64), 0)
        sizes = np.maximum(sizes, kind == 0)
        which = perm[r.g.choice(npool, size=nreq, p=pz)]
        qoff = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
        nq = int(qoff[-1])
        # queries S(u,v) + N(0,1e-3) n on each request's surface, formed on the GPU
        uvq = torch.as_tensor(np.stack([r.uniform(nq), r.uniform(nq)], 1), device="cuda")
        req_ids = ids[which].astype(np.int32)
        # upload requests own empty query ranges
        E = pool.eval(gn.Batch(req_ids, qoff), uvq, gn.S | gn.SU | gn.SV)
        nrm = torch.linalg.cross(E[3:6].T, E[6:9].T, dim=1)
        nrm = nrm / nrm.norm(dim=1, keepdim=True)
        off = torch.as_tensor(r.normal(nq, 1e-3), device="cuda")
        P = (E[0:3].T + off[:, None] * nrm).cpu().numpy()
        arrival = np.cumsum(r.g.exponential(1e6 / rate, nreq))
        uidx = np.cumsum(kind) - 1
        uidx = np.where(kind == 1, uidx % len(upload_bank), 0).astype(np.int32)
        return arrival, kind, req_ids, qoff, P, uidx, sizes

    def serve(rate, nreq, precision):
        arrival, kind, req_ids, qoff, P, uidx, sizes = trace(rate, nreq)
        srv = gn.Server(pool, slots=a.slots, max_batch_queries=a.max_batch_queries, max_batch_requests=4096,
                        precision=precision)
        clocks = Clocks(0)
        uv, st, res, lat, results, uids = srv.replay(arrival, kind, req_ids, qoff, P, upload_bank, uidx,
                                                     timeout_ms=600000)
        clk = clocks.stop()
        stats = srv.stats()
        srv.close()
        # uploaded surfaces are released again so every rate starts from the same pool
        for u in np.unique(uids[uids >= 0]):
            pool.remove(int(u))
        inv = kind == 0
        ok = results == 0
        done = arrival + lat
        # inversion throughput over the inversion requests' own span (uploads are reported apart)
        span_s = (done[inv].max() - arrival[inv].min()) / 1e6
        li = lat[inv & ok] / 1e3
        lu = lat[(kind == 1) & ok] / 1e3
        return {"rate_req_s": rate, "requests": int(nreq), "queries": int(sizes.sum()),
                "ok_frac": float(ok.mean()), "achieved_req_s": int(inv.sum()) / span_s,
                "achieved_queries_s": float(sizes.sum()) / span_s,
                "p50_ms": float(np.percentile(li, 50)), "p99_ms": float(np.percentile(li, 99)),
                "upload_p50_ms": float(np.percentile(lu, 50)) if lu.size else None,
                "upload_p99_ms": float(np.percentile(lu, 99)) if lu.size else None,
                "batches": int(stats.batches), "mean_batch_queries": stats.batch_queries / max(1, stats.batches),
                "gpu_ms_per_batch": stats.gpu_ms / max(1, stats.batches),
                "dispatch_us_per_batch": stats.dispatch_us / max(1, stats.batches),
                "retire_us_per_batch": stats.retire_us / max(1, stats.batches),
                "found_frac": float((st[np.repeat(inv, sizes)] == 0).mean()) if sizes.sum() else None,
                "clocks": clk}

    sweep = []
    for rate in rates:
        nreq = int(min(max(rate * serve_seconds, 2000), a.max_requests))
        sweep.append(serve(rate, nreq, gn.PREC_MIXED))
        phase(f"rate {rate:.0f}: p50 {sweep[-1]['p50_ms']:.3f} ms p99 {sweep[-1]['p99_ms']:.3f} ms, "
              f"{sweep[-1]['achieved_queries_s'] / 1e6:.1f} M queries/s")
    peak = max(sweep, key=lambda d: d["achieved_req_s"])
    half_rate = peak["achieved_req_s"] / 2
    half = serve(half_rate, int(min(max(half_rate * serve_seconds, 2000), a.max_requests)), gn.PREC_MIXED)
    phase(f"half peak {half_rate:.0f} req/s: p99 {half['p99_ms']:.3f} ms")
    fp64_peak = serve(rates[-1], int(min(max(rates[-1] * serve_seconds, 2000), a.max_requests) // 4), gn.PREC_FP64)
    phase("fp64 peak measured")
    rec = {
        "metric": "serve p99 latency at half of peak throughput (mixed)", "value": half["p99_ms"], "unit": "ms",
        "n_gpus": 1, "steps": len(rates) + 2, "warmup": 0, "ms_per_step": None, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp32+fp64 (mixed)", "data": "synthetic (seeded)",
        "config": {"workload": f"serving: pool of {npool} surfaces (batched-workload distribution), 20 GB budget, "
                               "Poisson arrivals, Zipf(1.1) surfaces, 1..4096 queries/request log-uniform, "
                               "10% uploads", "slots": a.slots, "max_batch_queries": a.max_batch_queries,
                   "queries_per_warp_chunk": a.serve_chunk, "rates_req_s": rates, "seconds_per_rate": serve_seconds},
        "peak": {"req_s": peak["achieved_req_s"], "queries_s": peak["achieved_queries_s"]},
        "half_peak": half, "sweep": sweep,
        "fp64_server_at_top_rate": fp64_peak,
        "mixed_vs_fp64_peak_queries_s": peak["achieved_queries_s"] / fp64_peak["achieved_queries_s"],
        "clocks": half["clocks"],
        "gpu_launches": None,
    }
    if compact:
        rec = {"value": rec["value"], "unit": "ms", "metric": rec["metric"], "peak": rec["peak"],
               "half_peak": {k: half[k] for k in ("rate_req_s", "achieved_req_s", "achieved_queries_s", "p50_ms",
                                                  "p99_ms", "ok_frac", "found_frac", "upload_p99_ms", "clocks")},
               "fp64_peak_queries_s": fp64_peak["achieved_queries_s"],
               "mixed_vs_fp64_peak_queries_s": rec["mixed_vs_fp64_peak_queries_s"],
               "sweep": [{k: d[k] for k in ("rate_req_s", "achieved_req_s", "achieved_queries_s", "p50_ms", "p99_ms")}
                         for d in sweep],
               "config": rec["config"], "clocks": half["clocks"]}
    return rec


def run_serving(a):
    print(json.dumps(serving_record(a)))


def cpu_baseline(surf, P, sample, g_uv, g_st, g_res):
    """The oracle (C restatement of the reference FP64 path) on all host cores, bounded sample;
    its results on that sample also check this run's mixed-precision results.  `one_core`: the
    same inversion on one host thread over the first eighth of the sample."""
    import oracle as O
    Ps = P[:sample]
    par, dt = oracle_parity_sample(surf, Ps, g_uv[:sample], g_st[:sample], g_res[:sample])
    o1 = O.OracleSurface(surf)
    o1.tree()
    P1 = Ps[:max(1, len(Ps) // 8)]
    t0 = time.perf_counter()
    o1.invert(P1, threads=1)
    dt1 = time.perf_counter() - t0
    return ({"value": len(Ps) / dt, "unit": "inversions/s", "cores": host_cores(), "kind": "port",
             "sample": f"{len(Ps)} queries of the same workload, the oracle's inversion, {dt:.2f} s wall",
             "one_core": {"value": len(P1) / dt1, "unit": "inversions/s", "sample": f"{len(P1)} queries, 1 thread"}},
            par)


def run_reference(a):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    load_pkg()
    from gpu_nurbs_gb300 import synth
    import oracle as O
    surf = {"large": synth.surface_large, "quintic": synth.surface_quintic}.get(a.workload, synth.surface_small)()
    o = O.OracleSurface(surf)
    uv, off = synth.query_params(a.cpu_sample, 1000, "large" if a.workload == "large" else "small")
    E = o.eval(uv, 7)
    P = synth.form_queries(E[0:3].T, E[3:6].T, E[6:9].T, off)
    o.tree()
    cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()
    for _ in range(min(a.warmup, 1)):
        o.invert(P[:1024], threads=cores)
    ts = []
    for _ in range(a.steps):
        t0 = time.perf_counter()
        o.invert(P, threads=cores)
        ts.append(time.perf_counter() - t0)
    dt = sum(ts) / len(ts)
    v = len(P) / dt
    kind = "port"  # the oracle's C restatement of the reference's FP64 algorithm is what runs
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": "inversions/s", "n_gpus": world,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp64", "data": "synthetic (seeded)",
        "config": {"workload": workload_label(a.workload if a.workload in ("large", "small", "quintic") else "small",
                                              a.queries or ((1 << 24) if a.workload == "quintic" else (1 << 20))),
                   "queries_per_step": len(P), "note": "each step inverts a bounded sample of the workload"},
        "cpu_baseline": {"value": v, "unit": "inversions/s", "cores": cores, "kind": kind,
                         "sample": f"{len(P)} queries per step (bounded sample of the workload), all host cores"},
        "e2e": {"value": v, "unit": "inversions/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="large",
                    choices=["large", "small", "quintic", "batched", "eval-small", "eval-large", "serving", "project", "quadtree", "pcurve"])
    ap.add_argument("--rates", default="1000,10000,30000,100000,300000,1000000")
    ap.add_argument("--serve-seconds", type=float, default=1.0)
    ap.add_argument("--max-requests", type=int, default=40000)
    ap.add_argument("--slots", type=int, default=4)
    ap.add_argument("--max-batch-queries", type=int, default=1 << 16, help="serving: queries per batch at most")
    ap.add_argument("--upload-frac", type=float, default=0.10)
    ap.add_argument("--serve-chunk", type=int, default=16, help="queries per warp chunk when serving")
    ap.add_argument("--surfaces", type=int, default=4096)
    ap.add_argument("--tune-queries", type=int, default=4 << 20)
    ap.add_argument("--queries", type=int, default=None,
                    help="points per step (default: 2^20; quintic 2^24; eval-large 2^26)")
    ap.add_argument("--cpu-sample", type=int, default=1 << 14)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--headline-only", action="store_true",
                    help="the large workload's line without the batched/quintic/eval/serving sub-records")
    a = ap.parse_args()
    if a.impl == "reference":
        run_reference(a)
    elif a.workload == "batched":
        run_batched(a)
    elif a.workload.startswith("eval"):
        run_eval(a)
    elif a.workload == "serving":
        run_serving(a)
    elif a.workload == "project":
        run_project(a)
    elif a.workload == "quadtree":
        run_quadtree(a)
    elif a.workload == "pcurve":
        run_pcurve(a)
    else:
        run_ours(a)


if __name__ == "__main__":
    main()
