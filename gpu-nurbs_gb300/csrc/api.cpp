// C-ABI of the GB300 NURBS engine (declared in include/gpu_nurbs.h).
//
// Host-side duties: argument validation, the per-surface device arena, breakpoint tables,
// launches on the caller's stream, and status codes.  Nothing here calls exit().
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "gpu_nurbs.h"
#include "nurbs_internal.h"
#include "surface_host.h"

using namespace gnurbs;

namespace {
thread_local std::string g_last_error;
}  // namespace

namespace gnurbs {

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  return fail(NURBS_E_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

}  // namespace gnurbs

namespace {

#define CUDA_TRY(expr, what)                         \
  do {                                               \
    cudaError_t e_ = (expr);                         \
    if (e_ != cudaSuccess) return cuda_fail(e_, what); \
  } while (0)

// Temporary device buffers of a call (host-buffer inversion, p-curve scratch, ...) come from
// a stream-ordered pool of the library's own, one per device, that keeps up to kTmpKeepBytes
// of freed memory between calls.  The device's default pool keeps none: it returns freed
// memory to the system at every synchronisation, and mapping it again on the next call costs
// more than the host<->device copies of a 2^20-query call.  The pools live as long as the
// process's contexts: like every handle of this library, they do not survive cudaDeviceReset.
constexpr int kTmpDevices = 64;
constexpr uint64_t kTmpKeepBytes = 512ull << 20;

cudaError_t tmp_alloc(void** p, size_t bytes, cudaStream_t st) {
  static std::mutex mu;
  static cudaMemPool_t pools[kTmpDevices] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kTmpDevices) return cudaMallocAsync(p, bytes, st);
  cudaMemPool_t pool;
  {
    std::lock_guard<std::mutex> lock(mu);
    if (!pools[dev]) {
      cudaMemPoolProps props{};
      props.allocType = cudaMemAllocationTypePinned;
      props.location.type = cudaMemLocationTypeDevice;
      props.location.id = dev;
      cudaMemPool_t created;
      if ((e = cudaMemPoolCreate(&created, &props)) != cudaSuccess) return e;
      uint64_t keep = kTmpKeepBytes;
      if ((e = cudaMemPoolSetAttribute(created, cudaMemPoolAttrReleaseThreshold, &keep)) != cudaSuccess) {
        cudaMemPoolDestroy(created);
        return e;
      }
      pools[dev] = created;
    }
    pool = pools[dev];
  }
  return cudaMallocFromPoolAsync(p, bytes, pool, st);
}

int validate_dims(int p, int q, int nu, int nv) {
  if (p < 1 || q < 1 || p > NURBS_MAX_DEGREE || q > NURBS_MAX_DEGREE)
    return fail(NURBS_E_INVALID, "degrees (%d,%d) outside 1..%d", p, q, NURBS_MAX_DEGREE);
  if (nu < p + 1 || nv < q + 1) return fail(NURBS_E_INVALID, "control net %dx%d too small for degree (%d,%d)", nu, nv, p, q);
  if ((int64_t)nu * nv > (int64_t)1 << 28) return fail(NURBS_E_UNSUPPORTED, "control net %dx%d too large", nu, nv);
  return NURBS_OK;
}

int validate_knots(const double* k, int p, int cp, const char* name) {
  int nk = p + cp + 1;
  for (int i = 0; i < nk; ++i)
    if (!std::isfinite(k[i])) return fail(NURBS_E_INVALID, "%s[%d] is not finite", name, i);
  for (int i = 0; i + 1 < nk; ++i)
    if (k[i] > k[i + 1]) return fail(NURBS_E_INVALID, "%s is not non-decreasing at %d", name, i);
  if (!(k[p] < k[cp])) return fail(NURBS_E_INVALID, "%s: empty parameter domain [k[%d], k[%d]]", name, p, cp);
  return NURBS_OK;
}

// Host copy of a buffer given as host or device pointer.
int fetch(const double* src, size_t n, int kind, std::vector<double>& dst, cudaStream_t st) {
  dst.resize(n);
  if (kind == NURBS_PTR_HOST) {
    std::memcpy(dst.data(), src, n * sizeof(double));
    return NURBS_OK;
  }
  CUDA_TRY(cudaMemcpyAsync(dst.data(), src, n * sizeof(double), cudaMemcpyDeviceToHost, st), "copy to host");
  CUDA_TRY(cudaStreamSynchronize(st), "stream sync");
  return NURBS_OK;
}

}  // namespace

// Inversion launches take their chunk counter from a ring of device words.  A slot is reused
// only after the launch that used it before has finished on the GPU (an event per slot), so
// calls on several streams at once never share a counter.
constexpr int kCounterRing = 16;

struct nurbs_surface_s {
  SurfDev dev{};
  void* arena = nullptr;
  size_t arena_bytes = 0;
  double* basis_u = nullptr;
  double* basis_v = nullptr;
  int device = 0;
  bool tree_built = false;
  unsigned* counters = nullptr;  // kCounterRing device words
  cudaEvent_t done[kCounterRing] = {};
  unsigned next_slot = 0;
  std::mutex mu;
};

// The persistent query kernels that take their work from a launch counter.
enum class QueryOp { kInvert, kProject, kQuadtree };

// Enqueues one launch of a query kernel on `st`: waits for the previous user of the counter
// slot, zeroes the counter, launches, marks the slot.  Inside a stream capture the slot is used
// without the event handshake (capture cannot wait on work recorded outside it).  precision:
// NURBS_PREC_FP64 or NURBS_PREC_MIXED; max_edge: the quadtree inversion's.
static cudaError_t invert_on(nurbs_surface_s* s, const double* P, int64_t n, double* uv, int* status, double* res,
                             int precision, cudaStream_t st, QueryOp op = QueryOp::kInvert, double max_edge = 0) {
  std::lock_guard<std::mutex> lk(s->mu);
  const int slot = (int)(s->next_slot++ % kCounterRing);
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  cudaError_t e = cudaStreamIsCapturing(st, &cap);
  if (e != cudaSuccess) return e;
  const bool capturing = cap != cudaStreamCaptureStatusNone;
  if (!capturing) {
    if (!s->done[slot]) {
      e = cudaEventCreateWithFlags(&s->done[slot], cudaEventDisableTiming);
      if (e != cudaSuccess) return e;
    } else {
      e = cudaStreamWaitEvent(st, s->done[slot], 0);
      if (e != cudaSuccess) return e;
    }
  }
  e = cudaMemsetAsync(s->counters + slot, 0, sizeof(unsigned), st);
  if (e == cudaSuccess) {
    if (op == QueryOp::kQuadtree)
      e = launch_invert_quadtree(s->dev, P, n, max_edge, uv, status, res, precision, s->counters + slot, st);
    else if (op == QueryOp::kProject)
      e = launch_project(s->dev, P, n, uv, status, res, precision, s->counters + slot, st);
    else
      e = launch_invert(s->dev, P, n, uv, status, res, precision, s->counters + slot, st);
  }
  if (e == cudaSuccess && !capturing) e = cudaEventRecord(s->done[slot], st);
  return e;
}

static void release_surface(nurbs_surface_s* s) {
  for (cudaEvent_t& ev : s->done)
    if (ev) cudaEventDestroy(ev);
  if (s->counters) cudaFree(s->counters);
}

extern "C" {

const char* nurbs_status_string(int status) {
  switch (status) {
    case NURBS_OK: return "ok";
    case NURBS_E_INVALID: return "invalid argument";
    case NURBS_E_CUDA: return "CUDA error";
    case NURBS_E_NOMEM: return "out of memory";
    case NURBS_E_IO: return "I/O error";
    case NURBS_E_PARSE: return "parse error";
    case NURBS_E_UNSUPPORTED: return "unsupported";
    case NURBS_E_BUDGET: return "memory budget exceeded";
    case NURBS_E_TIMEOUT: return "timeout";
    case NURBS_E_STATE: return "invalid state";
    default: return "unknown status";
  }
}

const char* nurbs_last_error(void) { return g_last_error.c_str(); }
const char* nurbs_version(void) { return "gpu-nurbs-gb300 0.1 (sm_103a)"; }

int64_t nurbs_matrix_n_size(int p, int q, int nu, int nv) {
  return (int64_t)(p + nu) * (q + nv) * 4 * (p + 1) * (q + 1);
}

int64_t nurbs_matrix_n_position(int i, int j, int p, int q, int nu, int nv, int c) {
  (void)nu;
  return (((int64_t)i * (q + nv) + j) * 4 + c) * (int64_t)(p + 1) * (q + 1);
}

int nurbs_surface_create(int p, int q, int nu, int nv, const double* knots_u, const double* knots_v,
                         const double* cps, const double* weights, int ptr_kind, void* stream,
                         nurbs_surface_t* out) {
  if (!out) return fail(NURBS_E_INVALID, "out is NULL");
  *out = nullptr;
  if (!knots_u || !knots_v || !cps || !weights) return fail(NURBS_E_INVALID, "NULL surface array");
  if (ptr_kind != NURBS_PTR_HOST && ptr_kind != NURBS_PTR_DEVICE) return fail(NURBS_E_INVALID, "bad ptr_kind");
  int rc = validate_dims(p, q, nu, nv);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  // device inputs are read back once: validation and breakpoint tables are host work
  std::vector<double> ku, kv, hc, hw;
  const size_t ncp = (size_t)nu * nv;
  if ((rc = fetch(knots_u, p + nu + 1, ptr_kind, ku, st))) return rc;
  if ((rc = fetch(knots_v, q + nv + 1, ptr_kind, kv, st))) return rc;
  if ((rc = fetch(cps, ncp * 3, ptr_kind, hc, st))) return rc;
  if ((rc = fetch(weights, ncp, ptr_kind, hw, st))) return rc;
  SurfaceHost S;
  std::string err;
  if ((rc = prepare_surface(p, q, nu, nv, ku.data(), kv.data(), hc.data(), hw.data(), S, err)))
    return fail(rc, "%s", err.c_str());
  nurbs_surface_s* s = new (std::nothrow) nurbs_surface_s();
  if (!s) return fail(NURBS_E_NOMEM, "host allocation failed");
  cudaGetDevice(&s->device);
  const size_t total = S.in_bytes + S.out_bytes;
  cudaError_t e = cudaMalloc(&s->arena, total);
  if (e != cudaSuccess) {
    delete s;
    cudaGetLastError();
    return fail(NURBS_E_NOMEM, "device allocation of %zu bytes failed: %s", total, cudaGetErrorString(e));
  }
  s->arena_bytes = total;
  char* A = (char*)s->arena;
  std::vector<char> img(S.in_bytes, 0);
  fill_surface(S, img.data(), A, A + S.in_bytes, s->dev);
  SurfDev& d = s->dev;
  s->basis_u = d.basis_u;
  s->basis_v = d.basis_v;
  e = cudaMemcpyAsync(A, img.data(), S.in_bytes, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = launch_basis(d.knots_u, p, d.knot_u, d.ns_u, s->basis_u, st);
  if (e == cudaSuccess) e = launch_basis(d.knots_v, q, d.knot_v, d.ns_v, s->basis_v, st);
  if (e == cudaSuccess) e = launch_span_matrices(d, s->basis_u, s->basis_v, (double*)d.m64, (float*)d.m32, st);
  if (e == cudaSuccess) e = launch_tree(d, st);
  if (e == cudaSuccess) e = launch_centre_ders(d, st);
  if (e == cudaSuccess) e = launch_cones(d, st);
  if (e == cudaSuccess) e = launch_quadtree_boxes(d, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // img must outlive the copy
  if (e != cudaSuccess) {
    cudaFree(s->arena);
    delete s;
    return cuda_fail(e, "matrix-form conversion");
  }
  s->tree_built = true;
  e = cudaMalloc((void**)&s->counters, sizeof(unsigned) * kCounterRing);
  if (e != cudaSuccess) {
    cudaFree(s->arena);
    delete s;
    cudaGetLastError();
    return fail(NURBS_E_NOMEM, "device allocation of the launch counters failed: %s", cudaGetErrorString(e));
  }
  *out = s;
  return NURBS_OK;
}

int nurbs_surface_destroy(nurbs_surface_t s) {
  if (!s) return NURBS_OK;
  release_surface(s);
  cudaError_t e = cudaFree(s->arena);
  delete s;
  if (e != cudaSuccess) return cuda_fail(e, "cudaFree");
  return NURBS_OK;
}

int nurbs_surface_info(nurbs_surface_t s, nurbs_surface_info_t* info) {
  if (!s || !info) return fail(NURBS_E_INVALID, "NULL argument");
  info->degree_u = s->dev.p;
  info->degree_v = s->dev.q;
  info->cp_u = s->dev.nu;
  info->cp_v = s->dev.nv;
  info->spans_u = s->dev.ns_u;
  info->spans_v = s->dev.ns_v;
  info->device_bytes = (int64_t)s->arena_bytes;
  info->tree_built = s->tree_built ? 1 : 0;
  return NURBS_OK;
}

int nurbs_get_matrix_n(nurbs_surface_t s, double* matrix_n_dev, void* stream) {
  if (!s || !matrix_n_dev) return fail(NURBS_E_INVALID, "NULL argument");
  CUDA_TRY(launch_export_ref_layout(s->dev, matrix_n_dev, (cudaStream_t)stream), "export MatrixN");
  return NURBS_OK;
}

int nurbs_get_matrix_n_raw(double* matrix_n_dev, int p, int q, int nu, int nv, const double* knots_u_dev,
                           const double* knots_v_dev, const double* control_points_dev, const double* weights_dev,
                           void* stream) {
  if (!matrix_n_dev || !knots_u_dev || !knots_v_dev || !control_points_dev || !weights_dev)
    return fail(NURBS_E_INVALID, "NULL argument");
  int rc = validate_dims(p, q, nu, nv);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  std::vector<double> ku, kv;
  if ((rc = fetch(knots_u_dev, p + nu + 1, NURBS_PTR_DEVICE, ku, st))) return rc;
  if ((rc = fetch(knots_v_dev, q + nv + 1, NURBS_PTR_DEVICE, kv, st))) return rc;
  if ((rc = validate_knots(ku.data(), p, nu, "knots_u"))) return rc;
  if ((rc = validate_knots(kv.data(), q, nv, "knots_v"))) return rc;
  std::vector<double> bu, bv;
  std::vector<int> iu, iv;
  breakpoints(ku.data(), p, nu, bu, iu);
  breakpoints(kv.data(), q, nv, bv, iv);
  const int nsu = (int)iu.size(), nsv = (int)iv.size(), k1 = p + 1, k2 = q + 1;
  size_t o_iu = 0, o_iv = align256(nsu * 4), o_bu = o_iv + align256(nsv * 4);
  size_t o_bv = o_bu + align256((size_t)nsu * k1 * k1 * 8);
  size_t total = o_bv + align256((size_t)nsv * k2 * k2 * 8);
  char* tmp = nullptr;
  CUDA_TRY(tmp_alloc((void**)&tmp, total, st), "temporary allocation");
  SurfDev d{};
  d.p = p; d.q = q; d.nu = nu; d.nv = nv; d.ns_u = nsu; d.ns_v = nsv;
  d.knot_u = (const int*)(tmp + o_iu);
  d.knot_v = (const int*)(tmp + o_iv);
  d.cps = control_points_dev;
  d.weights = weights_dev;
  cudaError_t e = cudaMemcpyAsync(tmp + o_iu, iu.data(), nsu * 4, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(tmp + o_iv, iv.data(), nsv * 4, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = launch_basis(knots_u_dev, p, d.knot_u, nsu, (double*)(tmp + o_bu), st);
  if (e == cudaSuccess) e = launch_basis(knots_v_dev, q, d.knot_v, nsv, (double*)(tmp + o_bv), st);
  if (e == cudaSuccess)
    e = launch_span_matrices(d, (double*)(tmp + o_bu), (double*)(tmp + o_bv), matrix_n_dev, nullptr, st);
  // the host vectors above must outlive the async copies
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFreeAsync(tmp, st);
  if (e != cudaSuccess) return cuda_fail(e, "GetMatrixN");
  return NURBS_OK;
}

int nurbs_eval(nurbs_surface_t s, const double* uv_dev, int64_t n, unsigned mask, double* out_dev, int precision,
               void* stream) {
  if (!s) return fail(NURBS_E_INVALID, "NULL surface");
  if (n < 0) return fail(NURBS_E_INVALID, "negative count");
  if (mask == 0 || mask > 1023u) return fail(NURBS_E_INVALID, "mask 0x%x outside 1..1023", mask);
  if (precision != NURBS_PREC_FP64 && precision != NURBS_PREC_EXACT)
    return fail(NURBS_E_INVALID, "nurbs_eval computes in FP64 (NURBS_PREC_FP64 or NURBS_PREC_EXACT); use nurbs_eval_f32");
  if (precision == NURBS_PREC_EXACT && mask > 63u)
    return fail(NURBS_E_INVALID, "NURBS_PREC_EXACT evaluates to second order (mask <= 63)");
  if (n == 0) return NURBS_OK;
  if (!uv_dev || !out_dev) return fail(NURBS_E_INVALID, "NULL buffer");
  if (precision == NURBS_PREC_EXACT)
    CUDA_TRY(launch_eval_exact(s->dev, uv_dev, n, mask, out_dev, (cudaStream_t)stream), "eval launch");
  else
    CUDA_TRY(launch_eval_f64(s->dev, uv_dev, n, mask, out_dev, (cudaStream_t)stream), "eval launch");
  return NURBS_OK;
}

int nurbs_eval_f32(nurbs_surface_t s, const float* uv_dev, int64_t n, unsigned mask, float* out_dev, void* stream) {
  if (!s) return fail(NURBS_E_INVALID, "NULL surface");
  if (n < 0) return fail(NURBS_E_INVALID, "negative count");
  if (mask == 0 || mask > 1023u) return fail(NURBS_E_INVALID, "mask 0x%x outside 1..1023", mask);
  if (n == 0) return NURBS_OK;
  if (!uv_dev || !out_dev) return fail(NURBS_E_INVALID, "NULL buffer");
  CUDA_TRY(launch_eval_f32(s->dev, uv_dev, n, mask, out_dev, (cudaStream_t)stream), "eval launch");
  return NURBS_OK;
}

int nurbs_eval_normal(nurbs_surface_t s, const double* uv_dev, int64_t n, unsigned mask, double* out_dev,
                      void* stream) {
  if (!s) return fail(NURBS_E_INVALID, "NULL surface");
  if (n < 0) return fail(NURBS_E_INVALID, "negative count");
  if (mask == 0 || mask > 63u) return fail(NURBS_E_INVALID, "normal mask 0x%x outside 1..63", mask);
  if (n == 0) return NURBS_OK;
  if (!uv_dev || !out_dev) return fail(NURBS_E_INVALID, "NULL buffer");
  CUDA_TRY(launch_eval_normal(s->dev, uv_dev, n, mask, out_dev, (cudaStream_t)stream), "normal launch");
  return NURBS_OK;
}

int nurbs_evaluate_random(const double* uv_dev, double* xyz_dev, int64_t n, const double* matrix_n_dev, int p, int q,
                          int nu, int nv, const double* knots_u_dev, const double* knots_v_dev, void* stream) {
  int rc = validate_dims(p, q, nu, nv);
  if (rc) return rc;
  if (n < 0) return fail(NURBS_E_INVALID, "negative count");
  if (n == 0) return NURBS_OK;
  if (!uv_dev || !xyz_dev || !matrix_n_dev || !knots_u_dev || !knots_v_dev) return fail(NURBS_E_INVALID, "NULL buffer");
  CUDA_TRY(launch_evaluate_random(uv_dev, xyz_dev, n, matrix_n_dev, p, q, nu, nv, knots_u_dev, knots_v_dev,
                                  (cudaStream_t)stream),
           "EvaluateRandom launch");
  return NURBS_OK;
}

int nurbs_build_tree(nurbs_surface_t s, int levels, void* stream) {
  if (!s) return fail(NURBS_E_INVALID, "NULL surface");
  if (levels != 2) return fail(NURBS_E_UNSUPPORTED, "only the 2-level tree is supported (got %d)", levels);
  cudaStream_t st = (cudaStream_t)stream;
  CUDA_TRY(launch_tree(s->dev, st), "tree launch");
  CUDA_TRY(launch_centre_ders(s->dev, st), "seed-centre derivatives");
  CUDA_TRY(launch_cones(s->dev, st), "normal cones");
  CUDA_TRY(launch_quadtree_boxes(s->dev, st), "quadtree boxes");
  CUDA_TRY(cudaStreamSynchronize(st), "tree sync");
  s->tree_built = true;
  return NURBS_OK;
}

int nurbs_tree_export(nurbs_surface_t s, double* nodes_host, unsigned char* divided_host, unsigned char* built_host) {
  if (!s || !nodes_host || !divided_host || !built_host) return fail(NURBS_E_INVALID, "NULL argument");
  static_assert(sizeof(TreeNodeDev) == 80, "TreeNodeDev layout");
  CUDA_TRY(cudaMemcpy(nodes_host, s->dev.tree, kTreeNodes * sizeof(TreeNodeDev), cudaMemcpyDeviceToHost), "tree copy");
  CUDA_TRY(cudaMemcpy(divided_host, s->dev.divided, kTreeNodes, cudaMemcpyDeviceToHost), "divided copy");
  CUDA_TRY(cudaMemcpy(built_host, s->dev.built, kTreeNodes, cudaMemcpyDeviceToHost), "built copy");
  return NURBS_OK;
}

int nurbs_normal_cones_export(nurbs_surface_t s, double* nbox_host, float* cone_host, float* lattice_host) {
  if (!s || !nbox_host || !cone_host || !lattice_host) return fail(NURBS_E_INVALID, "NULL argument");
  CUDA_TRY(cudaMemcpy(nbox_host, s->dev.nbox, kTreeNodes * 6 * sizeof(double), cudaMemcpyDeviceToHost), "cone copy");
  CUDA_TRY(cudaMemcpy(cone_host, s->dev.cone, kTreeNodes * kConeStride * sizeof(float), cudaMemcpyDeviceToHost),
           "cone copy");
  CUDA_TRY(cudaMemcpy(lattice_host, s->dev.lattice, kTreeNodes * kPts * kPts * 3 * sizeof(float),
                      cudaMemcpyDeviceToHost),
           "lattice copy");
  return NURBS_OK;
}

int nurbs_project(nurbs_surface_t s, const double* P_dev, int64_t n, double* uv_dev, int* status_dev,
                  double* residual_dev, int precision, void* stream) {
  if (!s) return fail(NURBS_E_INVALID, "NULL surface");
  if (n < 0) return fail(NURBS_E_INVALID, "negative count");
  if (precision != NURBS_PREC_FP64 && precision != NURBS_PREC_MIXED)
    return fail(NURBS_E_INVALID, "precision %d is not FP64 or MIXED", precision);
  if (n == 0) return NURBS_OK;
  if (!P_dev || !uv_dev || !status_dev || !residual_dev) return fail(NURBS_E_INVALID, "NULL buffer");
  CUDA_TRY(invert_on(s, P_dev, n, uv_dev, status_dev, residual_dev, precision, (cudaStream_t)stream,
                     QueryOp::kProject),
           "project launch");
  return NURBS_OK;
}

int nurbs_invert_quadtree(nurbs_surface_t s, const double* P_dev, int64_t n, double max_edge, double* uv_dev,
                          int* status_dev, double* residual_dev, int precision, void* stream) {
  if (!s) return fail(NURBS_E_INVALID, "NULL surface");
  if (n < 0) return fail(NURBS_E_INVALID, "negative count");
  if (precision != NURBS_PREC_FP64 && precision != NURBS_PREC_MIXED)
    return fail(NURBS_E_INVALID, "precision %d is not FP64 or MIXED", precision);
  if (!(max_edge > 0) || !std::isfinite(max_edge)) return fail(NURBS_E_INVALID, "max_edge must be positive");
  if (n > 0xffffffffLL) return fail(NURBS_E_INVALID, "more than 2^32 - 1 queries");
  if (n == 0) return NURBS_OK;
  if (!P_dev || !uv_dev || !status_dev || !residual_dev) return fail(NURBS_E_INVALID, "NULL buffer");
  CUDA_TRY(invert_on(s, P_dev, n, uv_dev, status_dev, residual_dev, precision, (cudaStream_t)stream,
                     QueryOp::kQuadtree, max_edge),
           "quadtree inversion launch");
  return NURBS_OK;
}

int nurbs_candidates(nurbs_surface_t s, const double* P_dev, int64_t n, int* list_dev, int* counts_dev, void* stream) {
  if (!s) return fail(NURBS_E_INVALID, "NULL surface");
  if (n < 0) return fail(NURBS_E_INVALID, "negative count");
  if (n == 0) return NURBS_OK;
  if (!P_dev || !list_dev || !counts_dev) return fail(NURBS_E_INVALID, "NULL buffer");
  CUDA_TRY(launch_candidates(s->dev, P_dev, n, list_dev, counts_dev, (cudaStream_t)stream), "candidates launch");
  return NURBS_OK;
}

int nurbs_invert(nurbs_surface_t s, const double* P_dev, int64_t n, double* uv_dev, int* status_dev,
                 double* residual_dev, int precision, void* stream) {
  if (!s) return fail(NURBS_E_INVALID, "NULL surface");
  if (n < 0) return fail(NURBS_E_INVALID, "negative count");
  if (precision != NURBS_PREC_FP64 && precision != NURBS_PREC_MIXED)
    return fail(NURBS_E_INVALID, "precision %d is not FP64 or MIXED", precision);
  if (n == 0) return NURBS_OK;
  if (!P_dev || !uv_dev || !status_dev || !residual_dev) return fail(NURBS_E_INVALID, "NULL buffer");
  CUDA_TRY(invert_on(s, P_dev, n, uv_dev, status_dev, residual_dev, precision, (cudaStream_t)stream),
           "invert launch");
  return NURBS_OK;
}

int nurbs_pcurve(nurbs_surface_t s, const double* C_dev, int64_t n, double* uv_dev, int* status_dev,
                 double* residual_dev, int* flags_dev, int precision, void* stream) {
  if (!s) return fail(NURBS_E_INVALID, "NULL surface");
  if (n < 0) return fail(NURBS_E_INVALID, "negative count");
  if (precision != NURBS_PREC_FP64 && precision != NURBS_PREC_MIXED)
    return fail(NURBS_E_INVALID, "precision %d is not FP64 or MIXED", precision);
  if (n == 0) return NURBS_OK;
  if (!C_dev || !uv_dev || !status_dev || !residual_dev || !flags_dev) return fail(NURBS_E_INVALID, "NULL buffer");
  cudaStream_t st = (cudaStream_t)stream;
  // pass-1 answers in scratch: uv (16 n), status (4 n), residual (8 n)
  const size_t oS = align256((size_t)n * 16), oR = oS + align256((size_t)n * 4), total = oR + align256((size_t)n * 8);
  char* buf = nullptr;
  CUDA_TRY(tmp_alloc((void**)&buf, total, st), "p-curve scratch");
  double* uv0 = (double*)buf;
  int* st0 = (int*)(buf + oS);
  double* res0 = (double*)(buf + oR);
  cudaError_t e = invert_on(s, C_dev, n, uv0, st0, res0, precision, st);
  if (e == cudaSuccess)
    e = launch_pcurve_passes(s->dev, C_dev, n, uv0, st0, res0, uv_dev, status_dev, residual_dev, flags_dev, st);
  cudaError_t e2 = cudaFreeAsync(buf, st);
  if (e == cudaSuccess) e = e2;
  if (e != cudaSuccess) return cuda_fail(e, "p-curve");
  return NURBS_OK;
}

int nurbs_invert_count(nurbs_surface_t s, const double* P_dev, int64_t n, int precision,
                       unsigned long long* counts_host, void* stream) {
  if (!s || !counts_host) return fail(NURBS_E_INVALID, "NULL argument");
  if (n < 0) return fail(NURBS_E_INVALID, "negative count");
  if (precision != NURBS_PREC_FP64 && precision != NURBS_PREC_MIXED)
    return fail(NURBS_E_INVALID, "precision %d is not FP64 or MIXED", precision);
  counts_host[0] = counts_host[1] = 0;
  if (n == 0) return NURBS_OK;
  if (!P_dev) return fail(NURBS_E_INVALID, "NULL buffer");
  cudaStream_t st = (cudaStream_t)stream;
  const size_t oUV = 256, oS = oUV + align256((size_t)n * 16), oR = oS + align256((size_t)n * 4),
               total = oR + align256((size_t)n * 8);
  char* buf = nullptr;
  CUDA_TRY(tmp_alloc((void**)&buf, total, st), "device buffers");
  unsigned* counter = (unsigned*)buf;
  unsigned long long* counts = (unsigned long long*)(buf + 64);
  cudaError_t e = cudaMemsetAsync(buf, 0, 256, st);
  if (e == cudaSuccess)
    e = launch_invert_count(s->dev, P_dev, n, (double*)(buf + oUV), (int*)(buf + oS), (double*)(buf + oR), precision,
                            counter, counts, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(counts_host, counts, 16, cudaMemcpyDeviceToHost, st);
  cudaError_t e2 = cudaFreeAsync(buf, st);
  if (e == cudaSuccess) e = e2;
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "counting inversion");
  return NURBS_OK;
}

int nurbs_invert_host(nurbs_surface_t s, const double* P_host, int64_t n, double* uv_host, int* status_host,
                      double* residual_host, int precision, void* stream) {
  if (!s) return fail(NURBS_E_INVALID, "NULL surface");
  if (n < 0) return fail(NURBS_E_INVALID, "negative count");
  if (n == 0) return NURBS_OK;
  if (precision != NURBS_PREC_FP64 && precision != NURBS_PREC_MIXED)
    return fail(NURBS_E_INVALID, "precision %d is not FP64 or MIXED", precision);
  if (!P_host || !uv_host || !status_host || !residual_host) return fail(NURBS_E_INVALID, "NULL buffer");
  cudaStream_t st = (cudaStream_t)stream;
  size_t bP = (size_t)n * 24, bUV = (size_t)n * 16, bS = (size_t)n * 4, bR = (size_t)n * 8;
  size_t oUV = align256(bP), oS = oUV + align256(bUV), oR = oS + align256(bS), total = oR + align256(bR);
  char* buf = nullptr;
  CUDA_TRY(tmp_alloc((void**)&buf, total, st), "device buffers");
  cudaError_t e = cudaMemcpyAsync(buf, P_host, bP, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = invert_on(s, (const double*)buf, n, (double*)(buf + oUV), (int*)(buf + oS), (double*)(buf + oR),
                  precision, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(uv_host, buf + oUV, bUV, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(status_host, buf + oS, bS, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(residual_host, buf + oR, bR, cudaMemcpyDeviceToHost, st);
  cudaFreeAsync(buf, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "invert (host buffers)");
  return NURBS_OK;
}

}  // extern "C"
