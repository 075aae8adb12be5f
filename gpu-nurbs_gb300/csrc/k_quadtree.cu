// Adaptive quadtree inversion (nurbs_invert_quadtree): the reference's first inversion, which
// needs no tree build — per query a breadth-first quadtree over the parameter domain, culled by
// control-net boxes (Inverse, src/kernel/kernel.cu:4-104; BoundingBoxCheck :106-149;
// getSplitType :251-298; NODE_MAX_SIZE 64, src/kernel/kernel.cuh:13).
//
// A persistent grid whose warps take chunks of 32 queries from a counter.  The first layer (the
// root: its precomputed box and one trajectory from the domain's centre) runs lane per query and
// answers most queries.  A query it leaves open is then searched by the whole warp.  With MODE
// mixed every node's trajectory runs in FP32 and its end takes FP64 Newton steps (the mixed
// inversion's final steps); the box checks and split decisions stay exact FP64:
//   * a layer's nodes live in shared memory; each node's control-point box is reduced by the
//     whole warp (lanes stride over the node's control-point rows and columns, min/max by
//     shuffles: exact, so the pass/fail decisions equal the oracle's);
//   * the passing nodes' trajectories run one per lane (from the node centre); a result counts
//     when it converged inside the domain within max_edge of P;
//   * the first layer with a result answers (its closest result; AMBIGUOUS as in the inversion);
//     otherwise each passing node is split by the reference's getSplitType, decided in FP32 where
//     its lengths are clearly off max_edge and else evaluated with the reference-order FP64
//     functions (this translation unit is compiled with --fmad=false, so the split decisions,
//     and with them the tree, are the oracle's; the v-length uses the v-derivative, which the
//     reference takes with MatrixSurfaceDerivativeU), and the children are compacted into the
//     next layer in the reference's order by a warp prefix sum.
// Culled nodes are not split (their control-point box does not hold P, so neither does their
// surface); a layer of more than 64 nodes or 60 layers ends the query unanswered.
#include "invert_core.cuh"

namespace gnurbs {
namespace {

using namespace inv;

constexpr int kQtMax = 64;     // nodes per layer (NODE_MAX_SIZE)
constexpr int kQtLayers = 60;

struct QtWarp {
  double node[2][kQtMax + 4][4];  // two layers: lb.u, lb.v, rt.u, rt.v
  int code[2][kQtMax + 4];        // index of the node's precomputed box, -1 when it has none
  double su[kQtMax], sv[kQtMax], sr[kQtMax];
  unsigned char pass[kQtMax], ok[kQtMax];
};

__device__ __forceinline__ int knot_span(const int* knot_idx, const double* b, int ns, double x) {
  return knot_idx[exact::find_seg(b, ns, x)];  // findSpan (Evaluate.cu:504-533) over the breakpoints
}

// getSplitType: 0 NOT_SPLIT, 1 SPLIT_V, 2 SPLIT_U, 3 SPLIT_UV
__device__ int split_type(const SurfDev& s, const double* nd, double max_edge) {
  const int p = s.p, q = s.q, k2 = q + 1, k12 = (p + 1) * (q + 1);
  const double iu = (nd[2] - nd[0]) / 4, iv = (nd[3] - nd[1]) / 4;
  double ul = 0, vl = 0;
  for (int i = 0; i < 4; ++i) {
    const double x = nd[0] + i * iu, y = nd[1] + i * iv;
    const int su = exact::find_seg(s.bu, s.ns_u, x), sv = exact::find_seg(s.bv, s.ns_v, y);
    const double du = s.bu[su + 1] - s.bu[su], dv = s.bv[sv + 1] - s.bv[sv];
    const double u = (x - s.bu[su]) / du, v = (y - s.bv[sv]) / dv;
    exact::DenseSpan M{s.m64 + (size_t)(su * s.ns_v + sv) * k12 * 4, k2};
    const v4<double> R = exact::point_r(M, p, q, u, v);
    const v3<double> a = exact::der_u(M, p, q, u, v, R, s.range_u / du);
    const v3<double> b = exact::der_v(M, p, q, u, v, R, s.range_v / dv);
    ul += sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
    vl += sqrt(b.x * b.x + b.y * b.y + b.z * b.z);
  }
  ul *= (nd[2] - nd[0]) * 0.25;
  vl *= (nd[3] - nd[1]) * 0.25;
  if (ul < max_edge && vl < max_edge) return 0;
  if (nd[2] - nd[0] > 0.25 || nd[3] - nd[1] > 0.25) return 3;
  if (ul < max_edge) return 1;
  if (vl < max_edge) return 2;
  return 3;
}

// getSplitType decided in FP32 where that is safe: the lengths from the FP32 tables' derivatives,
// used when each differs from max_edge by more than 1 % of max_edge plus 0.1 % of itself and every
// sample falls in the same span as in FP64; otherwise the reference-order FP64 evaluation above.
// Measured against the FP64 lengths over 20,000 nodes (depths 0-8) of six surfaces up to degree 5
// and 256x256 nets, the FP32 lengths err by at most 1.4e-4 of themselves, so both give the same
// decision; the FP32 one costs a fraction of the FP64 work (the FP64 split types took most of a
// launch).
template <int P, int Q>
__device__ int split_type_fast(const SurfDev& s, const Ctx& cx, const double* nd, double max_edge) {
  const double iu = (nd[2] - nd[0]) / 4, iv = (nd[3] - nd[1]) / 4;
  float ul = 0, vl = 0;
  bool exact = false;
  for (int i = 0; i < 4; ++i) {
    const double x = nd[0] + i * iu, y = nd[1] + i * iv;
    const int su = exact::find_seg(s.bu, s.ns_u, x), sv = exact::find_seg(s.bv, s.ns_v, y);
    int hu = su, hv = sv;
    const fast::SDer<float> d = fast::eval_at<float, P, Q, 1, true>(cx.L32, cx.m32, cx.p, cx.q, (float)x, (float)y,
                                                                  hu, hv);
    exact = exact || hu != su || hv != sv;
    ul += sqrtf(dot3(d.Su, d.Su));
    vl += sqrtf(dot3(d.Sv, d.Sv));
  }
  ul *= (float)((nd[2] - nd[0]) * 0.25);
  vl *= (float)((nd[3] - nd[1]) * 0.25);
  const float me = (float)max_edge;
  exact = exact || !(fabsf(ul - me) > 0.01f * me + 1e-3f * ul) || !(fabsf(vl - me) > 0.01f * me + 1e-3f * vl);
  if (exact) return split_type(s, nd, max_edge);
  const bool us = ul < me, vs = vl < me;
  if (us && vs) return 0;
  if (nd[2] - nd[0] > 0.25 || nd[3] - nd[1] > 0.25) return 3;
  if (us) return 1;
  if (vs) return 2;
  return 3;
}

__device__ __forceinline__ void put_node(double* o, double a, double b, double c, double d) {
  o[0] = a;
  o[1] = b;
  o[2] = c;
  o[3] = d;
}

// Precomputed boxes of the top kQtDepth levels of square children (depth d, u index a, v index b:
// code = base(d) + a * 2^d + b; base = 0, 1, 5), written when the surface is converted.  Deeper
// nodes, and the halves of U / V splits, scan their control points.
constexpr int kQtDepth = 3;
constexpr int kQtBoxes = 1 + 4 + 16;
__device__ __forceinline__ int code_depth(int c) { return c == 0 ? 0 : (c < 5 ? 1 : 2); }
__device__ __forceinline__ int child_code(int pc, int hu, int hv) {
  if (pc < 0) return -1;
  const int d = code_depth(pc);
  if (d + 1 >= kQtDepth) return -1;
  const int base = d == 0 ? 0 : 1, side = 1 << d, idx = pc - base;
  const int a = idx / side, b = idx % side;
  return (d == 0 ? 1 : 5) + (2 * a + hu) * (2 * side) + (2 * b + hv);
}

// Partial box over a node's control points (the rows findSpan(lb.u) - p .. findSpan(rt.u), the
// same in v: BoundingBoxCheck's range), over elements t, t + stride, ...; starts from the first
// control point of the range, as the reference does.
__device__ void node_box(const SurfDev& s, const double* nd, int t, int stride, double* mn, double* mx) {
  const int i0 = knot_span(s.knot_u, s.bu, s.ns_u, nd[0]) - s.p, i1 = knot_span(s.knot_u, s.bu, s.ns_u, nd[2]);
  const int j0 = knot_span(s.knot_v, s.bv, s.ns_v, nd[1]) - s.q, j1 = knot_span(s.knot_v, s.bv, s.ns_v, nd[3]);
  const int nb = j1 - j0 + 1, cnt = (i1 - i0 + 1) * nb;
  for (int c = 0; c < 3; ++c) {
    mn[c] = s.cps[3 * ((size_t)i0 * s.nv + j0) + c];
    mx[c] = mn[c];
  }
  for (int e = t; e < cnt; e += stride) {
    const double* x = s.cps + 3 * ((size_t)(i0 + e / nb) * s.nv + (j0 + e % nb));
    for (int c = 0; c < 3; ++c) {
      mn[c] = mn[c] > x[c] ? x[c] : mn[c];
      mx[c] = mx[c] < x[c] ? x[c] : mx[c];
    }
  }
}

// One CTA per precomputed box: the node's rectangle by the same midpoint splits as the search.
__global__ void __launch_bounds__(256) k_quadtree_boxes(SurfDev s, double* __restrict__ qtbox) {
  const int code = blockIdx.x;
  const int d = code_depth(code), side = 1 << d, idx = code - (d == 0 ? 0 : (d == 1 ? 1 : 5));
  const int a = idx / side, b = idx % side;
  double nd[4] = {s.dom_u0, s.dom_v0, s.dom_u1, s.dom_v1};
  for (int l = d - 1; l >= 0; --l) {
    const int hu = (a >> l) & 1, hv = (b >> l) & 1;
    const double mu = (nd[0] + nd[2]) / 2, mv = (nd[1] + nd[3]) / 2;
    if (hu) nd[0] = mu; else nd[2] = mu;
    if (hv) nd[1] = mv; else nd[3] = mv;
  }
  double mn[3], mx[3];
  node_box(s, nd, threadIdx.x, blockDim.x, mn, mx);
  __shared__ double red[256][6];
  for (int c = 0; c < 3; ++c) {
    red[threadIdx.x][c] = mn[c];
    red[threadIdx.x][3 + c] = mx[c];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int j = 1; j < (int)blockDim.x; ++j)
      for (int c = 0; c < 3; ++c) {
        mn[c] = fmin(mn[c], red[j][c]);
        mx[c] = fmax(mx[c], red[j][3 + c]);
      }
    for (int c = 0; c < 3; ++c) {
      qtbox[6 * code + c] = mn[c];
      qtbox[6 * code + 3 + c] = mx[c];
    }
  }
}

// One node's trajectory from (u, v): FP64 (the inversion's FP64 iteration), or MIXED (the mixed
// inversion's FP32 iteration, the point relative to the control net's centre, then its FP64
// final steps).  True when it converged inside the domain within max_edge of P; (u, v, rr) the
// result.
template <int P, int Q, int MODE>
__device__ bool node_trajectory(const SurfDev& s, const Ctx& cx, double px, double py, double pz, double max_edge,
                                double& u, double& v, double& rr) {
  if constexpr (MODE == kModeMixed) {
    Seed<float> sd;
    sd.u = (float)u;
    sd.v = (float)v;
    sd.prev = INFINITY;
    sd.it = 0;
    sd.hu = 0;
    sd.hv = 0;
    sd.newton = false;
    const float tx = (float)(px - s.org[0]), ty = (float)(py - s.org[1]), tz = (float)(pz - s.org[2]);
    const float eu = 2.0f * (float)(s.dom_u1 - s.dom_u0), ev = 2.0f * (float)(s.dom_v1 - s.dom_v0);
    const float far[4] = {(float)s.dom_u0 - eu, (float)s.dom_u1 + eu, (float)s.dom_v0 - ev, (float)s.dom_v1 + ev};
    float dist;
    int r = kContinue;
    while (r == kContinue) {
      r = iterate32<P, Q>(cx, tx, ty, tz, sd, dist);
      if (r == kContinue && !(sd.u >= far[0] && sd.u <= far[1] && sd.v >= far[2] && sd.v <= far[3])) r = kFailed;
    }
    if (r != kConverged) return false;
    u = sd.u;
    v = sd.v;
    return final64<P, Q>(cx, px, py, pz, u, v, rr) && rr < max_edge;
  } else {
    Seed<double> sd;
    sd.u = u;
    sd.v = v;
    sd.prev = INFINITY;
    sd.it = 0;
    sd.hu = 0;
    sd.hv = 0;
    sd.newton = false;
    int r = kContinue;
    while (r == kContinue) r = iterate64<P, Q>(cx, px, py, pz, sd);
    u = sd.u;
    v = sd.v;
    return r == kConverged && finish64<P, Q>(cx, px, py, pz, u, v, sd.hu, sd.hv, rr) && rr < max_edge;
  }
}

// The whole warp searches one query's tree.  root_failed: the root passed and its trajectory had
// no result (the chunk's lane-per-query first layer found that), so layer 0 goes straight to the
// split.
template <int P, int Q, int MODE>
__device__ void quadtree_query(const SurfDev& s, const Ctx& cx, QtWarp& w, const double* __restrict__ qtbox,
                               const double* __restrict__ Pq, int64_t qi, double max_edge, bool root_failed,
                               double* __restrict__ uv_out, int* __restrict__ st_out, double* __restrict__ res_out) {
  const int lane = threadIdx.x & 31;
  const unsigned FULL = 0xffffffffu;
  const double px = Pq[3 * qi], py = Pq[3 * qi + 1], pz = Pq[3 * qi + 2];
  int cur = 0, size = 1, status = 3;
  bool passed_any = false;
  double ou = __longlong_as_double(0x7ff8000000000000ll), ov = ou, orr = ou;
  if (lane == 0) {
    put_node(w.node[0][0], s.dom_u0, s.dom_v0, s.dom_u1, s.dom_v1);
    w.code[0][0] = 0;
  }
  __syncwarp();
  for (int layer = 0; layer < kQtLayers && size > 0; ++layer) {
    const bool known = layer == 0 && root_failed;
    if (known) {
      if (lane == 0) {
        w.pass[0] = 1;
        w.ok[0] = 0;
      }
      passed_any = true;
    }
    // ---- control-point boxes (BoundingBoxCheck), one node at a time, the warp striding over it
    for (int i = 0; i < (known ? 0 : size); ++i) {
      const double* nd = w.node[cur][i];
      double mn[3], mx[3];
      if (w.code[cur][i] >= 0) {  // the top levels' boxes, written with the surface
        const double* b = qtbox + 6 * w.code[cur][i];
        for (int c = 0; c < 3; ++c) {
          mn[c] = b[c];
          mx[c] = b[3 + c];
        }
      } else {
        node_box(s, nd, lane, 32, mn, mx);
        for (int o = 16; o > 0; o >>= 1)
          for (int c = 0; c < 3; ++c) {
            mn[c] = fmin(mn[c], __shfl_xor_sync(FULL, mn[c], o));
            mx[c] = fmax(mx[c], __shfl_xor_sync(FULL, mx[c], o));
          }
      }
      const bool pass = px >= mn[0] - max_edge && px <= mx[0] + max_edge && py >= mn[1] - max_edge &&
                        py <= mx[1] + max_edge && pz >= mn[2] - max_edge && pz <= mx[2] + max_edge;
      if (lane == 0) w.pass[i] = pass ? 1 : 0;
      passed_any = passed_any || pass;
    }
    __syncwarp();
    // ---- trajectories of the passing nodes, one per lane
    for (int i = lane; i < (known ? 0 : size); i += 32) {
      w.ok[i] = 0;
      if (!w.pass[i]) continue;
      const double* nd = w.node[cur][i];
      double u = (nd[0] + nd[2]) / 2, v = (nd[1] + nd[3]) / 2, rr;
      if (node_trajectory<P, Q, MODE>(s, cx, px, py, pz, max_edge, u, v, rr)) {
        w.ok[i] = 1;
        w.su[i] = u;
        w.sv[i] = v;
        w.sr[i] = rr;
      }
    }
    __syncwarp();
    // ---- the layer's closest result (ties: the lower node), if any
    int best = -1;
    for (int i = 0; i < size; ++i)
      if (w.ok[i] && (best < 0 || w.sr[i] < w.sr[best])) best = i;
    if (best >= 0) {
      status = 0;
      for (int i = 0; i < size; ++i)
        if (w.ok[i] && i != best && w.sr[i] <= w.sr[best] * (1 + 1e-6) + 1e-12 &&
            (fabs(w.su[i] - w.su[best]) > 1e-7 || fabs(w.sv[i] - w.sv[best]) > 1e-7))
          status = 1;
      ou = w.su[best];
      ov = w.sv[best];
      orr = w.sr[best];
      break;
    }
    // ---- split the passing nodes (getSplitType) and compact their children in node order
    int nch[2] = {0, 0}, typ[2] = {0, 0};
    for (int r = 0; r < 2; ++r) {
      const int i = lane + 32 * r;
      if (i < size && w.pass[i]) {
        typ[r] = split_type_fast<P, Q>(s, cx, w.node[cur][i], max_edge);
        nch[r] = typ[r] == 3 ? 4 : (typ[r] == 0 ? 0 : 2);
      }
    }
    int total = 0, off[2];
    for (int r = 0; r < 2; ++r) {
      int incl = nch[r];
      for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(FULL, incl, o);
        if (lane >= o) incl += t;
      }
      off[r] = total + incl - nch[r];
      total += __shfl_sync(FULL, incl, 31);
    }
    if (total > kQtMax) break;  // layer overflow: unanswered
    if (total == 0) {
      status = passed_any ? 3 : 2;
      break;
    }
    for (int r = 0; r < 2; ++r) {
      const int i = lane + 32 * r;
      if (nch[r] == 0) continue;
      const double* nd = w.node[cur][i];
      const double lx = nd[0], ly = nd[1], rx = nd[2], ry = nd[3];
      const double mxu = (lx + rx) / 2, myv = (ly + ry) / 2;
      double* o = w.node[cur ^ 1][off[r]];
      int* oc = w.code[cur ^ 1] + off[r];
      const int pc = w.code[cur][i];
      if (typ[r] == 3) {
        put_node(o, lx, ly, mxu, myv);
        put_node(o + 4, lx, myv, mxu, ry);
        put_node(o + 8, mxu, myv, rx, ry);
        put_node(o + 12, mxu, ly, rx, myv);
        const int hu[4] = {0, 0, 1, 1}, hv[4] = {0, 1, 1, 0};
        for (int c = 0; c < 4; ++c) oc[c] = child_code(pc, hu[c], hv[c]);
      } else {
        if (typ[r] == 2) {
          put_node(o, lx, ly, mxu, ry);
          put_node(o + 4, mxu, ly, rx, ry);
        } else {
          put_node(o, lx, ly, rx, myv);
          put_node(o + 4, lx, myv, rx, ry);
        }
        oc[0] = oc[1] = -1;
      }
    }
    __syncwarp();
    cur ^= 1;
    size = total;
  }
  if (lane == 0) {
    uv_out[2 * qi] = ou;
    uv_out[2 * qi + 1] = ov;
    st_out[qi] = status;
    res_out[qi] = orr;
  }
  __syncwarp();
}

template <int P, int Q, int MODE>
__global__ void __launch_bounds__(kThreads)
    k_invert_quadtree(SurfDev s, const double* __restrict__ qtbox, const double* __restrict__ Pq, int64_t n,
                      double max_edge, double* __restrict__ uv_out, int* __restrict__ st_out,
                      double* __restrict__ res_out, unsigned* __restrict__ counter) {
  __shared__ QtWarp ww[kWarps];
  Ctx cx;
  cx.L32 = fast::global_locator<float>(s);
  cx.L64 = fast::global_locator<double>(s);
  cx.m32 = s.m32;
  cx.m64 = s.m64;
  cx.p = s.p;
  cx.q = s.q;
  cx.dom_u0 = s.dom_u0;
  cx.dom_u1 = s.dom_u1;
  cx.dom_v0 = s.dom_v0;
  cx.dom_v1 = s.dom_v1;
  QtWarp& w = ww[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  const unsigned FULL = 0xffffffffu;
  // chunks of 32 queries: the first layer (the root, one node) lane per query, which answers most
  // queries; the warp then searches the rest one by one from the root's split
  const int64_t chunks = (n + 31) / 32;
  for (;;) {
    unsigned ch = 0;
    if (lane == 0) ch = atomicAdd(counter, 1u);
    ch = __shfl_sync(FULL, ch, 0);
    if ((int64_t)ch >= chunks) break;
    const int64_t qi = (int64_t)ch * 32 + lane;
    bool rest = false;
    if (qi < n) {
      const double px = Pq[3 * qi], py = Pq[3 * qi + 1], pz = Pq[3 * qi + 2];
      const bool pass = px >= qtbox[0] - max_edge && px <= qtbox[3] + max_edge && py >= qtbox[1] - max_edge &&
                        py <= qtbox[4] + max_edge && pz >= qtbox[2] - max_edge && pz <= qtbox[5] + max_edge;
      int status = 2;  // the root alone does not pass: no node ever passes
      double ou = __longlong_as_double(0x7ff8000000000000ll), ov = ou, orr = ou;
      if (pass) {
        double u = (s.dom_u0 + s.dom_u1) / 2, v = (s.dom_v0 + s.dom_v1) / 2, rr = 0;
        const bool ok = node_trajectory<P, Q, MODE>(s, cx, px, py, pz, max_edge, u, v, rr);
        if (ok) {
          status = 0;
          ou = u;
          ov = v;
          orr = rr;
        } else {
          rest = true;
        }
      }
      if (!rest) {
        uv_out[2 * qi] = ou;
        uv_out[2 * qi + 1] = ov;
        st_out[qi] = status;
        res_out[qi] = orr;
      }
    }
    unsigned m = __ballot_sync(FULL, rest);
    while (m) {
      const int j = __ffs(m) - 1;
      m &= m - 1;
      quadtree_query<P, Q, MODE>(s, cx, w, qtbox, Pq, (int64_t)ch * 32 + j, max_edge, true, uv_out, st_out,
                                 res_out);
    }
  }
}

template <int P, int Q, int MODE>
cudaError_t launch_quadtree_mode(const SurfDev& s, const double* P_, int64_t n, double max_edge, double* uv, int* st_,
                                 double* res, unsigned* counter, cudaStream_t st) {
  if ((n + 31) / 32 > 0xffffffffLL) return cudaErrorInvalidValue;  // chunk ids are 32-bit
  static int cached[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) dev = 0;
  if (!cached[dev]) {
    int sms = 0, per_sm = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_invert_quadtree<P, Q, MODE>, kThreads, 0);
    cached[dev] = (sms > 0 ? sms : 1) * (per_sm > 0 ? per_sm : 1);
  }
  int64_t blocks = ((n + 31) / 32 + kWarps - 1) / kWarps;
  if (blocks > cached[dev]) blocks = cached[dev];
  k_invert_quadtree<P, Q, MODE><<<(unsigned)blocks, kThreads, 0, st>>>(s, s.qtbox, P_, n, max_edge, uv, st_, res,
                                                                       counter);
  return cudaGetLastError();
}

template <int P, int Q>
cudaError_t launch_quadtree_pq(const SurfDev& s, const double* P_, int64_t n, double max_edge, double* uv, int* st_,
                               double* res, int precision, unsigned* counter, cudaStream_t st) {
  if (precision == kModeMixed)
    return launch_quadtree_mode<P, Q, kModeMixed>(s, P_, n, max_edge, uv, st_, res, counter, st);
  return launch_quadtree_mode<P, Q, kModeFP64>(s, P_, n, max_edge, uv, st_, res, counter, st);
}

}  // namespace

cudaError_t launch_quadtree_boxes(const SurfDev& s, cudaStream_t st) {
  k_quadtree_boxes<<<kQtBoxes, 256, 0, st>>>(s, s.qtbox);
  return cudaGetLastError();
}

cudaError_t launch_invert_quadtree(const SurfDev& s, const double* P, int64_t n, double max_edge, double* uv,
                                   int* status, double* residual, int precision, unsigned* counter, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  if (s.p == 3 && s.q == 3)
    return launch_quadtree_pq<3, 3>(s, P, n, max_edge, uv, status, residual, precision, counter, st);
  return launch_quadtree_pq<0, 0>(s, P, n, max_edge, uv, status, residual, precision, counter, st);
}

}  // namespace gnurbs
