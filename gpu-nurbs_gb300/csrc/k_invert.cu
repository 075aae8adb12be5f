// Stage d: candidate culling + Gauss-Newton point inversion (K4 invert), one fused kernel.
//
// Replaces NewInverse + GaussNewton (src/kernel/kernel.cu:433-469, 151-249).  Per query:
//   1. cull: the built tree nodes sit in shared memory as FP32 boxes rounded outward (a point
//      outside is outside the exact box) and inward (a point strictly inside is inside it); only
//      coordinates within an FP32 ulp of a face are decided by the exact FP64 box, so the
//      candidate set equals the reference's NewBoundingBoxCheck scan bit for bit;
//   2. each candidate is seeded at its node's uv-centre (kernel.cu:154) and iterated with the
//      reference's Gauss-Newton update  C <- C - (J^T J)^-1 J^T (S(C) - P)  (kernel.cu:195-243)
//      until the step is small, then with Newton steps (Hessian J^T J + sum r_k d2S_k) whose
//      fixed point is the same stationary point but which converge quadratically;
//   3. results inside the knot domain are kept; the closest wins.
//
// Work distribution.  The grid is persistent (as many CTAs as fit on the GPU at once) and each
// warp takes chunks of consecutive queries from a global counter until none are left, so
// warps that drew expensive queries do not hold up the end of the launch.  Chunks hold 32
// queries; on large launches the last two rounds hold 8, which shortens the tail in which the
// last warps finish while the others idle.  A query has anywhere from 0 to 65 candidate seeds
// and a seed needs from 2 to 24 iterations, so one thread per query leaves most lanes of a warp
// idle.  Each warp flattens its chunk's (query, seed) pairs into a task list (warp prefix sum
// over the candidate counts) and lanes pull the next tasks as their seeds converge or fail, so
// all 32 lanes iterate until the warp's list is exhausted: at once in the FP64 schedule, in
// batches of eight free lanes in the mixed one (the start is divergent work, cheaper done once
// for several lanes than every iteration for the two or three that just finished).  Finished
// seeds are merged
// into per-query records in shared memory (only results that can change a record, one lane at
// a time).  Every seed runs to its own end (convergence, failure, the iteration cap, or an FP32
// iterate two domain extents outside the domain), decided by the seed alone, so a query's result
// does not depend on which other queries share its warp: results are the same alone and in any
// batch.
//
// Precision schedules (template MODE):
//   FP64  — every evaluation, solve and update in FP64.
//   MIXED — the seed exploration in FP32 (FP32 span matrices, FP32 breakpoints); the best
//           minimum (plus a distinct runner-up within 5 % of its distance, and the closest
//           minimum just outside the domain when as close) then takes the final Newton steps in
//           FP64: S, Su, Sv and the gradient J^T r in FP64, for the first three steps the
//           Hessian's curvature term from FP32 second derivatives (it only sets the convergence
//           rate; two steps normally reach the tolerance), the 2x2 solve and the residual
//           |S - P| at the returned point in FP64 (from the last step's S, Su, Sv and the step, a
//           first-order update whose error is far below FP64 rounding).  Later steps (at most 24
//           in all) take the curvature in FP64 too, for nearly degenerate minima.
#include "invert_core.cuh"

namespace gnurbs {
namespace {

using namespace inv;

// Register budget: 6 CTAs per SM (80 registers) for the mixed kernel of degrees up to 3; degree 5
// keeps 128 registers (4 CTAs per SM), its larger Horner state spilling at 80.
template <int P, int Q, int MODE>
__global__ void __launch_bounds__(kThreads, MODE == kModeMixed ? ((P == 5 || Q == 5) ? 4 : kMinBlocksMixed) : 4)
    k_invert(SurfDev s, const double* __restrict__ Pq, int64_t n, double* __restrict__ uv_out,
             int* __restrict__ st_out, double* __restrict__ res_out, unsigned* __restrict__ counter,
             int64_t n_big) {
  __shared__ Staged<kSmemSpans, MODE> sm;           // one surface for the whole CTA
  __shared__ WarpWork<MODE> ww[kWarps];
  Ctx cx;
  stage_surface<kSmemSpans>(s, sm, cx, threadIdx.x, blockDim.x);
  __syncthreads();
  const int warp = threadIdx.x >> 5;
  // queries [0, n_big) in chunks of 32, then [n_big, n) in chunks of 8
  const int64_t big = n_big / 32, units = big + (n - n_big + 7) / 8;
  for (;;) {
    unsigned ch = 0;
    if ((threadIdx.x & 31) == 0) ch = atomicAdd(counter, 1u);
    ch = __shfl_sync(0xffffffffu, ch, 0);
    if ((int64_t)ch >= units) break;
    const int64_t q0 = (int64_t)ch < big ? (int64_t)ch * 32 : n_big + ((int64_t)ch - big) * 8;
    const int64_t q1 = (int64_t)ch < big ? q0 + 32 : min(q0 + 8, n);
    invert_chunk<P, Q, MODE, kSmemSpans>(sm, ww[warp], cx, Pq, q0, q1, uv_out, st_out, res_out);
  }
}

// The work-counting variant: the same per-query computation, 32-query chunks from the counter,
// FP32/FP64 seed iterations and final FP64 polishes added to counts[0..1].  Diagnostic only.
template <int P, int Q, int MODE>
__global__ void __launch_bounds__(kThreads, 4)
    k_invert_count(SurfDev s, const double* __restrict__ Pq, int64_t n, double* __restrict__ uv_out,
                   int* __restrict__ st_out, double* __restrict__ res_out, unsigned* __restrict__ counter,
                   unsigned long long* __restrict__ counts) {
  __shared__ Staged<kSmemSpans, MODE> sm;
  __shared__ WarpWork<MODE> ww[kWarps];
  Ctx cx;
  stage_surface<kSmemSpans>(s, sm, cx, threadIdx.x, blockDim.x);
  __syncthreads();
  const int warp = threadIdx.x >> 5;
  const int64_t units = (n + 31) / 32;
  for (;;) {
    unsigned ch = 0;
    if ((threadIdx.x & 31) == 0) ch = atomicAdd(counter, 1u);
    ch = __shfl_sync(0xffffffffu, ch, 0);
    if ((int64_t)ch >= units) break;
    const int64_t q0 = (int64_t)ch * 32;
    invert_chunk<P, Q, MODE, kSmemSpans, true>(sm, ww[warp], cx, Pq, q0, min(q0 + 32, n), uv_out, st_out, res_out,
                                               counts);
  }
}

template <int P, int Q, int MODE>
cudaError_t launch_count_mode(const SurfDev& s, const double* P_, int64_t n, double* uv, int* st_, double* res,
                              unsigned* counter, unsigned long long* counts, cudaStream_t st) {
  if ((n + 31) / 32 > 0x3fffffffLL) return cudaErrorInvalidValue;
  int sms = 0;
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int64_t blocks = std::min<int64_t>((n + 32 * kWarps - 1) / (32 * kWarps), (int64_t)(sms > 0 ? sms : 1) * 4);
  k_invert_count<P, Q, MODE><<<(unsigned)blocks, kThreads, 0, st>>>(s, P_, n, uv, st_, res, counter, counts);
  return cudaGetLastError();
}

template <int P, int Q>
cudaError_t launch_count_pq(const SurfDev& s, const double* P_, int64_t n, double* uv, int* st_, double* res,
                            int prec, unsigned* counter, unsigned long long* counts, cudaStream_t st) {
  if (prec == 1) return launch_count_mode<P, Q, kModeMixed>(s, P_, n, uv, st_, res, counter, counts, st);
  return launch_count_mode<P, Q, kModeFP64>(s, P_, n, uv, st_, res, counter, counts, st);
}

// CTAs of a kernel that fit on the current GPU at once (queried once per kernel and device).
template <class K>
int64_t resident_ctas(K kernel) {
  static int cached[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) dev = 0;
  if (!cached[dev]) {
    int sms = 0, per_sm = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kThreads, 0);
    cached[dev] = (sms > 0 ? sms : 1) * (per_sm > 0 ? per_sm : 1);
  }
  return cached[dev];
}

template <int P, int Q, int MODE>
cudaError_t launch_mode(const SurfDev& s, const double* P_, int64_t n, double* uv, int* st_, double* res,
                        unsigned* counter, cudaStream_t st) {
  const int64_t chunks = (n + 31) / 32;
  if (chunks > 0x3fffffffLL) return cudaErrorInvalidValue;  // chunk ids are 32-bit
  int64_t blocks = (chunks + kWarps - 1) / kWarps;
  const int64_t cap = resident_ctas(k_invert<P, Q, MODE>);
  if (blocks > cap) blocks = cap;
  // small chunks for the last two rounds of warps, when there are at least four rounds
  const int64_t warps = cap * kWarps, tail = 2 * warps * 8;
  const int64_t n_big = ((n >= 4 * warps * 32 ? n - tail : n) / 32) * 32;  // a multiple of 32
  k_invert<P, Q, MODE><<<(unsigned)blocks, kThreads, 0, st>>>(s, P_, n, uv, st_, res, counter, n_big);
  return cudaGetLastError();
}

template <int P, int Q>
cudaError_t launch_pq(const SurfDev& s, const double* P_, int64_t n, double* uv, int* st_, double* res, int prec,
                      unsigned* counter, cudaStream_t st) {
  if (prec == 1) return launch_mode<P, Q, kModeMixed>(s, P_, n, uv, st_, res, counter, st);
  return launch_mode<P, Q, kModeFP64>(s, P_, n, uv, st_, res, counter, st);
}

// S, Su, Sv at the uv-centre of every built node, FP32 and FP64: the first iteration of every
// seed starts there, and its evaluation does not depend on the query.  Computed with the same
// device functions and arguments as the seed iterations, so the values are the same bits.
template <int P, int Q>
__device__ void centre_ders(const SurfDev& s, int k) {
  if (k >= kTreeNodes || !s.built[k]) return;
  const TreeNodeDev& T = s.tree[k];
  const double cu = (T.uv_lb[0] + T.uv_rt[0]) / 2, cv = (T.uv_lb[1] + T.uv_rt[1]) / 2;  // kernel.cu:154
  const fast::Locator<float> L32 = fast::global_locator<float>(s);
  const fast::Locator<double> L64 = fast::global_locator<double>(s);
  int hu = 0, hv = 0;
  fast::SDer<float> d = fast::eval_at<float, P, Q, 2, true>(L32, s.m32, s.p, s.q, (float)cu, (float)cv, hu, hv);
  hu = hv = 0;
  fast::SDer<double> e = fast::eval_at<double, P, Q, 2>(L64, s.m64, s.p, s.q, cu, cv, hu, hv);
  const float f[9] = {d.S.x, d.S.y, d.S.z, d.Su.x, d.Su.y, d.Su.z, d.Sv.x, d.Sv.y, d.Sv.z};
  const double g[9] = {e.S.x, e.S.y, e.S.z, e.Su.x, e.Su.y, e.Su.z, e.Sv.x, e.Sv.y, e.Sv.z};
  for (int c = 0; c < 9; ++c) {
    s.cd32[9 * k + c] = f[c];
    s.cd64[9 * k + c] = g[c];
  }
}

template <int P, int Q>
__global__ void k_centre_ders(SurfDev s) {
  centre_ders<P, Q>(s, threadIdx.x);
}

__global__ void k_centre_ders_batched(const SurfDev* __restrict__ table, const int* __restrict__ ids) {
  const SurfDev s = table[ids[blockIdx.x]];
  if (s.p == 3 && s.q == 3) centre_ders<3, 3>(s, threadIdx.x);
  else if (s.p == 5 && s.q == 5) centre_ders<5, 5>(s, threadIdx.x);
  else if (s.p == 2 && s.q == 2) centre_ders<2, 2>(s, threadIdx.x);
  else centre_ders<0, 0>(s, threadIdx.x);
}

}  // namespace

cudaError_t launch_centre_ders(const SurfDev& s, cudaStream_t st) {
  if (s.p == 3 && s.q == 3) k_centre_ders<3, 3><<<1, 96, 0, st>>>(s);
  else if (s.p == 5 && s.q == 5) k_centre_ders<5, 5><<<1, 96, 0, st>>>(s);
  else if (s.p == 2 && s.q == 2) k_centre_ders<2, 2><<<1, 96, 0, st>>>(s);
  else k_centre_ders<0, 0><<<1, 96, 0, st>>>(s);
  return cudaGetLastError();
}

cudaError_t launch_centre_ders_batched(const SurfDev* table, const int* ids, int count, cudaStream_t st) {
  for (int off = 0; off < count; off += 65535) {
    const int c = count - off < 65535 ? count - off : 65535;
    k_centre_ders_batched<<<c, 96, 0, st>>>(table, ids + off);
  }
  return cudaGetLastError();
}

cudaError_t launch_invert_count(const SurfDev& s, const double* P, int64_t n, double* uv, int* status,
                                double* residual, int precision, unsigned* counter, unsigned long long* counts,
                                cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  if (s.p == 3 && s.q == 3) return launch_count_pq<3, 3>(s, P, n, uv, status, residual, precision, counter, counts, st);
  if (s.p == 5 && s.q == 5) return launch_count_pq<5, 5>(s, P, n, uv, status, residual, precision, counter, counts, st);
  return launch_count_pq<0, 0>(s, P, n, uv, status, residual, precision, counter, counts, st);
}

cudaError_t launch_invert(const SurfDev& s, const double* P, int64_t n, double* uv, int* status, double* residual,
                          int precision, unsigned* counter, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  if (s.p == 3 && s.q == 3) return launch_pq<3, 3>(s, P, n, uv, status, residual, precision, counter, st);
  if (s.p == 5 && s.q == 5) return launch_pq<5, 5>(s, P, n, uv, status, residual, precision, counter, st);
  if (s.p == 2 && s.q == 2) return launch_pq<2, 2>(s, P, n, uv, status, residual, precision, counter, st);
  return launch_pq<0, 0>(s, P, n, uv, status, residual, precision, counter, st);
}

}  // namespace gnurbs
