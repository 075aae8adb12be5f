// Batched inversion over a pool of many surfaces of uneven degree, net size and query count,
// in one persistent launch.
//
// The batch is cut on the host into tiles (surface, query range of at most tile_q queries);
// persistent CTAs (a fixed number per SM) take tiles from a global atomic counter.  A CTA
// stages the tile's surface (tree boxes, seeds, breakpoint tables) in shared memory when it
// differs from the previous tile's, then its warps invert 32-query chunks of the tile with the
// same per-warp task scheduler as the single-surface kernel (invert_core.cuh), dispatching on
// the surface's degrees: (p,q) in {2,3,5}^2 run degree-specialised code, other degrees a
// run-time-degree path.  Tile size and CTAs per SM are chosen by the pool's autotuner.
#include "invert_core.cuh"

namespace gnurbs {
namespace {

using namespace inv;

// Each degree variant is its own (not inlined) function, so that it keeps its own register
// allocation instead of the kernel taking the union of all variants' live ranges.
template <int P, int Q, int MODE>
__device__ __noinline__ void chunk_variant(InvSmem<MODE>& sm, const Ctx& cx, const double* __restrict__ P_,
                                           int64_t q0, int64_t qend, double* __restrict__ uv, int* __restrict__ st,
                                           double* __restrict__ res) {
  invert_chunk<P, Q, MODE>(sm, cx, P_, q0, qend, uv, st, res);
}

template <int MODE>
__device__ __forceinline__ void dispatch_chunk(InvSmem<MODE>& sm, const Ctx& cx, const double* __restrict__ P,
                                               int64_t q0, int64_t qend, double* __restrict__ uv, int* __restrict__ st,
                                               double* __restrict__ res) {
#define GN_CASE(A, B)                                                 \
  if (cx.p == A && cx.q == B) {                                       \
    chunk_variant<A, B, MODE>(sm, cx, P, q0, qend, uv, st, res);      \
    return;                                                           \
  }
  GN_CASE(3, 3)
  GN_CASE(2, 2)
  GN_CASE(5, 5)
  GN_CASE(2, 3)
  GN_CASE(3, 2)
  GN_CASE(2, 5)
  GN_CASE(5, 2)
  GN_CASE(3, 5)
  GN_CASE(5, 3)
#undef GN_CASE
  chunk_variant<0, 0, MODE>(sm, cx, P, q0, qend, uv, st, res);
}

template <int MODE>
__global__ void __launch_bounds__(kThreads, 4) k_invert_pool(const SurfDev* __restrict__ table,
                                                          const InvTile* __restrict__ tiles, int ntiles,
                                                          int* __restrict__ counter, const double* __restrict__ P,
                                                          double* __restrict__ uv, int* __restrict__ st,
                                                          double* __restrict__ res) {
  __shared__ InvSmem<MODE> sm;
  __shared__ int s_tile;
  Ctx cx;
  int cur = -1;
  const int warp = threadIdx.x >> 5;
  for (;;) {
    if (threadIdx.x == 0) s_tile = atomicAdd(counter, 1);
    __syncthreads();
    const int t = s_tile;
    if (t >= ntiles) break;
    const InvTile T = tiles[t];
    if (T.surf != cur) {
      const SurfDev s = table[T.surf];
      stage_surface<MODE>(s, sm, cx);
      cur = T.surf;
      __syncthreads();
    }
    const int nch = (T.count + 31) >> 5;
    for (int c = warp; c < nch; c += kWarps)
      dispatch_chunk<MODE>(sm, cx, P, T.begin + 32 * (int64_t)c, T.begin + T.count, uv, st, res);
    __syncthreads();
  }
}

// Batched FP64 evaluation over tiles: one CTA per tile, one thread per (u,v), run-time degrees.
template <int ORDER>
__global__ void __launch_bounds__(128) k_eval_pool(const SurfDev* __restrict__ table, const InvTile* __restrict__ tiles,
                                                   const double* __restrict__ uv, int64_t n, unsigned mask,
                                                   double* __restrict__ out) {
  const InvTile T = tiles[blockIdx.x];
  const SurfDev s = table[T.surf];
  const fast::Locator<double> L = fast::global_locator<double>(s);
  for (int k = threadIdx.x; k < T.count; k += blockDim.x) {
    const int64_t i = T.begin + k;
    int hu = 0, hv = 0;
    fast::SDer<double> d = fast::eval_at<double, 0, 0, ORDER>(L, s.m64, s.p, s.q, uv[2 * i], uv[2 * i + 1], hu, hv);
    int o = 0;
    auto put = [&](const v3<double>& a) {
      out[(int64_t)(3 * o + 0) * n + i] = a.x;
      out[(int64_t)(3 * o + 1) * n + i] = a.y;
      out[(int64_t)(3 * o + 2) * n + i] = a.z;
      ++o;
    };
    if (mask & 1u) put(d.S);
    if (ORDER >= 1) {
      if (mask & 2u) put(d.Su);
      if (mask & 4u) put(d.Sv);
    }
    if (ORDER >= 2) {
      if (mask & 8u) put(d.Suu);
      if (mask & 16u) put(d.Suv);
      if (mask & 32u) put(d.Svv);
    }
  }
}

}  // namespace

cudaError_t launch_eval_pool(const SurfDev* table, const InvTile* tiles, int ntiles, const double* uv, int64_t n,
                             unsigned mask, double* out, cudaStream_t st) {
  if (ntiles <= 0) return cudaSuccess;
  int order = (mask & 56u) ? 2 : ((mask & 6u) ? 1 : 0);
  if (order == 0) k_eval_pool<0><<<ntiles, 128, 0, st>>>(table, tiles, uv, n, mask, out);
  else if (order == 1) k_eval_pool<1><<<ntiles, 128, 0, st>>>(table, tiles, uv, n, mask, out);
  else k_eval_pool<2><<<ntiles, 128, 0, st>>>(table, tiles, uv, n, mask, out);
  return cudaGetLastError();
}

cudaError_t launch_invert_pool(const SurfDev* table, const InvTile* tiles, int ntiles, int* counter, const double* P,
                               double* uv, int* status, double* residual, int precision, int ctas, int /*unused*/,
                               cudaStream_t st) {
  if (ntiles <= 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(int), st);
  if (e != cudaSuccess) return e;
  if (ctas > ntiles) ctas = ntiles;
  if (precision == 1)
    k_invert_pool<kModeMixed><<<ctas, kThreads, 0, st>>>(table, tiles, ntiles, counter, P, uv, status, residual);
  else
    k_invert_pool<kModeFP64><<<ctas, kThreads, 0, st>>>(table, tiles, ntiles, counter, P, uv, status, residual);
  return cudaGetLastError();
}

}  // namespace gnurbs
