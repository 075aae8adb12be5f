// Batched inversion over a pool of many surfaces of uneven degree, net size and query count,
// in one persistent launch.
//
// The batch is cut on the host into chunks (surface, query range of at most 32 queries, fewer
// when the pool is configured for latency); every warp of the persistent CTAs takes chunks from
// a global atomic counter on its own, stages the chunk's surface (tree boxes, seeds, breakpoint
// tables for up to 64 spans per direction) in its own shared-memory area when it differs from
// its previous chunk's, and inverts the chunk with the same task scheduler as the
// single-surface kernel (invert_core.cuh).  Warps never wait for one another, so a batch of a
// few thousand queries spreads over all SMs.  Degree dispatch: (p,q) in {2,3,5}^2 run
// degree-specialised code, other degrees a run-time-degree path.  Chunk size and CTAs per SM
// are chosen by the pool's autotuner.
#include "invert_core.cuh"

namespace gnurbs {
namespace {

using namespace inv;

// Each degree variant is its own (not inlined) function, so that it keeps its own register
// allocation instead of the kernel taking the union of all variants' live ranges.
constexpr int kPoolSpans = 64;  // breakpoint tables staged per warp up to this many spans

template <int P, int Q, int MODE>
__device__ __noinline__ void chunk_variant(Staged<kPoolSpans, MODE>& sm, WarpWork<MODE>& ww, const Ctx& cx,
                                           const double* __restrict__ P_, int64_t q0, int64_t qend,
                                           double* __restrict__ uv, int* __restrict__ st, double* __restrict__ res) {
  invert_chunk<P, Q, MODE, kPoolSpans>(sm, ww, cx, P_, q0, qend, uv, st, res);
}

template <int MODE>
__device__ __forceinline__ void dispatch_chunk(Staged<kPoolSpans, MODE>& sm, WarpWork<MODE>& ww, const Ctx& cx,
                                               const double* __restrict__ P,
                                               int64_t q0, int64_t qend, double* __restrict__ uv, int* __restrict__ st,
                                               double* __restrict__ res) {
#define GN_CASE(A, B)                                                 \
  if (cx.p == A && cx.q == B) {                                       \
    chunk_variant<A, B, MODE>(sm, ww, cx, P, q0, qend, uv, st, res);  \
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
  chunk_variant<0, 0, MODE>(sm, ww, cx, P, q0, qend, uv, st, res);
}

template <int MODE>
__global__ void __launch_bounds__(kThreads, 4) k_invert_pool(const SurfDev* __restrict__ table,
                                                          const InvTile* __restrict__ tiles, int ntiles,
                                                          int* __restrict__ counter, const double* __restrict__ P,
                                                          double* __restrict__ uv, int* __restrict__ st,
                                                          double* __restrict__ res, int group) {
  __shared__ Staged<kPoolSpans, MODE> sm[kWarps];
  __shared__ WarpWork<MODE> ww[kWarps];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  Ctx cx;
  int cur = -1;
  for (;;) {
    // a group of consecutive chunks (mostly of one surface: chunks are listed surface by
    // surface) per grab, so a warp restages rarely
    int t0 = 0;
    if (lane == 0) t0 = atomicAdd(counter, group);
    t0 = __shfl_sync(0xffffffffu, t0, 0);
    if (t0 >= ntiles) break;
    const int t1 = min(t0 + group, ntiles);
    for (int t = t0; t < t1; ++t) {
      const InvTile T = tiles[t];
      if (T.surf != cur) {
        __syncwarp();
        const SurfDev s = table[T.surf];
        stage_surface<kPoolSpans>(s, sm[warp], cx, lane, 32);
        cur = T.surf;
        __syncwarp();
      }
      dispatch_chunk<MODE>(sm[warp], ww[warp], cx, P, T.begin, T.begin + T.count, uv, st, res);
      __syncwarp();
    }
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

// CTA-granular schedule for large batches: a CTA takes a tile of up to 32*kWarps*k queries of
// one surface, stages the surface once for its four warps, and the warps split the tile's
// 32-query chunks.
constexpr int kCtaSpans = 256;

template <int P, int Q, int MODE>
__device__ __noinline__ void chunk_variant_cta(Staged<kCtaSpans, MODE>& sm, WarpWork<MODE>& ww, const Ctx& cx,
                                               const double* __restrict__ P_, int64_t q0, int64_t qend,
                                               double* __restrict__ uv, int* __restrict__ st,
                                               double* __restrict__ res) {
  invert_chunk<P, Q, MODE, kCtaSpans>(sm, ww, cx, P_, q0, qend, uv, st, res);
}

template <int MODE>
__device__ __forceinline__ void dispatch_chunk_cta(Staged<kCtaSpans, MODE>& sm, WarpWork<MODE>& ww, const Ctx& cx,
                                                   const double* __restrict__ P, int64_t q0, int64_t qend,
                                                   double* __restrict__ uv, int* __restrict__ st,
                                                   double* __restrict__ res) {
#define GN_CASE(A, B)                                                     \
  if (cx.p == A && cx.q == B) {                                           \
    chunk_variant_cta<A, B, MODE>(sm, ww, cx, P, q0, qend, uv, st, res);  \
    return;                                                               \
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
  chunk_variant_cta<0, 0, MODE>(sm, ww, cx, P, q0, qend, uv, st, res);
}

template <int MODE>
__global__ void __launch_bounds__(kThreads, MODE == kModeMixed ? kMinBlocksMixed : 4)
    k_invert_pool_cta(const SurfDev* __restrict__ table,
                                                              const InvTile* __restrict__ tiles, int ntiles,
                                                              int* __restrict__ counter, const double* __restrict__ P,
                                                              double* __restrict__ uv, int* __restrict__ st,
                                                              double* __restrict__ res) {
  __shared__ Staged<kCtaSpans, MODE> sm;
  __shared__ WarpWork<MODE> ww[kWarps];
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
      stage_surface<kCtaSpans>(s, sm, cx, threadIdx.x, blockDim.x);
      cur = T.surf;
      __syncthreads();
    }
    const int nch = (T.count + 31) >> 5;
    for (int c = warp; c < nch; c += kWarps)
      dispatch_chunk_cta<MODE>(sm, ww[warp], cx, P, T.begin + 32 * (int64_t)c, T.begin + T.count, uv, st, res);
    __syncthreads();
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
                               double* uv, int* status, double* residual, int precision, int ctas, int tile_queries,
                               cudaStream_t st) {
  if (ntiles <= 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(int), st);
  if (e != cudaSuccess) return e;
  if (tile_queries > 32) {  // CTA tiles
    if (ctas > ntiles) ctas = ntiles;
    if (precision == 1)
      k_invert_pool_cta<kModeMixed><<<ctas, kThreads, 0, st>>>(table, tiles, ntiles, counter, P, uv, status, residual);
    else
      k_invert_pool_cta<kModeFP64><<<ctas, kThreads, 0, st>>>(table, tiles, ntiles, counter, P, uv, status, residual);
    return cudaGetLastError();
  }
  const int warps_needed = ntiles;
  if (ctas * kWarps > warps_needed) ctas = (warps_needed + kWarps - 1) / kWarps;
  // chunks per grab: large batches take up to 8 at a time, while every warp still gets about
  // eight grabs so the tail stays short
  int group = ntiles / (ctas * kWarps * 8);
  group = group < 1 ? 1 : (group > 8 ? 8 : group);
  if (precision == 1)
    k_invert_pool<kModeMixed><<<ctas, kThreads, 0, st>>>(table, tiles, ntiles, counter, P, uv, status, residual,
                                                          group);
  else
    k_invert_pool<kModeFP64><<<ctas, kThreads, 0, st>>>(table, tiles, ntiles, counter, P, uv, status, residual,
                                                         group);
  return cudaGetLastError();
}

}  // namespace gnurbs
