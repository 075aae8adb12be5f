// Stage b: batched evaluation of points and derivatives up to second order (K2 eval).
//
// Replaces MatrixSurfacePoint / MatrixSurfaceDerivative{U,V,UU,UV,VV}
// (src/NURBS/Evaluate.cu:159-227, 535-930) driven per point as EvaluateRandom does
// (:1023-1038).  The reference recontracts the span matrix once per requested quantity from
// local-memory arrays; here one thread per point streams the span's (p+1)(q+1) 4-vectors of
// coefficients once (two 16-byte __ldg per coefficient, L1/L2-resident span table) through a
// Horner scheme that yields R and all its derivatives to the requested order together, then
// applies the quotient rule once.  Output is SoA, one coalesced streaming store per value.
//
// FP64 cost per point for p = q = 3: 60 / 112 / 152 FMAs for order 0 / 1 / 2 (the
// reference's formulation spends 80 / 176 / 288), plus one reciprocal.
#include "nurbs_internal.h"
#include "nurbs_math.cuh"

namespace gnurbs {

template <typename T>
__device__ __forceinline__ void st_stream(T* p, T v) {
  __stcs(p, v);
}

template <typename T, int P, int Q, int ORDER>
__global__ void __launch_bounds__(256) k_eval(SurfDev s, const T* __restrict__ uv, int64_t n, unsigned mask,
                                              T* __restrict__ out) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    T u = uv[2 * i], v = uv[2 * i + 1];
    fast::SDer<T> d = fast::eval_point<T, P, Q, ORDER>(s, u, v);
    if constexpr (sizeof(T) == 4) {  // FP32 tables hold the surface relative to org
      d.S.x += s.org32[0];
      d.S.y += s.org32[1];
      d.S.z += s.org32[2];
    }
    int o = 0;
    auto put = [&](const v3<T>& a) {
      st_stream(out + (int64_t)(3 * o + 0) * n + i, a.x);
      st_stream(out + (int64_t)(3 * o + 1) * n + i, a.y);
      st_stream(out + (int64_t)(3 * o + 2) * n + i, a.z);
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
    if (ORDER >= 3) {
      if (mask & 64u) put(d.Suuu);
      if (mask & 128u) put(d.Suuv);
      if (mask & 256u) put(d.Suvv);
      if (mask & 512u) put(d.Svvv);
    }
  }
}

// Surface normal N = Su x Sv (not normalised, as the reference's TrueNormal, Evaluate.cu:
// 1111-1117) and its first and second derivatives, the latter as the reference's
// SurfaceNormalDerivative{UU,UV,VV} (Evaluate.cu:1125-1135) with correct third derivatives:
//   Nu = Suu x Sv + Su x Suv,  Nv = Suv x Sv + Su x Svv,
//   Nuu = Suuu x Sv + 2 Suu x Suv + Su x Suuv,  Nuv = Suuv x Sv + Suu x Svv + Su x Suvv,
//   Nvv = Suvv x Sv + 2 Suv x Svv + Su x Svvv.
__device__ __forceinline__ v3<double> cross(const v3<double>& a, const v3<double>& b) {
  return {fast::mad(a.y, b.z, -(a.z * b.y)), fast::mad(a.z, b.x, -(a.x * b.z)), fast::mad(a.x, b.y, -(a.y * b.x))};
}
__device__ __forceinline__ v3<double> add3(const v3<double>& a, const v3<double>& b, double sb, const v3<double>& c) {
  return {fast::mad(sb, b.x, a.x) + c.x, fast::mad(sb, b.y, a.y) + c.y, fast::mad(sb, b.z, a.z) + c.z};
}

template <int P, int Q, int ORDER>
__global__ void __launch_bounds__(256) k_eval_normal(SurfDev s, const double* __restrict__ uv, int64_t n,
                                                     unsigned mask, double* __restrict__ out) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const fast::SDer<double> d = fast::eval_point<double, P, Q, ORDER>(s, uv[2 * i], uv[2 * i + 1]);
    int o = 0;
    auto put = [&](const v3<double>& a) {
      st_stream(out + (int64_t)(3 * o + 0) * n + i, a.x);
      st_stream(out + (int64_t)(3 * o + 1) * n + i, a.y);
      st_stream(out + (int64_t)(3 * o + 2) * n + i, a.z);
      ++o;
    };
    if (mask & 1u) put(cross(d.Su, d.Sv));
    if (ORDER >= 2) {
      if (mask & 2u) put(add3(cross(d.Suu, d.Sv), cross(d.Su, d.Suv), 1.0, {0, 0, 0}));
      if (mask & 4u) put(add3(cross(d.Suv, d.Sv), cross(d.Su, d.Svv), 1.0, {0, 0, 0}));
    }
    if (ORDER >= 3) {
      if (mask & 8u) put(add3(cross(d.Suuu, d.Sv), cross(d.Suu, d.Suv), 2.0, cross(d.Su, d.Suuv)));
      if (mask & 16u) put(add3(cross(d.Suuv, d.Sv), cross(d.Suu, d.Svv), 1.0, cross(d.Su, d.Suvv)));
      if (mask & 32u) put(add3(cross(d.Suvv, d.Sv), cross(d.Suv, d.Svv), 2.0, cross(d.Su, d.Svvv)));
    }
  }
}

static int order_of(unsigned mask) {
  if (mask & (64u | 128u | 256u | 512u)) return 3;
  if (mask & (8u | 16u | 32u)) return 2;
  if (mask & (2u | 4u)) return 1;
  return 0;
}

template <typename T, int P, int Q>
static cudaError_t launch_pq(const SurfDev& s, const T* uv, int64_t n, unsigned mask, T* out, cudaStream_t st) {
  int64_t blocks = (n + 255) / 256;
  const int64_t cap = 152 * 64;
  if (blocks > cap) blocks = cap;
  switch (order_of(mask)) {
    case 0: k_eval<T, P, Q, 0><<<(unsigned)blocks, 256, 0, st>>>(s, uv, n, mask, out); break;
    case 1: k_eval<T, P, Q, 1><<<(unsigned)blocks, 256, 0, st>>>(s, uv, n, mask, out); break;
    case 2: k_eval<T, P, Q, 2><<<(unsigned)blocks, 256, 0, st>>>(s, uv, n, mask, out); break;
    default: k_eval<T, P, Q, 3><<<(unsigned)blocks, 256, 0, st>>>(s, uv, n, mask, out); break;
  }
  return cudaGetLastError();
}

template <int P, int Q>
static cudaError_t launch_normal_pq(const SurfDev& s, const double* uv, int64_t n, unsigned mask, double* out,
                                    cudaStream_t st) {
  int64_t blocks = (n + 255) / 256;
  const int64_t cap = 152 * 64;
  if (blocks > cap) blocks = cap;
  if (mask & (8u | 16u | 32u)) k_eval_normal<P, Q, 3><<<(unsigned)blocks, 256, 0, st>>>(s, uv, n, mask, out);
  else if (mask & (2u | 4u)) k_eval_normal<P, Q, 2><<<(unsigned)blocks, 256, 0, st>>>(s, uv, n, mask, out);
  else k_eval_normal<P, Q, 1><<<(unsigned)blocks, 256, 0, st>>>(s, uv, n, mask, out);
  return cudaGetLastError();
}

template <typename T>
static cudaError_t dispatch(const SurfDev& s, const T* uv, int64_t n, unsigned mask, T* out, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  if (s.p == 3 && s.q == 3) return launch_pq<T, 3, 3>(s, uv, n, mask, out, st);
  if (s.p == 5 && s.q == 5) return launch_pq<T, 5, 5>(s, uv, n, mask, out, st);
  if (s.p == 2 && s.q == 2) return launch_pq<T, 2, 2>(s, uv, n, mask, out, st);
  return launch_pq<T, 0, 0>(s, uv, n, mask, out, st);
}

cudaError_t launch_eval_f64(const SurfDev& s, const double* uv, int64_t n, unsigned mask, double* out,
                            cudaStream_t st) {
  return dispatch<double>(s, uv, n, mask, out, st);
}
cudaError_t launch_eval_f32(const SurfDev& s, const float* uv, int64_t n, unsigned mask, float* out,
                            cudaStream_t st) {
  return dispatch<float>(s, uv, n, mask, out, st);
}
cudaError_t launch_eval_normal(const SurfDev& s, const double* uv, int64_t n, unsigned mask, double* out,
                               cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  if (s.p == 3 && s.q == 3) return launch_normal_pq<3, 3>(s, uv, n, mask, out, st);
  if (s.p == 5 && s.q == 5) return launch_normal_pq<5, 5>(s, uv, n, mask, out, st);
  return launch_normal_pq<0, 0>(s, uv, n, mask, out, st);
}

}  // namespace gnurbs
