// Drop-in kernels with the reference's own argument lists, working on the reference MatrixN
// layout and raw knot vectors.  Compiled with --fmad=false and written with the
// reference-order functions, so results are bit-identical to its FP64 arithmetic.
#include "nurbs_internal.h"
#include "nurbs_math.cuh"

namespace gnurbs {

// findSpan (src/NURBS/Evaluate.cu:504-533) with the same bisection; the loop is bounded so
// unsorted knots cannot hang a thread (it then returns the last probe).
__device__ int ref_find_span(int degree, int cp, const double* __restrict__ knots, double u) {
  int n = cp - 1;
  if (u >= knots[n + 1]) return n;
  if (u <= knots[degree]) return degree;
  int low = degree, high = n + 1;
  int mid = (int)((low + high) / 2.0);
  for (int guard = 0; guard < 64 && (u < knots[mid] || u >= knots[mid + 1]); ++guard) {
    if (u < knots[mid]) high = mid;
    else low = mid;
    mid = (int)((low + high) / 2.0);
  }
  return mid;
}

// EvaluateRandom (src/NURBS/Evaluate.cu:1023-1038), with the index < n guard the reference lacks.
__global__ void k_evaluate_random(const double* __restrict__ uv, double* __restrict__ xyz, int64_t n,
                                  const double* __restrict__ matrix_n, int p, int q, int nu, int nv,
                                  const double* __restrict__ ku, const double* __restrict__ kv) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double u = uv[2 * i], v = uv[2 * i + 1];
  int m = ref_find_span(p, nu, ku, u);
  int nn = ref_find_span(q, nv, kv, v);
  u = (u - ku[m]) / (ku[m + 1] - ku[m]);
  v = (v - kv[nn]) / (kv[nn + 1] - kv[nn]);
  const int k1 = p + 1, k2 = q + 1;
  size_t pos = (((size_t)m * (q + nv) + nn) * 4) * (size_t)(k1 * k2);  // MatrixNPosition(m, nn, ..., 0)
  exact::RefSpan M{matrix_n + pos, k1, k2};
  v3<double> S = exact::cart(exact::point_r(M, p, q, u, v));
  xyz[3 * i] = S.x;
  xyz[3 * i + 1] = S.y;
  xyz[3 * i + 2] = S.z;
}

// nurbs_eval with NURBS_PREC_EXACT: S and the old-style derivatives to second order
// (MatrixSurfacePoint, MatrixSurfaceDerivative{U,V,UU,UV,VV}, Evaluate.cu:159-227, 535-930) term by
// term, over the surface's span table; bit-identical to the reference's FP64 functions at every
// degree (the Horner path is within 1e-12 for degree <= 3 and within the conditioning of the
// power basis above).
__global__ void __launch_bounds__(128) k_eval_exact(SurfDev s, const double* __restrict__ uv, int64_t n, unsigned mask,
                                                   double* __restrict__ out) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int p = s.p, q = s.q, k2 = q + 1, k12 = (p + 1) * (q + 1);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const double x = uv[2 * i], y = uv[2 * i + 1];
    const int su = exact::find_seg(s.bu, s.ns_u, x), sv = exact::find_seg(s.bv, s.ns_v, y);
    const double du = s.bu[su + 1] - s.bu[su], dv = s.bv[sv + 1] - s.bv[sv];
    const double u = (x - s.bu[su]) / du, v = (y - s.bv[sv]) / dv;
    const double spanU = s.range_u / du, spanV = s.range_v / dv;
    exact::DenseSpan M{s.m64 + (size_t)(su * s.ns_v + sv) * k12 * 4, k2};
    const v4<double> R = exact::point_r(M, p, q, u, v);
    int o = 0;
    auto put = [&](const v3<double>& a) {
      out[(int64_t)(3 * o + 0) * n + i] = a.x;
      out[(int64_t)(3 * o + 1) * n + i] = a.y;
      out[(int64_t)(3 * o + 2) * n + i] = a.z;
      ++o;
    };
    if (mask & 1u) put(exact::cart(R));
    if (mask & 2u) put(exact::der_u(M, p, q, u, v, R, spanU));
    if (mask & 4u) put(exact::der_v(M, p, q, u, v, R, spanV));
    if (mask & 8u) put(exact::der_uu(M, p, q, u, v, R, spanU));
    if (mask & 16u) put(exact::der_uv(M, p, q, u, v, R, spanU, spanV));
    if (mask & 32u) put(exact::der_vv(M, p, q, u, v, R, spanV));
  }
}

cudaError_t launch_eval_exact(const SurfDev& s, const double* uv, int64_t n, unsigned mask, double* out,
                              cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  int64_t blocks = (n + 127) / 128;
  if (blocks > 152 * 64) blocks = 152 * 64;
  k_eval_exact<<<(unsigned)blocks, 128, 0, st>>>(s, uv, n, mask, out);
  return cudaGetLastError();
}

cudaError_t launch_evaluate_random(const double* uv, double* xyz, int64_t n, const double* matrix_n, int p, int q,
                                   int nu, int nv, const double* knots_u, const double* knots_v, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  k_evaluate_random<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(uv, xyz, n, matrix_n, p, q, nu, nv, knots_u,
                                                                  knots_v);
  return cudaGetLastError();
}

}  // namespace gnurbs
