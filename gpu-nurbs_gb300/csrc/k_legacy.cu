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

cudaError_t launch_evaluate_random(const double* uv, double* xyz, int64_t n, const double* matrix_n, int p, int q,
                                   int nu, int nv, const double* knots_u, const double* knots_v, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  k_evaluate_random<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(uv, xyz, n, matrix_n, p, q, nu, nv, knots_u,
                                                                  knots_v);
  return cudaGetLastError();
}

}  // namespace gnurbs
