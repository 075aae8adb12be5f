// Stage a: knot vectors -> per-span rational power-basis matrices (K1 span_convert).
//
// Replaces GetMatrixN (src/NURBS/Evaluate.cu:3-88).  The reference launches one thread per
// knot pair (i,j), recomputes both basis-to-power matrices per thread with the 4^p-way Nrc
// recursion (:90-103), allocates temporaries on the device heap and multiplies through eight
// dynamic-parallelism child grids.  Here:
//   1. k_basis: one thread per (direction, span, column) evaluates Nrc bottom-up over the
//      recursion depth (each state once, O(p^3) per column); each direction's spans are done
//      once, not once per (i,j).
//   2. k_span_matrices: one thread per (span, homogeneous component) forms W.P_c on the span's
//      (p+1)x(q+1) control net and applies N_u . (W.P_c) . N_v^T with the reference's
//      summation order.
// This translation unit is compiled with --fmad=false: every product and sum rounds as in
// the reference's unfused FP64 arithmetic, so the matrices are bit-identical to GetMatrixN's.
#include "nurbs_internal.h"
#include "nurbs_math.cuh"

namespace gnurbs {

// Nrc table for one span and one column c (1-based): the reference's recurrence
// (src/NURBS/Evaluate.cu:90-103) evaluated bottom-up, each (r, j) entry once, in the
// reference's expression order.  N[r-1][c-1] = Nrc(knot, d, r, c, I, I, d), I = span - (d-1);
// out is the span's (d+1)^2 matrix.
__device__ void basis_column(const double* __restrict__ knot, int d, int span, int c, double* __restrict__ out) {
  const int k = d + 1;
  const int I = span - (d - 1);
  const int R0 = 1 - d, RN = 2 * d + 1;
  const int J0 = I - d, JN = d + 1;
  double prev[(2 * kMaxDegree + 1) * (kMaxDegree + 1)];
  double cur[(2 * kMaxDegree + 1) * (kMaxDegree + 1)];
  for (int ri = 0; ri < RN; ++ri)
    for (int ji = 0; ji < JN; ++ji) {
      int r = R0 + ri, j = J0 + ji;
      prev[ri * JN + ji] = (((I + c - 1) == (j + d)) && (r == 1)) ? 1.0 : 0.0;  // Evaluate.cu:91-95
    }
  // A = Nabla(knot, d, I, 1) = knot[I+d] - knot[I+d-1] (the span length)
  const double A = knot[I + d] - knot[I + d - 1];
  for (int m = 1; m <= d; ++m) {
    for (int r = 1 - (d - m); r <= d + 1; ++r) {
      int ri = r - R0;
      for (int j = I - (d - m); j <= I; ++j) {
        int ji = j - J0;
        double n1 = prev[(ri - 1) * JN + ji];
        double n2 = prev[ri * JN + ji];
        double n3 = prev[ri * JN + (ji - 1)];
        double n4 = prev[(ri - 1) * JN + (ji - 1)];
        // B = Nabla(knot, d, j, d-m+1), C = Nabla(knot, d, j, I-j)   (Evaluate.cu:105-108)
        double B = knot[j + d - 1 + (d - m + 1)] - knot[j + d - 1];
        double C = knot[j + d - 1 + (I - j)] - knot[j + d - 1];
        cur[ri * JN + ji] = A / B * n1 + C / B * n2 + (1 - C / B) * n3 + (-A / B) * n4;  // :98-101
      }
    }
    for (int r = 1 - (d - m); r <= d + 1; ++r)
      for (int j = I - (d - m); j <= I; ++j) prev[(r - R0) * JN + (j - J0)] = cur[(r - R0) * JN + (j - J0)];
  }
  for (int r = 1; r <= d + 1; ++r) out[(r - 1) * k + (c - 1)] = prev[(r - R0) * JN + (I - J0)];
}

__global__ void k_basis(const double* __restrict__ knot, int d, const int* __restrict__ knot_idx, int nspans,
                        double* __restrict__ basis) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  int k = d + 1;
  if (t >= nspans * k) return;
  int sidx = t / k;
  basis_column(knot, d, knot_idx[sidx], t % k + 1, basis + (size_t)sidx * k * k);
}

// Batched over many (surface, direction) jobs: item t belongs to the job with the largest item0 <= t.
__global__ void k_basis_batched(const BasisJob* __restrict__ jobs, int njobs, int64_t nitems) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nitems) return;
  int lo = 0, hi = njobs - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (jobs[mid].item0 <= t) lo = mid;
    else hi = mid - 1;
  }
  const BasisJob J = jobs[lo];
  const int k = J.degree + 1;
  int64_t local = t - J.item0;
  int sidx = (int)(local / k);
  basis_column(J.knots, J.degree, J.knot_idx[sidx], (int)(local % k) + 1, J.out + (size_t)sidx * k * k);
}

// out_c = Nu . (Mid_c . NvT) for one (span, component).  Dense output (m64/m32) or, when
// ref_out != nullptr, the reference MatrixN layout.
__device__ void span_component(const SurfDev& s, const double* __restrict__ basis_u,
                               const double* __restrict__ basis_v, int span, int c, double* __restrict__ m64,
                               float* __restrict__ m32, double* __restrict__ ref_out) {
  int su = span / s.ns_v, sv = span % s.ns_v;
  const int p = s.p, q = s.q, k1 = p + 1, k2 = q + 1;
  const int i = s.knot_u[su], j = s.knot_v[sv];
  const double* Nu = basis_u + (size_t)su * k1 * k1;
  const double* Nv = basis_v + (size_t)sv * k2 * k2;
  double mid[(kMaxDegree + 1) * (kMaxDegree + 1)];
  double tmp[(kMaxDegree + 1) * (kMaxDegree + 1)];
  for (int a = 0; a <= p; ++a)  // Middle_c = P_c * w   (Evaluate.cu:35-43)
    for (int b = 0; b <= q; ++b) {
      size_t idx = (size_t)(a + i - p) * s.nv + (b + j - q);
      double w = s.weights[idx];
      mid[a * k2 + b] = (c < 3) ? s.cps[3 * idx + c] * w : w;
    }
  // temp = Middle . NvT with NvT[t][l] = Nv[l][t]   (matrix_mult, Matrix.cu:43-52 order)
  for (int a = 0; a < k1; ++a)
    for (int l = 0; l < k2; ++l) {
      double acc = 0;
      for (int tt = 0; tt < k2; ++tt) acc += mid[a * k2 + tt] * Nv[l * k2 + tt];
      tmp[a * k2 + l] = acc;
    }
  // out = Nu . temp
  for (int a = 0; a < k1; ++a)
    for (int l = 0; l < k2; ++l) {
      double acc = 0;
      for (int ss = 0; ss < k1; ++ss) acc += Nu[a * k1 + ss] * tmp[ss * k2 + l];
      if (ref_out) {
        // MatrixNPosition(i, j, p, q, nu, nv, c) + a*k2 + l   (Evaluate.cu:110-112)
        size_t pos = (((size_t)i * (q + s.nv) + j) * 4 + c) * (size_t)(k1 * k2) + a * k2 + l;
        ref_out[pos] = acc;
      } else {
        m64[((size_t)span * k1 * k2 + a * k2 + l) * 4 + c] = acc;
        if (c == 3) m32[((size_t)span * span_coefs32(p, q) + a * k2 + l) * 4 + c] = (float)acc;
      }
    }
  if (ref_out || c == 3) return;
  // FP32 table: the same span matrix for the surface translated by -org (the matrix form is
  // linear in the weighted control points: Middle_c = (P_c - org_c) * w), computed in FP64 and
  // rounded once
  for (int a = 0; a <= p; ++a)
    for (int b = 0; b <= q; ++b) {
      size_t idx = (size_t)(a + i - p) * s.nv + (b + j - q);
      mid[a * k2 + b] = (s.cps[3 * idx + c] - s.org[c]) * s.weights[idx];
    }
  for (int a = 0; a < k1; ++a)
    for (int l = 0; l < k2; ++l) {
      double acc = 0;
      for (int tt = 0; tt < k2; ++tt) acc += mid[a * k2 + tt] * Nv[l * k2 + tt];
      tmp[a * k2 + l] = acc;
    }
  for (int a = 0; a < k1; ++a)
    for (int l = 0; l < k2; ++l) {
      double acc = 0;
      for (int ss = 0; ss < k1; ++ss) acc += Nu[a * k1 + ss] * tmp[ss * k2 + l];
      m32[((size_t)span * span_coefs32(p, q) + a * k2 + l) * 4 + c] = (float)acc;
    }
}

__global__ void k_span_matrices(SurfDev s, const double* __restrict__ basis_u, const double* __restrict__ basis_v,
                                double* __restrict__ m64, float* __restrict__ m32, double* __restrict__ ref_out) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= s.ns_u * s.ns_v * 4) return;
  span_component(s, basis_u, basis_v, t >> 2, t & 3, m64, m32, ref_out);
}

__global__ void k_span_matrices_batched(const SurfDev* __restrict__ table, const SpanJob* __restrict__ jobs,
                                        int njobs, int64_t nitems) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nitems) return;
  int lo = 0, hi = njobs - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (jobs[mid].item0 <= t) lo = mid;
    else hi = mid - 1;
  }
  const SurfDev s = table[jobs[lo].surf];
  int64_t local = t - jobs[lo].item0;
  span_component(s, s.basis_u, s.basis_v, (int)(local >> 2), (int)(local & 3), const_cast<double*>(s.m64),
                 const_cast<float*>(s.m32), nullptr);
}

// Dense -> reference MatrixN layout, one thread per double.
__global__ void k_export_ref(SurfDev s, double* __restrict__ ref_out) {
  const int k1 = s.p + 1, k2 = s.q + 1, k12 = k1 * k2;
  int64_t total = (int64_t)s.ns_u * s.ns_v * k12 * 4;
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= total) return;
  int c = (int)(t & 3);
  int64_t e = t >> 2;
  int ab = (int)(e % k12);
  int64_t span = e / k12;
  int su = (int)(span / s.ns_v), sv = (int)(span % s.ns_v);
  int i = s.knot_u[su], j = s.knot_v[sv];
  size_t pos = (((size_t)i * (s.q + s.nv) + j) * 4 + c) * (size_t)k12 + ab;
  ref_out[pos] = s.m64[t];
}

cudaError_t launch_basis(const double* knots, int degree, const int* knot_idx, int nspans, double* basis,
                         cudaStream_t st) {
  int threads = nspans * (degree + 1);
  if (threads <= 0) return cudaSuccess;
  k_basis<<<(threads + 127) / 128, 128, 0, st>>>(knots, degree, knot_idx, nspans, basis);
  return cudaGetLastError();
}

cudaError_t launch_span_matrices(const SurfDev& s, const double* basis_u, const double* basis_v, double* m64,
                                 float* m32, cudaStream_t st) {
  int threads = s.ns_u * s.ns_v * 4;
  if (threads <= 0) return cudaSuccess;
  double* ref_out = (m32 == nullptr) ? m64 : nullptr;
  k_span_matrices<<<(threads + 127) / 128, 128, 0, st>>>(s, basis_u, basis_v, ref_out ? nullptr : m64, m32,
                                                          ref_out);
  return cudaGetLastError();
}

cudaError_t launch_basis_batched(const BasisJob* jobs, int njobs, int64_t nitems, cudaStream_t st) {
  if (nitems <= 0) return cudaSuccess;
  k_basis_batched<<<(unsigned)((nitems + 127) / 128), 128, 0, st>>>(jobs, njobs, nitems);
  return cudaGetLastError();
}

cudaError_t launch_span_matrices_batched(const SurfDev* table, const SpanJob* jobs, int njobs, int64_t nitems,
                                         cudaStream_t st) {
  if (nitems <= 0) return cudaSuccess;
  k_span_matrices_batched<<<(unsigned)((nitems + 127) / 128), 128, 0, st>>>(table, jobs, njobs, nitems);
  return cudaGetLastError();
}

cudaError_t launch_export_ref_layout(const SurfDev& s, double* matrix_n, cudaStream_t st) {
  int64_t total = (int64_t)s.ns_u * s.ns_v * (s.p + 1) * (s.q + 1) * 4;
  if (total <= 0) return cudaSuccess;
  k_export_ref<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(s, matrix_n);
  return cudaGetLastError();
}

}  // namespace gnurbs
