// gpu_nurbs_device.cuh — header-only __host__ __device__ NURBS functions under the reference's
// names, for device code that calls them per point the way the reference's kernels do.
//
// They operate on the reference MatrixN layout (GetMatrixN output, or nurbs_get_matrix_n):
// `middle` points at component 0 of a span, MatrixN + MatrixNPosition(m, n, ...), and holds four
// (p+1)x(q+1) row-major matrices (x.w, y.w, z.w, w).  Arithmetic follows the reference's
// expression order (src/NURBS/Evaluate.cu, src/util/Matrix.cu, src/util/ExtraMath.cu); compiled
// with --fmad=false the values are bit-identical to the reference's FP64 functions, with pow(h,2)
// and pow(h,3) rounded once (h*h and an error-free cube).  The mixed derivative is the correct
// old-style MatrixSurfaceDerivativeUV (Evaluate.cu:743-847); the new-style one with the sign
// error (:956-960) is not provided.
//
//   int     findSpan(degree, cp, knots, u)                               Evaluate.cu:504-533
//   long long MatrixNPosition(i, j, degree_u, degree_v, cp_u, cp_v, c)   Evaluate.cu:110-112
//   d4  MatrixSurfacePoint(middle, degree_u, degree_v, u, v)             Evaluate.cu:159-227
//   d3  homogenousToCartesian(R)                                         ExtraMath.cu:3-5
//   d3  MatrixSurfaceDerivativeU / V (middle, p, q, u, v, R, span)       Evaluate.cu:535-665
//   d3  MatrixSurfaceDerivativeUU / UV / VV (middle, p, q, u, v, R, spanU, spanV)
//                                                                        Evaluate.cu:667-930
// (u, v) are local parameters in [0,1] of the span and spanU = (k[last]-k[0]) / (k[m+1]-k[m]),
// as the reference computes them (e.g. src/kernel/kernel.cu:165-168).  MatrixNPosition returns
// a 64-bit offset (the reference's int wraps past 2^31 doubles).  d4/d3 are plain structs with
// the members of double4/double3.
#pragma once
#include <cuda_runtime.h>

#include "../gpu-nurbs_gb300/csrc/nurbs_math.cuh"

namespace nurbs_device {

struct d4 {
  double x, y, z, w;
};
struct d3 {
  double x, y, z;
};

GN_HD int findSpan(int degree, int cp, const double* knots, double u) {
  int n = cp - 1;
  if (u >= knots[n + 1]) return n;
  if (u <= knots[degree]) return degree;
  int low = degree, high = n + 1;
  int mid = (int)((low + high) / 2.0);
  // bounded bisection: unsorted knots cannot hang the caller
  for (int guard = 0; guard < 64 && (u < knots[mid] || u >= knots[mid + 1]); ++guard) {
    if (u < knots[mid]) high = mid;
    else low = mid;
    mid = (int)((low + high) / 2.0);
  }
  return mid;
}

GN_HD long long MatrixNPosition(int i, int j, int degree_u, int degree_v, int cp_u, int cp_v, int index) {
  (void)cp_u;
  long long k12 = (long long)(degree_u + 1) * (degree_v + 1);
  return (((long long)i * (degree_v + cp_v) + j) * 4 + index) * k12;
}

namespace detail {
GN_HD gnurbs::exact::RefSpan span(const double* middle, int p, int q) { return {middle, p + 1, q + 1}; }
GN_HD d3 to3(const gnurbs::v3<double>& a) { return {a.x, a.y, a.z}; }
GN_HD gnurbs::v4<double> from4(const d4& a) { return {a.x, a.y, a.z, a.w}; }
}  // namespace detail

GN_HD d4 MatrixSurfacePoint(const double* middle, int degree_u, int degree_v, double u, double v) {
  gnurbs::v4<double> r = gnurbs::exact::point_r(detail::span(middle, degree_u, degree_v), degree_u, degree_v, u, v);
  return {r.x, r.y, r.z, r.w};
}
GN_HD d3 homogenousToCartesian(const d4& R) { return {R.x / R.w, R.y / R.w, R.z / R.w}; }

GN_HD d3 MatrixSurfaceDerivativeU(const double* middle, int p, int q, double u, double v, const d4& R, double spanU) {
  return detail::to3(gnurbs::exact::der_u(detail::span(middle, p, q), p, q, u, v, detail::from4(R), spanU));
}
GN_HD d3 MatrixSurfaceDerivativeV(const double* middle, int p, int q, double u, double v, const d4& R, double spanV) {
  return detail::to3(gnurbs::exact::der_v(detail::span(middle, p, q), p, q, u, v, detail::from4(R), spanV));
}
GN_HD d3 MatrixSurfaceDerivativeUU(const double* middle, int p, int q, double u, double v, const d4& R, double spanU,
                                   double /*spanV*/) {
  return detail::to3(gnurbs::exact::der_uu(detail::span(middle, p, q), p, q, u, v, detail::from4(R), spanU));
}
GN_HD d3 MatrixSurfaceDerivativeUV(const double* middle, int p, int q, double u, double v, const d4& R, double spanU,
                                   double spanV) {
  return detail::to3(gnurbs::exact::der_uv(detail::span(middle, p, q), p, q, u, v, detail::from4(R), spanU, spanV));
}
GN_HD d3 MatrixSurfaceDerivativeVV(const double* middle, int p, int q, double u, double v, const d4& R,
                                   double /*spanU*/, double spanV) {
  return detail::to3(gnurbs::exact::der_vv(detail::span(middle, p, q), p, q, u, v, detail::from4(R), spanV));
}

}  // namespace nurbs_device
