// Device math of the GB300 NURBS engine.
//
// Two families:
//  * gnurbs::exact — the reference's FP64 expressions term by term (power vectors by running
//    product, matrix_mult sums from 0 in ascending order, the old-style quotient-rule
//    derivatives of src/NURBS/Evaluate.cu:535-930).  Used where results must be bit-identical
//    to the reference (span conversion, subdivision tree); the translation units that use
//    them are compiled with --fmad=false so that no product is fused into a sum.
//  * gnurbs::fast — Horner contractions of the same span matrices for batched evaluation and
//    Gauss-Newton: one pass over the (p+1)(q+1) coefficient vectors yields R and its
//    derivatives up to second order for all four homogeneous components at once.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include "nurbs_internal.h"

#define GN_HD __host__ __device__ __forceinline__

namespace gnurbs {

template <typename T>
struct v4 {
  T x, y, z, w;
};
template <typename T>
struct v3 {
  T x, y, z;
};

// ------------------------------------------------------------------ exact (reference order)
namespace exact {

// Once-rounded x^3 from an error-free product expansion (TwoProduct via fma).  Equals a
// correctly rounded pow(x, 3) (the reference writes pow(h, 3), Evaluate.cu:737, 844, 926).
GN_HD double cube(double x) {
  double a = x * x;
  double b = fma(x, x, -a);
  double c = a * x;
  double d = fma(a, x, -c);
  double e = b * x;
  return c + (d + e);
}
GN_HD double sq(double x) { return x * x; }  // pow(x, 2): the square rounded once

// Coefficient accessor over the dense span layout [a][b][c].
struct DenseSpan {
  const double* m;
  int k2;
  GN_HD double operator()(int c, int a, int b) const { return m[((a * k2) + b) * 4 + c]; }
};
// Coefficient accessor over the reference MatrixN layout (4 planes of k1 x k2 row-major).
struct RefSpan {
  const double* m;
  int k1, k2;
  GN_HD double operator()(int c, int a, int b) const { return m[(c * k1 + a) * k2 + b]; }
};

GN_HD void power_vec(double t, int k, double* out) {  // Evaluate.cu:172-181
  double now = 1;
  for (int i = 0; i < k; i++) {
    out[i] = now;
    now *= t;
  }
}
GN_HD void dpower_vec(double t, int k, double* out) {  // Evaluate.cu:540-545
  double now = 1;
  out[0] = 0;
  for (int i = 0; i < k - 1; i++) {
    out[i + 1] = (i + 1) * now;
    now *= t;
  }
}
GN_HD void ddpower_vec(double t, int k, double* out) {  // Evaluate.cu:680-685
  double now = 1;
  out[0] = 0;
  if (k > 1) out[1] = 0;
  for (int i = 0; i < k - 2; i++) {
    out[i + 2] = (i + 2) * (i + 1) * now;
    now *= t;
  }
}

// temp_c[a] = sum_b M_c[a][b] * vec[b]  (matrix_mult(middle_c, vec, temp_c, k1, k2, 1))
template <class Acc>
GN_HD void mv(const Acc& M, int k1, int k2, const double* vec, double (*tmp)[kMaxDegree + 1]) {
  for (int c = 0; c < 4; ++c)
    for (int a = 0; a < k1; ++a) {
      double acc = 0;
      for (int b = 0; b < k2; ++b) acc += M(c, a, b) * vec[b];
      tmp[c][a] = acc;
    }
}
// temp_c[b] = sum_a vec[a] * M_c[a][b]  (matrix_mult(vectorUT, middle_c, temp_c, 1, k1, k2))
template <class Acc>
GN_HD void vm(const Acc& M, int k1, int k2, const double* vec, double (*tmp)[kMaxDegree + 1]) {
  for (int c = 0; c < 4; ++c)
    for (int b = 0; b < k2; ++b) {
      double acc = 0;
      for (int a = 0; a < k1; ++a) acc += vec[a] * M(c, a, b);
      tmp[c][b] = acc;
    }
}
GN_HD double dotk(const double* a, const double* b, int k) {
  double acc = 0;
  for (int l = 0; l < k; ++l) acc += a[l] * b[l];
  return acc;
}
GN_HD v4<double> dot4(const double* vec, double (*tmp)[kMaxDegree + 1], int k) {
  return {dotk(vec, tmp[0], k), dotk(vec, tmp[1], k), dotk(vec, tmp[2], k), dotk(vec, tmp[3], k)};
}

// MatrixSurfacePoint (Evaluate.cu:159-227)
template <class Acc>
GN_HD v4<double> point_r(const Acc& M, int p, int q, double u, double v) {
  double U[kMaxDegree + 1], V[kMaxDegree + 1], tmp[4][kMaxDegree + 1];
  power_vec(u, p + 1, U);
  power_vec(v, q + 1, V);
  mv(M, p + 1, q + 1, V, tmp);
  return dot4(U, tmp, p + 1);
}
GN_HD v3<double> cart(v4<double> R) { return {R.x / R.w, R.y / R.w, R.z / R.w}; }  // ExtraMath.cu:3-5

// old MatrixSurfaceDerivativeU (Evaluate.cu:535-598)
template <class Acc>
GN_HD v3<double> der_u(const Acc& M, int p, int q, double u, double v, v4<double> R, double spanU) {
  double dU[kMaxDegree + 1], V[kMaxDegree + 1], tmp[4][kMaxDegree + 1];
  dpower_vec(u, p + 1, dU);
  power_vec(v, q + 1, V);
  mv(M, p + 1, q + 1, V, tmp);
  v4<double> RdU = dot4(dU, tmp, p + 1);
  double h = R.w, hdU = RdU.w, s = -hdU / sq(h);
  return {(R.x * s + RdU.x / h) * spanU, (R.y * s + RdU.y / h) * spanU, (R.z * s + RdU.z / h) * spanU};
}
// old MatrixSurfaceDerivativeV (Evaluate.cu:600-665)
template <class Acc>
GN_HD v3<double> der_v(const Acc& M, int p, int q, double u, double v, v4<double> R, double spanV) {
  double U[kMaxDegree + 1], dV[kMaxDegree + 1], tmp[4][kMaxDegree + 1];
  power_vec(u, p + 1, U);
  dpower_vec(v, q + 1, dV);
  mv(M, p + 1, q + 1, dV, tmp);
  v4<double> RdV = dot4(U, tmp, p + 1);
  double h = R.w, hdV = RdV.w, s = -hdV / sq(h);
  return {(R.x * s + RdV.x / h) * spanV, (R.y * s + RdV.y / h) * spanV, (R.z * s + RdV.z / h) * spanV};
}
// old MatrixSurfaceDerivativeUU (Evaluate.cu:667-741)
template <class Acc>
GN_HD v3<double> der_uu(const Acc& M, int p, int q, double u, double v, v4<double> R, double spanU) {
  double dU[kMaxDegree + 1], ddU[kMaxDegree + 1], V[kMaxDegree + 1], tmp[4][kMaxDegree + 1];
  dpower_vec(u, p + 1, dU);
  ddpower_vec(u, p + 1, ddU);
  power_vec(v, q + 1, V);
  mv(M, p + 1, q + 1, V, tmp);
  v4<double> RdU = dot4(dU, tmp, p + 1);
  v4<double> RdUU = dot4(ddU, tmp, p + 1);
  double h = R.w, hdU = RdU.w, hdUU = RdUU.w;
  double s1 = (2 * sq(hdU) / cube(h)) - (hdUU / sq(h));
  double s2 = -hdU / sq(h);
  return {((R.x * s1 + (2 * RdU.x) * s2) + RdUU.x / h) * spanU * spanU,
          ((R.y * s1 + (2 * RdU.y) * s2) + RdUU.y / h) * spanU * spanU,
          ((R.z * s1 + (2 * RdU.z) * s2) + RdUU.z / h) * spanU * spanU};
}
// old MatrixSurfaceDerivativeUV (Evaluate.cu:743-847) — the correct-sign mixed derivative
template <class Acc>
GN_HD v3<double> der_uv(const Acc& M, int p, int q, double u, double v, v4<double> R, double spanU,
                        double spanV) {
  double U[kMaxDegree + 1], dU[kMaxDegree + 1], V[kMaxDegree + 1], dV[kMaxDegree + 1];
  double tmp[4][kMaxDegree + 1];
  power_vec(u, p + 1, U);
  dpower_vec(u, p + 1, dU);
  power_vec(v, q + 1, V);
  dpower_vec(v, q + 1, dV);
  mv(M, p + 1, q + 1, V, tmp);
  v4<double> RdU = dot4(dU, tmp, p + 1);
  mv(M, p + 1, q + 1, dV, tmp);
  v4<double> RdV = dot4(U, tmp, p + 1);
  v4<double> RdUV = dot4(dU, tmp, p + 1);
  double h = R.w, hdU = RdU.w, hdV = RdV.w, hdUV = RdUV.w;
  double h2 = sq(h), h3 = cube(h);
  return {((((RdUV.x * h - hdV * RdU.x) - RdV.x * hdU) - R.x * hdUV) / h2 + ((2 * R.x) * hdU * hdV) / h3) * spanU * spanV,
          ((((RdUV.y * h - hdV * RdU.y) - RdV.y * hdU) - R.y * hdUV) / h2 + ((2 * R.y) * hdU * hdV) / h3) * spanU * spanV,
          ((((RdUV.z * h - hdV * RdU.z) - RdV.z * hdU) - R.z * hdUV) / h2 + ((2 * R.z) * hdU * hdV) / h3) * spanU * spanV};
}
// old MatrixSurfaceDerivativeVV (Evaluate.cu:849-930): contracts U first
template <class Acc>
GN_HD v3<double> der_vv(const Acc& M, int p, int q, double u, double v, v4<double> R, double spanV) {
  double U[kMaxDegree + 1], dV[kMaxDegree + 1], ddV[kMaxDegree + 1], tmp[4][kMaxDegree + 1];
  power_vec(u, p + 1, U);
  dpower_vec(v, q + 1, dV);
  ddpower_vec(v, q + 1, ddV);
  vm(M, p + 1, q + 1, U, tmp);
  v4<double> RdV = dot4(dV, tmp, q + 1);
  v4<double> RdVV = dot4(ddV, tmp, q + 1);
  double h = R.w, hdV = RdV.w, hdVV = RdVV.w;
  double s1 = (2 * sq(hdV) / cube(h)) - (hdVV / sq(h));
  double s2 = -hdV / sq(h);
  return {((R.x * s1 + (2 * RdV.x) * s2) + RdVV.x / h) * spanV * spanV,
          ((R.y * s1 + (2 * RdV.y) * s2) + RdVV.y / h) * spanV * spanV,
          ((R.z * s1 + (2 * RdV.z) * s2) + RdVV.z / h) * spanV * spanV};
}

// ---- third order and normals in the new-style quotient rule (the normal-cone build)
// Power vectors and their derivatives (GetVector, src/kernel/kernel.cu:1386-1450), R-derivatives
// as U^(a) . (M_c . V^(b)) scaled by spanU^a spanV^b, S = R.xyz / h and the quotient rule with
// its signs (the reference's mixed third derivatives, Evaluate.cu:963-1020, add two of the terms
// they subtract).  Term order as written, so the normal cones are bit-identical to the oracle's.
GN_HD void vectors_k(double t, int k, double* V0, double* V1, double* V2, double* V3) {
  double now = 1;
  for (int i = 0; i < k; i++) {
    V0[i] = now;
    now *= t;
  }
  V1[0] = 0;
  for (int i = 0; i < k - 1; i++) V1[i + 1] = (i + 1) * V0[i];
  V2[0] = 0;
  if (k > 1) V2[1] = 0;
  for (int i = 0; i < k - 2; i++) V2[i + 2] = (i + 2) * (i + 1) * V0[i];
  V3[0] = 0;
  if (k > 1) V3[1] = 0;
  if (k > 2) V3[2] = 0;
  for (int i = 0; i < k - 3; i++) V3[i + 3] = (i + 3) * (i + 2) * (i + 1) * V0[i];
}
template <class Acc>
GN_HD v4<double> rd(const Acc& M, int k1, int k2, const double* vu, const double* vv) {
  double tmp[4][kMaxDegree + 1];
  mv(M, k1, k2, vv, tmp);
  return dot4(vu, tmp, k1);
}
// the same contracting u first (MatrixSurfaceRdVV, Evaluate.cu:384-405)
template <class Acc>
GN_HD v4<double> rd_ufirst(const Acc& M, int k1, int k2, const double* vu, const double* vv) {
  double tmp[4][kMaxDegree + 1];
  vm(M, k1, k2, vu, tmp);
  return dot4(vv, tmp, k2);
}
GN_HD v4<double> scale4(v4<double> a, double s) { return {a.x * s, a.y * s, a.z * s, a.w * s}; }
GN_HD v3<double> cross(v3<double> a, v3<double> b) {  // cross_product, src/util/Matrix.cu:62-64
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
GN_HD v3<double> add(v3<double> a, v3<double> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
GN_HD v3<double> twice(v3<double> a) { return {2 * a.x, 2 * a.y, 2 * a.z}; }

// d[0..9] = S, Su, Sv, Suu, Suv, Svv, Suuu, Suuv, Suvv, Svvv at local (u, v) of span M.
template <class Acc>
GN_HD void ders3(const Acc& M, int p, int q, double u, double v, double su, double sv, v3<double>* d) {
  const int k1 = p + 1, k2 = q + 1;
  double U[4][kMaxDegree + 1], V[4][kMaxDegree + 1];
  vectors_k(u, k1, U[0], U[1], U[2], U[3]);
  vectors_k(v, k2, V[0], V[1], V[2], V[3]);
  const v4<double> R = rd(M, k1, k2, U[0], V[0]);
  const v4<double> Ru = scale4(rd(M, k1, k2, U[1], V[0]), su);
  const v4<double> Rv = scale4(rd(M, k1, k2, U[0], V[1]), sv);
  const v4<double> Ruu = scale4(scale4(rd(M, k1, k2, U[2], V[0]), su), su);
  const v4<double> Ruv = scale4(scale4(rd(M, k1, k2, U[1], V[1]), su), sv);
  const v4<double> Rvv = scale4(scale4(rd_ufirst(M, k1, k2, U[0], V[2]), sv), sv);
  const v4<double> Ruuu = scale4(scale4(scale4(rd(M, k1, k2, U[3], V[0]), su), su), su);
  const v4<double> Ruuv = scale4(scale4(scale4(rd(M, k1, k2, U[2], V[1]), su), su), sv);
  const v4<double> Ruvv = scale4(scale4(scale4(rd(M, k1, k2, U[1], V[2]), su), sv), sv);
  const v4<double> Rvvv = scale4(scale4(scale4(rd(M, k1, k2, U[0], V[3]), sv), sv), sv);
  const double h = R.w, hu = Ru.w, hv = Rv.w, huu = Ruu.w, huv = Ruv.w, hvv = Rvv.w;
  const double Rs[10][3] = {{R.x, R.y, R.z},          {Ru.x, Ru.y, Ru.z},       {Rv.x, Rv.y, Rv.z},
                            {Ruu.x, Ruu.y, Ruu.z},    {Ruv.x, Ruv.y, Ruv.z},    {Rvv.x, Rvv.y, Rvv.z},
                            {Ruuu.x, Ruuu.y, Ruuu.z}, {Ruuv.x, Ruuv.y, Ruuv.z}, {Ruvv.x, Ruvv.y, Ruvv.z},
                            {Rvvv.x, Rvvv.y, Rvvv.z}};
  double o[10][3];
  for (int c = 0; c < 3; ++c) {
    o[0][c] = Rs[0][c] / h;
    o[1][c] = (Rs[1][c] - hu * o[0][c]) / h;
    o[2][c] = (Rs[2][c] - hv * o[0][c]) / h;
    o[3][c] = ((Rs[3][c] - 2 * hu * o[1][c]) - huu * o[0][c]) / h;
    o[4][c] = (((Rs[4][c] - hv * o[1][c]) - hu * o[2][c]) - huv * o[0][c]) / h;
    o[5][c] = ((Rs[5][c] - 2 * hv * o[2][c]) - hvv * o[0][c]) / h;
    o[6][c] = (((Rs[6][c] - 3 * hu * o[3][c]) - 3 * huu * o[1][c]) - Ruuu.w * o[0][c]) / h;
    o[7][c] = (((((Rs[7][c] - hv * o[3][c]) - 2 * hu * o[4][c]) - 2 * huv * o[1][c]) - huu * o[2][c]) -
               Ruuv.w * o[0][c]) / h;
    o[8][c] = (((((Rs[8][c] - hu * o[5][c]) - 2 * hv * o[4][c]) - 2 * huv * o[2][c]) - hvv * o[1][c]) -
               Ruvv.w * o[0][c]) / h;
    o[9][c] = (((Rs[9][c] - 3 * hv * o[5][c]) - 3 * hvv * o[2][c]) - Rvvv.w * o[0][c]) / h;
  }
  for (int b = 0; b < 10; ++b) d[b] = {o[b][0], o[b][1], o[b][2]};
}

// N = Su x Sv and N_uu, N_uv, N_vv (n[0..3]) from ders3's d.
GN_HD void normal_ders2(const v3<double>* d, v3<double>* n) {
  n[0] = cross(d[1], d[2]);
  n[1] = add(add(cross(d[6], d[2]), twice(cross(d[3], d[4]))), cross(d[1], d[7]));
  n[2] = add(add(add(cross(d[7], d[2]), cross(d[3], d[5])), cross(d[4], d[4])), cross(d[1], d[8]));
  n[3] = add(add(cross(d[8], d[2]), twice(cross(d[4], d[5]))), cross(d[1], d[9]));
}

// findSpan semantics over the breakpoints of the domain: the largest s in [0, ns-1] with
// b[s] <= x (x below the domain -> 0, at or above its end -> ns-1), i.e. the knot span m with
// k[m] <= x < k[m+1] that findSpan (Evaluate.cu:504-533) returns.  Bounded; NaN -> 0.
GN_HD int find_seg(const double* b, int ns, double x) {
  int lo = 0;
  int step = 1;
  while ((step << 1) <= ns) step <<= 1;
  for (; step > 0; step >>= 1) {
    int t = lo + step;
    if (t < ns && b[t] <= x) lo = t;
  }
  return lo;
}

}  // namespace exact

// ------------------------------------------------------------------------ fast (Horner)
namespace fast {

GN_HD double mad(double a, double b, double c) { return fma(a, b, c); }
GN_HD float mad(float a, float b, float c) { return fmaf(a, b, c); }

template <typename T>
GN_HD v4<T> vmad(const v4<T>& a, T s, const v4<T>& c) {
  return {mad(a.x, s, c.x), mad(a.y, s, c.y), mad(a.z, s, c.z), mad(a.w, s, c.w)};
}
// FP32 on the device: two packed two-wide FMAs (sm_100 and later) instead of four, each
// component the same round-to-nearest fused multiply-add as fmaf, so no result changes.
template <>
GN_HD v4<float> vmad<float>(const v4<float>& a, float s, const v4<float>& c) {
#ifdef __CUDA_ARCH__
  const float2 ss = make_float2(s, s);
  const float2 lo = __ffma2_rn(make_float2(a.x, a.y), ss, make_float2(c.x, c.y));
  const float2 hi = __ffma2_rn(make_float2(a.z, a.w), ss, make_float2(c.z, c.w));
  return {lo.x, lo.y, hi.x, hi.y};
#else
  return {mad(a.x, s, c.x), mad(a.y, s, c.y), mad(a.z, s, c.z), mad(a.w, s, c.w)};
#endif
}

// Coefficient loads through the read-only path.  An FP64 coefficient (32 bytes, 32-byte
// aligned) is one 256-bit load; two adjacent FP32 coefficients starting at an even index of a
// 32-byte aligned table are one 256-bit load too, halving the load instructions and the L1
// wavefronts of the gathers, which bound the FP32 evaluation.
__device__ __forceinline__ v4<double> load_coef(const double* m, int idx) {
  v4<double> c;
  asm("ld.global.nc.v4.f64 {%0, %1, %2, %3}, [%4];"
      : "=d"(c.x), "=d"(c.y), "=d"(c.z), "=d"(c.w)
      : "l"(m + 4 * idx));
  return c;
}
__device__ __forceinline__ v4<float> load_coef(const float* m, int idx) {
  float4 f = __ldg(reinterpret_cast<const float4*>(m + 4 * idx));
  return {f.x, f.y, f.z, f.w};
}
// coefficients idx (lo) and idx + 1 (hi); idx even, table 32-byte aligned
__device__ __forceinline__ void load_coef_pair(const float* m, int idx, v4<float>& lo, v4<float>& hi) {
  asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=f"(lo.x), "=f"(lo.y), "=f"(lo.z), "=f"(lo.w), "=f"(hi.x), "=f"(hi.y), "=f"(hi.z), "=f"(hi.w)
      : "l"(m + 4 * idx));
}
__device__ __forceinline__ void load_coef_pair(const double* m, int idx, v4<double>& lo, v4<double>& hi) {
  lo = load_coef(m, idx);
  hi = load_coef(m, idx + 1);
}

// Horner accumulator tracking value and D derivatives (D <= 3).  Coefficients are pushed from
// the highest power down; after all pushes p = f(x), dp = f'(x), ddp = f''(x)/2 and dddp = the
// third derivative / 6.  The first pushes are peeled so no FMA is spent on zero accumulators.
template <typename T, int D>
struct Horner {
  v4<T> p, dp, ddp, dddp;
  int k;
  // dp/ddp/dddp start at zero: a polynomial of degree < D has vanishing higher derivatives
  GN_HD Horner()
      : dp{T(0), T(0), T(0), T(0)}, ddp{T(0), T(0), T(0), T(0)}, dddp{T(0), T(0), T(0), T(0)}, k(0) {}
  GN_HD void push(const v4<T>& c, T x) {
    if (k == 0) {
      p = c;
    } else {
      if (D >= 3) {
        if (k == 3) dddp = ddp;
        else if (k > 3) dddp = vmad(dddp, x, ddp);
      }
      if (D >= 2) {
        if (k == 2) ddp = dp;
        else if (k > 2) ddp = vmad(ddp, x, dp);
      }
      if (D >= 1) {
        if (k == 1) dp = p;
        else dp = vmad(dp, x, p);
      }
      p = vmad(p, x, c);
    }
    ++k;
  }
};

template <typename T>
GN_HD v4<T> zero4() {
  return {T(0), T(0), T(0), T(0)};
}

// Homogeneous R and its local derivatives at local (u,v) in one span.
//   ORDER 0: R; ORDER 1: + Ru, Rv; ORDER 2: + Ruu, Ruv, Rvv.
// P, Q > 0 fix the degrees at compile time; P = Q = 0 reads p, q at run time.
template <typename T>
struct RDer {
  v4<T> R, Ru, Rv, Ruu, Ruv, Rvv, Ruuu, Ruuv, Ruvv, Rvvv;
};

template <typename T, int P, int Q, int ORDER>
__device__ __forceinline__ RDer<T> span_contract(const T* __restrict__ m, int p_rt, int q_rt, T u, T v) {
  const int pp = P > 0 ? P : p_rt;
  const int qq = Q > 0 ? Q : q_rt;
  const int k2 = qq + 1;
  constexpr int DR = ORDER;                  // derivatives of the u-Horner over t_a
  constexpr int DV = ORDER >= 1 ? ORDER - 1 : 0;
  constexpr int DVV = ORDER >= 2 ? ORDER - 2 : 0;
  Horner<T, DR> colR;
  Horner<T, DV> colV;
  Horner<T, DVV> colVV;
  Horner<T, 0> colVVV;
#pragma unroll
  for (int a = (P > 0 ? P : kMaxDegree); a >= 0; --a) {
    if (P == 0 && a > pp) continue;
    Horner<T, ORDER> row;
    if constexpr (P > 0 && Q > 0) {
      // Spans start at an even coefficient index, so coefficients (a, b-1) and (a, b) share
      // one aligned 256-bit load when a*(q+1) + b - 1 is even; a coefficient left over at
      // either end of the row is loaded alone.
      int b = Q;
      if (((a * k2 + b - 1) & 1) && b >= 0) {  // row starts on an unpaired coefficient
        row.push(load_coef(m, a * k2 + b), v);
        --b;
      }
#pragma unroll
      for (; b >= 1; b -= 2) {
        v4<T> lo, hi;
        load_coef_pair(m, a * k2 + b - 1, lo, hi);
        row.push(hi, v);
        row.push(lo, v);
      }
      if (b == 0) row.push(load_coef(m, a * k2), v);
    } else {
#pragma unroll
      for (int b = (Q > 0 ? Q : kMaxDegree); b >= 0; --b) {
        if (Q == 0 && b > qq) continue;
        row.push(load_coef(m, a * k2 + b), v);
      }
    }
    colR.push(row.p, u);
    if (ORDER >= 1) colV.push(row.dp, u);
    if (ORDER >= 2) colVV.push(row.ddp, u);
    if (ORDER >= 3) colVVV.push(row.dddp, u);
  }
  RDer<T> o;
  o.R = colR.p;
  if (ORDER >= 1) {
    o.Ru = colR.dp;
    o.Rv = colV.p;
  }
  if (ORDER >= 2) {
    o.Ruu = {T(2) * colR.ddp.x, T(2) * colR.ddp.y, T(2) * colR.ddp.z, T(2) * colR.ddp.w};
    o.Ruv = colV.dp;
    o.Rvv = {T(2) * colVV.p.x, T(2) * colVV.p.y, T(2) * colVV.p.z, T(2) * colVV.p.w};
  }
  if (ORDER >= 3) {
    o.Ruuu = {T(6) * colR.dddp.x, T(6) * colR.dddp.y, T(6) * colR.dddp.z, T(6) * colR.dddp.w};
    o.Ruuv = {T(2) * colV.ddp.x, T(2) * colV.ddp.y, T(2) * colV.ddp.z, T(2) * colV.ddp.w};
    o.Ruvv = {T(2) * colVV.dp.x, T(2) * colVV.dp.y, T(2) * colVV.dp.z, T(2) * colVV.dp.w};
    o.Rvvv = {T(6) * colVVV.p.x, T(6) * colVVV.p.y, T(6) * colVVV.p.z, T(6) * colVVV.p.w};
  }
  return o;
}

// Cartesian point and derivatives with respect to the global parameters.
template <typename T>
struct SDer {
  v3<T> S, Su, Sv, Suu, Suv, Svv, Suuu, Suuv, Suvv, Svvv;
};

template <typename T>
GN_HD v3<T> xyz(const v4<T>& a) {
  return {a.x, a.y, a.z};
}
// (a - s*b) * f, componentwise, s scalar
template <typename T>
GN_HD v3<T> sub_scaled(const v3<T>& a, T s, const v3<T>& b, T f) {
  return {mad(-s, b.x, a.x) * f, mad(-s, b.y, a.y) * f, mad(-s, b.z, a.z) * f};
}

// 1/x: IEEE in FP64; in FP32 either IEEE or the hardware approximation (about 1 ulp), which the
// FP32 exploration of the inversion uses since its results are refined in FP64 anyway.
template <bool FAST>
__device__ __forceinline__ float rcp(float x) {
  if constexpr (FAST) return __fdividef(1.0f, x);
  else return 1.0f / x;
}
template <bool FAST>
__device__ __forceinline__ double rcp(double x) {
  return 1.0 / x;
}

// Quotient rule S = R.xyz / h and its derivatives (h = R.w), mapped to global parameters
// by su = d(local u)/du and sv.  Every product that feeds a sum is an explicit FMA, so the
// results do not depend on how the compiler contracts the surrounding code.
template <typename T, int ORDER, bool FAST = false>
__device__ __forceinline__ SDer<T> quotient(const RDer<T>& d, T su, T sv) {
  SDer<T> o;
  T ih = rcp<FAST>(d.R.w);
  o.S = {d.R.x * ih, d.R.y * ih, d.R.z * ih};
  if (ORDER >= 1) {
    v3<T> Au = sub_scaled(xyz(d.Ru), d.Ru.w, o.S, ih);  // local dS/du
    v3<T> Av = sub_scaled(xyz(d.Rv), d.Rv.w, o.S, ih);
    if (ORDER >= 2) {
      T hu2 = T(2) * d.Ru.w, hv2 = T(2) * d.Rv.w, hu = d.Ru.w, hv = d.Rv.w;
      v3<T> Auu = {mad(-d.Ruu.w, o.S.x, mad(-hu2, Au.x, d.Ruu.x)) * ih,
                   mad(-d.Ruu.w, o.S.y, mad(-hu2, Au.y, d.Ruu.y)) * ih,
                   mad(-d.Ruu.w, o.S.z, mad(-hu2, Au.z, d.Ruu.z)) * ih};
      v3<T> Auv = {mad(-d.Ruv.w, o.S.x, mad(-hv, Au.x, mad(-hu, Av.x, d.Ruv.x))) * ih,
                   mad(-d.Ruv.w, o.S.y, mad(-hv, Au.y, mad(-hu, Av.y, d.Ruv.y))) * ih,
                   mad(-d.Ruv.w, o.S.z, mad(-hv, Au.z, mad(-hu, Av.z, d.Ruv.z))) * ih};
      v3<T> Avv = {mad(-d.Rvv.w, o.S.x, mad(-hv2, Av.x, d.Rvv.x)) * ih,
                   mad(-d.Rvv.w, o.S.y, mad(-hv2, Av.y, d.Rvv.y)) * ih,
                   mad(-d.Rvv.w, o.S.z, mad(-hv2, Av.z, d.Rvv.z)) * ih};
      T suu = su * su, suv = su * sv, svv = sv * sv;
      o.Suu = {Auu.x * suu, Auu.y * suu, Auu.z * suu};
      o.Suv = {Auv.x * suv, Auv.y * suv, Auv.z * suv};
      o.Svv = {Avv.x * svv, Avv.y * svv, Avv.z * svv};
      if (ORDER >= 3) {
        // R = S h differentiated three times (the reference's UUV/UVV forms, Evaluate.cu:963-1020,
        // carry two wrong signs; these are the quotient rule's):
        //   S_uuu = (R_uuu - 3 h_u S_uu - 3 h_uu S_u - h_uuu S) / h
        //   S_uuv = (R_uuv - h_v S_uu - 2 h_u S_uv - 2 h_uv S_u - h_uu S_v - h_uuv S) / h
        const T huu = d.Ruu.w, huv = d.Ruv.w, hvv = d.Rvv.w;
        const T hu3 = T(3) * hu, hv3 = T(3) * hv, huu3 = T(3) * huu, hvv3 = T(3) * hvv, huv2 = T(2) * huv;
        auto c3 = [&](T r, T a2, T a1, T s, T k2, T k1, T k0) { return mad(-k0, s, mad(-k1, a1, mad(-k2, a2, r))) * ih; };
        v3<T> Auuu = {c3(d.Ruuu.x, Auu.x, Au.x, o.S.x, hu3, huu3, d.Ruuu.w),
                      c3(d.Ruuu.y, Auu.y, Au.y, o.S.y, hu3, huu3, d.Ruuu.w),
                      c3(d.Ruuu.z, Auu.z, Au.z, o.S.z, hu3, huu3, d.Ruuu.w)};
        v3<T> Avvv = {c3(d.Rvvv.x, Avv.x, Av.x, o.S.x, hv3, hvv3, d.Rvvv.w),
                      c3(d.Rvvv.y, Avv.y, Av.y, o.S.y, hv3, hvv3, d.Rvvv.w),
                      c3(d.Rvvv.z, Avv.z, Av.z, o.S.z, hv3, hvv3, d.Rvvv.w)};
        auto c5 = [&](T r, T a_aa, T a_ab, T a_a, T a_b, T s, T hb, T ha2, T hab2, T haa, T h3w) {
          return mad(-h3w, s, mad(-haa, a_b, mad(-hab2, a_a, mad(-ha2, a_ab, mad(-hb, a_aa, r))))) * ih;
        };
        v3<T> Auuv = {c5(d.Ruuv.x, Auu.x, Auv.x, Au.x, Av.x, o.S.x, hv, hu2, huv2, huu, d.Ruuv.w),
                      c5(d.Ruuv.y, Auu.y, Auv.y, Au.y, Av.y, o.S.y, hv, hu2, huv2, huu, d.Ruuv.w),
                      c5(d.Ruuv.z, Auu.z, Auv.z, Au.z, Av.z, o.S.z, hv, hu2, huv2, huu, d.Ruuv.w)};
        v3<T> Auvv = {c5(d.Ruvv.x, Avv.x, Auv.x, Av.x, Au.x, o.S.x, hu, hv2, huv2, hvv, d.Ruvv.w),
                      c5(d.Ruvv.y, Avv.y, Auv.y, Av.y, Au.y, o.S.y, hu, hv2, huv2, hvv, d.Ruvv.w),
                      c5(d.Ruvv.z, Avv.z, Auv.z, Av.z, Au.z, o.S.z, hu, hv2, huv2, hvv, d.Ruvv.w)};
        T suuu = suu * su, suuv = suu * sv, suvv = su * svv, svvv = svv * sv;
        o.Suuu = {Auuu.x * suuu, Auuu.y * suuu, Auuu.z * suuu};
        o.Suuv = {Auuv.x * suuv, Auuv.y * suuv, Auuv.z * suuv};
        o.Suvv = {Auvv.x * suvv, Auvv.y * suvv, Auvv.z * suvv};
        o.Svvv = {Avvv.x * svvv, Avvv.y * svvv, Avvv.z * svvv};
      }
    }
    o.Su = {Au.x * su, Au.y * su, Au.z * su};
    o.Sv = {Av.x * sv, Av.y * sv, Av.z * sv};
  }
  return o;
}

// Breakpoint search with __ldg (see exact::find_seg for the semantics).
template <typename T>
__device__ __forceinline__ int find_seg(const T* __restrict__ b, int ns, T x) {
  int lo = 0;
  int step = 1 << (31 - __clz(ns));
  for (; step > 0; step >>= 1) {
    int t = lo + step;
    if (t < ns && __ldg(b + t) <= x) lo = t;
  }
  return lo;
}

// Locates (u,v) and evaluates S and derivatives up to ORDER in precision T.
template <typename T, int P, int Q, int ORDER>
__device__ __forceinline__ SDer<T> eval_point(const SurfDev& s, T u, T v) {
  const T* bu;
  const T* bv;
  const T* iu;
  const T* iv;
  const T* m;
  if constexpr (sizeof(T) == 8) {
    bu = reinterpret_cast<const T*>(s.bu);
    bv = reinterpret_cast<const T*>(s.bv);
    iu = reinterpret_cast<const T*>(s.inv_du);
    iv = reinterpret_cast<const T*>(s.inv_dv);
    m = reinterpret_cast<const T*>(s.m64);
  } else {
    bu = reinterpret_cast<const T*>(s.bu32);
    bv = reinterpret_cast<const T*>(s.bv32);
    iu = reinterpret_cast<const T*>(s.inv_du32);
    iv = reinterpret_cast<const T*>(s.inv_dv32);
    m = reinterpret_cast<const T*>(s.m32);
  }
  int su = find_seg(bu, s.ns_u, u);
  int sv = find_seg(bv, s.ns_v, v);
  T idu = __ldg(iu + su), idv = __ldg(iv + sv);
  T lu = (u - __ldg(bu + su)) * idu;
  T lv = (v - __ldg(bv + sv)) * idv;
  const int k12 = sizeof(T) == 4 ? span_coefs32(s.p, s.q) : (s.p + 1) * (s.q + 1);
  const T* span = m + (size_t)(su * s.ns_v + sv) * k12 * 4;
  RDer<T> d = span_contract<T, P, Q, ORDER>(span, s.p, s.q, lu, lv);
  T ru, rv;
  if constexpr (sizeof(T) == 8) {
    ru = s.range_u;
    rv = s.range_v;
  } else {
    ru = s.range_u32;
    rv = s.range_v32;
  }
  T scu = ru * idu, scv = rv * idv;
  return quotient<T, ORDER>(d, scu, scv);
}

// Breakpoint tables of one precision, wherever they live (global memory, or a copy the calling
// kernel staged in shared memory).
template <typename T>
struct Locator {
  const T* bu;
  const T* bv;
  const T* iu;
  const T* iv;
  int ns_u, ns_v;
  T ru, rv;
};

template <typename T>
__device__ __forceinline__ Locator<T> global_locator(const SurfDev& s) {
  Locator<T> L;
  if constexpr (sizeof(T) == 8) {
    L.bu = s.bu; L.bv = s.bv; L.iu = s.inv_du; L.iv = s.inv_dv; L.ru = s.range_u; L.rv = s.range_v;
  } else {
    L.bu = s.bu32; L.bv = s.bv32; L.iu = s.inv_du32; L.iv = s.inv_dv32; L.ru = s.range_u32; L.rv = s.range_v32;
  }
  L.ns_u = s.ns_u;
  L.ns_v = s.ns_v;
  return L;
}

// find_seg with a warm start: keeps `hint` when it is still the span of x, else bisects.
template <typename T>
__device__ __forceinline__ int find_seg_hint(const T* b, int ns, T x, int hint) {
  if ((hint == 0 || b[hint] <= x) && (hint == ns - 1 || x < b[hint + 1])) return hint;
  int lo = 0;
  int step = 1 << (31 - __clz(ns));
  for (; step > 0; step >>= 1) {
    int t = lo + step;
    if (t < ns && b[t] <= x) lo = t;
  }
  return lo;
}

// eval_point with explicit breakpoint tables and span hints (updated in place).
template <typename T, int P, int Q, int ORDER, bool FAST = false>
__device__ __forceinline__ SDer<T> eval_at(const Locator<T>& L, const T* __restrict__ m, int p, int q, T u, T v,
                                           int& hu, int& hv) {
  hu = find_seg_hint(L.bu, L.ns_u, u, hu);
  hv = find_seg_hint(L.bv, L.ns_v, v, hv);
  T idu = L.iu[hu], idv = L.iv[hv];
  T lu = (u - L.bu[hu]) * idu;
  T lv = (v - L.bv[hv]) * idv;
  const int k12 = sizeof(T) == 4 ? span_coefs32(p, q) : (p + 1) * (q + 1);
  const T* span = m + (size_t)(hu * L.ns_v + hv) * k12 * 4;
  RDer<T> d = span_contract<T, P, Q, ORDER>(span, p, q, lu, lv);
  return quotient<T, ORDER, FAST>(d, L.ru * idu, L.rv * idv);
}

}  // namespace fast
}  // namespace gnurbs
