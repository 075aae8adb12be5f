// Stage d: candidate culling + Gauss-Newton point inversion (K4 invert), one fused kernel.
//
// Replaces NewInverse + GaussNewton (src/kernel/kernel.cu:433-469, 151-249).  Per query:
//   1. cull: the built tree nodes sit in shared memory twice — as FP32 boxes rounded outward
//      (a necessary test that never rejects a true hit) and as the exact FP64 boxes that decide
//      it — so the candidate set equals the reference's NewBoundingBoxCheck scan bit for bit;
//   2. each candidate is seeded at its node's uv-centre (kernel.cu:154) and iterated with the
//      reference's Gauss-Newton update  C <- C - (J^T J)^-1 J^T (S(C) - P)  (kernel.cu:195-243)
//      until the step is small, then with Newton steps (Hessian J^T J + sum r_k d2S_k) whose
//      fixed point is the same stationary point but which converge quadratically;
//   3. results inside the knot domain are kept; the closest wins (ties: first in node order).
//
// Precision schedules (template MODE):
//   FP64  — every evaluation, solve and update in FP64.
//   MIXED — phase 1 for every candidate in FP32 (FP32 span matrices, FP32 breakpoints); the
//           best candidate (plus a second one when it is nearly as close) then takes the final
//           two Newton steps in FP64: S, Su, Sv and the gradient J^T r in FP64, the Hessian's
//           curvature term from FP32 second derivatives (it only sets the convergence rate),
//           the 2x2 solve and the residual |S - P| in FP64.  Extra FP64 steps (at most 4) run
//           only when the second step is not yet below tolerance (near-singular or boundary
//           cases).  FP64 work per query is thus ~2 evaluations instead of ~20.
#include "nurbs_internal.h"
#include "nurbs_math.cuh"

namespace gnurbs {

namespace {

constexpr int kModeFP64 = 0;
constexpr int kModeMixed = 1;

constexpr int kMaxIter32 = 24;     // FP32 phase iterations per candidate
constexpr int kMaxIter64 = 40;     // FP64-mode iterations per candidate
constexpr int kMaxFinal64 = 6;     // MIXED: FP64 steps (2 normally)
constexpr float kNewtonSwitch32 = 1e-3f;
constexpr double kNewtonSwitch64 = 1e-3;
constexpr float kTol32 = 3e-7f;    // FP32 phase: stop when the step is at FP32 resolution
constexpr double kTolNewton64 = 1e-10;  // a Newton step this small leaves < 1e-19 error
constexpr double kTolAny64 = 1e-14;
constexpr double kDistinct = 1e-7;      // two solutions are the same minimum within this (uv)
constexpr float kDistinct32 = 1e-4f;

struct Sol {
  double u, v, r;
  bool ok;
};

template <typename T>
__device__ __forceinline__ T dot3(const v3<T>& a, const v3<T>& b) {
  return a.x * b.x + a.y * b.y + a.z * b.z;
}

// One (Gauss-)Newton step from the derivatives at C.  Returns false when the system is
// singular.  Newton uses H = J^T J + r.d2S when that H is positive definite.
template <typename T, typename TH>
__device__ __forceinline__ bool solve_step(const v3<T>& r, const v3<T>& Su, const v3<T>& Sv, const v3<TH>& Suu,
                                           const v3<TH>& Suv, const v3<TH>& Svv, bool newton, T& du, T& dv) {
  T a00 = dot3(Su, Su), a01 = dot3(Su, Sv), a11 = dot3(Sv, Sv);
  T g0 = dot3(Su, r), g1 = dot3(Sv, r);
  if (newton) {
    v3<T> rr = r;
    T h00 = a00 + (T)(rr.x * (T)Suu.x + rr.y * (T)Suu.y + rr.z * (T)Suu.z);
    T h01 = a01 + (T)(rr.x * (T)Suv.x + rr.y * (T)Suv.y + rr.z * (T)Suv.z);
    T h11 = a11 + (T)(rr.x * (T)Svv.x + rr.y * (T)Svv.y + rr.z * (T)Svv.z);
    T det = h00 * h11 - h01 * h01;
    if (h00 > T(0) && det > T(0)) {
      du = (h11 * g0 - h01 * g1) / det;
      dv = (h00 * g1 - h01 * g0) / det;
      return true;
    }
  }
  T det = a00 * a11 - a01 * a01;
  if (!(det > T(0))) return false;
  du = (a11 * g0 - a01 * g1) / det;
  dv = (a00 * g1 - a01 * g0) / det;
  return true;
}

// FP32 phase from seed (u,v).  On success returns the iterate and its distance.
template <int P, int Q>
__device__ bool phase32(const SurfDev& s, float px, float py, float pz, float& u, float& v, float& dist) {
  bool newton = false;
  float prev = INFINITY;
  for (int it = 0; it < kMaxIter32; ++it) {
    fast::SDer<float> d = fast::eval_point<float, P, Q, 2>(s, u, v);
    v3<float> r = {d.S.x - px, d.S.y - py, d.S.z - pz};
    float du, dv;
    if (!solve_step<float, float>(r, d.Su, d.Sv, d.Suu, d.Suv, d.Svv, newton, du, dv)) return false;
    if (!(isfinite(du) && isfinite(dv))) return false;
    u -= du;
    v -= dv;
    float step = fmaxf(fabsf(du), fabsf(dv));
    dist = sqrtf(dot3(r, r));
    // FP32 resolution of the parameters here: the rounding of S (relative 2^-24 of its
    // magnitude) mapped through the smaller tangent length
    float smag = fmaxf(fmaxf(fabsf(d.S.x), fabsf(d.S.y)), fmaxf(fabsf(d.S.z), 1.0f));
    float tmin = sqrtf(fminf(dot3(d.Su, d.Su), dot3(d.Sv, d.Sv)));
    float floor32 = 8.0f * 5.96e-8f * smag / fmaxf(tmin, 1e-30f);
    if (step <= fmaxf(kTol32, floor32)) return true;
    // Newton steps that stop shrinking have reached the rounding floor
    if (newton && step < 1e-4f && step > 0.5f * prev) return true;
    prev = step;
    newton = step < kNewtonSwitch32;
  }
  return false;
}

// FP64 iterations from (u,v).  MIXED: curvature from FP32 second derivatives and at most
// kMaxFinal64 steps; FP64: full FP64 with the GN -> Newton switch.
template <int P, int Q, int MODE>
__device__ Sol phase64(const SurfDev& s, double px, double py, double pz, double u, double v) {
  Sol o = {u, v, 0.0, false};
  bool newton = (MODE == kModeMixed);
  const int maxit = MODE == kModeMixed ? kMaxFinal64 : kMaxIter64;
  bool converged = false;
  for (int it = 0; it < maxit; ++it) {
    double du, dv;
    if (MODE == kModeMixed) {
      fast::SDer<double> d = fast::eval_point<double, P, Q, 1>(s, u, v);
      fast::SDer<float> c = fast::eval_point<float, P, Q, 2>(s, (float)u, (float)v);
      v3<double> r = {d.S.x - px, d.S.y - py, d.S.z - pz};
      if (!solve_step<double, float>(r, d.Su, d.Sv, c.Suu, c.Suv, c.Svv, true, du, dv)) return o;
    } else {
      fast::SDer<double> d = fast::eval_point<double, P, Q, 2>(s, u, v);
      v3<double> r = {d.S.x - px, d.S.y - py, d.S.z - pz};
      if (!solve_step<double, double>(r, d.Su, d.Sv, d.Suu, d.Suv, d.Svv, newton, du, dv)) return o;
    }
    if (!(isfinite(du) && isfinite(dv))) return o;
    u -= du;
    v -= dv;
    double step = fmax(fabs(du), fabs(dv));
    if ((newton && step <= kTolNewton64) || step <= kTolAny64) {
      converged = true;
      break;
    }
    if (MODE != kModeMixed) newton = step < kNewtonSwitch64;
  }
  if (!converged) return o;
  // residual check in FP64 at the returned point: |S(C) - P|
  fast::SDer<double> d = fast::eval_point<double, P, Q, 0>(s, u, v);
  v3<double> r = {d.S.x - px, d.S.y - py, d.S.z - pz};
  o.u = u;
  o.v = v;
  o.r = sqrt(dot3(r, r));
  o.ok = (u >= s.dom_u0 && u <= s.dom_u1 && v >= s.dom_v0 && v <= s.dom_v1) && isfinite(o.r);
  return o;
}

struct Best {
  Sol sol[4];
  int n;
};

__device__ __forceinline__ void add_solution(Best& b, const Sol& s) {
  // merge with an existing copy of the same minimum (keep the closer estimate)
  for (int k = 0; k < b.n; ++k) {
    if (fabs(b.sol[k].u - s.u) <= kDistinct && fabs(b.sol[k].v - s.v) <= kDistinct) {
      if (s.r < b.sol[k].r) b.sol[k] = s;
      return;
    }
  }
  if (b.n < 4) {
    b.sol[b.n++] = s;
    return;
  }
  int worst = 0;
  for (int k = 1; k < 4; ++k)
    if (b.sol[k].r > b.sol[worst].r) worst = k;
  if (s.r < b.sol[worst].r) b.sol[worst] = s;
}

// best solution and status (FOUND / AMBIGUOUS), as the oracle decides it
__device__ __forceinline__ int finish(const Best& b, double& u, double& v, double& r) {
  int bi = 0;
  for (int k = 1; k < b.n; ++k)
    if (b.sol[k].r < b.sol[bi].r) bi = k;
  u = b.sol[bi].u;
  v = b.sol[bi].v;
  r = b.sol[bi].r;
  for (int k = 0; k < b.n; ++k) {
    if (k == bi) continue;
    if (b.sol[k].r <= r * (1 + 1e-6) + 1e-12) return 1;  // NURBS_INV_AMBIGUOUS
  }
  return 0;
}

__device__ __forceinline__ float round_down_f(double x) { return __double2float_rd(x); }
__device__ __forceinline__ float round_up_f(double x) { return __double2float_ru(x); }

template <int P, int Q, int MODE>
__global__ void __launch_bounds__(128) k_invert(SurfDev s, const double* __restrict__ Pq, int64_t n,
                                                double* __restrict__ uv_out, int* __restrict__ st_out,
                                                double* __restrict__ res_out) {
  __shared__ float box32[kTreeNodes][6];
  __shared__ double box64[kTreeNodes][6];
  __shared__ double ctr[kTreeNodes][2];
  __shared__ float ctr32[kTreeNodes][2];
  __shared__ float dom32[4];
  __shared__ int nb;
  if (threadIdx.x == 0) {
    int c = 0;
    for (int k = 0; k < kTreeNodes; ++k) {
      if (!s.built[k]) continue;
      const TreeNodeDev& T = s.tree[k];
      for (int j = 0; j < 3; ++j) {
        box64[c][j] = T.lb[j];
        box64[c][3 + j] = T.rt[j];
        box32[c][j] = round_down_f(T.lb[j]);
        box32[c][3 + j] = round_up_f(T.rt[j]);
      }
      ctr[c][0] = (T.uv_lb[0] + T.uv_rt[0]) / 2;  // kernel.cu:154
      ctr[c][1] = (T.uv_lb[1] + T.uv_rt[1]) / 2;
      ctr32[c][0] = (float)ctr[c][0];
      ctr32[c][1] = (float)ctr[c][1];
      ++c;
    }
    nb = c;
    const float slack = 1e-4f;  // FP32 domain test is a prefilter; the FP64 phase decides
    dom32[0] = (float)s.dom_u0 - slack;
    dom32[1] = (float)s.dom_u1 + slack;
    dom32[2] = (float)s.dom_v0 - slack;
    dom32[3] = (float)s.dom_v1 + slack;
  }
  __syncthreads();
  const int nbl = nb;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const double px = Pq[3 * i], py = Pq[3 * i + 1], pz = Pq[3 * i + 2];
    const float fx = (float)px, fy = (float)py, fz = (float)pz;
    // ---- cull (exact candidate set, ascending node order)
    uint64_t m0 = 0, m1 = 0;
    for (int k = 0; k < nbl; ++k) {
      if (fx >= box32[k][0] && fy >= box32[k][1] && fz >= box32[k][2] && fx <= box32[k][3] && fy <= box32[k][4] &&
          fz <= box32[k][5]) {
        if (px >= box64[k][0] && py >= box64[k][1] && pz >= box64[k][2] && px <= box64[k][3] &&
            py <= box64[k][4] && pz <= box64[k][5]) {
          if (k < 64) m0 |= 1ull << k;
          else m1 |= 1ull << (k - 64);
        }
      }
    }
    int status;
    double ou = __longlong_as_double(0x7ff8000000000000ll), ov = ou, orr = ou;
    if (m0 == 0 && m1 == 0) {
      status = 2;  // NURBS_INV_NO_CANDIDATE
    } else if (MODE == kModeFP64) {
      Best b;
      b.n = 0;
      for (int w = 0; w < 2; ++w) {
        uint64_t m = w == 0 ? m0 : m1;
        while (m) {
          int k = __ffsll((long long)m) - 1 + 64 * w;
          m &= m - 1;
          Sol so = phase64<P, Q, kModeFP64>(s, px, py, pz, ctr[k][0], ctr[k][1]);
          if (so.ok) add_solution(b, so);
        }
      }
      if (b.n == 0) status = 3;
      else status = finish(b, ou, ov, orr);
    } else {
      // FP32 phase over all candidates: keep the best and the best distinct runner-up
      float bu1 = 0, bv1 = 0, bd1 = INFINITY, bu2 = 0, bv2 = 0, bd2 = INFINITY;
      for (int w = 0; w < 2; ++w) {
        uint64_t m = w == 0 ? m0 : m1;
        while (m) {
          int k = __ffsll((long long)m) - 1 + 64 * w;
          m &= m - 1;
          float u = ctr32[k][0], v = ctr32[k][1], d;
          if (!phase32<P, Q>(s, fx, fy, fz, u, v, d)) continue;
          if (!(u >= dom32[0] && u <= dom32[1] && v >= dom32[2] && v <= dom32[3])) continue;
          bool same1 = fabsf(u - bu1) <= kDistinct32 && fabsf(v - bv1) <= kDistinct32 && bd1 < INFINITY;
          if (same1) {
            if (d < bd1) { bu1 = u; bv1 = v; bd1 = d; }
          } else if (d < bd1) {
            bu2 = bu1; bv2 = bv1; bd2 = bd1;
            bu1 = u; bv1 = v; bd1 = d;
          } else if (d < bd2) {
            bu2 = u; bv2 = v; bd2 = d;
          }
        }
      }
      Best b;
      b.n = 0;
      if (bd1 < INFINITY) {
        Sol s1 = phase64<P, Q, kModeMixed>(s, px, py, pz, (double)bu1, (double)bv1);
        if (s1.ok) add_solution(b, s1);
        if (bd2 < INFINITY && (!s1.ok || bd2 <= bd1 * 1.001f + 1e-5f)) {
          Sol s2 = phase64<P, Q, kModeMixed>(s, px, py, pz, (double)bu2, (double)bv2);
          if (s2.ok) add_solution(b, s2);
        }
      }
      if (b.n == 0) status = 3;
      else status = finish(b, ou, ov, orr);
    }
    uv_out[2 * i] = ou;
    uv_out[2 * i + 1] = ov;
    st_out[i] = status;
    res_out[i] = orr;
  }
}

template <int P, int Q>
cudaError_t launch_pq(const SurfDev& s, const double* P_, int64_t n, double* uv, int* st_, double* res, int prec,
                      cudaStream_t st) {
  int64_t blocks = (n + 127) / 128;
  const int64_t cap = 152 * 64;
  if (blocks > cap) blocks = cap;
  if (prec == 1)
    k_invert<P, Q, kModeMixed><<<(unsigned)blocks, 128, 0, st>>>(s, P_, n, uv, st_, res);
  else
    k_invert<P, Q, kModeFP64><<<(unsigned)blocks, 128, 0, st>>>(s, P_, n, uv, st_, res);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_invert(const SurfDev& s, const double* P, int64_t n, double* uv, int* status, double* residual,
                          int precision, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  if (s.p == 3 && s.q == 3) return launch_pq<3, 3>(s, P, n, uv, status, residual, precision, st);
  if (s.p == 5 && s.q == 5) return launch_pq<5, 5>(s, P, n, uv, status, residual, precision, st);
  if (s.p == 2 && s.q == 2) return launch_pq<2, 2>(s, P, n, uv, status, residual, precision, st);
  return launch_pq<0, 0>(s, P, n, uv, status, residual, precision, st);
}

}  // namespace gnurbs
