// Device core of the point inversion (stage d), shared by the single-surface kernel
// (k_invert.cu) and the pooled persistent kernel (k_pool.cu): per-seed FP32/FP64 iterations,
// the per-warp task scheduler over (query, seed) pairs and the final FP64 steps.  The
// algorithm and its precision schedules are described in k_invert.cu.
#pragma once
#include <type_traits>

#include "nurbs_internal.h"
#include "nurbs_math.cuh"

namespace gnurbs {
namespace inv {

constexpr int kModeFP64 = 0;
constexpr int kModeMixed = 1;

constexpr int kWarps = 4;          // warps per CTA
constexpr int kThreads = 32 * kWarps;
constexpr int kMinBlocksMixed = 6;  // CTAs per SM the mixed kernels are register-budgeted for (80 registers)
constexpr int kMaxIter32 = 40;     // FP32 iterations per seed (the FP64 cap: the oracle's too)
constexpr int kMaxIter64 = 40;     // FP64-mode iterations per seed
constexpr int kMaxFinal64 = 24;    // MIXED: FP64 steps (2 normally)
constexpr int kFinal32Curv = 3;    // MIXED: FP64 steps with the FP32 curvature term before the FP64 one
constexpr float kPolishMargin = 0.05f;  // MIXED: a runner-up this close to the best also takes the FP64 steps
constexpr double kNewtonSwitch = 1e-2;  // GN while the step is larger, Newton below
constexpr float kTol32 = 3e-7f;
constexpr double kTolNewton64 = 1e-10;  // a Newton step this small leaves < 1e-19 error
constexpr double kTolAny64 = 1e-14;
constexpr double kDistinct = 1e-7;      // FP64 minima: grid cell size, times the domain's extent
constexpr float kDistinct32 = 1e-4f;    // FP32 minima: the same
// Every seed runs to its own end, decided by the seed alone.  Stopping a seed once it nears a
// minimum its query already found saves ~15-20 % of the iterations, but whether that other seed
// has finished first depends on the other queries sharing the warp, so results would depend on
// the batch.
constexpr int kSols = 4;                // FP64 mode: distinct minima kept per query
constexpr int kSmemSpans = 256;         // breakpoint tables staged in shared memory up to this
// MIXED: lanes whose seed has ended wait until this many are free (or no lane still iterates)
// and then start their next seeds together, so that the divergent start (task decode, the first
// step from the node centre) runs once for several lanes instead of every iteration for ~3.
// Which lane runs which seed, and when, does not change any seed's arithmetic, and the
// records are independent of arrival order, so results are the same for every value.
constexpr int kStartBatch = 8;

// Arithmetic below writes every product that feeds a sum as an explicit FMA (the translation
// units are compiled with --fmad=false), so a seed's trajectory is the same bit for bit in
// every kernel that runs it: results do not depend on the kernel, the batch or the schedule.
template <typename T>
__device__ __forceinline__ T dot3(const v3<T>& a, const v3<T>& b) {
  return fast::mad(a.z, b.z, fast::mad(a.y, b.y, a.x * b.x));
}
template <typename T, typename TH>
__device__ __forceinline__ T dot3c(const v3<T>& a, const v3<TH>& b) {  // b converted to T
  return fast::mad(a.z, (T)b.z, fast::mad(a.y, (T)b.y, a.x * (T)b.x));
}
template <typename T>
__device__ __forceinline__ T det2(T h00, T h01, T h11) {
  return fast::mad(h00, h11, -(h01 * h01));
}

// One (Gauss-)Newton step from the derivatives at C.  Newton uses H = J^T J + r.d2S when that
// H is positive definite, else the Gauss-Newton matrix J^T J (the reference's update,
// kernel.cu:195-243).  Returns kSingular when the system is singular, kStepGN or kStepNewton
// for the matrix it used.  FAST: FP32 reciprocal by the hardware approximation.
enum StepKind { kSingular = 0, kStepGN = 1, kStepNewton = 2 };
template <typename T, typename TH, bool FAST>
__device__ __forceinline__ int solve_step(const v3<T>& r, const v3<T>& Su, const v3<T>& Sv, const v3<TH>& Suu,
                                          const v3<TH>& Suv, const v3<TH>& Svv, bool newton, T& du, T& dv) {
  T h00 = dot3(Su, Su), h01 = dot3(Su, Sv), h11 = dot3(Sv, Sv);
  const T g0 = dot3(Su, r), g1 = dot3(Sv, r);
  int kind = kStepGN;
  if (newton) {
    const T n00 = h00 + dot3c(r, Suu), n01 = h01 + dot3c(r, Suv), n11 = h11 + dot3c(r, Svv);
    if (n00 > T(0) && det2(n00, n01, n11) > T(0)) {
      h00 = n00;
      h01 = n01;
      h11 = n11;
      kind = kStepNewton;
    }
  }
  const T det = det2(h00, h01, h11);
  if (!(det > T(0))) return kSingular;
  const T inv = fast::rcp<FAST>(det);
  du = fast::mad(h11, g0, -(h01 * g1)) * inv;
  dv = fast::mad(h00, g1, -(h01 * g0)) * inv;
  return kind;
}

// Where one kernel finds the span tables: breakpoints in shared memory when they fit.
struct Ctx {
  fast::Locator<float> L32;
  fast::Locator<double> L64;
  const float* m32;
  const double* m64;
  int p, q;
  double dom_u0, dom_u1, dom_v0, dom_v1;
};

// Per-seed iteration state (hu/hv: span hints for the warm-started span search).
template <typename T>
struct Seed {
  T u, v, prev;
  int it, hu, hv;
  bool newton;
};

enum StepResult { kContinue = 0, kConverged = 1, kFailed = 2 };

// One FP32 iteration of a seed.  Convergence: the step is at the FP32 resolution of the
// parameters (the change of S it makes, |Su du + Sv dv|, is within 8 ulp(|S|)), or Newton steps
// (with a positive definite Hessian) stop shrinking.  Where the Hessian is not
// positive definite the iterate is near a saddle of the distance, from which the GN steps creep
// away slowly: steps that do not shrink there are no sign of convergence.  dist2 = |S - P|^2
// before the step.
template <int P, int Q>
__device__ __forceinline__ int iterate32(const Ctx& c, float px, float py, float pz, Seed<float>& st, float& dist2) {
  fast::SDer<float> d = fast::eval_at<float, P, Q, 2, true>(c.L32, c.m32, c.p, c.q, st.u, st.v, st.hu, st.hv);
  v3<float> r = {d.S.x - px, d.S.y - py, d.S.z - pz};
  float du, dv;
  const int kind = solve_step<float, float, true>(r, d.Su, d.Sv, d.Suu, d.Suv, d.Svv, st.newton, du, dv);
  if (kind == kSingular) return kFailed;
  if (!(isfinite(du) && isfinite(dv))) return kFailed;
  st.u -= du;
  st.v -= dv;
  float step = fmaxf(fabsf(du), fabsf(dv));
  dist2 = dot3(r, r);
  float smag = fmaxf(fmaxf(fabsf(d.S.x), fabsf(d.S.y)), fmaxf(fabsf(d.S.z), 1.0f));
  const v3<float> dS = {fast::mad(d.Sv.x, dv, d.Su.x * du), fast::mad(d.Sv.y, dv, d.Su.y * du),
                        fast::mad(d.Sv.z, dv, d.Su.z * du)};
  float fl = 8.0f * 5.96e-8f * smag;
  if (step <= kTol32 || dot3(dS, dS) <= fl * fl) return kConverged;
  if (kind == kStepNewton && step < 1e-4f && step > 0.5f * st.prev) return kConverged;
  st.prev = step;
  st.newton = step < (float)kNewtonSwitch;
  if (++st.it >= kMaxIter32) return kFailed;
  return kContinue;
}

// One FP64 iteration of a seed (FP64 mode).
template <int P, int Q>
__device__ __forceinline__ int iterate64(const Ctx& c, double px, double py, double pz, Seed<double>& st) {
  fast::SDer<double> d = fast::eval_at<double, P, Q, 2>(c.L64, c.m64, c.p, c.q, st.u, st.v, st.hu, st.hv);
  v3<double> r = {d.S.x - px, d.S.y - py, d.S.z - pz};
  double du, dv;
  if (!solve_step<double, double, false>(r, d.Su, d.Sv, d.Suu, d.Suv, d.Svv, st.newton, du, dv)) return kFailed;
  if (!(isfinite(du) && isfinite(dv))) return kFailed;
  st.u -= du;
  st.v -= dv;
  double step = fmax(fabs(du), fabs(dv));
  if ((st.newton && step <= kTolNewton64) || step <= kTolAny64) return kConverged;
  st.prev = step;
  st.newton = step < kNewtonSwitch;
  if (++st.it >= kMaxIter64) return kFailed;
  return kContinue;
}

// The first iteration of a seed from its node centre's precomputed S, Su, Sv (cd = 9 values,
// the same bits the evaluation there gives): the seed advances to its second iteration when the
// first one continues it, and is left at the centre otherwise, for iterate32/iterate64 to repeat
// that first iteration and end the seed.  The step is the GN update (the Newton phase starts
// after a step below kNewtonSwitch).
template <typename T>
__device__ __forceinline__ void first_step(const T* __restrict__ cd, T px, T py, T pz, const float far[4],
                                           Seed<T>& st) {
  const v3<T> S = {cd[0], cd[1], cd[2]}, Su = {cd[3], cd[4], cd[5]}, Sv = {cd[6], cd[7], cd[8]};
  const v3<T> r = {S.x - px, S.y - py, S.z - pz};
  T du, dv;
  if (solve_step<T, T, sizeof(T) == 4>(r, Su, Sv, Su, Su, Su, false, du, dv) == kSingular) return;
  if (!(isfinite(du) && isfinite(dv))) return;
  const T u = st.u - du, v = st.v - dv;
  T step;
  if constexpr (sizeof(T) == 4) step = fmaxf(fabsf(du), fabsf(dv));
  else step = fmax(fabs(du), fabs(dv));
  if constexpr (sizeof(T) == 4) {
    const float smag = fmaxf(fmaxf(fabsf(S.x), fabsf(S.y)), fmaxf(fabsf(S.z), 1.0f));
    const v3<float> dS = {fast::mad(Sv.x, dv, Su.x * du), fast::mad(Sv.y, dv, Su.y * du),
                          fast::mad(Sv.z, dv, Su.z * du)};
    const float fl = 8.0f * 5.96e-8f * smag;
    if (step <= kTol32 || dot3(dS, dS) <= fl * fl) return;  // converged at once: left to iterate32
    if (!(u >= far[0] && u <= far[1] && v >= far[2] && v <= far[3])) return;
  } else {
    if (step <= kTolAny64) return;
  }
  st.u = u;
  st.v = v;
  st.prev = step;
  st.newton = step < (T)kNewtonSwitch;
  st.it = 1;
}

// FP64 residual at (u,v), with the domain test.
template <int P, int Q>
__device__ __forceinline__ bool finish64(const Ctx& c, double px, double py, double pz, double u, double v,
                                         int hu, int hv, double& res) {
  fast::SDer<double> d = fast::eval_at<double, P, Q, 0>(c.L64, c.m64, c.p, c.q, u, v, hu, hv);
  v3<double> r = {d.S.x - px, d.S.y - py, d.S.z - pz};
  res = sqrt(dot3(r, r));
  return (u >= c.dom_u0 && u <= c.dom_u1 && v >= c.dom_v0 && v <= c.dom_v1) && isfinite(res);
}

// MIXED: the final FP64 Newton steps from an FP32 minimum, then the residual.  The first
// kFinal32Curv steps take the Hessian's curvature term from FP32 second derivatives (it only
// sets the rate of convergence, and two steps normally reach the tolerance); later steps take
// it in FP64, which converges where the minimum is nearly degenerate (a flat valley, where the
// FP32 term's error is comparable to the Hessian's smallest eigenvalue).
template <int P, int Q>
__device__ bool final64(const Ctx& c, double px, double py, double pz, double& u, double& v, double& res) {
  // span hints from the FP32 tables (shared memory when staged): the FP64 search then only
  // confirms them with two reads instead of bisecting the FP64 tables in global memory
  int hu = fast::find_seg_hint(c.L32.bu, c.L32.ns_u, (float)u, 0);
  int hv = fast::find_seg_hint(c.L32.bv, c.L32.ns_v, (float)v, 0);
  int hu32 = hu, hv32 = hv;
  for (int it = 0; it < kMaxFinal64; ++it) {
    fast::SDer<double> d;
    double du, dv;
    int kind;
    v3<double> r;
    if (it < kFinal32Curv) {
      d = fast::eval_at<double, P, Q, 1>(c.L64, c.m64, c.p, c.q, u, v, hu, hv);
      fast::SDer<float> e = fast::eval_at<float, P, Q, 2, true>(c.L32, c.m32, c.p, c.q, (float)u, (float)v, hu32, hv32);
      r = {d.S.x - px, d.S.y - py, d.S.z - pz};
      kind = solve_step<double, float, false>(r, d.Su, d.Sv, e.Suu, e.Suv, e.Svv, true, du, dv);
    } else {
      d = fast::eval_at<double, P, Q, 2>(c.L64, c.m64, c.p, c.q, u, v, hu, hv);
      r = {d.S.x - px, d.S.y - py, d.S.z - pz};
      kind = solve_step<double, double, false>(r, d.Su, d.Sv, d.Suu, d.Suv, d.Svv, true, du, dv);
    }
    if (kind == kSingular) return false;
    if (!(isfinite(du) && isfinite(dv))) return false;
    u -= du;
    v -= dv;
    if (fmax(fabs(du), fabs(dv)) <= kTolNewton64) {
      // Residual at the returned point from this step's FP64 S, Su, Sv: S(u - du, v - dv) =
      // S - Su du - Sv dv + O(|S''| 1e-20), below the rounding of S itself.
      const v3<double> r2 = {fast::mad(-d.Sv.x, dv, fast::mad(-d.Su.x, du, r.x)),
                             fast::mad(-d.Sv.y, dv, fast::mad(-d.Su.y, du, r.y)),
                             fast::mad(-d.Sv.z, dv, fast::mad(-d.Su.z, du, r.z))};
      res = sqrt(dot3(r2, r2));
      return (u >= c.dom_u0 && u <= c.dom_u1 && v >= c.dom_v0 && v <= c.dom_v1) && isfinite(res);
    }
  }
  return false;
}

// Position of the k-th (0-based) set bit of m, which has more than k set bits: a fixed
// five-step bisection on bit counts of the lower half of each window.
__device__ __forceinline__ int select_bit(uint64_t m, int k) {
  const unsigned lo = (unsigned)m;
  const int clo = __popc(lo);
  unsigned w32 = k < clo ? lo : (unsigned)(m >> 32);
  int pos = k < clo ? 0 : 32;
  if (k >= clo) k -= clo;
#pragma unroll
  for (int w = 16; w > 0; w >>= 1) {
    const int c = __popc(w32 & ((1u << w) - 1u));
    if (k >= c) {
      k -= c;
      w32 >>= w;
      pos += w;
    }
  }
  return pos;
}

struct Rec32 {  // per-query FP32 record: best and best distinct runner-up (squared distances)
  float u1, v1, d1, u2, v2, d2;
  int cu1, cv1;  // grid cell of the best
  float ue, ve, de;  // the closest FP32 minimum just outside the domain (edge record)
};

// Total order on results (distance, then u, then v): the minimum of a set does not depend on
// the order in which its members arrive, so per-query records are schedule independent.
template <typename T>
__device__ __forceinline__ bool before(T d, T u, T v, T d0, T u0, T v0) {
  return d < d0 || (d == d0 && (u < u0 || (u == u0 && v < v0)));
}
struct Rec64 {  // per-query FP64 record: distinct minima and their grid cells
  double u[kSols], v[kSols], r[kSols];
  int cu[kSols], cv[kSols];
  int n;
};

// Results are grouped into minima by a fixed grid over the parameter domain (cells of
// kDistinct32 / kDistinct times the domain's extent): a grouping that depends on each result
// alone, unlike "within a distance of the current representative", so the records below hold
// the same values whatever order the seeds finish in.
template <typename T>
struct Cells {
  T u0, v0, iu, iv;  // domain origin, cells per parameter unit
};
// cell indices of an in-domain result (rounded down; saturating)
__device__ __forceinline__ int cell_index(float x) { return __float2int_rd(x); }
__device__ __forceinline__ int cell_index(double x) { return __double2int_rd(x); }
template <typename T>
__device__ __forceinline__ void cell_of(const Cells<T>& g, T u, T v, int& cu, int& cv) {
  cu = cell_index((u - g.u0) * g.iu);
  cv = cell_index((v - g.v0) * g.iv);
}

// R.1 = the minimum of all results (total order); R.2 = the minimum of the results outside
// R.1's cell.  Exact for any arrival order: a new overall minimum in another cell makes the
// old minimum (smaller than everything else seen) the runner-up.
__device__ __forceinline__ void merge32(Rec32& R, int cu, int cv, float u, float v, float d) {
  if (R.d1 < INFINITY && cu == R.cu1 && cv == R.cv1) {
    if (before(d, u, v, R.d1, R.u1, R.v1)) { R.u1 = u; R.v1 = v; R.d1 = d; }
  } else if (before(d, u, v, R.d1, R.u1, R.v1)) {
    R.u2 = R.u1; R.v2 = R.v1; R.d2 = R.d1;
    R.u1 = u; R.v1 = v; R.d1 = d; R.cu1 = cu; R.cv1 = cv;
  } else if (before(d, u, v, R.d2, R.u2, R.v2)) {
    R.u2 = u; R.v2 = v; R.d2 = d;
  }
}

// The kSols cells with the smallest minima, each with its minimum.  A cell evicted earlier can
// only come back with a smaller value than the one it was evicted with, so the kept values are
// exact cell minima whatever the arrival order.
__device__ __forceinline__ void merge64(Rec64& R, int cu, int cv, double u, double v, double r) {
  for (int k = 0; k < R.n; ++k)
    if (cu == R.cu[k] && cv == R.cv[k]) {
      if (before(r, u, v, R.r[k], R.u[k], R.v[k])) { R.u[k] = u; R.v[k] = v; R.r[k] = r; }
      return;
    }
  int slot = R.n;
  if (R.n >= kSols) {
    slot = 0;
    for (int k = 1; k < kSols; ++k)
      if (before(R.r[slot], R.u[slot], R.v[slot], R.r[k], R.u[k], R.v[k])) slot = k;
    if (!before(r, u, v, R.r[slot], R.u[slot], R.v[slot])) return;
  } else {
    ++R.n;
  }
  R.u[slot] = u; R.v[slot] = v; R.r[slot] = r; R.cu[slot] = cu; R.cv[slot] = cv;
}

// best minimum and status (FOUND / AMBIGUOUS): FOUND unless another distinct minimum is as
// close within 1e-6 relative
// A minimum within (tu, tv) of the best is the same minimum: results that converged to one
// point can fall on both sides of a grid-cell boundary (an exact parameter such as 0.5 is one).
__device__ __forceinline__ int finish_status(const double* us, const double* vs, const double* rs, int n, double tu,
                                             double tv, double& u, double& v, double& r) {
  int bi = 0;
  for (int k = 1; k < n; ++k)
    if (before(rs[k], us[k], vs[k], rs[bi], us[bi], vs[bi])) bi = k;
  u = us[bi];
  v = vs[bi];
  r = rs[bi];
  for (int k = 0; k < n; ++k)
    if (k != bi && rs[k] <= r * (1 + 1e-6) + 1e-12 && (fabs(us[k] - u) > tu || fabs(vs[k] - v) > tv))
      return 1;  // NURBS_INV_AMBIGUOUS
  return 0;
}

// One surface staged in shared memory: tree boxes (FP32 outward-rounded and exact FP64), seed
// centres, domain, and breakpoint tables when the surface has at most KS spans per direction.
// FP64 breakpoint tables are staged only for the FP64 schedule: the mixed schedule reads them in
// its few final FP64 steps from global memory, which leaves more of the SM's memory to L1.
template <int KS, int MODE>
struct Staged {
  static constexpr int KS64 = MODE == kModeMixed ? 1 : KS;
  float box32[kTreeNodes][6];   // rounded outward: a point outside is outside the exact box
  float box32i[kTreeNodes][6];  // rounded inward: a point strictly inside is inside the exact box
  const TreeNodeDev* tree;     // exact FP64 boxes, read only near a face (global memory, L2)
  double ctr[kTreeNodes][2];
  float ctr32[kTreeNodes][2];
  double org[3];    // origin of the FP32 tables: FP32 iterations see P - org
  const float* cd32;   // S, Su, Sv at the node centres (FP32, relative to org), 9 per node
  const double* cd64;  // the same in FP64
  float dom32[4];
  float near32[4];  // 1 % of the extent around the domain: FP32 minima here are edge records
  float far32[4];  // two domain extents around the domain: an FP32 iterate beyond is abandoned
  Cells<float> cell32;
  Cells<double> cell64;
  int nb;
  float sb32[2][KS + 1], si32[2][KS];
  double sb64[2][KS64 + 1], si64[2][KS64];
};

// Per-warp bookkeeping of the task scheduler: candidate masks, task-order tables, per-query
// records and query coordinates of the warp's (up to) 32 queries.
template <int MODE>
struct WarpWork {
  unsigned long long smask0[32];
  unsigned char smask1[32];
  // round-major task order and the queries' FP64 coordinates: FP64 schedule only
  unsigned srmask[MODE == kModeMixed ? 1 : kTreeNodes];
  int srpref[MODE == kModeMixed ? 1 : kTreeNodes + 1];
  int slpref[32];
  typename std::conditional<MODE == kModeMixed, Rec32, Rec64>::type rec[32];
  float sp32[32][3];
  double sp64[MODE == kModeMixed ? 1 : 32][3];
};

// Cooperative over `nthreads` threads (index tid): stages one surface and fills the context.
// The callers synchronise the participating threads before and after.
template <int KS, int MODE>
__device__ __forceinline__ void stage_surface(const SurfDev& s, Staged<KS, MODE>& sm, Ctx& cx, int tid, int nthreads) {
  constexpr int KS64 = Staged<KS, MODE>::KS64;
  const bool smem_tables = s.ns_u <= KS && s.ns_v <= KS;
  const bool smem_tables64 = s.ns_u <= KS64 && s.ns_v <= KS64;
  if (smem_tables) {
    for (int k = tid; k <= s.ns_u; k += nthreads) {
      sm.sb32[0][k] = s.bu32[k];
      if (smem_tables64) sm.sb64[0][k] = s.bu[k];
      if (k < s.ns_u) {
        sm.si32[0][k] = s.inv_du32[k];
        if (smem_tables64) sm.si64[0][k] = s.inv_du[k];
      }
    }
    for (int k = tid; k <= s.ns_v; k += nthreads) {
      sm.sb32[1][k] = s.bv32[k];
      if (smem_tables64) sm.sb64[1][k] = s.bv[k];
      if (k < s.ns_v) {
        sm.si32[1][k] = s.inv_dv32[k];
        if (smem_tables64) sm.si64[1][k] = s.inv_dv[k];
      }
    }
  }
  cx.L32 = fast::global_locator<float>(s);
  cx.L64 = fast::global_locator<double>(s);
  if (smem_tables) {
    cx.L32.bu = sm.sb32[0]; cx.L32.bv = sm.sb32[1]; cx.L32.iu = sm.si32[0]; cx.L32.iv = sm.si32[1];
    if (smem_tables64) {
      cx.L64.bu = sm.sb64[0]; cx.L64.bv = sm.sb64[1]; cx.L64.iu = sm.si64[0]; cx.L64.iv = sm.si64[1];
    }
  }
  cx.m32 = s.m32;
  cx.m64 = s.m64;
  cx.p = s.p;
  cx.q = s.q;
  cx.dom_u0 = s.dom_u0; cx.dom_u1 = s.dom_u1; cx.dom_v0 = s.dom_v0; cx.dom_v1 = s.dom_v1;
  // built nodes are the root alone, or the root and all 64 children (the children of the
  // 2-level tree are built together when the root is divided), so node k keeps index k
  const int nb = s.built[1] ? kTreeNodes : (s.built[0] ? 1 : 0);
  for (int k = tid; k < nb; k += nthreads) {
    const TreeNodeDev& T = s.tree[k];
    for (int j = 0; j < 3; ++j) {
      sm.box32[k][j] = __double2float_rd(T.lb[j]);
      sm.box32[k][3 + j] = __double2float_ru(T.rt[j]);
      sm.box32i[k][j] = __double2float_ru(T.lb[j]);
      sm.box32i[k][3 + j] = __double2float_rd(T.rt[j]);
    }
    sm.ctr[k][0] = (T.uv_lb[0] + T.uv_rt[0]) / 2;  // kernel.cu:154
    sm.ctr[k][1] = (T.uv_lb[1] + T.uv_rt[1]) / 2;
    sm.ctr32[k][0] = (float)sm.ctr[k][0];
    sm.ctr32[k][1] = (float)sm.ctr[k][1];
  }
  if (tid == 0) {
    sm.nb = nb;
    sm.tree = s.tree;
    sm.cd32 = s.cd32;
    sm.cd64 = s.cd64;
    sm.org[0] = s.org[0];
    sm.org[1] = s.org[1];
    sm.org[2] = s.org[2];
    const float slack = 1e-4f;  // FP32 domain test is a prefilter; the FP64 phase decides
    sm.dom32[0] = (float)s.dom_u0 - slack;
    sm.dom32[1] = (float)s.dom_u1 + slack;
    sm.dom32[2] = (float)s.dom_v0 - slack;
    sm.dom32[3] = (float)s.dom_v1 + slack;
    const float fu = 2.0f * (float)(s.dom_u1 - s.dom_u0), fv = 2.0f * (float)(s.dom_v1 - s.dom_v0);
    sm.near32[0] = (float)s.dom_u0 - 5e-3f * fu;
    sm.near32[1] = (float)s.dom_u1 + 5e-3f * fu;
    sm.near32[2] = (float)s.dom_v0 - 5e-3f * fv;
    sm.near32[3] = (float)s.dom_v1 + 5e-3f * fv;
    sm.far32[0] = (float)s.dom_u0 - fu;
    sm.far32[1] = (float)s.dom_u1 + fu;
    sm.far32[2] = (float)s.dom_v0 - fv;
    sm.far32[3] = (float)s.dom_v1 + fv;
    const double eu = s.dom_u1 - s.dom_u0, ev = s.dom_v1 - s.dom_v0;
    sm.cell32 = {(float)s.dom_u0, (float)s.dom_v0, (float)(1.0 / ((double)kDistinct32 * eu)),
                 (float)(1.0 / ((double)kDistinct32 * ev))};
    sm.cell64 = {s.dom_u0, s.dom_v0, 1.0 / (kDistinct * eu), 1.0 / (kDistinct * ev)};
  }
}

// One warp inverts the queries [q0, min(q0+32, qend)) of the staged surface.
// COUNT: the work-counting variant (nurbs_invert_count): seed iterations and final FP64 polishes
// are added to counts[0] and counts[1]; the results are the same.
template <int P, int Q, int MODE, int KS, bool COUNT = false>
__device__ __forceinline__ void invert_chunk(Staged<KS, MODE>& sm, WarpWork<MODE>& ww, const Ctx& cx,
                                             const double* __restrict__ Pq,
                                             int64_t q0, int64_t qend, double* __restrict__ uv_out,
                                             int* __restrict__ st_out, double* __restrict__ res_out,
                                             unsigned long long* __restrict__ counts = nullptr) {
  unsigned n_iter = 0, n_final = 0;
  const int lane = threadIdx.x & 31;
  const unsigned FULL = 0xffffffffu;
  const unsigned lt_mask = (1u << lane) - 1u;
  const int nbl = sm.nb;
  {
    const int64_t q = q0 + lane;
    const bool valid = q < qend;
    double px = 0, py = 0, pz = 0;
    if (valid) {
      px = Pq[3 * q];
      py = Pq[3 * q + 1];
      pz = Pq[3 * q + 2];
    }
    const float fx = (float)px, fy = (float)py, fz = (float)pz;
    // ---- cull (exact candidate set, ascending node order).  With f = fl(x) rounded to nearest,
    // f < rd(lb) implies x < lb and f > ru(lb) implies x > lb (rounding is monotone), so the
    // FP64 comparison only runs for coordinates within an FP32 ulp of a box face.
    uint64_t m0 = 0;
    unsigned m1 = 0;
    if (valid) {
      for (int k = 0; k < nbl; ++k) {
        if (fx >= sm.box32[k][0] && fy >= sm.box32[k][1] && fz >= sm.box32[k][2] && fx <= sm.box32[k][3] &&
            fy <= sm.box32[k][4] && fz <= sm.box32[k][5]) {
          const bool surely = fx > sm.box32i[k][0] && fy > sm.box32i[k][1] && fz > sm.box32i[k][2] &&
                              fx < sm.box32i[k][3] && fy < sm.box32i[k][4] && fz < sm.box32i[k][5];
          const TreeNodeDev* B = sm.tree + k;
          if (surely || (px >= B->lb[0] && py >= B->lb[1] && pz >= B->lb[2] && px <= B->rt[0] && py <= B->rt[1] &&
                         pz <= B->rt[2])) {
            if (k < 64) m0 |= 1ull << k;
            else m1 = 1u;
          }
        }
      }
    }
    const int cnt = __popcll(m0) + (int)m1;
    // Task lists.  FP64 schedule: round-major, round r holds seed r of every query with more
    // than r seeds (rmask[r] = lanes with a seed in round r, rpref[r] = tasks before round r), so
    // a warp's concurrent seeds come from different queries.  Mixed schedule: lane-major, a
    // query's seeds consecutive (slpref = exclusive prefix of the candidate counts).
    const int maxc = __reduce_max_sync(FULL, (unsigned)cnt);
    int total = 0;
    for (int r = 0; r < maxc; ++r) {
      unsigned m = __ballot_sync(FULL, cnt > r);
      if (MODE != kModeMixed && lane == 0) {
        ww.srmask[r] = m;
        ww.srpref[r] = total;
      }
      total += __popc(m);
    }
    if (MODE != kModeMixed && lane == 0) ww.srpref[maxc] = total;
    if constexpr (MODE == kModeMixed) {
      int incl = cnt;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(FULL, incl, o);
        if (lane >= o) incl += t;
      }
      ww.slpref[lane] = incl - cnt;
    }
    // the FP32 iterations work relative to the FP32 tables' origin
    ww.sp32[lane][0] = (float)(px - sm.org[0]);
    ww.sp32[lane][1] = (float)(py - sm.org[1]);
    ww.sp32[lane][2] = (float)(pz - sm.org[2]);
    if constexpr (MODE != kModeMixed) {
      ww.sp64[lane][0] = px;
      ww.sp64[lane][1] = py;
      ww.sp64[lane][2] = pz;
    }
    ww.smask0[lane] = m0;
    ww.smask1[lane] = (unsigned char)m1;
    if constexpr (MODE == kModeMixed) {
      Rec32& R = ww.rec[lane];
      R.d1 = INFINITY;
      R.d2 = INFINITY;
      R.de = INFINITY;
      R.u1 = R.v1 = R.u2 = R.v2 = R.ue = R.ve = 0.f;
      R.cu1 = R.cv1 = 0;
    } else {
      ww.rec[lane].n = 0;
    }
    __syncwarp();

    // decode task t -> (owner lane, node)
    auto decode = [&](int t, int& ql, int& node) {
      if constexpr (MODE == kModeMixed) {
        // lane-major: the largest lane whose exclusive prefix is <= t owns task t (a lane with
        // no candidates shares its prefix with the next lane and is never the largest)
        int lo = 0;
#pragma unroll
        for (int step = 16; step > 0; step >>= 1)
          if (ww.slpref[lo + step] <= t) lo += step;
        ql = lo;
        uint64_t mm = ww.smask0[ql];
        int k = t - ww.slpref[lo];
        if (k < __popcll(mm)) {
          node = select_bit(mm, k);
        } else {
          node = 64;
        }
        return;
      }
      // round: the largest r with rpref[r] <= t (rounds are non-empty, so rpref is increasing)
      int r = 0;
#pragma unroll
      for (int step = 64; step > 0; step >>= 1)
        if (r + step < maxc && ww.srpref[r + step] <= t) r += step;
      // lane: the (t - rpref[r])-th set bit of rmask[r]
      const unsigned m = ww.srmask[r];
      int i = t - ww.srpref[r], pos = 0;
#pragma unroll
      for (int w = 16; w > 0; w >>= 1)
        if (__popc(m & ((1u << (pos + w)) - 1u)) <= i) pos += w;
      ql = pos;
      int k = r;  // seed r of that query: its r-th candidate node in ascending order
      uint64_t mm = ww.smask0[ql];
      int c0 = __popcll(mm);
      if (k < c0) {
        node = select_bit(mm, k);
      } else {
        node = 64;
      }
    };

    int next = 32;
    int task = lane;
    bool active = task < total;
    int ql = 0, node = 0;
    if constexpr (MODE == kModeMixed) {
      Seed<float> sd;
      float dist = 0.f;
      float tx = 0, ty = 0, tz = 0;
      auto start = [&]() {
        decode(task, ql, node);
        tx = ww.sp32[ql][0];
        ty = ww.sp32[ql][1];
        tz = ww.sp32[ql][2];
        sd.u = sm.ctr32[node][0];
        sd.v = sm.ctr32[node][1];
        sd.prev = INFINITY;
        sd.it = 0;
        sd.hu = 0;
        sd.hv = 0;
        sd.newton = false;
        first_step<float>(sm.cd32 + 9 * node, tx, ty, tz, sm.far32, sd);
      };
      if (active) start();
      bool waiting = false;  // finished, waiting for the next batch of starts
      while (__any_sync(FULL, active || waiting)) {
        int res = kContinue;
        if (active) {
          res = iterate32<P, Q>(cx, tx, ty, tz, sd, dist);
          if constexpr (COUNT) ++n_iter;
          if (res == kContinue && !(sd.u >= sm.far32[0] && sd.u <= sm.far32[1] && sd.v >= sm.far32[2] &&
                                    sd.v <= sm.far32[3]))
            res = kFailed;
        }
        const bool done = active && res != kContinue;
        const bool keep = res == kConverged && sd.u >= sm.dom32[0] && sd.u <= sm.dom32[1] && sd.v >= sm.dom32[2] &&
                          sd.v <= sm.dom32[3];
        // An FP32 minimum within 1 % of the extent outside the domain: near an edge FP32 arithmetic
        // can end outside while FP64 steps from there reach a minimum inside.  The closest such
        // result of a query is kept apart and takes the final FP64 steps too when it is close.
        const bool edge = done && res == kConverged && !keep && sd.u >= sm.near32[0] && sd.u <= sm.near32[1] &&
                          sd.v >= sm.near32[2] && sd.v <= sm.near32[3];
        __syncwarp();
        int cu = 0, cv = 0;
        bool upd = done && keep;
        if (upd) {
          // Records only improve, so a result that cannot change its query's record now never
          // will: only the others are merged, one lane at a time.
          cell_of(sm.cell32, sd.u, sd.v, cu, cv);
          const Rec32& R = ww.rec[ql];
          if (R.d1 < INFINITY && cu == R.cu1 && cv == R.cv1)
            upd = before(dist, sd.u, sd.v, R.d1, R.u1, R.v1);
          else
            upd = before(dist, sd.u, sd.v, R.d1, R.u1, R.v1) || before(dist, sd.u, sd.v, R.d2, R.u2, R.v2);
        }
        const bool upe = edge && before(dist, sd.u, sd.v, ww.rec[ql].de, ww.rec[ql].ue, ww.rec[ql].ve);
        unsigned fm = __ballot_sync(FULL, upd || upe);
        while (fm) {
          int j = __ffs(fm) - 1;
          if (lane == j) {
            Rec32& R = ww.rec[ql];
            if (upd) merge32(R, cu, cv, sd.u, sd.v, dist);
            else if (before(dist, sd.u, sd.v, R.de, R.ue, R.ve)) { R.ue = sd.u; R.ve = sd.v; R.de = dist; }
          }
          __syncwarp();
          fm &= fm - 1;
        }
        if (done) {
          active = false;
          waiting = true;
        }
        const unsigned wm = __ballot_sync(FULL, waiting);
        if (wm && (__popc(wm) >= kStartBatch || !__any_sync(FULL, active))) {
          if (waiting) {
            task = next + __popc(wm & lt_mask);
            active = task < total;
            waiting = false;
            if (active) start();
          }
          next += __popc(wm);
        }
      }
    } else {
      Seed<double> sd;
      double tx = 0, ty = 0, tz = 0;
      auto start = [&]() {
        decode(task, ql, node);
        tx = ww.sp64[ql][0];
        ty = ww.sp64[ql][1];
        tz = ww.sp64[ql][2];
        sd.u = sm.ctr[node][0];
        sd.v = sm.ctr[node][1];
        sd.prev = INFINITY;
        sd.it = 0;
        sd.hu = 0;
        sd.hv = 0;
        sd.newton = false;
        first_step<double>(sm.cd64 + 9 * node, tx, ty, tz, sm.far32, sd);
      };
      if (active) start();
      while (__any_sync(FULL, active)) {
        int res = kContinue;
        double rr = 0;
        bool keep = false;
        if (active) {
          res = iterate64<P, Q>(cx, tx, ty, tz, sd);
          if constexpr (COUNT) ++n_iter;
          if (res == kConverged) keep = finish64<P, Q>(cx, tx, ty, tz, sd.u, sd.v, sd.hu, sd.hv, rr);
        }
        const bool done = active && res != kContinue;
        __syncwarp();
        int cu = 0, cv = 0;
        if (done && keep) cell_of(sm.cell64, sd.u, sd.v, cu, cv);
        unsigned fm = __ballot_sync(FULL, done && keep);
        while (fm) {
          int j = __ffs(fm) - 1;
          if (lane == j) merge64(ww.rec[ql], cu, cv, sd.u, sd.v, rr);
          __syncwarp();
          fm &= fm - 1;
        }
        unsigned dm = __ballot_sync(FULL, done);
        if (done) {
          task = next + __popc(dm & lt_mask);
          active = task < total;
          if (active) start();
        }
        next += __popc(dm);
      }
    }
    __syncwarp();

    // ---- per query: final FP64 steps (MIXED) and the result
    int status;
    double ou = __longlong_as_double(0x7ff8000000000000ll), ov = ou, orr = ou;
    if (cnt == 0) {
      status = 2;  // NURBS_INV_NO_CANDIDATE
    } else if constexpr (MODE == kModeMixed) {
      // the query's FP64 coordinates again (not kept in registers through the seed loop)
      px = Pq[3 * q];
      py = Pq[3 * q + 1];
      pz = Pq[3 * q + 2];
      double us[3], vs[3], rs[3];
      int ns = 0;
      // FP64 minima reached from the records; two within kDistinct are one minimum (split by a
      // cell boundary), which keeps its smaller residual
      auto add = [&](double u, double v, double r) {
        for (int k = 0; k < ns; ++k)
          if (fabs(u - us[k]) <= kDistinct && fabs(v - vs[k]) <= kDistinct) {
            if (r < rs[k]) { us[k] = u; vs[k] = v; rs[k] = r; }
            return;
          }
        us[ns] = u; vs[ns] = v; rs[ns] = r; ++ns;
      };
      const Rec32& R = ww.rec[lane];
      const float dbest = fminf(R.d1, R.de);
      if (dbest < INFINITY) {
        // the runner-up also takes the FP64 steps when the best fails there, or when it is within
        // kPolishMargin of the best (an FP32 iterate that stopped in a flat valley overstates its
        // minimum's distance); one next to the best is the same minimum split by a cell boundary.
        // The edge record takes them when it is within the same margin.
        const float e1 = sqrtf(dbest) * (1.0f + kPolishMargin) + 1e-5f;
        if (R.d1 < INFINITY) {
          const bool second =
              R.d2 < INFINITY && !(fabsf(R.u2 - R.u1) <= kDistinct32 && fabsf(R.v2 - R.v1) <= kDistinct32);
          const bool tie = second && R.d2 <= e1 * e1;
          double u = R.u1, v = R.v1, r;
          const bool ok1 = final64<P, Q>(cx, px, py, pz, u, v, r);
          if constexpr (COUNT) ++n_final;
          if (ok1) add(u, v, r);
          if (ok1 ? tie : second) {
            double u2 = R.u2, v2 = R.v2, r2;
            if constexpr (COUNT) ++n_final;
            if (final64<P, Q>(cx, px, py, pz, u2, v2, r2)) add(u2, v2, r2);
          }
        }
        if (R.de <= e1 * e1) {
          double u3 = R.ue, v3 = R.ve, r3;
          if constexpr (COUNT) ++n_final;
          if (final64<P, Q>(cx, px, py, pz, u3, v3, r3)) add(u3, v3, r3);
        }
      }
      status = ns == 0 ? 3 : finish_status(us, vs, rs, ns, kDistinct, kDistinct, ou, ov, orr);
    } else {
      const Rec64& R = ww.rec[lane];
      status = R.n == 0 ? 3 : finish_status(R.u, R.v, R.r, R.n, 2.0 / sm.cell64.iu, 2.0 / sm.cell64.iv, ou, ov, orr);
    }
    if (valid) {
      uv_out[2 * q] = ou;
      uv_out[2 * q + 1] = ov;
      st_out[q] = status;
      res_out[q] = orr;
    }
    __syncwarp();
  }
  if constexpr (COUNT) {
    unsigned long long a = n_iter, b = n_final;
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_xor_sync(0xffffffffu, a, o);
      b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    if ((threadIdx.x & 31) == 0) {
      atomicAdd(counts, a);
      atomicAdd(counts + 1, b);
    }
  }
}

}  // namespace inv
}  // namespace gnurbs
