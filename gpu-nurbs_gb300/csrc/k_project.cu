// Point projection (nurbs_project): the closest point of the surface over its closed knot domain,
// for query points near the surface or far from it.
//
// Replaces the reference's unfinished projection (Project, src/kernel/kernel.cu:471-485, a
// <<<1,1>>> launch for one constant point; NormalBoundingBoxCheck :487-513; NormalBoundingBox
// :623-704; NormalBoxToNormalTreeNode :1613-1636) with one fused persistent kernel:
//   1. cull (FP32, relative to the control net's centre, the same operations and roundings as
//      the oracle's cull, so both select the same nodes): the distance bound UB is the
//      least distance from P to the 3x3 sub-lattice surface points of every built node; a node is
//      a candidate when its bound box is within UB of P and its normal cone, taken with both
//      signs, can face P from some point of the box's bounding ball;
//   2. each candidate is seeded at its 9x9 lattice point closest to P and iterated with projected
//      Newton steps and a line search inside the domain (the full Hessian J^T J + r.d2S where it
//      is positive definite, J^T J elsewhere; a coordinate held at a bound whose descent points
//      out of the domain, the other taking the 1-D step; every step halved until |S - P| does not
//      grow), so minima on the boundary, where S - P is not normal to the surface, are found too;
//   3. the converged results are merged into per-query records (grid cells of the domain, as in
//      the inversion) and the closest wins; AMBIGUOUS when another minimum is as close.
// The warp's (query, seed) pairs are flattened into a task list as in the FP64 inversion
// (round-major), every lane pulling the next task when its seed ends.  Two schedules (template
// MODE): FP64 — every trajectory in FP64; MIXED — the trajectories in FP32 (tables relative to
// the control net's centre; steps below kWholeStep32 skip the line search, whose distance
// comparisons are rounding noise there), each query's best result and best of another grid cell
// kept, then FP64 projected Newton steps from the best, and from the other when it is within
// kPolishMargin of it or the best fails (project_polish64, the FP64 schedule's iteration where
// those steps do not converge).
#include "invert_core.cuh"

namespace gnurbs {
namespace {

using namespace inv;

constexpr int kMaxIterProj = 40;  // projected Newton iterations per seed (the oracle's cap)
constexpr int kMaxHalvings = 30;  // line-search halvings per iteration
// a Newton move this small ends a seed (far points have flat minima, where Newton converges
// slowly: the inversion's 1e-10 would leave the parameters ~1e-9 from the minimum)
constexpr double kTolNewtonProj = 1e-12;
constexpr double kWholeStep = 1e-6;  // steps below this skip the line search
constexpr int kLattice = kPts * kPts;

struct ProjStaged {
  float cone[kTreeNodes][kConeStride];
  float sub[kTreeNodes][9][3];  // the 3x3 sub-lattice (1, 4, 7)^2 of every node
};

template <int MODE>
struct ProjWarp {
  unsigned long long smask0[32];
  unsigned char smask1[32];
  unsigned srmask[kTreeNodes];
  int srpref[kTreeNodes + 1];
  unsigned char psub[32][kTreeNodes];  // seed lattice index of (query, node)
  typename std::conditional<MODE == kModeMixed, Rec32, Rec64>::type rec[32];
  double sp64[32][3];  // the query
  float sp32[32][3];   // the query relative to the control net's centre, FP32
};

__device__ __forceinline__ float fdot3(const float* a, const float* b) {
  return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2];
}
__device__ __forceinline__ double clampd(double x, double lo, double hi) { return x < lo ? lo : (x > hi ? hi : x); }

struct PSeed {
  double u, v;
  int it, hu, hv;
};
struct PSeed32 {
  float u, v;
  int it, hu, hv;
};

constexpr float kWholeStep32 = 3e-4f;  // mixed: FP32 steps below this skip the line search
constexpr float kTolMove32 = 1e-6f;    // mixed: an FP32 move this small ends the exploration

// One FP32 projected Newton iteration of the mixed schedule's exploration (the FP64 rules, the
// point and the tables relative to the control net's centre).  dist2 = |S - P|^2 before the step.
template <int P, int Q>
__device__ __forceinline__ int project_iterate32(const Ctx& c, const float dom[4], float px, float py, float pz,
                                                 PSeed32& sd, float& dist2) {
  fast::SDer<float> d = fast::eval_at<float, P, Q, 2, true>(c.L32, c.m32, c.p, c.q, sd.u, sd.v, sd.hu, sd.hv);
  const v3<float> r = {d.S.x - px, d.S.y - py, d.S.z - pz};
  const float f = dot3(r, r);
  dist2 = f;
  const float g0 = dot3(d.Su, r), g1 = dot3(d.Sv, r);
  const float a00 = dot3(d.Su, d.Su), a01 = dot3(d.Su, d.Sv), a11 = dot3(d.Sv, d.Sv);
  const float n00 = a00 + dot3(r, d.Suu), n01 = a01 + dot3(r, d.Suv), n11 = a11 + dot3(r, d.Svv);
  const bool fu = !((sd.u <= dom[0] && g0 > 0) || (sd.u >= dom[1] && g0 < 0));
  const bool fv = !((sd.v <= dom[2] && g1 > 0) || (sd.v >= dom[3] && g1 < 0));
  float d0 = 0, d1 = 0;
  if (fu && fv) {
    const bool newton = n00 > 0 && det2(n00, n01, n11) > 0;
    const float h00 = newton ? n00 : a00, h01 = newton ? n01 : a01, h11 = newton ? n11 : a11;
    const float det = det2(h00, h01, h11);
    if (!(det > 0)) return kFailed;
    const float inv = fast::rcp<true>(det);
    d0 = fast::mad(h11, g0, -(h01 * g1)) * inv;
    d1 = fast::mad(h00, g1, -(h01 * g0)) * inv;
  } else if (fu) {
    const float h = n00 > 0 ? n00 : a00;
    if (!(h > 0)) return kFailed;
    d0 = g0 / h;
  } else if (fv) {
    const float h = n11 > 0 ? n11 : a11;
    if (!(h > 0)) return kFailed;
    d1 = g1 / h;
  } else {
    return kConverged;
  }
  if (!(isfinite(d0) && isfinite(d1))) return kFailed;
  float un = fminf(fmaxf(sd.u - d0, dom[0]), dom[1]), vn = fminf(fmaxf(sd.v - d1, dom[2]), dom[3]);
  if (fmaxf(fabsf(d0), fabsf(d1)) > kWholeStep32) {
    float alpha = 1;
    for (int ls = 0;; ++ls) {
      int hu = sd.hu, hv = sd.hv;
      fast::SDer<float> e = fast::eval_at<float, P, Q, 0, true>(c.L32, c.m32, c.p, c.q, un, vn, hu, hv);
      const v3<float> rn = {e.S.x - px, e.S.y - py, e.S.z - pz};
      if (dot3(rn, rn) <= f || ls == kMaxHalvings) break;
      alpha *= 0.5f;
      un = fminf(fmaxf(sd.u - alpha * d0, dom[0]), dom[1]);
      vn = fminf(fmaxf(sd.v - alpha * d1, dom[2]), dom[3]);
    }
  }
  const float moved = fmaxf(fabsf(un - sd.u), fabsf(vn - sd.v));
  sd.u = un;
  sd.v = vn;
  if (moved <= kTolMove32) return kConverged;
  if (++sd.it >= kMaxIterProj) return kFailed;
  return kContinue;
}

// One projected Newton iteration with its line search (see above).
template <int P, int Q>
__device__ __forceinline__ int project_iterate(const Ctx& c, double px, double py, double pz, PSeed& sd) {
  fast::SDer<double> d = fast::eval_at<double, P, Q, 2>(c.L64, c.m64, c.p, c.q, sd.u, sd.v, sd.hu, sd.hv);
  const v3<double> r = {d.S.x - px, d.S.y - py, d.S.z - pz};
  const double f = dot3(r, r);
  const double g0 = dot3(d.Su, r), g1 = dot3(d.Sv, r);
  const double a00 = dot3(d.Su, d.Su), a01 = dot3(d.Su, d.Sv), a11 = dot3(d.Sv, d.Sv);
  const double n00 = a00 + dot3(r, d.Suu), n01 = a01 + dot3(r, d.Suv), n11 = a11 + dot3(r, d.Svv);
  const bool fu = !((sd.u <= c.dom_u0 && g0 > 0) || (sd.u >= c.dom_u1 && g0 < 0));
  const bool fv = !((sd.v <= c.dom_v0 && g1 > 0) || (sd.v >= c.dom_v1 && g1 < 0));
  double d0 = 0, d1 = 0;
  bool newton;
  if (fu && fv) {
    newton = n00 > 0 && det2(n00, n01, n11) > 0;
    const double h00 = newton ? n00 : a00, h01 = newton ? n01 : a01, h11 = newton ? n11 : a11;
    const double det = det2(h00, h01, h11);
    if (!(det > 0)) return kFailed;
    d0 = fast::mad(h11, g0, -(h01 * g1)) / det;
    d1 = fast::mad(h00, g1, -(h01 * g0)) / det;
  } else if (fu) {
    newton = n00 > 0;
    const double h = newton ? n00 : a00;
    if (!(h > 0)) return kFailed;
    d0 = g0 / h;
  } else if (fv) {
    newton = n11 > 0;
    const double h = newton ? n11 : a11;
    if (!(h > 0)) return kFailed;
    d1 = g1 / h;
  } else {
    return kConverged;  // a corner where the distance grows into the domain
  }
  if (!(isfinite(d0) && isfinite(d1))) return kFailed;
  // line search; a step below kWholeStep is taken whole (its decrease is below the rounding of
  // the distance, so comparing distances would stop it at random near the minimum)
  double un = clampd(sd.u - d0, c.dom_u0, c.dom_u1), vn = clampd(sd.v - d1, c.dom_v0, c.dom_v1);
  if (fmax(fabs(d0), fabs(d1)) > kWholeStep) {
    double alpha = 1;
    for (int ls = 0;; ++ls) {
      int hu = sd.hu, hv = sd.hv;
      fast::SDer<double> e = fast::eval_at<double, P, Q, 0>(c.L64, c.m64, c.p, c.q, un, vn, hu, hv);
      const v3<double> rn = {e.S.x - px, e.S.y - py, e.S.z - pz};
      if (dot3(rn, rn) <= f || ls == kMaxHalvings) break;
      alpha *= 0.5;
      un = clampd(sd.u - alpha * d0, c.dom_u0, c.dom_u1);
      vn = clampd(sd.v - alpha * d1, c.dom_v0, c.dom_v1);
    }
  }
  const double moved = fmax(fabs(un - sd.u), fabs(vn - sd.v));
  sd.u = un;
  sd.v = vn;
  if (moved <= kTolAny64 || (newton && moved <= kTolNewtonProj)) return kConverged;
  if (++sd.it >= kMaxIterProj) return kFailed;
  return kContinue;
}

// MIXED: the final FP64 steps from an FP32 result, as the inversion's (final64): S, Su, Sv in FP64
// and the Hessian's curvature term from FP32 second derivatives, projected onto the domain as the
// trajectories are, without a line search (the FP32 result lies in its minimum's basin); at most
// kPolishSteps, converged at a move <= kTolNewtonProj, the residual from the last step's S, Su, Sv.
// False when it does not converge: the caller then runs the FP64 schedule's iteration.
constexpr int kPolishSteps = 8;
template <int P, int Q>
__device__ bool project_polish64(const Ctx& c, double px, double py, double pz, double& u, double& v, double& res) {
  int hu = fast::find_seg_hint(c.L32.bu, c.L32.ns_u, (float)u, 0);
  int hv = fast::find_seg_hint(c.L32.bv, c.L32.ns_v, (float)v, 0);
  int hu32 = hu, hv32 = hv;
  for (int it = 0; it < kPolishSteps; ++it) {
    const fast::SDer<double> d = fast::eval_at<double, P, Q, 1>(c.L64, c.m64, c.p, c.q, u, v, hu, hv);
    const fast::SDer<float> e = fast::eval_at<float, P, Q, 2, true>(c.L32, c.m32, c.p, c.q, (float)u, (float)v, hu32,
                                                                  hv32);
    const v3<double> r = {d.S.x - px, d.S.y - py, d.S.z - pz};
    const double g0 = dot3(d.Su, r), g1 = dot3(d.Sv, r);
    const double a00 = dot3(d.Su, d.Su), a01 = dot3(d.Su, d.Sv), a11 = dot3(d.Sv, d.Sv);
    const double n00 = a00 + dot3c(r, e.Suu), n01 = a01 + dot3c(r, e.Suv), n11 = a11 + dot3c(r, e.Svv);
    const bool fu = !((u <= c.dom_u0 && g0 > 0) || (u >= c.dom_u1 && g0 < 0));
    const bool fv = !((v <= c.dom_v0 && g1 > 0) || (v >= c.dom_v1 && g1 < 0));
    double d0 = 0, d1 = 0;
    if (fu && fv) {
      const bool newton = n00 > 0 && det2(n00, n01, n11) > 0;
      const double h00 = newton ? n00 : a00, h01 = newton ? n01 : a01, h11 = newton ? n11 : a11;
      const double det = det2(h00, h01, h11);
      if (!(det > 0)) return false;
      d0 = fast::mad(h11, g0, -(h01 * g1)) / det;
      d1 = fast::mad(h00, g1, -(h01 * g0)) / det;
    } else if (fu) {
      const double h = n00 > 0 ? n00 : a00;
      if (!(h > 0)) return false;
      d0 = g0 / h;
    } else if (fv) {
      const double h = n11 > 0 ? n11 : a11;
      if (!(h > 0)) return false;
      d1 = g1 / h;
    }
    if (!(isfinite(d0) && isfinite(d1))) return false;
    const double un = clampd(u - d0, c.dom_u0, c.dom_u1), vn = clampd(v - d1, c.dom_v0, c.dom_v1);
    const double du = u - un, dv = v - vn;
    u = un;
    v = vn;
    if (fmax(fabs(du), fabs(dv)) <= kTolNewtonProj) {
      const v3<double> r2 = {fast::mad(-d.Sv.x, dv, fast::mad(-d.Su.x, du, r.x)),
                             fast::mad(-d.Sv.y, dv, fast::mad(-d.Su.y, du, r.y)),
                             fast::mad(-d.Sv.z, dv, fast::mad(-d.Su.z, du, r.z))};
      res = sqrt(dot3(r2, r2));
      return isfinite(res);
    }
  }
  return false;
}

// One warp projects the queries [q0, min(q0+32, qend)).
template <int P, int Q, int MODE>
__device__ __forceinline__ void project_chunk(const Staged<kSmemSpans, MODE>& sm, const ProjStaged& ps,
                                              const float* __restrict__ lattice, ProjWarp<MODE>& ww, const Ctx& cx,
                                              const double* __restrict__ Pq, int64_t q0, int64_t qend,
                                              double* __restrict__ uv_out, int* __restrict__ st_out,
                                              double* __restrict__ res_out) {
  const int lane = threadIdx.x & 31;
  const unsigned FULL = 0xffffffffu;
  const unsigned lt_mask = (1u << lane) - 1u;
  const int nbl = sm.nb;
  const int64_t q = q0 + lane;
  const bool valid = q < qend;
  double px = 0, py = 0, pz = 0;
  if (valid) {
    px = Pq[3 * q];
    py = Pq[3 * q + 1];
    pz = Pq[3 * q + 2];
  }
  const float Pf[3] = {(float)(px - sm.org[0]), (float)(py - sm.org[1]), (float)(pz - sm.org[2])};
  // ---- cull (the oracle's arithmetic, operation for operation)
  uint64_t m0 = 0;
  unsigned m1 = 0;
  if (valid) {
    float ub2 = INFINITY;
    for (int k = 0; k < nbl; ++k)
      for (int j = 0; j < 9; ++j) {
        const float dd3[3] = {ps.sub[k][j][0] - Pf[0], ps.sub[k][j][1] - Pf[1], ps.sub[k][j][2] - Pf[2]};
        const float dd = fdot3(dd3, dd3);
        ub2 = ub2 < dd ? ub2 : dd;
      }
    ub2 = ub2 * (1.0f + 0x1p-10f);
    for (int k = 0; k < nbl; ++k) {
      const float* rc = ps.cone[k];
      float g[3];
      for (int c = 0; c < 3; ++c) {
        const float lo = rc[9 + c] - Pf[c], hi = Pf[c] - rc[12 + c];
        g[c] = lo > hi ? lo : hi;
        g[c] = g[c] > 0.0f ? g[c] : 0.0f;
      }
      const bool nearb = fdot3(g, g) <= ub2;
      const float dv[3] = {Pf[0] - rc[0], Pf[1] - rc[1], Pf[2] - rc[2]};
      const float dd = fdot3(dv, dv), r = rc[3];
      float e = dd - r * r;
      e = e > 0.0f ? e : 0.0f;
      const bool seen = rc[7] * sqrtf(e) <= fabsf(fdot3(dv, rc + 4)) + rc[8] * r;
      if (nearb && seen) {
        // seed: the node's lattice point closest to P (first of equals)
        const float* L = lattice + (size_t)k * kLattice * 3;
        float best = INFINITY;
        int bi = 0;
        for (int j = 0; j < kLattice; ++j) {
          const float x[3] = {__ldg(L + 3 * j) - Pf[0], __ldg(L + 3 * j + 1) - Pf[1], __ldg(L + 3 * j + 2) - Pf[2]};
          const float ee = fdot3(x, x);
          if (ee < best) {
            best = ee;
            bi = j;
          }
        }
        ww.psub[lane][k] = (unsigned char)bi;
        if (k < 64) m0 |= 1ull << k;
        else m1 = 1u;
      }
    }
  }
  const int cnt = __popcll(m0) + (int)m1;
  // round-major task list: round r holds seed r of every query with more than r seeds
  const int maxc = __reduce_max_sync(FULL, (unsigned)cnt);
  int total = 0;
  for (int r = 0; r < maxc; ++r) {
    unsigned m = __ballot_sync(FULL, cnt > r);
    if (lane == 0) {
      ww.srmask[r] = m;
      ww.srpref[r] = total;
    }
    total += __popc(m);
  }
  if (lane == 0) ww.srpref[maxc] = total;
  ww.sp64[lane][0] = px;
  ww.sp64[lane][1] = py;
  ww.sp64[lane][2] = pz;
  ww.sp32[lane][0] = Pf[0];
  ww.sp32[lane][1] = Pf[1];
  ww.sp32[lane][2] = Pf[2];
  ww.smask0[lane] = m0;
  ww.smask1[lane] = (unsigned char)m1;
  if constexpr (MODE == kModeMixed) {
    Rec32& R = ww.rec[lane];
    R.d1 = R.d2 = R.de = INFINITY;
    R.u1 = R.v1 = R.u2 = R.v2 = R.ue = R.ve = 0.f;
    R.cu1 = R.cv1 = 0;
  } else {
    ww.rec[lane].n = 0;
  }
  __syncwarp();

  auto decode = [&](int t, int& ql, int& node) {
    int r = 0;
#pragma unroll
    for (int step = 64; step > 0; step >>= 1)
      if (r + step < maxc && ww.srpref[r + step] <= t) r += step;
    const unsigned m = ww.srmask[r];
    int i = t - ww.srpref[r], pos = 0;
#pragma unroll
    for (int w = 16; w > 0; w >>= 1)
      if (__popc(m & ((1u << (pos + w)) - 1u)) <= i) pos += w;
    ql = pos;
    const uint64_t mm = ww.smask0[ql];
    node = r < __popcll(mm) ? select_bit(mm, r) : 64;
  };
  // the seed of (query, node): its lattice point's parameters, as the samples compute them
  auto seed_of = [&](int ql, int node, double& u, double& v) {
    const int j = ww.psub[ql][node];
    const unsigned g = node == 0 ? 1u : (unsigned)kGap;
    const unsigned bx = node == 0 ? 0u : (unsigned)(node - 1) / kGap, by = node == 0 ? 0u : (unsigned)(node - 1) % kGap;
    const double base_unit = 1.0 / g, unit = base_unit / kGap;
    u = clampd(base_unit * bx + (j / kPts) * unit, cx.dom_u0, cx.dom_u1);
    v = clampd(base_unit * by + (j % kPts) * unit, cx.dom_v0, cx.dom_v1);
  };

  int next = 32;
  int task = lane;
  bool active = task < total;
  int ql = 0, node = 0;
  if constexpr (MODE == kModeMixed) {
    // ---- FP32 exploration; per query the best result and the best outside its cell
    const float dom32[4] = {(float)cx.dom_u0, (float)cx.dom_u1, (float)cx.dom_v0, (float)cx.dom_v1};
    PSeed32 sd;
    float tx = 0, ty = 0, tz = 0, dist = 0;
    auto start = [&]() {
      decode(task, ql, node);
      tx = ww.sp32[ql][0];
      ty = ww.sp32[ql][1];
      tz = ww.sp32[ql][2];
      double u, v;
      seed_of(ql, node, u, v);
      sd.u = fminf(fmaxf((float)u, dom32[0]), dom32[1]);
      sd.v = fminf(fmaxf((float)v, dom32[2]), dom32[3]);
      sd.it = 0;
      sd.hu = 0;
      sd.hv = 0;
    };
    if (active) start();
    bool waiting = false;  // finished, waiting for the next batch of starts (as the inversion's)
    while (__any_sync(FULL, active || waiting)) {
      int res = kContinue;
      if (active) res = project_iterate32<P, Q>(cx, dom32, tx, ty, tz, sd, dist);
      const bool done = active && res != kContinue;
      __syncwarp();
      int cu = 0, cv = 0;
      bool upd = done && res == kConverged;
      if (upd) {
        cell_of(sm.cell32, sd.u, sd.v, cu, cv);
        const Rec32& R = ww.rec[ql];
        if (R.d1 < INFINITY && cu == R.cu1 && cv == R.cv1)
          upd = before(dist, sd.u, sd.v, R.d1, R.u1, R.v1);
        else
          upd = before(dist, sd.u, sd.v, R.d1, R.u1, R.v1) || before(dist, sd.u, sd.v, R.d2, R.u2, R.v2);
      }
      unsigned fm = __ballot_sync(FULL, upd);
      while (fm) {
        const int j = __ffs(fm) - 1;
        if (lane == j) merge32(ww.rec[ql], cu, cv, sd.u, sd.v, dist);
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
    PSeed sd;
    double tx = 0, ty = 0, tz = 0;
    auto start = [&]() {
      decode(task, ql, node);
      tx = ww.sp64[ql][0];
      ty = ww.sp64[ql][1];
      tz = ww.sp64[ql][2];
      seed_of(ql, node, sd.u, sd.v);
      sd.it = 0;
      sd.hu = 0;
      sd.hv = 0;
    };
    if (active) start();
    while (__any_sync(FULL, active)) {
      int res = kContinue;
      double rr = 0;
      bool keep = false;
      if (active) {
        res = project_iterate<P, Q>(cx, tx, ty, tz, sd);
        if (res == kConverged) keep = finish64<P, Q>(cx, tx, ty, tz, sd.u, sd.v, sd.hu, sd.hv, rr);
      }
      const bool done = active && res != kContinue;
      __syncwarp();
      int cu = 0, cv = 0;
      if (done && keep) cell_of(sm.cell64, sd.u, sd.v, cu, cv);
      unsigned fm = __ballot_sync(FULL, done && keep);
      while (fm) {
        const int j = __ffs(fm) - 1;
        if (lane == j) merge64(ww.rec[ql], cu, cv, sd.u, sd.v, rr);
        __syncwarp();
        fm &= fm - 1;
      }
      const unsigned dm = __ballot_sync(FULL, done);
      if (done) {
        task = next + __popc(dm & lt_mask);
        active = task < total;
        if (active) start();
      }
      next += __popc(dm);
    }
  }
  __syncwarp();
  int status;
  double ou = __longlong_as_double(0x7ff8000000000000ll), ov = ou, orr = ou;
  if (cnt == 0) {
    status = 2;  // NURBS_INV_NO_CANDIDATE (non-finite P)
  } else if constexpr (MODE == kModeMixed) {
    // ---- the FP64 projected Newton steps from the best FP32 result (and from the best outside
    // its cell when that one is as close within kPolishMargin, or when the best fails)
    double us[2], vs[2], rs[2];
    int ns = 0;
    auto polish = [&](float u0, float v0) {
      PSeed sd;
      sd.u = u0;
      sd.v = v0;
      sd.it = 0;
      sd.hu = 0;
      sd.hv = 0;
      double rr;
      if (!project_polish64<P, Q>(cx, px, py, pz, sd.u, sd.v, rr)) {
        sd.u = u0;
        sd.v = v0;
        int r = kContinue;
        while (r == kContinue) r = project_iterate<P, Q>(cx, px, py, pz, sd);
        if (r != kConverged || !finish64<P, Q>(cx, px, py, pz, sd.u, sd.v, sd.hu, sd.hv, rr)) return false;
      }
      if (ns == 1 && fabs(sd.u - us[0]) <= kDistinct && fabs(sd.v - vs[0]) <= kDistinct) {
        if (rr < rs[0]) { us[0] = sd.u; vs[0] = sd.v; rs[0] = rr; }
        return true;
      }
      us[ns] = sd.u;
      vs[ns] = sd.v;
      rs[ns] = rr;
      ++ns;
      return true;
    };
    const Rec32& R = ww.rec[lane];
    if (R.d1 < INFINITY) {
      const float e1 = sqrtf(R.d1) * (1.0f + kPolishMargin) + 1e-5f;
      const bool second = R.d2 < INFINITY && !(fabsf(R.u2 - R.u1) <= kDistinct32 && fabsf(R.v2 - R.v1) <= kDistinct32);
      const bool ok1 = polish(R.u1, R.v1);
      if (second && (!ok1 || R.d2 <= e1 * e1)) polish(R.u2, R.v2);
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

// Shared memory (dynamic, above the 48 KB of static allocations): the staged surface, the cone
// records and sub-lattice points, and the warps' bookkeeping.
template <int MODE>
struct ProjSmem {
  static constexpr size_t ps = (sizeof(Staged<kSmemSpans, MODE>) + 15) / 16 * 16;
  static constexpr size_t ww = ps + (sizeof(ProjStaged) + 15) / 16 * 16;
  static constexpr size_t bytes = ww + sizeof(ProjWarp<MODE>) * kWarps;
};

// Register budget: the FP64 schedule keeps 168 registers (3 CTAs per SM); the mixed one of a
// specialised degree is held to 5 CTAs per SM, its FP32 exploration latency-bound at 3 (the
// generic-degree variant would spill 18 KB at that budget and keeps 3).
template <int P, int Q, int MODE>
__global__ void __launch_bounds__(kThreads, (MODE == kModeMixed && P != 0) ? 5 : 3)
    k_project(SurfDev s, const double* __restrict__ Pq, int64_t n, double* __restrict__ uv_out,
              int* __restrict__ st_out, double* __restrict__ res_out, unsigned* __restrict__ counter) {
  extern __shared__ __align__(16) unsigned char smem[];
  Staged<kSmemSpans, MODE>& sm = *reinterpret_cast<Staged<kSmemSpans, MODE>*>(smem);
  ProjStaged& ps = *reinterpret_cast<ProjStaged*>(smem + ProjSmem<MODE>::ps);
  ProjWarp<MODE>* ww = reinterpret_cast<ProjWarp<MODE>*>(smem + ProjSmem<MODE>::ww);
  Ctx cx;
  stage_surface<kSmemSpans>(s, sm, cx, threadIdx.x, blockDim.x);
  for (int e = threadIdx.x; e < kTreeNodes * kConeStride; e += blockDim.x)
    ps.cone[e / kConeStride][e % kConeStride] = s.cone[e];
  for (int e = threadIdx.x; e < kTreeNodes * 9; e += blockDim.x) {
    const int k = e / 9, j = e % 9, a = 1 + 3 * (j / 3), b = 1 + 3 * (j % 3);
    const float* x = s.lattice + ((size_t)k * kLattice + kPts * a + b) * 3;
    ps.sub[k][j][0] = x[0];
    ps.sub[k][j][1] = x[1];
    ps.sub[k][j][2] = x[2];
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5;
  const int64_t units = (n + 31) / 32;
  for (;;) {
    unsigned ch = 0;
    if ((threadIdx.x & 31) == 0) ch = atomicAdd(counter, 1u);
    ch = __shfl_sync(0xffffffffu, ch, 0);
    if ((int64_t)ch >= units) break;
    const int64_t q0 = (int64_t)ch * 32;
    project_chunk<P, Q, MODE>(sm, ps, s.lattice, ww[warp], cx, Pq, q0, min(q0 + 32, n), uv_out, st_out, res_out);
  }
}

template <int P, int Q, int MODE>
cudaError_t launch_project_mode(const SurfDev& s, const double* P_, int64_t n, double* uv, int* st_, double* res,
                                unsigned* counter, cudaStream_t st) {
  const int64_t chunks = (n + 31) / 32;
  if (chunks > 0x3fffffffLL) return cudaErrorInvalidValue;  // chunk ids are 32-bit
  constexpr size_t bytes = ProjSmem<MODE>::bytes;
  static int cached[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) dev = 0;
  if (!cached[dev]) {
    cudaError_t e = cudaFuncSetAttribute(k_project<P, Q, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e != cudaSuccess) return e;
    int sms = 0, per_sm = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_project<P, Q, MODE>, kThreads, bytes);
    cached[dev] = (sms > 0 ? sms : 1) * (per_sm > 0 ? per_sm : 1);
  }
  int64_t blocks = (chunks + kWarps - 1) / kWarps;
  if (blocks > cached[dev]) blocks = cached[dev];
  k_project<P, Q, MODE><<<(unsigned)blocks, kThreads, bytes, st>>>(s, P_, n, uv, st_, res, counter);
  return cudaGetLastError();
}

template <int P, int Q>
cudaError_t launch_project_pq(const SurfDev& s, const double* P_, int64_t n, double* uv, int* st_, double* res,
                              int precision, unsigned* counter, cudaStream_t st) {
  if (precision == kModeMixed) return launch_project_mode<P, Q, kModeMixed>(s, P_, n, uv, st_, res, counter, st);
  return launch_project_mode<P, Q, kModeFP64>(s, P_, n, uv, st_, res, counter, st);
}

}  // namespace

cudaError_t launch_project(const SurfDev& s, const double* P, int64_t n, double* uv, int* status, double* residual,
                           int precision, unsigned* counter, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  if (s.p == 3 && s.q == 3) return launch_project_pq<3, 3>(s, P, n, uv, status, residual, precision, counter, st);
  if (s.p == 5 && s.q == 5) return launch_project_pq<5, 5>(s, P, n, uv, status, residual, precision, counter, st);
  return launch_project_pq<0, 0>(s, P, n, uv, status, residual, precision, counter, st);
}

}  // namespace gnurbs
