// p-curves: the parameter-space image of a 3-D curve that lies on (or near) a surface, from its
// ordered samples.  The reference names p-curve calculation as the use of its inversion
// (README.md:10) but has no code for it; this is the caller on the far side of stage d.
//
// Three passes over the samples, all on the caller's stream:
//   1. every sample is inverted as nurbs_invert does (tree candidates, GN then Newton, FP64 or
//      mixed precision);
//   2. continuation: each sample also takes Newton steps (FP64, with the FP32 curvature term
//      first) from its two neighbours' pass-1 parameters, and keeps such a minimum when it is
//      strictly closer than its own (a curve
//      sample's closest point is usually next to its neighbour's, even where the tree seeds miss
//      it); a sample without an answer takes the closer of the two;
//   3. flags per sample: NURBS_PCURVE_JUMP when the parameter step from the previous sample is
//      more than four times what the chord allows (|duv| > 4 |C_i - C_i-1| / sigma_min(J)), the
//      mark of a seam, a fold or a sample that found another sheet; NURBS_PCURVE_AMBIGUOUS and
//      NURBS_PCURVE_NOT_FOUND from the inversion status.
// Pass 2 reads only pass-1 results and pass 3 only pass-2 results, so every sample's answer
// depends on its own and its neighbours' inputs alone.
#include "gpu_nurbs.h"
#include "invert_core.cuh"

namespace gnurbs {
namespace {

using namespace inv;

__device__ __forceinline__ Ctx global_ctx(const SurfDev& s) {
  Ctx cx;
  cx.L32 = fast::global_locator<float>(s);
  cx.L64 = fast::global_locator<double>(s);
  cx.m32 = s.m32;
  cx.m64 = s.m64;
  cx.p = s.p;
  cx.q = s.q;
  cx.dom_u0 = s.dom_u0;
  cx.dom_u1 = s.dom_u1;
  cx.dom_v0 = s.dom_v0;
  cx.dom_v1 = s.dom_v1;
  return cx;
}

// Newton steps (GN where the Hessian is not positive definite) from (u, v) toward the minimum of
// |S - P|; true when they converge inside the domain, with the residual.  First the mixed
// inversion's final steps (S, Su, Sv in FP64, the curvature term from FP32 second derivatives:
// a neighbour's answer is next to the sample's minimum, where those converge as the FP64 steps
// do at a fraction of the FP64 work), then, where they do not converge, FP64 Newton steps.
template <int P, int Q>
__device__ bool continue_from(const Ctx& cx, double px, double py, double pz, double& u, double& v, double& res) {
  {
    double uu = u, vv = v;
    if (final64<P, Q>(cx, px, py, pz, uu, vv, res)) {
      u = uu;
      v = vv;
      return true;
    }
  }
  Seed<double> sd;
  sd.u = u;
  sd.v = v;
  sd.prev = INFINITY;
  sd.it = 0;
  sd.hu = 0;
  sd.hv = 0;
  sd.newton = true;
  int r = kContinue;
  while (r == kContinue) r = iterate64<P, Q>(cx, px, py, pz, sd);
  if (r != kConverged) return false;
  u = sd.u;
  v = sd.v;
  return finish64<P, Q>(cx, px, py, pz, u, v, sd.hu, sd.hv, res);
}

template <int P, int Q>
__global__ void k_pcurve_continue(SurfDev s, const double* __restrict__ C, int64_t n, const double* __restrict__ uv0,
                                  const int* __restrict__ st0, const double* __restrict__ res0,
                                  double* __restrict__ uv, int* __restrict__ st, double* __restrict__ res) {
  const Ctx cx = global_ctx(s);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double px = C[3 * i], py = C[3 * i + 1], pz = C[3 * i + 2];
    double bu = uv0[2 * i], bv = uv0[2 * i + 1], br = res0[i];
    int bs = st0[i];
    const double scale = fmax(1.0, fmax(fabs(px), fmax(fabs(py), fabs(pz))));
    for (int side = 0; side < 2; ++side) {
      const int64_t j = side == 0 ? i - 1 : i + 1;
      if (j < 0 || j >= n || st0[j] > NURBS_INV_AMBIGUOUS) continue;
      double u = uv0[2 * j], v = uv0[2 * j + 1], r;
      if (!continue_from<P, Q>(cx, px, py, pz, u, v, r)) continue;
      const bool found = bs <= NURBS_INV_AMBIGUOUS;
      // strictly closer (beyond rounding of the residual), and another minimum than the own one
      if (!found || (r < br - (1e-12 * br + 1e-14 * scale) && (fabs(u - bu) > 1e-7 || fabs(v - bv) > 1e-7))) {
        bu = u;
        bv = v;
        br = r;
        bs = NURBS_INV_FOUND;
      }
    }
    uv[2 * i] = bu;
    uv[2 * i + 1] = bv;
    res[i] = br;
    st[i] = bs;
  }
}

template <int P, int Q>
__global__ void k_pcurve_flags(SurfDev s, const double* __restrict__ C, int64_t n, const double* __restrict__ uv,
                               const int* __restrict__ st, int* __restrict__ flags) {
  const Ctx cx = global_ctx(s);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    int f = 0;
    if (st[i] > NURBS_INV_AMBIGUOUS) f |= NURBS_PCURVE_NOT_FOUND;
    if (st[i] == NURBS_INV_AMBIGUOUS) f |= NURBS_PCURVE_AMBIGUOUS;
    if (i > 0 && st[i] <= NURBS_INV_AMBIGUOUS && st[i - 1] <= NURBS_INV_AMBIGUOUS) {
      const double u = uv[2 * i], v = uv[2 * i + 1];
      int hu = 0, hv = 0;
      const fast::SDer<double> d = fast::eval_at<double, P, Q, 1>(cx.L64, cx.m64, cx.p, cx.q, u, v, hu, hv);
      // smallest singular value of J = [Su Sv]: sqrt of the smaller eigenvalue of J^T J
      const double a = dot3(d.Su, d.Su), b = dot3(d.Su, d.Sv), c = dot3(d.Sv, d.Sv);
      const double m = 0.5 * (a + c), h = 0.5 * (a - c);
      const double lmin = m - sqrt(fast::mad(h, h, b * b));
      const double dx = C[3 * i] - C[3 * i - 3], dy = C[3 * i + 1] - C[3 * i - 2], dz = C[3 * i + 2] - C[3 * i - 1];
      const double chord = sqrt(fast::mad(dz, dz, fast::mad(dy, dy, dx * dx)));
      const double du = u - uv[2 * i - 2], dv = v - uv[2 * i - 1];
      const double step = sqrt(fast::mad(dv, dv, du * du));
      if (!(lmin > 0) || step * sqrt(lmin) > 4.0 * chord + 1e-12) f |= NURBS_PCURVE_JUMP;
    }
    flags[i] = f;
  }
}

template <int P, int Q>
cudaError_t launch_pq(const SurfDev& s, const double* C, int64_t n, const double* uv0, const int* st0,
                      const double* res0, double* uv, int* st, double* res, int* flags, cudaStream_t stream) {
  const int64_t blocks = std::min<int64_t>((n + 127) / 128, 152 * 16);
  k_pcurve_continue<P, Q><<<(unsigned)blocks, 128, 0, stream>>>(s, C, n, uv0, st0, res0, uv, st, res);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_pcurve_flags<P, Q><<<(unsigned)blocks, 128, 0, stream>>>(s, C, n, uv, st, flags);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_pcurve_passes(const SurfDev& s, const double* C, int64_t n, const double* uv0, const int* st0,
                                 const double* res0, double* uv, int* st, double* res, int* flags,
                                 cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  if (s.p == 3 && s.q == 3) return launch_pq<3, 3>(s, C, n, uv0, st0, res0, uv, st, res, flags, stream);
  if (s.p == 5 && s.q == 5) return launch_pq<5, 5>(s, C, n, uv0, st0, res0, uv, st, res, flags, stream);
  if (s.p == 2 && s.q == 2) return launch_pq<2, 2>(s, C, n, uv0, st0, res0, uv, st, res, flags, stream);
  return launch_pq<0, 0>(s, C, n, uv0, st0, res0, uv, st, res, flags, stream);
}

}  // namespace gnurbs
