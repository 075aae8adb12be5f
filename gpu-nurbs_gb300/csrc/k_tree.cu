// Stage c: 2-level subdivision tree of AABBs and candidate selection (K3 tree_build).
//
// Replaces, per level, the reference's chain GetPoints -> 3x GetSecondDerivatives ->
// 3x Max_Sequential_Addressing_Shared -> TightBoundingBox (src/kernel/kernel.cu:375-431,
// 544-621, 707-733; driven by src/main.cu:280-309) with one fused kernel: one CTA per node,
// one thread per lattice sample (9x9), samples and second-derivative maxima kept in shared
// memory, box inflation K = (M1 + 2 M2 + M3) sqrt(3) / (8 (8g)^2), clip to the parent box,
// flatness test NeedDivide (kernel.cu:859-878).
// Compiled with --fmad=false and evaluated with the reference-order functions of
// gnurbs::exact, so boxes and Divided flags are bit-identical to the reference's FP64 math.
#include "nurbs_internal.h"
#include "nurbs_math.cuh"

namespace gnurbs {

__device__ __forceinline__ bool need_divide(const TreeNodeDev& n) {  // kernel.cu:859-878
  double dx = n.rt[0] - n.lb[0], dy = n.rt[1] - n.lb[1], dz = n.rt[2] - n.lb[2], t;
  if (dx > dy) { t = dx; dx = dy; dy = t; }
  if (dx > dz) { t = dx; dx = dz; dz = t; }
  if ((dx < 0.5 * dy) && (dx < 0.5 * dz)) return false;
  return true;
}

// One node of the given level for CTA index blk (block linear index bx*g + by); 96 threads.
__device__ __forceinline__ void tree_node(const SurfDev& s, int level, unsigned blk) {
  const unsigned g = level == 0 ? 1u : (unsigned)kGap;
  const unsigned bx = blk / g, by = blk % g;
  const int tree_index = level == 0 ? 0 : 1 + (int)blk;
  if (level == 1 && !s.divided[0]) {  // parent not divided: node not built
    if (threadIdx.x == 0) s.built[tree_index] = 0;
    return;
  }
  __shared__ double sM[3][kPts * kPts];
  __shared__ double sS[3][kPts * kPts];
  const int t = threadIdx.x;
  const int p = s.p, q = s.q, k2 = q + 1, k12 = (p + 1) * (q + 1);
  if (t < kPts * kPts) {
    const int tx = t / kPts, ty = t % kPts;
    // GetPoints / GetSecondDerivatives sample (kernel.cu:383-388, 412-417)
    double base_unit = 1.0 / g;
    double unit = base_unit / kGap;
    double base_u = base_unit * bx, base_v = base_unit * by;
    double p1 = base_u + tx * unit, p2 = base_v + ty * unit;
    int su = exact::find_seg(s.bu, s.ns_u, p1);
    int sv = exact::find_seg(s.bv, s.ns_v, p2);
    double du = s.bu[su + 1] - s.bu[su], dv = s.bv[sv + 1] - s.bv[sv];
    double u = (p1 - s.bu[su]) / du;
    double v = (p2 - s.bv[sv]) / dv;
    double spanU = s.range_u / du;
    double spanV = s.range_v / dv;
    exact::DenseSpan M{s.m64 + (size_t)(su * s.ns_v + sv) * k12 * 4, k2};
    v4<double> R = exact::point_r(M, p, q, u, v);
    v3<double> a = exact::der_uu(M, p, q, u, v, R, spanU);
    v3<double> b = exact::der_uv(M, p, q, u, v, R, spanU, spanV);
    v3<double> c = exact::der_vv(M, p, q, u, v, R, spanV);
    sM[0][t] = fmax(fabs(a.x), fmax(fabs(a.y), fabs(a.z)));  // kernel.cu:399
    sM[1][t] = fmax(fabs(b.x), fmax(fabs(b.y), fabs(b.z)));
    sM[2][t] = fmax(fabs(c.x), fmax(fabs(c.y), fabs(c.z)));
    v3<double> S = exact::cart(R);
    sS[0][t] = S.x;
    sS[1][t] = S.y;
    sS[2][t] = S.z;
  }
  __syncthreads();
  if (t < 9) {
    // t in 0..2: max of M_t; 3..5: max of S_(t-3); 6..8: min of S_(t-6).  Exact, so the
    // order (sequential here, a strided tree in the reference) does not change the value.
    const double* src = t < 3 ? sM[t] : sS[t < 6 ? t - 3 : t - 6];
    double acc = src[0];
    if (t < 6) {
      for (int k = 1; k < kPts * kPts; ++k) acc = acc < src[k] ? src[k] : acc;  // kernel.cu:725
    } else {
      for (int k = 1; k < kPts * kPts; ++k) acc = acc > src[k] ? src[k] : acc;  // kernel.cu:593-595
    }
    __syncwarp(0x1ffu);
    // reuse slot 0 of each array for the reduced value
    __shared__ double red[9];
    red[t] = acc;
    __syncwarp(0x1ffu);
    if (t == 0) {
      unsigned den = 8u * kGap * g * kGap * g;
      double K = (red[0] + 2 * red[1] + red[2]) * 1.7320508075688772 / den;  // sqrt(3), kernel.cu:574
      TreeNodeDev n;
      n.rt[0] = red[3] + K;
      n.rt[1] = red[4] + K;
      n.rt[2] = red[5] + K;
      n.lb[0] = red[6] - K;
      n.lb[1] = red[7] - K;
      n.lb[2] = red[8] - K;
      double uunit = 1.0 / g;  // kernel.cu:604-605
      n.uv_lb[0] = bx * uunit;
      n.uv_lb[1] = by * uunit;
      n.uv_rt[0] = (bx + 1) * uunit;
      n.uv_rt[1] = (by + 1) * uunit;
      if (level == 1) {  // min/max(TreeNode) against the parent (kernel.cu:606-611, 885-901)
        const TreeNodeDev& P = s.tree[0];
        for (int k = 0; k < 3; ++k) {
          n.rt[k] = fmin(n.rt[k], P.rt[k]);
          n.lb[k] = fmax(n.lb[k], P.lb[k]);
        }
      }
      s.tree[tree_index] = n;
      s.divided[tree_index] = need_divide(n) ? 1 : 0;
      s.built[tree_index] = 1;
    }
  }
}

__global__ void __launch_bounds__(96) k_tree_level(SurfDev s, int level) { tree_node(s, level, blockIdx.x); }

// Many surfaces: blockIdx.y selects the surface of ids[] in the device table.
__global__ void __launch_bounds__(96) k_tree_level_batched(const SurfDev* __restrict__ table,
                                                            const int* __restrict__ ids, int level) {
  const SurfDev s = table[ids[blockIdx.y]];
  tree_node(s, level, blockIdx.x);
}

// NewInverse's scan (kernel.cu:456-457) over built nodes, NewBoundingBoxCheck (:466-469).
__global__ void k_candidates(SurfDev s, const double* __restrict__ P, int64_t n, int* __restrict__ list,
                             int* __restrict__ counts) {
  __shared__ double box[kTreeNodes][6];
  __shared__ unsigned char built[kTreeNodes];
  for (int k = threadIdx.x; k < kTreeNodes; k += blockDim.x) {
    built[k] = s.built[k];
    for (int c = 0; c < 3; ++c) {
      box[k][c] = s.tree[k].lb[c];
      box[k][3 + c] = s.tree[k].rt[c];
    }
  }
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double x = P[3 * i], y = P[3 * i + 1], z = P[3 * i + 2];
    int cnt = 0;
    for (int k = 0; k < kTreeNodes; ++k) {
      if (!built[k]) continue;
      if ((x >= box[k][0]) && (y >= box[k][1]) && (z >= box[k][2]) && (x <= box[k][3]) && (y <= box[k][4]) &&
          (z <= box[k][5]))
        list[i * kTreeNodes + cnt++] = k;
    }
    counts[i] = cnt;
  }
}

// ---- normal cones of the built nodes (the projection's culling data)
// Per node: the normal N = Su x Sv and its second derivatives at the node's 9x9 lattice (the box
// tree's samples, evaluated by exact::ders3), the normal box widened by the box tree's bound K
// applied to N and clipped to the parent's, the cone around the box centre, the node's bound box
// (its box intersected with the box of the control points acting on its parameter rectangle)
// and the lattice's surface points; everything in the oracle's order of operations, so the
// records are bit-identical to the oracle's.  Record layout: nurbs_internal.h.
__device__ __forceinline__ float round_down(double x) { return __double2float_rd(x); }
__device__ __forceinline__ float round_up(double x) { return __double2float_ru(x); }

__device__ __forceinline__ void cone_node(const SurfDev& s, int level, unsigned blk) {
  const unsigned g = level == 0 ? 1u : (unsigned)kGap;
  const unsigned bx = blk / g, by = blk % g;
  const int k = level == 0 ? 0 : 1 + (int)blk;
  if (!s.built[k]) return;
  __shared__ double sN[6][kPts * kPts];  // N xyz, then max |N_uu|, |N_uv|, |N_vv| components
  __shared__ double red[9];
  __shared__ double hull[96][6];
  const int t = threadIdx.x;
  const int p = s.p, q = s.q, k2 = q + 1, k12 = (p + 1) * (q + 1);
  if (t < kPts * kPts) {
    const int tx = t / kPts, ty = t % kPts;
    double base_unit = 1.0 / g;
    double unit = base_unit / kGap;
    double base_u = base_unit * bx, base_v = base_unit * by;
    double p1 = base_u + tx * unit, p2 = base_v + ty * unit;
    int su = exact::find_seg(s.bu, s.ns_u, p1);
    int sv = exact::find_seg(s.bv, s.ns_v, p2);
    double du = s.bu[su + 1] - s.bu[su], dv = s.bv[sv + 1] - s.bv[sv];
    double u = (p1 - s.bu[su]) / du;
    double v = (p2 - s.bv[sv]) / dv;
    exact::DenseSpan M{s.m64 + (size_t)(su * s.ns_v + sv) * k12 * 4, k2};
    v3<double> d[10], n[4];
    exact::ders3(M, p, q, u, v, s.range_u / du, s.range_v / dv, d);
    exact::normal_ders2(d, n);
    sN[0][t] = n[0].x;
    sN[1][t] = n[0].y;
    sN[2][t] = n[0].z;
    sN[3][t] = fmax(fabs(n[1].x), fmax(fabs(n[1].y), fabs(n[1].z)));
    sN[4][t] = fmax(fabs(n[2].x), fmax(fabs(n[2].y), fabs(n[2].z)));
    sN[5][t] = fmax(fabs(n[3].x), fmax(fabs(n[3].y), fabs(n[3].z)));
    float* o = s.lattice + (size_t)(k * kPts * kPts + t) * 3;
    o[0] = (float)(d[0].x - s.org[0]);
    o[1] = (float)(d[0].y - s.org[1]);
    o[2] = (float)(d[0].z - s.org[2]);
  }
  // control points acting on the node's parameter rectangle (uv_lb, uv_rt of the tree node)
  {
    const TreeNodeDev& T = s.tree[k];
    int i0 = exact::find_seg(s.bu, s.ns_u, T.uv_lb[0]), i1 = exact::find_seg(s.bu, s.ns_u, T.uv_rt[0]);
    int j0 = exact::find_seg(s.bv, s.ns_v, T.uv_lb[1]), j1 = exact::find_seg(s.bv, s.ns_v, T.uv_rt[1]);
    if (i1 > i0 && s.bu[i1] >= T.uv_rt[0]) --i1;  // the span starting at the right end
    if (j1 > j0 && s.bv[j1] >= T.uv_rt[1]) --j1;
    const int a0 = s.knot_u[i0] - p, a1 = s.knot_u[i1], b0 = s.knot_v[j0] - q, b1 = s.knot_v[j1];
    const int nb = b1 - b0 + 1, cnt = (a1 - a0 + 1) * nb;
    double h[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
    for (int e = t; e < cnt; e += blockDim.x) {
      const double* x = s.cps + 3 * ((size_t)(a0 + e / nb) * s.nv + (b0 + e % nb));
      for (int c = 0; c < 3; ++c) {
        h[c] = h[c] > x[c] ? x[c] : h[c];
        h[3 + c] = h[3 + c] < x[c] ? x[c] : h[3 + c];
      }
    }
    for (int c = 0; c < 6; ++c) hull[t][c] = h[c];
  }
  __syncthreads();
  if (t < 9) {
    // 0..2: max of the N_uu, N_uv, N_vv maxima; 3..5: max of N; 6..8: min of N (exact, any order)
    const double* src = t < 3 ? sN[3 + t] : sN[t < 6 ? t - 3 : t - 6];
    double acc = src[0];
    if (t < 6) {
      for (int j = 1; j < kPts * kPts; ++j) acc = acc < src[j] ? src[j] : acc;
    } else {
      for (int j = 1; j < kPts * kPts; ++j) acc = acc > src[j] ? src[j] : acc;
    }
    red[t] = acc;
  }
  __syncthreads();
  if (t == 0) {
    unsigned den = 8u * kGap * g * kGap * g;
    double K = (red[0] + 2 * red[1] + red[2]) * 1.7320508075688772 / den;
    double nb[6];
    for (int c = 0; c < 3; ++c) {
      nb[c] = red[6 + c] - K;
      nb[3 + c] = red[3 + c] + K;
      if (level == 1) {
        nb[c] = fmax(nb[c], s.nbox[c]);
        nb[3 + c] = fmin(nb[3 + c], s.nbox[3 + c]);
      }
    }
    for (int c = 0; c < 6; ++c) s.nbox[6 * k + c] = nb[c];
    double hb[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
    for (int j = 0; j < (int)blockDim.x; ++j)
      for (int c = 0; c < 3; ++c) {
        hb[c] = hb[c] > hull[j][c] ? hull[j][c] : hb[c];
        hb[3 + c] = hb[3 + c] < hull[j][3 + c] ? hull[j][3 + c] : hb[3 + c];
      }
    // the node's own box where it is narrower
    const TreeNodeDev& T = s.tree[k];
    double xb[6];
    bool empty = false;
    for (int c = 0; c < 3; ++c) {
      xb[c] = hb[c] > T.lb[c] ? hb[c] : T.lb[c];
      xb[3 + c] = hb[3 + c] < T.rt[c] ? hb[3 + c] : T.rt[c];
      empty = empty || xb[c] > xb[3 + c];
    }
    const double* bb = empty ? hb : xb;
    float* rec = s.cone + kConeStride * k;
    double ctr[3], hh[3];
    for (int c = 0; c < 3; ++c) {
      ctr[c] = (bb[c] + bb[3 + c]) / 2;
      hh[c] = (bb[3 + c] - bb[c]) / 2;
    }
    const double r = sqrt(hh[0] * hh[0] + hh[1] * hh[1] + hh[2] * hh[2]);
    const double cm = fmax(fabs(ctr[0] - s.org[0]), fmax(fabs(ctr[1] - s.org[1]), fabs(ctr[2] - s.org[2])));
    for (int c = 0; c < 3; ++c) rec[c] = (float)(ctr[c] - s.org[c]);
    rec[3] = (float)(r * (1 + 0x1p-20) + cm * 0x1p-20);
    bool all = nb[0] > nb[3] || nb[1] > nb[4] || nb[2] > nb[5];
    all = all || (nb[0] <= 0 && nb[3] >= 0 && nb[1] <= 0 && nb[4] >= 0 && nb[2] <= 0 && nb[5] >= 0);
    double cosA = 0, sinA = 1, ax[3] = {0, 0, 1};
    if (!all) {
      const double m[3] = {(nb[0] + nb[3]) / 2, (nb[1] + nb[4]) / 2, (nb[2] + nb[5]) / 2};
      const double mm = sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]);
      double cmin = 1;
      for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j)
          for (int l = 0; l < 2; ++l) {
            const double c[3] = {nb[3 * i], nb[3 * j + 1], nb[3 * l + 2]};
            const double cc = (m[0] * c[0] + m[1] * c[1] + m[2] * c[2]) / (mm * sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]));
            cmin = cmin < cc ? cmin : cc;
          }
      if (cmin > 0) {
        const double sn = sqrt(fmax(0.0, 1 - cmin * cmin));
        const double tt = 0x1p-11, cd = (1 - tt * tt) / (1 + tt * tt), sd = (2 * tt) / (1 + tt * tt);
        const double ca = cmin * cd - sn * sd, sa = sn * cd + cmin * sd;
        if (ca > 0) {
          cosA = ca;
          sinA = sa;
          ax[0] = m[0] / mm;
          ax[1] = m[1] / mm;
          ax[2] = m[2] / mm;
        }
      }
    }
    for (int c = 0; c < 3; ++c) rec[4 + c] = (float)ax[c];
    rec[7] = (float)cosA;
    rec[8] = (float)sinA;
    for (int c = 0; c < 3; ++c) {
      rec[9 + c] = round_down(bb[c] - s.org[c]);
      rec[12 + c] = round_up(bb[3 + c] - s.org[c]);
    }
    for (int c = 15; c < kConeStride; ++c) rec[c] = 0;
  }
}

__global__ void __launch_bounds__(96) k_cone_level(SurfDev s, int level) { cone_node(s, level, blockIdx.x); }

cudaError_t launch_cones(const SurfDev& s, cudaStream_t st) {
  k_cone_level<<<1, 96, 0, st>>>(s, 0);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_cone_level<<<kGap * kGap, 96, 0, st>>>(s, 1);
  return cudaGetLastError();
}

cudaError_t launch_tree(const SurfDev& s, cudaStream_t st) {
  k_tree_level<<<1, 96, 0, st>>>(s, 0);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_tree_level<<<kGap * kGap, 96, 0, st>>>(s, 1);
  return cudaGetLastError();
}

cudaError_t launch_tree_batched(const SurfDev* table, const int* ids, int count, cudaStream_t st) {
  for (int off = 0; off < count; off += 65535) {
    int c = count - off < 65535 ? count - off : 65535;
    k_tree_level_batched<<<dim3(1, c), 96, 0, st>>>(table, ids + off, 0);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  for (int off = 0; off < count; off += 65535) {
    int c = count - off < 65535 ? count - off : 65535;
    k_tree_level_batched<<<dim3(kGap * kGap, c), 96, 0, st>>>(table, ids + off, 1);
  }
  return cudaGetLastError();
}

cudaError_t launch_candidates(const SurfDev& s, const double* P, int64_t n, int* list, int* counts,
                              cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  int64_t blocks = (n + 255) / 256;
  if (blocks > 152 * 32) blocks = 152 * 32;
  k_candidates<<<(unsigned)blocks, 256, 0, st>>>(s, P, n, list, counts);
  return cudaGetLastError();
}

}  // namespace gnurbs
