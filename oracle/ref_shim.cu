// REFERENCE SHIM — test infrastructure only; builds oracle/_ref/libnurbs_ref.so.
//
// Compiles the reference's own FP64 device functions (Qiang-Zou/GPU-NURBS, GPLv3) for the
// host by including its sources by path from REF_DIR — nothing is copied into this
// repository.  `__device__` is re-marked `__host__ __device__` before the includes so that
// Nrc, findSpan, MatrixSurfacePoint, the old MatrixSurfaceDerivative{U,V,UU,UV,VV},
// GaussNewton, NeedDivide, min/max(TreeNode) and NewBoundingBoxCheck become host-callable.
// The __global__ bodies that drive them are restated below as host loops (a few lines each).
// Used only to pin the C oracle (nurbs_oracle.c) and to generate golden fixtures.
#include <cuda_runtime.h>
#include <cublas_v2.h>
#include <cuda_fp16.h>
#include <curand_kernel.h>
#include <device_launch_parameters.h>
#include <cuda.h>
#include <cstring>

#undef __device__
#define __device__ __host__ __location__(device)

#include "src/util/Operator.cu"
#include "src/util/ExtraMath.cu"
#include "src/util/Matrix.cu"
#include "src/NURBS/Evaluate.cu"
#include "src/kernel/kernel.cu"

static double3* make_cps(const double* cps, int n) {
  double3* p = new double3[n];
  for (int k = 0; k < n; ++k) p[k] = {cps[3 * k], cps[3 * k + 1], cps[3 * k + 2]};
  return p;
}

extern "C" {

// GetMatrixN (src/NURBS/Evaluate.cu:3-88) as a host loop; the eight child
// gpu_matrix_mult launches become matrix_mult calls in the same order.
int ref_matrix_n(int p, int q, int nu, int nv, const double* ku_c, const double* kv_c,
                 const double* cps, const double* w_c, double* MatrixN) {
  double* ku = const_cast<double*>(ku_c);
  double* kv = const_cast<double*>(kv_c);
  double* weights = const_cast<double*>(w_c);
  double3* control_points = make_cps(cps, nu * nv);
  int written = 0;
  for (int i = 0; i < p + nu; ++i)
    for (int j = 0; j < q + nv; ++j) {
      if (ku[i] == ku[i + 1] || kv[j] == kv[j + 1]) continue;
      if (i < p || i >= nu || j < q || j >= nv) continue;  // outside the clamped domain
      int k1 = p + 1, k2 = q + 1;
      double* Nu = new double[k1 * k1];
      double* NvT = new double[k2 * k2];
      for (int m = 0; m < k1; m++)
        for (int n = 0; n < k1; n++) Nu[m * k1 + n] = Nrc(ku, p, m + 1, n + 1, i - (p - 1), i - (p - 1), p);
      for (int m = 0; m < k2; m++)
        for (int n = 0; n < k2; n++) NvT[n * k2 + m] = Nrc(kv, q, m + 1, n + 1, j - (q - 1), j - (q - 1), q);
      double* Mid[4];
      double* Tmp[4];
      for (int c = 0; c < 4; ++c) { Mid[c] = new double[k1 * k2]; Tmp[c] = new double[k1 * k2]; }
      for (int s = 0; s <= p; s++)
        for (int l = 0; l <= q; l++) {
          double w = weights[(s + i - p) * nv + (l + j - q)];
          Mid[0][s * k2 + l] = control_points[(s + i - p) * nv + (l + j - q)].x * w;
          Mid[1][s * k2 + l] = control_points[(s + i - p) * nv + (l + j - q)].y * w;
          Mid[2][s * k2 + l] = control_points[(s + i - p) * nv + (l + j - q)].z * w;
          Mid[3][s * k2 + l] = w;
        }
      for (int c = 0; c < 4; ++c) matrix_mult(Mid[c], NvT, Tmp[c], k1, k2, k2);
      for (int c = 0; c < 4; ++c)
        matrix_mult(Nu, Tmp[c], MatrixN + MatrixNPosition(i, j, p, q, nu, nv, c), k1, k1, k2);
      for (int c = 0; c < 4; ++c) { delete[] Mid[c]; delete[] Tmp[c]; }
      delete[] Nu;
      delete[] NvT;
      ++written;
    }
  delete[] control_points;
  return written;
}

// Point + old-style derivatives at n parameter pairs; out is SoA blocks in the order
// S, Su, Sv, Suu, Suv, Svv restricted to the mask bits (1,2,4,8,16,32).
void ref_eval(int p, int q, int nu, int nv, const double* ku_c, const double* kv_c, const double* MN_c,
              const double* uv, long long n, unsigned mask, double* out) {
  double* knots_u = const_cast<double*>(ku_c);
  double* knots_v = const_cast<double*>(kv_c);
  double* MatrixN = const_cast<double*>(MN_c);
  for (long long k = 0; k < n; ++k) {
    double uu = uv[2 * k], vv = uv[2 * k + 1];
    int m = findSpan(p, nu, knots_u, uu);
    int nn = findSpan(q, nv, knots_v, vv);
    double u = (uu - knots_u[m]) / (knots_u[m + 1] - knots_u[m]);
    double v = (vv - knots_v[nn]) / (knots_v[nn + 1] - knots_v[nn]);
    double spanU = (knots_u[p + nu] - knots_u[0]) / (knots_u[m + 1] - knots_u[m]);
    double spanV = (knots_v[q + nv] - knots_v[0]) / (knots_v[nn + 1] - knots_v[nn]);
    double* middle = MatrixN + MatrixNPosition(m, nn, p, q, nu, nv, 0);
    double4 R = MatrixSurfacePoint(middle, p, q, nu, nv, knots_u, knots_v, u, v);
    double3 blk[6];
    blk[0] = homogenousToCartesian(R);
    if (mask & 2) blk[1] = MatrixSurfaceDerivativeU(middle, p, q, nu, nv, knots_u, knots_v, u, v, R, spanU);
    if (mask & 4) blk[2] = MatrixSurfaceDerivativeV(middle, p, q, nu, nv, knots_u, knots_v, u, v, R, spanV);
    if (mask & 8) blk[3] = MatrixSurfaceDerivativeUU(middle, p, q, nu, nv, knots_u, knots_v, u, v, R, spanU, spanV);
    if (mask & 16) blk[4] = MatrixSurfaceDerivativeUV(middle, p, q, nu, nv, knots_u, knots_v, u, v, R, spanU, spanV);
    if (mask & 32) blk[5] = MatrixSurfaceDerivativeVV(middle, p, q, nu, nv, knots_u, knots_v, u, v, R, spanU, spanV);
    int o = 0;
    for (int b = 0; b < 6; ++b) {
      if (!((mask >> b) & 1u)) continue;
      out[(3 * o + 0) * n + k] = blk[b].x;
      out[(3 * o + 1) * n + k] = blk[b].y;
      out[(3 * o + 2) * n + k] = blk[b].z;
      ++o;
    }
  }
}

// The 2-level build of src/main.cu:280-309 with the bodies of GetPoints (kernel.cu:404-431),
// GetSecondDerivatives (:375-402), Max_Sequential_Addressing_Shared (:707-733) and
// TightBoundingBox (:544-621) restated per node.  tree: 65 nodes x 10 doubles
// (uv lb, uv rt, lb xyz, rt xyz); divided/built: 65 bytes.
void ref_build_tree(int p, int q, int nu, int nv, const double* ku_c, const double* kv_c, const double* MN_c,
                    double* tree_out, unsigned char* divided_out, unsigned char* built_out) {
  double* knots_u = const_cast<double*>(ku_c);
  double* knots_v = const_cast<double*>(kv_c);
  double* MatrixN = const_cast<double*>(MN_c);
  TreeNode Tree[TwoLayerTree];
  bool Divided[TwoLayerTree];
  memset(Tree, 0, sizeof(Tree));
  memset(Divided, 0, sizeof(Divided));
  memset(built_out, 0, TwoLayerTree);
  Divided[0] = true;  // src/main.cu:153
  int base = 0;
  unsigned g = 1;
  for (int level = 0; level < 2; ++level) {
    for (unsigned bx = 0; bx < g; ++bx)
      for (unsigned by = 0; by < g; ++by) {
        int block_linear = (int)(bx * g + by);
        int parent_index = (base + block_linear - 1) / ChildrenNumber;
        if (!(parent_index < 0 || Divided[parent_index])) continue;
        double base_unit = 1.0 / g;
        double unit = base_unit / GapPerEdge;
        double base_u = base_unit * bx, base_v = base_unit * by;
        double d1[PointsPerBlock], d2[PointsPerBlock], d3v[PointsPerBlock];
        double3 S[PointsPerBlock];
        for (unsigned tx = 0; tx < PointsPerEdge; ++tx)
          for (unsigned ty = 0; ty < PointsPerEdge; ++ty) {
            int idx = tx * PointsPerEdge + ty;
            double p1 = base_u + tx * unit, p2 = base_v + ty * unit;
            int m = findSpan(p, nu, knots_u, p1);
            int n = findSpan(q, nv, knots_v, p2);
            double u = (p1 - knots_u[m]) / (knots_u[m + 1] - knots_u[m]);
            double v = (p2 - knots_v[n]) / (knots_v[n + 1] - knots_v[n]);
            double spanU = (knots_u[p + nu] - knots_u[0]) / (knots_u[m + 1] - knots_u[m]);
            double spanV = (knots_v[q + nv] - knots_v[0]) / (knots_v[n + 1] - knots_v[n]);
            double* middle = MatrixN + MatrixNPosition(m, n, p, q, nu, nv, 0);
            double4 R = MatrixSurfacePoint(middle, p, q, nu, nv, knots_u, knots_v, u, v);
            double3 a = MatrixSurfaceDerivativeUU(middle, p, q, nu, nv, knots_u, knots_v, u, v, R, spanU, spanV);
            double3 b = MatrixSurfaceDerivativeUV(middle, p, q, nu, nv, knots_u, knots_v, u, v, R, spanU, spanV);
            double3 c = MatrixSurfaceDerivativeVV(middle, p, q, nu, nv, knots_u, knots_v, u, v, R, spanU, spanV);
            d1[idx] = fmax(fabs(a.x), fmax(fabs(a.y), fabs(a.z)));
            d2[idx] = fmax(fabs(b.x), fmax(fabs(b.y), fabs(b.z)));
            d3v[idx] = fmax(fabs(c.x), fmax(fabs(c.y), fabs(c.z)));
            S[idx] = homogenousToCartesian(R);
          }
        // the shared-memory tree reductions of the reference, sequentially (exact)
        double M1 = d1[0], M2 = d2[0], M3 = d3v[0];
        double3 mx = S[0], mn = S[0];
        for (int k = 1; k < PointsPerBlock; ++k) {
          M1 = M1 < d1[k] ? d1[k] : M1;
          M2 = M2 < d2[k] ? d2[k] : M2;
          M3 = M3 < d3v[k] ? d3v[k] : M3;
          mx.x = mx.x < S[k].x ? S[k].x : mx.x;
          mx.y = mx.y < S[k].y ? S[k].y : mx.y;
          mx.z = mx.z < S[k].z ? S[k].z : mx.z;
          mn.x = mn.x > S[k].x ? S[k].x : mn.x;
          mn.y = mn.y > S[k].y ? S[k].y : mn.y;
          mn.z = mn.z > S[k].z ? S[k].z : mn.z;
        }
        int tree_index = base + block_linear;
        double K = (M1 + 2 * M2 + M3) * sqrt(3.0) / (8 * GapPerEdge * g * GapPerEdge * g);
        Tree[tree_index].right_top = {mx.x + K, mx.y + K, mx.z + K};
        Tree[tree_index].left_bottom = {mn.x - K, mn.y - K, mn.z - K};
        double uunit = 1.0 / g;
        Tree[tree_index].uv = {{bx * uunit, by * uunit}, {(bx + 1) * uunit, (by + 1) * uunit}};
        int pidx = (tree_index - 1) / ChildrenNumber;
        if (pidx >= 0) {
          Tree[tree_index] = min(Tree[tree_index], Tree[pidx]);
          Tree[tree_index] = max(Tree[tree_index], Tree[pidx]);
        }
        Divided[tree_index] = NeedDivide(Tree[tree_index]);
        built_out[tree_index] = 1;
      }
    base += g * g;
    g *= GapPerEdge;
  }
  for (int t = 0; t < TwoLayerTree; ++t) {
    double* o = tree_out + 10 * t;
    o[0] = Tree[t].uv.left_bottom.x; o[1] = Tree[t].uv.left_bottom.y;
    o[2] = Tree[t].uv.right_top.x; o[3] = Tree[t].uv.right_top.y;
    o[4] = Tree[t].left_bottom.x; o[5] = Tree[t].left_bottom.y; o[6] = Tree[t].left_bottom.z;
    o[7] = Tree[t].right_top.x; o[8] = Tree[t].right_top.y; o[9] = Tree[t].right_top.z;
    divided_out[t] = Divided[t] ? 1 : 0;
  }
}

// NewBoundingBoxCheck (kernel.cu:466-469) for one node given as 10 doubles.
int ref_box_check(const double* node10, const double* P) {
  TreeNode T;
  T.uv = {{node10[0], node10[1]}, {node10[2], node10[3]}};
  T.left_bottom = {node10[4], node10[5], node10[6]};
  T.right_top = {node10[7], node10[8], node10[9]};
  return NewBoundingBoxCheck(T, double3{P[0], P[1], P[2]}) ? 1 : 0;
}

// The reference GaussNewton exactly as shipped (kernel.cu:151-249).
int ref_gauss_newton(int p, int q, int nu, int nv, const double* ku_c, const double* kv_c, const double* MN_c,
                     const double* node_uv4, const double* P, double max_edge, double* uv_out) {
  Node node = {{node_uv4[0], node_uv4[1]}, {node_uv4[2], node_uv4[3]}};
  bool flag = false;
  double2 result = {0, 0};
  bool ok = GaussNewton(node, double3{P[0], P[1], P[2]}, max_edge, const_cast<double*>(MN_c), p, q, nu, nv,
                        const_cast<double*>(ku_c), const_cast<double*>(kv_c), nullptr, nullptr, &flag, &result, 0);
  uv_out[0] = result.x;
  uv_out[1] = result.y;
  return ok ? 1 : 0;
}

// findSpan (Evaluate.cu:504-533)
int ref_find_span(int degree, int cp, const double* knots, double u) {
  return findSpan(degree, cp, const_cast<double*>(knots), u);
}

// The projection path's derivatives at (uu, vv): GetVector's power vectors (kernel.cu:1386-1450,
// restated for one point), MatrixSurfaceRd* (Evaluate.cu:288-502), the new-style quotient forms
// (:932-1020) and SurfaceNormalDerivative{UU,UV,VV} (:1125-1135).  out[42]: S, Su, Sv, Suu, Suv,
// Svv, Suuu, Suuv, Suvv, Svvv, N = Su x Sv, Nuu, Nuv, Nvv (xyz each).
void ref_ders3(int p, int q, int nu, int nv, const double* ku_c, const double* kv_c, const double* MN_c, double uu,
               double vv, double* out) {
  double* knots_u = const_cast<double*>(ku_c);
  double* knots_v = const_cast<double*>(kv_c);
  double* MatrixN = const_cast<double*>(MN_c);
  int m = findSpan(p, nu, knots_u, uu);
  int n = findSpan(q, nv, knots_v, vv);
  double u = (uu - knots_u[m]) / (knots_u[m + 1] - knots_u[m]);
  double v = (vv - knots_v[n]) / (knots_v[n + 1] - knots_v[n]);
  double spanU = (knots_u[p + nu] - knots_u[0]) / (knots_u[m + 1] - knots_u[m]);
  double spanV = (knots_v[q + nv] - knots_v[0]) / (knots_v[n + 1] - knots_v[n]);
  double* middle = MatrixN + MatrixNPosition(m, n, p, q, nu, nv, 0);
  const int k1 = p + 1, k2 = q + 1;
  double U[4][MAX_DEGREE], V[4][MAX_DEGREE];
  for (int d = 0; d < 2; ++d) {
    double* W = d == 0 ? U[0] : V[0];
    double* W1 = d == 0 ? U[1] : V[1];
    double* W2 = d == 0 ? U[2] : V[2];
    double* W3 = d == 0 ? U[3] : V[3];
    const int k = d == 0 ? k1 : k2;
    const double t = d == 0 ? u : v;
    double now = 1;
    for (int i = 0; i < k; i++) { W[i] = now; now *= t; }
    W1[0] = 0;
    for (int i = 0; i < k - 1; i++) W1[i + 1] = (i + 1) * W[i];
    W2[0] = W2[1] = 0;
    for (int i = 0; i < k - 2; i++) W2[i + 2] = (i + 2) * (i + 1) * W[i];
    W3[0] = W3[1] = W3[2] = 0;
    for (int i = 0; i < k - 3; i++) W3[i + 3] = (i + 3) * (i + 2) * (i + 1) * W[i];
  }
  double4 R = MatrixSurfacePoint(middle, p, q, nu, nv, knots_u, knots_v, u, v);
  double4 RdU = MatrixSurfaceRdU(middle, p, q, nu, nv, knots_u, knots_v, u, v, U[1], V[0], spanU);
  double4 RdV = MatrixSurfaceRdV(middle, p, q, nu, nv, knots_u, knots_v, u, v, U[0], V[1], spanV);
  double4 RdUU = MatrixSurfaceRdUU(middle, p, q, nu, nv, knots_u, knots_v, u, v, U[2], V[0], spanU);
  double4 RdUV = MatrixSurfaceRdUV(middle, p, q, nu, nv, knots_u, knots_v, u, v, U[1], V[1], spanU, spanV);
  double4 RdVV = MatrixSurfaceRdVV(middle, p, q, nu, nv, knots_u, knots_v, u, v, U[0], V[2], spanV);
  double4 RdUUU = MatrixSurfaceRdUUU(middle, p, q, nu, nv, knots_u, knots_v, u, v, U[3], V[0], spanU);
  double4 RdUUV = MatrixSurfaceRdUUV(middle, p, q, nu, nv, knots_u, knots_v, u, v, U[2], V[1], spanU, spanV);
  double4 RdUVV = MatrixSurfaceRdUVV(middle, p, q, nu, nv, knots_u, knots_v, u, v, U[1], V[2], spanU, spanV);
  double4 RdVVV = MatrixSurfaceRdVVV(middle, p, q, nu, nv, knots_u, knots_v, u, v, U[0], V[3], spanV);
  const double h = R.w;
  double3 P = homogenousToCartesian(R);
  double3 PdU = MatrixSurfaceDerivativeU(RdU, P, h);
  double3 PdV = MatrixSurfaceDerivativeV(RdV, P, h);
  double3 PdUU = MatrixSurfaceDerivativeUU(RdUU, PdU, P, h, RdU.w);
  double3 PdUV = MatrixSurfaceDerivativeUV(RdUV, PdU, PdV, P, h, RdU.w, RdV.w);
  double3 PdVV = MatrixSurfaceDerivativeVV(RdVV, PdV, P, h, RdV.w);
  double3 PdUUU = MatrixSurfaceDerivativeUUU(RdUUU, PdUU, PdU, P, h, RdU.w, RdUU.w);
  double3 PdUUV = MatrixSurfaceDerivativeUUV(RdUUV, PdUU, PdUV, PdU, PdV, P, h, RdU.w, RdV.w, RdUU.w, RdUV.w);
  double3 PdUVV = MatrixSurfaceDerivativeUVV(RdUVV, PdUV, PdVV, PdU, PdV, P, h, RdU.w, RdV.w, RdUV.w, RdVV.w);
  double3 PdVVV = MatrixSurfaceDerivativeVVV(RdVVV, PdVV, PdV, P, h, RdV.w, RdVV.w);
  const double3 blk[14] = {P, PdU, PdV, PdUU, PdUV, PdVV, PdUUU, PdUUV, PdUVV, PdVVV, cross_product(PdU, PdV),
                           SurfaceNormalDerivativeUU(PdU, PdV, PdUU, PdUV, PdUUU, PdUUV),
                           SurfaceNormalDerivativeUV(PdU, PdV, PdUU, PdUV, PdVV, PdUUV, PdUVV),
                           SurfaceNormalDerivativeVV(PdU, PdV, PdUV, PdVV, PdUVV, PdVVV)};
  for (int b = 0; b < 14; ++b) {
    out[3 * b] = blk[b].x;
    out[3 * b + 1] = blk[b].y;
    out[3 * b + 2] = blk[b].z;
  }
}

// BoundingBoxCheck (kernel.cu:106-149) and getSplitType (:251-298) of the first inversion for one
// node given as 4 doubles (lb.u, lb.v, rt.u, rt.v).
int ref_qt_box_check(int p, int q, int nu, int nv, const double* ku_c, const double* kv_c, const double* cps,
                     const double* node4, const double* P, double max_edge) {
  double3* control_points = make_cps(cps, nu * nv);
  Node nd = {{node4[0], node4[1]}, {node4[2], node4[3]}};
  bool r = BoundingBoxCheck(nd, double3{P[0], P[1], P[2]}, max_edge, p, q, nu, nv, const_cast<double*>(ku_c),
                            const_cast<double*>(kv_c), control_points);
  delete[] control_points;
  return r ? 1 : 0;
}

int ref_qt_split_type(int p, int q, int nu, int nv, const double* ku_c, const double* kv_c, const double* MN_c,
                      const double* node4, double max_edge) {
  Node nd = {{node4[0], node4[1]}, {node4[2], node4[3]}};
  return (int)getSplitType(nd, max_edge, const_cast<double*>(MN_c), p, q, nu, nv, const_cast<double*>(ku_c),
                           const_cast<double*>(kv_c), nullptr, nullptr);
}

}  // extern "C"
