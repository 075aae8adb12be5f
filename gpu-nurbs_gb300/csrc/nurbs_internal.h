// Internal host/device declarations of the GB300 NURBS engine (not part of the C-ABI).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace gnurbs {

constexpr int kMaxDegree = 7;     // p, q <= 7 (reference MAX_DEGREE 8 = p+1)
constexpr int kTreeNodes = 65;    // root + 8x8 children

// Coefficients per span in the FP32 span table: (p+1)(q+1) rounded up to even, so every span
// starts 32-byte aligned and coefficient pairs can be read with one 256-bit load.
__host__ __device__ inline int span_coefs32(int p, int q) {
  const int k = (p + 1) * (q + 1);
  return k + (k & 1);
}
constexpr int kGap = 8;           // GapPerEdge (src/kernel/kernel.cuh:17)
constexpr int kPts = kGap + 1;    // PointsPerEdge
constexpr int kConeStride = 20;   // floats per normal-cone record

// Device view of one surface.  All pointers are device pointers into the surface's arena.
//
// HBM layout (one arena per surface, 256-byte aligned sub-buffers):
//   bu[ns_u+1], bv[ns_v+1]           breakpoints = distinct knots of the domain, ascending
//   inv_du[ns_u], inv_dv[ns_v]       1/(bu[s+1]-bu[s])
//   bu32/bv32, inv_du32/inv_dv32     the same in FP32 (mixed-precision seeding)
//   knot_u[ns_u], knot_v[ns_v]       knot index m of span s (k[m] = bu[s]) for the reference layout
//   m64[ns_u*ns_v][k1][k2][4]        span matrices, homogeneous components (xw, yw, zw, w)
//                                    innermost, so one (a,b) coefficient is one 32-byte vector
//   m32                              the same for the surface translated by -org, rounded to FP32
//                                    (16 bytes per coefficient): FP32 evaluation works in coordinates
//                                    relative to the control net's centre, so its resolution is set by
//                                    the surface's extent, not by its distance from the origin
//   tree[65]                         TreeNodeDev; divided[65], built[65]
//   cd32[65][9], cd64[65][9]         S, Su, Sv at every built node's uv-centre (the inversion seeds),
//                                    FP32 (relative to org) and FP64, written after the tree
//   nbox[65][6]                      normal boxes (lb xyz, rt xyz) of the built nodes
//   cone[65][kConeStride]            FP32 projection culling record of each built node, relative to
//                                    org: bound-box ball centre (0..2) and radius (3), normal-cone
//                                    axis (4..6), cos and sin of its half-angle (7, 8; 0 and 1 for
//                                    every direction), bound box rounded outward (lb 9..11,
//                                    rt 12..14), zero (15..19)
//   lattice[65][81][3]               surface points of each node's 9x9 lattice (index 9 tx + ty),
//                                    FP32 relative to org: distance bounds and projection seeds
//   qtbox[21][6]                     control-point boxes of the quadtree inversion's square nodes of
//                                    depth 0..2, written with the tree
struct SurfDev {
  int p, q, nu, nv;
  int ns_u, ns_v;
  double range_u, range_v;   // k[last]-k[0] (derivative scale numerator, kernel.cu:167-168)
  float range_u32, range_v32;
  double dom_u0, dom_u1, dom_v0, dom_v1;  // knot domain [k[p], k[nu]] x [k[q], k[nv]]
  double org[3];          // origin of the FP32 tables: centre of the control net's bounding box
  float org32[3];
  const double* bu;
  const double* bv;
  const double* inv_du;
  const double* inv_dv;
  const float* bu32;
  const float* bv32;
  const float* inv_du32;
  const float* inv_dv32;
  const int* knot_u;
  const int* knot_v;
  const double* m64;
  const float* m32;
  const double* cps;      // 3*nu*nv  (xyz interleaved)
  const double* weights;  // nu*nv
  const double* knots_u;  // p+nu+1
  const double* knots_v;  // q+nv+1
  struct TreeNodeDev* tree;
  unsigned char* divided;
  unsigned char* built;
  double* basis_u;        // per-span basis-to-power matrices (conversion scratch kept with the surface)
  double* basis_v;
  float* cd32;            // seed-centre derivatives (see above)
  double* cd64;
  double* nbox;           // normal cones (see above)
  float* cone;
  float* lattice;
  double* qtbox;          // control-point boxes of the quadtree inversion's top levels (21 x 6)
};

// Tree node in the reference TreeNode order (src/kernel/kernel.cuh:30-39), 80 bytes.
struct TreeNodeDev {
  double uv_lb[2], uv_rt[2];
  double lb[3], rt[3];
};

// ---- error text of the C-ABI (api.cpp): sets the calling thread's nurbs_last_error() message
// and returns `code` (cuda_fail: NURBS_E_CUDA with the runtime's error string) ----
int fail(int code, const char* fmt, ...);
int cuda_fail(cudaError_t e, const char* what);

// ---- launchers (each returns a cudaError_t from the launch) ----
// stage a
cudaError_t launch_basis(const double* knots, int degree, const int* knot_idx, int nspans,
                         double* basis_out, cudaStream_t st);
cudaError_t launch_span_matrices(const SurfDev& s, const double* basis_u, const double* basis_v,
                                 double* m64, float* m32, cudaStream_t st);
cudaError_t launch_export_ref_layout(const SurfDev& s, double* matrix_n, cudaStream_t st);
// stage b
cudaError_t launch_eval_f64(const SurfDev& s, const double* uv, int64_t n, unsigned mask, double* out,
                            cudaStream_t st);
cudaError_t launch_eval_f32(const SurfDev& s, const float* uv, int64_t n, unsigned mask, float* out,
                            cudaStream_t st);
cudaError_t launch_eval_exact(const SurfDev& s, const double* uv, int64_t n, unsigned mask, double* out,
                              cudaStream_t st);
cudaError_t launch_eval_normal(const SurfDev& s, const double* uv, int64_t n, unsigned mask, double* out,
                               cudaStream_t st);
cudaError_t launch_evaluate_random(const double* uv, double* xyz, int64_t n, const double* matrix_n, int p,
                                   int q, int nu, int nv, const double* knots_u, const double* knots_v,
                                   cudaStream_t st);
// stage c
cudaError_t launch_tree(const SurfDev& s, cudaStream_t st);
cudaError_t launch_candidates(const SurfDev& s, const double* P, int64_t n, int* list, int* counts,
                              cudaStream_t st);
// batched (pool) variants: surfaces are read from a device table of SurfDev records
struct BasisJob {        // one (surface, direction): its spans' columns are items [item0, item0 + ns*(d+1))
  const double* knots;
  const int* knot_idx;
  double* out;
  int degree, nspans;
  int64_t item0;
};
struct SpanJob {         // one surface: its spans x 4 components are items [item0, item0 + 4*ns_u*ns_v)
  int surf;
  int64_t item0;
};
struct InvTile {         // a range of queries of one surface
  int surf;
  int count;
  int64_t begin;
};
cudaError_t launch_basis_batched(const BasisJob* jobs, int njobs, int64_t nitems, cudaStream_t st);
cudaError_t launch_span_matrices_batched(const SurfDev* table, const SpanJob* jobs, int njobs, int64_t nitems,
                                         cudaStream_t st);
cudaError_t launch_tree_batched(const SurfDev* table, const int* ids, int count, cudaStream_t st);
cudaError_t launch_eval_pool(const SurfDev* table, const InvTile* tiles, int ntiles, const double* uv, int64_t n,
                             unsigned mask, double* out, cudaStream_t st);
cudaError_t launch_invert_pool(const SurfDev* table, const InvTile* tiles, int ntiles, int* counter,
                               const double* P, double* uv, int* status, double* residual, int precision,
                               int ctas, int tile_queries, cudaStream_t st);

// stage d.  counter: one device word, zero when the launch starts (the kernel's chunk counter).
cudaError_t launch_invert(const SurfDev& s, const double* P, int64_t n, double* uv, int* status,
                          double* residual, int precision, unsigned* counter, cudaStream_t st);
// p-curves: continuation from the neighbours' pass-1 answers, then flags (k_pcurve.cu)
cudaError_t launch_pcurve_passes(const SurfDev& s, const double* C, int64_t n, const double* uv0, const int* st0,
                                 const double* res0, double* uv, int* st, double* res, int* flags,
                                 cudaStream_t stream);
// normal cones, bound boxes and lattice points of the built nodes (after the tree and the span tables)
cudaError_t launch_cones(const SurfDev& s, cudaStream_t st);
// the projection: closest point over the closed domain (k_project.cu)
cudaError_t launch_project(const SurfDev& s, const double* P, int64_t n, double* uv, int* status,
                           double* residual, int precision, unsigned* counter, cudaStream_t st);
// adaptive quadtree inversion (k_quadtree.cu); its top levels' control-point boxes (qtbox), written
// with the tree
cudaError_t launch_quadtree_boxes(const SurfDev& s, cudaStream_t st);
cudaError_t launch_invert_quadtree(const SurfDev& s, const double* P, int64_t n, double max_edge, double* uv,
                                   int* status, double* residual, int precision, unsigned* counter, cudaStream_t st);
// S, Su, Sv at the built nodes' uv-centres (cd32/cd64), after the tree is built
cudaError_t launch_centre_ders(const SurfDev& s, cudaStream_t st);
cudaError_t launch_centre_ders_batched(const SurfDev* table, const int* ids, int count, cudaStream_t st);
// the work-counting variant; counts[0] += seed iterations, counts[1] += final FP64 polishes
cudaError_t launch_invert_count(const SurfDev& s, const double* P, int64_t n, double* uv, int* status,
                                double* residual, int precision, unsigned* counter, unsigned long long* counts,
                                cudaStream_t st);

}  // namespace gnurbs
