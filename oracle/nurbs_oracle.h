/*
 * CPU ORACLE — test infrastructure only.
 *
 * A plain-C restatement of the reference's FP64 NURBS path (Qiang-Zou/GPU-NURBS):
 * span-matrix conversion, point/derivative evaluation, the 2-level subdivision tree,
 * candidate selection and Gauss-Newton inversion.  Each function cites the reference
 * file:line it follows.  It is the checker for the CUDA library and the CPU baseline of
 * the benchmark; it is never linked into, or called by, the product library.
 *
 * Parity of this restatement is pinned against the reference's own sources compiled for
 * the host (oracle/_ref, built by oracle/Makefile from the reference tree) and against the
 * reference's known-answer points; the fixtures produced that way live in tests/golden/.
 *
 * Build: gcc -O2 -ffp-contract=off (no FMA contraction, so rounding follows the source
 * expression order exactly as the reference's unfused code does).
 */
#ifndef NURBS_ORACLE_H
#define NURBS_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* A rational B-spline surface as the reference's .nu reader leaves it
 * (src/main.cu:45-113): control points row-major over (u-index i, v-index j),
 * index i*cp_v + j, xyz interleaved; weights not pre-multiplied. */
typedef struct {
    int degree_u, degree_v, cp_u, cp_v;
    const double* knots_u;   /* degree_u + cp_u + 1 */
    const double* knots_v;   /* degree_v + cp_v + 1 */
    const double* cps;       /* 3 * cp_u * cp_v */
    const double* weights;   /* cp_u * cp_v */
} orc_surface;

/* Tree node in the reference layout (src/kernel/kernel.cuh:30-39). */
typedef struct {
    double uv_lb[2], uv_rt[2];
    double lb[3], rt[3];
} orc_tree_node;

#define ORC_TREE_NODES 65     /* root + 8x8 children: the reference's 2-level build */
#define ORC_MAX_DEGREE 7      /* MAX_DEGREE 8 = k, so p <= 7 (src/NURBS/Evaluate.cuh:15) */

/* Size in doubles of the reference MatrixN buffer (src/main.cu:182). */
int64_t orc_matrix_n_size(const orc_surface* s);
/* Offset of component c of span (i,j) in MatrixN (src/NURBS/Evaluate.cu:110-112). */
int64_t orc_matrix_n_position(int i, int j, int degree_u, int degree_v, int cp_u, int cp_v, int c);
/* findSpan (src/NURBS/Evaluate.cu:504-533). */
int orc_find_span(int degree, int cp, const double* knots, double u);
/* GetMatrixN (src/NURBS/Evaluate.cu:3-88) with the Nrc recursion (:90-108) memoised.
 * Writes every non-empty span with i in [degree_u, cp_u-1], j in [degree_v, cp_v-1];
 * other slots are left untouched.  Returns the number of spans written. */
int orc_matrix_n(const orc_surface* s, double* matrix_n);

/* Evaluation mask bits (output blocks, each 3 doubles per point). */
#define ORC_S   1u
#define ORC_SU  2u
#define ORC_SV  4u
#define ORC_SUU 8u
#define ORC_SUV 16u
#define ORC_SVV 32u
/* Evaluates the blocks in mask at n (u,v) pairs (interleaved).  out is SoA:
 * for each set bit b in ascending order, 3 planes x[n], y[n], z[n].
 * Follows EvaluateRandom (src/NURBS/Evaluate.cu:1023-1038) for S and the old-style
 * MatrixSurfaceDerivative{U,V,UU,UV,VV} (src/NURBS/Evaluate.cu:535-930) for derivatives. */
void orc_eval(const orc_surface* s, const double* matrix_n, const double* uv, int64_t n,
              unsigned mask, double* out, int threads);

/* Homogeneous point R at local (u,v) in a span (MatrixSurfacePoint, Evaluate.cu:159-227). */
void orc_point_r(const double* middle, int degree_u, int degree_v, double u, double v, double R[4]);

/* The 2-level tree of the reference's inversion test (src/main.cu:280-309; kernels
 * GetPoints, GetSecondDerivatives, Max_Sequential_Addressing_Shared, TightBoundingBox in
 * src/kernel/kernel.cu).  divided[k] is meaningful for built nodes only; built[k] is 1
 * for the root and, if divided[0], for nodes 1..64. */
void orc_build_tree(const orc_surface* s, const double* matrix_n, orc_tree_node* tree,
                    unsigned char* divided, unsigned char* built);

/* Candidate list of query P: ascending built node indices whose closed AABB contains P
 * (NewInverse loop, src/kernel/kernel.cu:456-457; NewBoundingBoxCheck :466-469).
 * Returns the count; list must hold ORC_TREE_NODES ints. */
int orc_candidates(const orc_tree_node* tree, const unsigned char* built, const double P[3], int* list);

/* Inversion status codes (shared with the CUDA library). */
#define ORC_FOUND_UNIQUE    0
#define ORC_FOUND_AMBIGUOUS 1
#define ORC_NO_CANDIDATE    2
#define ORC_NOT_CONVERGED   3

/* Converged inversion (the oracle's definition, nurbs_oracle.c): from the uv-centre of every
 * candidate node, the reference GN update (kernel.cu:151-249) while the last step was >= 1e-2
 * in max-norm, then Newton steps (the GN update where the Hessian is not positive definite)
 * until a Newton step is <= 1e-10 or any step <= 1e-14, at most max_iter iterations; results
 * inside the knot domain are kept and the one of least distance is returned.  uv[2n],
 * status[n], residual[n], iters[n] (total iterations; may be NULL). */
void orc_invert(const orc_surface* s, const double* matrix_n, const orc_tree_node* tree,
                const unsigned char* built, const double* P, int64_t n, int max_iter,
                double* uv, int* status, double* residual, int* iters, int threads);

/* Stability of the answer at FP32 resolution: for k in [0,K) every coordinate of P, taken
 * relative to the centre of the control net's bounding box, is scaled by (1 +- eps) (even k) or
 * (1 +- 4 eps) (odd k) with signs from a fixed hash; the perturbed point is inverted as
 * orc_invert does, and its answer is carried back to the true point by Newton steps.  Outputs
 * are K*n long (perturbation-major): uv[2Kn], found[Kn] (1 when the perturbed point had an
 * answer whose Newton polish converged in the domain), residual[Kn] at the true point. */
void orc_invert_perturbed(const orc_surface* s, const double* matrix_n, const orc_tree_node* tree,
                          const unsigned char* built, const double* P, int64_t n, int max_iter, int K,
                          double eps, double* uv, int* found, double* residual, int threads);

/* The same inversion with its exploration in FP32 arithmetic (nurbs_oracle.c): every
 * trajectory computed in float relative to the control net's centre and stopped at FP32
 * resolution, the distinct FP32 minima within 5 % of the closest carried to the true point's
 * minimum by FP64 Newton steps.  pk >= 0: the FP32 phase explores perturbation pk (as
 * orc_invert_perturbed makes it) of each point; pk < 0: the point itself.  uv[2n], found[n],
 * residual[n]; a query whose FP64 answer differs from this one has an answer that FP32
 * arithmetic cannot determine. */
void orc_invert_fp32_explore(const orc_surface* s, const double* matrix_n, const orc_tree_node* tree,
                             const unsigned char* built, const double* P, int64_t n, int max_iter, int pk,
                             double eps, double* uv, int* found, double* residual, int threads);

/* p-curve of ordered curve samples C[3n] (the oracle of nurbs_pcurve): orc_invert of every
 * sample, FP64 Newton steps from the neighbours' answers kept when strictly closer (or when the
 * sample had none), flags (1 jump, 2 ambiguous, 4 not found).  uv[2n], status[n], residual[n],
 * flags[n]. */
void orc_pcurve(const orc_surface* s, const double* matrix_n, const orc_tree_node* tree,
                const unsigned char* built, const double* C, int64_t n, int max_iter, double* uv,
                int* status, double* residual, int* flags, int threads);

/* S and derivatives to third order (out[30]: S, Su, Sv, Suu, Suv, Svv, Suuu, Suuv, Suvv, Svvv)
 * and the normal N = Su x Sv with its first and second derivatives (out[18]) at one global
 * parameter pair, from the homogeneous R-derivatives with the quotient rule's signs
 * (nurbs_oracle.c); orc_eval_normal is the batched SoA form of nurbs_eval_normal. */
void orc_ders3(const orc_surface* s, const double* matrix_n, double u, double v, double out[30]);
void orc_normals(const orc_surface* s, const double* matrix_n, double u, double v, double out[18]);
void orc_eval_normal(const orc_surface* s, const double* matrix_n, const double* uv, int64_t n, unsigned mask,
                     double* out, int threads);

/* Normal cones of the built nodes (the oracle of the CUDA cone build; nurbs_oracle.c states the
 * definition): nbox[6 * 65] = the normal boxes (lb xyz, rt xyz); cone[ORC_CONE_STRIDE * 65] =
 * per node in FP32, relative to the control net's centre: the bound box's bounding-ball centre
 * (0..2) and radius (3), cone axis (4..6), cos and sin of the half-angle (7, 8; 0 and 1 for
 * every direction), the bound box rounded outward (lb 9..11, rt 12..14), zero (15..19);
 * upts[3 * ORC_UPTS * 65] = the surface points of each node's 9x9 lattice (index 9 tx + ty), the
 * same way. */
#define ORC_CONE_STRIDE 20
#define ORC_UPTS 81
void orc_build_cones(const orc_surface* s, const double* matrix_n, const orc_tree_node* tree,
                     const unsigned char* built, double* nbox, float* cone, float* upts);
/* Projection candidates of one point P (128 * node + its seed's lattice index, ascending
 * nodes); org = the control net's centre.  Returns the candidate count. */
int orc_project_cull(const orc_tree_node* tree, const unsigned char* built, const float* cone, const float* upts,
                     const double* P, const double org[3], int* list);
/* cone arguments below: the cone records followed by upts (ORC_CONE_STRIDE * 65 + 3 * ORC_UPTS * 65
 * floats). */
/* Closest point of the surface over its closed domain (the oracle of nurbs_project), and the
 * stability set of its answers (the counterpart of orc_invert_perturbed). */
void orc_project(const orc_surface* s, const double* matrix_n, const orc_tree_node* tree,
                 const unsigned char* built, const float* cone, const double* P, int64_t n, int max_iter,
                 double* uv, int* status, double* residual, int* iters, int threads);
void orc_project_perturbed(const orc_surface* s, const double* matrix_n, const orc_tree_node* tree,
                           const unsigned char* built, const float* cone, const double* P, int64_t n, int max_iter,
                           int K, double eps, double* uv, int* found, double* residual, int threads);

/* Adaptive quadtree inversion (the reference's v1 Inverse with its control-net culling; the
 * oracle of nurbs_invert_quadtree, definition in nurbs_oracle.c): per query a breadth-first
 * quadtree over the domain, a trajectory from every node whose widened control-net box holds P,
 * the first layer with a result within max_edge answers.  uv[2n], status[n], residual[n],
 * layers[n] (layers visited; may be NULL). */
void orc_invert_quadtree(const orc_surface* s, const double* matrix_n, const double* P, int64_t n, double max_edge,
                         int max_iter, double* uv, int* status, double* residual, int* layers, int threads);

/* One node (lb.u, lb.v, rt.u, rt.v) of the quadtree inversion: its control-point box check and
 * its split type (as_reference = 1: the reference's v-length from MatrixSurfaceDerivativeU, for
 * pinning the definition against the reference's own getSplitType). */
int orc_qt_hull_check(const orc_surface* s, const double node4[4], const double P[3], double max_edge);
int orc_qt_split_type(const orc_surface* s, const double* matrix_n, const double node4[4], double max_edge,
                      int as_reference);

/* The reference's GaussNewton exactly as shipped (kernel.cu:151-249): <= 10 steps,
 * success when |S-P| < max_edge before a step.  Returns 1 on success and writes uv. */
int orc_gauss_newton_shipped(const orc_surface* s, const double* matrix_n, const double seed[2],
                             const double P[3], double max_edge, double uv[2]);

/* x*x*x rounded once (pow(x,3) of a correctly rounded libm), from an error-free
 * product expansion.  Exposed for the tests that compare it with libm pow. */
double orc_cube(double x);

#ifdef __cplusplus
}
#endif
#endif
