/*
 * gpu_nurbs.h — C-ABI of the GB300 NURBS evaluation / inverse-evaluation engine.
 *
 * Drop-in boundary for the reference Qiang-Zou/GPU-NURBS, whose "API" is its .nu reader,
 * its kernels and its __device__ functions (src/main.cu, src/NURBS/Evaluate.cu,
 * src/kernel/kernel.cu).  Each entry point below names the reference interface it replaces.
 *
 * Conventions
 *   - Every call returns an int status: NURBS_OK (0) or a negative NURBS_E_* code; nothing
 *     calls exit().  nurbs_last_error() gives a message for the calling thread.
 *   - Pointers named *_dev are device pointers owned by the caller; *_host are host pointers.
 *     Entry points that take a `stream` enqueue work on it and return without waiting, unless
 *     their comment says otherwise.  `stream` is a cudaStream_t passed as void* (NULL = the
 *     legacy default stream).
 *   - Layouts: (u,v) pairs and points are interleaved arrays of doubles (double2 / double3 in
 *     the reference).  Control points are row-major over (u-index i, v-index j): i*cp_v + j.
 *   - A surface handle may be used from several host threads; calls on one handle are
 *     serialised by the caller's stream order.
 */
#ifndef GPU_NURBS_H
#define GPU_NURBS_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ status codes */
#define NURBS_OK              0
#define NURBS_E_INVALID      -1   /* bad argument (degree, size, null pointer, knot order) */
#define NURBS_E_CUDA         -2   /* a CUDA runtime call failed */
#define NURBS_E_NOMEM        -3   /* device or host allocation failed */
#define NURBS_E_IO           -4   /* file could not be opened / written */
#define NURBS_E_PARSE        -5   /* malformed .nu text */
#define NURBS_E_UNSUPPORTED  -6   /* valid input outside what this build handles */
#define NURBS_E_BUDGET       -7   /* admission refused by a device-memory budget */
#define NURBS_E_TIMEOUT      -8   /* a bounded wait ran out */
#define NURBS_E_STATE        -9   /* call not valid in the object's current state */

#define NURBS_MAX_DEGREE 7        /* MAX_DEGREE 8 = p+1, src/NURBS/Evaluate.cuh:15 */
#define NURBS_TREE_NODES 65       /* root + 8x8 children (src/main.cu:283, kernel.cuh:23-25) */

/* evaluation output blocks (bit set => 3 planes x[n],y[n],z[n] in the output, in this order) */
#define NURBS_S    1u
#define NURBS_SU   2u
#define NURBS_SV   4u
#define NURBS_SUU  8u
#define NURBS_SUV 16u
#define NURBS_SVV 32u
/* third order (MatrixSurfaceRd{UUU,UUV,UVV,VVV} + MatrixSurfaceDerivative{UUU,UUV,UVV,VVV},
 * src/NURBS/Evaluate.cu:408-502, 963-1020; the reference's UUV/UVV quotient forms carry two wrong
 * signs, these follow the quotient rule) */
#define NURBS_SUUU  64u
#define NURBS_SUUV 128u
#define NURBS_SUVV 256u
#define NURBS_SVVV 512u
/* surface normal N = Su x Sv (not normalised, TrueNormal, src/NURBS/Evaluate.cu:1111-1117) and its
 * derivatives, for nurbs_eval_normal */
#define NURBS_N    1u
#define NURBS_NU   2u
#define NURBS_NV   4u
#define NURBS_NUU  8u
#define NURBS_NUV 16u
#define NURBS_NVV 32u

/* precision schedules */
#define NURBS_PREC_FP64   0   /* every iteration and contraction in FP64 */
#define NURBS_PREC_MIXED  1   /* FP32 seeding/early iterations, FP64 final 2 steps + residual */
#define NURBS_PREC_FP32   2   /* evaluation only: FP32 contraction of the FP32 span matrices */
#define NURBS_PREC_EXACT  3   /* nurbs_eval only: the reference's FP64 expressions term by term
                                 (bit-identical to its functions at every degree; mask <= 63) */

/* inversion status per query */
#define NURBS_INV_FOUND        0   /* converged, in-domain, best candidate unique */
#define NURBS_INV_AMBIGUOUS    1   /* converged; another distinct minimum is as close */
#define NURBS_INV_NO_CANDIDATE 2   /* P lies in no tree box (NewInverse leaves flag unset) */
#define NURBS_INV_NOT_CONVERGED 3  /* no candidate converged inside the knot domain */

const char* nurbs_status_string(int status);
const char* nurbs_last_error(void);
const char* nurbs_version(void);

/* ------------------------------------------------------------------- .nu files */
/* Replaces readNu (src/main.cu:45-113): same tags NU, CP, KNu, KNv, DP.  Allocates host
 * arrays owned by the descriptor; release with nurbs_nu_free.  Unlike the reference, a
 * missing tag or short line returns NURBS_E_PARSE instead of looping forever. */
typedef struct {
    int degree_u, degree_v, cp_u, cp_v;
    double* knots_u;   /* degree_u + cp_u + 1 */
    double* knots_v;   /* degree_v + cp_v + 1 */
    double* cps;       /* 3 * cp_u * cp_v, xyz interleaved, row-major i*cp_v + j */
    double* weights;   /* cp_u * cp_v */
} nurbs_nu_desc;

int nurbs_nu_read(const char* path, nurbs_nu_desc* out);
int nurbs_nu_parse(const char* text, int64_t len, nurbs_nu_desc* out);
int nurbs_nu_write(const char* path, const nurbs_nu_desc* desc);
void nurbs_nu_free(nurbs_nu_desc* desc);

/* --------------------------------------------------------------- surface handle */
typedef struct nurbs_surface_s* nurbs_surface_t;

#define NURBS_PTR_HOST   0   /* knots/cps/weights are host pointers */
#define NURBS_PTR_DEVICE 1   /* knots/cps/weights are device pointers */

/* Uploads a surface and converts it to matrix form (stage a; replaces the GetMatrixN launch
 * of src/main.cu:252): dense FP64 and FP32 span matrices over the non-empty spans.  Also
 * builds the 2-level subdivision tree (stage c).  Synchronous: returns when done. */
int nurbs_surface_create(int degree_u, int degree_v, int cp_u, int cp_v,
                         const double* knots_u, const double* knots_v,
                         const double* cps, const double* weights,
                         int ptr_kind, void* stream, nurbs_surface_t* out);
int nurbs_surface_destroy(nurbs_surface_t s);

typedef struct {
    int degree_u, degree_v, cp_u, cp_v;
    int spans_u, spans_v;          /* non-empty spans per direction */
    int64_t device_bytes;          /* device memory held by the handle */
    int tree_built;                /* 1 once the tree exists */
} nurbs_surface_info_t;
int nurbs_surface_info(nurbs_surface_t s, nurbs_surface_info_t* info);

/* ------------------------------------------------------------ stage a: matrix form */
/* Size in doubles of the reference's MatrixN buffer (src/main.cu:182). */
int64_t nurbs_matrix_n_size(int degree_u, int degree_v, int cp_u, int cp_v);
/* Offset of component c of knot span (i,j) in MatrixN: MatrixNPosition
 * (src/NURBS/Evaluate.cu:110-112). */
int64_t nurbs_matrix_n_position(int i, int j, int degree_u, int degree_v, int cp_u, int cp_v, int c);
/* Writes the handle's span matrices into a caller buffer in the reference's MatrixN layout
 * (slots of empty spans are left untouched, as GetMatrixN leaves them). */
int nurbs_get_matrix_n(nurbs_surface_t s, double* matrix_n_dev, void* stream);
/* Legacy GetMatrixN (src/NURBS/Evaluate.cu:3-88) with the reference's argument list; all
 * pointers are device pointers and control_points is double3[cp_u*cp_v].  No device heap and
 * no dynamic parallelism; values are bit-identical to the reference's FP64 arithmetic. */
int nurbs_get_matrix_n_raw(double* matrix_n_dev, int degree_u, int degree_v, int cp_u, int cp_v,
                           const double* knots_u_dev, const double* knots_v_dev,
                           const double* control_points_dev, const double* weights_dev, void* stream);

/* GetMatrixN into a caller buffer that allocates nothing.  No counterpart in the reference:
 * it is for callers that cannot allocate device memory when they convert a surface — code
 * running under a device allocator it does not own (an application's caching allocator, a
 * budget admitter that forbids allocations outside its pool) or a real-time / serving loop
 * that must not enter the allocator between requests.  Same arguments and bit-identical
 * output as nurbs_get_matrix_n_raw; its scratch (span tables and basis matrices) is a
 * file-scope device array of NURBS_NOALLOC_SCRATCH_BYTES held by every GPU that loads the
 * library until the process exits.  Surfaces whose worst-case scratch
 * (cp_u-degree_u + cp_v-degree_v) * 4 + (cp_u-degree_u)*(degree_u+1)^2*8 +
 * (cp_v-degree_v)*(degree_v+1)^2*8 bytes (plus alignment) exceeds it return
 * NURBS_E_UNSUPPORTED.  The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress, with that device current); make that first call before any stream
 * capture.  The looked-up address is cached per device: do not call this entry point again
 * after cudaDeviceReset in the same process (the reset frees the array the cache names).  All
 * calls share the array, so calls that overlap on the GPU race: serialise them.  Synchronises
 * `stream` once (to read the span counts back).  Errors set nurbs_last_error(). */
#define NURBS_NOALLOC_SCRATCH_BYTES (1u << 20)
int nurbs_get_matrix_n_noalloc(double* matrix_n_dev, int degree_u, int degree_v, int cp_u, int cp_v,
                               const double* knots_u_dev, const double* knots_v_dev,
                               const double* control_points_dev, const double* weights_dev, void* stream);

/* -------------------------------------------------------------- stage b: evaluation */
/* Batched evaluation at n parameter pairs uv_dev[2n] (global parameters).  out_dev is SoA:
 * for each set bit of mask, in the order S,Su,Sv,Suu,Suv,Svv,Suuu,Suuv,Suvv,Svvv, three planes
 * of n doubles.
 * Replaces MatrixSurfacePoint + MatrixSurfaceDerivative{U,V,UU,UV,VV}
 * (src/NURBS/Evaluate.cu:159-227, 535-930) driven per point as EvaluateRandom does
 * (:1023-1038).  precision NURBS_PREC_FP64 only (see nurbs_eval_f32). */
int nurbs_eval(nurbs_surface_t s, const double* uv_dev, int64_t n, unsigned mask,
               double* out_dev, int precision, void* stream);
/* Normal N = Su x Sv and its derivatives at n parameter pairs (FP64): for each set bit of mask
 * (NURBS_N, NU, NV, NUU, NUV, NVV, in that order) three planes of n doubles.  The second
 * derivatives are SurfaceNormalDerivative{UU,UV,VV} (src/NURBS/Evaluate.cu:1125-1135). */
int nurbs_eval_normal(nurbs_surface_t s, const double* uv_dev, int64_t n, unsigned mask, double* out_dev,
                      void* stream);
/* FP32 variant: float (u,v) in, float SoA out, contraction of the FP32 span matrices. */
int nurbs_eval_f32(nurbs_surface_t s, const float* uv_dev, int64_t n, unsigned mask,
                   float* out_dev, void* stream);
/* Legacy EvaluateRandom (src/NURBS/Evaluate.cu:1023-1038): S at n points straight from a
 * reference-layout MatrixN; xyz_dev is double3[n].  Guards index < n (the reference does not). */
int nurbs_evaluate_random(const double* uv_dev, double* xyz_dev, int64_t n, const double* matrix_n_dev,
                          int degree_u, int degree_v, int cp_u, int cp_v,
                          const double* knots_u_dev, const double* knots_v_dev, void* stream);

/* ------------------------------------------------ stage c: subdivision tree / culling */
/* (Re)builds the tree: GetPoints + GetSecondDerivatives + Max_Sequential_Addressing_Shared
 * + TightBoundingBox for levels 0..levels-1 (src/main.cu:280-309).  Only levels == 2 (the
 * reference's setting) is supported. */
int nurbs_build_tree(nurbs_surface_t s, int levels, void* stream);
/* Copies the tree to host memory in the reference TreeNode order (kernel.cuh:30-39):
 * per node 10 doubles {uv.lb.x, uv.lb.y, uv.rt.x, uv.rt.y, lb.x, lb.y, lb.z, rt.x, rt.y, rt.z},
 * plus Divided[] and built[] (1 where the node was computed).  Synchronous, on the legacy default
 * stream: a tree built on a non-blocking stream must be complete first (that stream synchronised). */
int nurbs_tree_export(nurbs_surface_t s, double* nodes_host, unsigned char* divided_host,
                      unsigned char* built_host);
/* Candidate lists (the NewInverse scan, src/kernel/kernel.cu:456-457, over built nodes):
 * for query k, counts_dev[k] ascending node indices in list_dev[k*65 ...]. */
int nurbs_candidates(nurbs_surface_t s, const double* P_dev, int64_t n, int* list_dev, int* counts_dev,
                     void* stream);

/* ----------------------------------------------------------- stage d: inversion */
/* Point inversion of n points P_dev[3n]: candidates from the tree, Gauss-Newton from each
 * candidate's uv-centre (GaussNewton, src/kernel/kernel.cu:151-249), converged and kept when
 * inside the knot domain; the closest wins.  Outputs uv_dev[2n], status_dev[n] (NURBS_INV_*),
 * residual_dev[n] = |S(uv) - P| in FP64.  precision: NURBS_PREC_FP64 or NURBS_PREC_MIXED. */
int nurbs_invert(nurbs_surface_t s, const double* P_dev, int64_t n, double* uv_dev, int* status_dev,
                 double* residual_dev, int precision, void* stream);
/* Point projection: the closest point of the surface over its closed knot domain for each of n
 * points P_dev[3n], near the surface or far from it.  Replaces the reference's unfinished
 * Project / NormalBoundingBox / NormalBoxToNormalTreeNode / NormalBoundingBoxCheck
 * (src/kernel/kernel.cu:471-513, 623-704, 1613-1641; src/main.cu:329-396).  Candidates are the
 * built nodes whose bound box (the node's box intersected with its control points' box) is within
 * a distance bound from lattice points and whose normal cone can face P (both signs); each is
 * seeded at its 9x9 lattice point closest to P and runs projected Newton steps with a line search
 * inside the domain, so minima on the domain's boundary are found too.  precision:
 * NURBS_PREC_FP64, or NURBS_PREC_MIXED (the trajectories in FP32, then FP64 projected Newton
 * steps from the best result, and from the best of another grid cell within 5 %).  Outputs as
 * nurbs_invert (NURBS_INV_NO_CANDIDATE only for non-finite P).  The cones are built with the tree
 * (nurbs_surface_create, nurbs_build_tree); single surfaces only (not the pool). */
int nurbs_project(nurbs_surface_t s, const double* P_dev, int64_t n, double* uv_dev, int* status_dev,
                  double* residual_dev, int precision, void* stream);
/* Adaptive quadtree inversion, the reference's first inversion (Inverse, BoundingBoxCheck,
 * getSplitType; src/kernel/kernel.cu:4-149, 251-298), which needs no tree: per query a
 * breadth-first quadtree over the domain; a node passes when P lies in the box of the control
 * points of its span range widened by max_edge, and seeds an FP64 trajectory at its centre
 * (nurbs_invert's iteration) that counts when it converges inside the domain within max_edge of
 * P; the first layer with such a result answers with its closest one.  Nodes that pass are split
 * by getSplitType (the v-length from the v-derivative); a layer of more than 64 nodes
 * (NODE_MAX_SIZE) ends the query unanswered.  For points on the surface or within max_edge of
 * it.  precision: NURBS_PREC_FP64, or NURBS_PREC_MIXED (the root's trajectory, which answers most
 * queries, in FP32 with FP64 final Newton steps and residual; the deeper layers in FP64).
 * Outputs as nurbs_invert; n < 2^32 * 32. */
int nurbs_invert_quadtree(nurbs_surface_t s, const double* P_dev, int64_t n, double max_edge, double* uv_dev,
                          int* status_dev, double* residual_dev, int precision, void* stream);
/* Copies the projection's culling data to host memory: nbox[65*6] normal boxes (lb xyz, rt xyz),
 * cone[65*20] FP32 records relative to the control net's centre (bound-box ball centre and radius,
 * cone axis, cos and sin of its half-angle (0 and 1: every direction), bound box rounded outward,
 * zero padding), lattice[65*81*3] the nodes' 9x9 lattice surface points (FP32, relative to the
 * same centre).  Synchronous, on the legacy default stream: cones built on a non-blocking stream
 * (nurbs_surface_create, nurbs_build_tree) must be complete first. */
int nurbs_normal_cones_export(nurbs_surface_t s, double* nbox_host, float* cone_host, float* lattice_host);

/* p-curve of a 3-D curve on the surface: the parameters of its n ordered samples C_dev[3n].
 * No counterpart in the reference's code (its README names p-curve calculation as the use of
 * the inversion).  Each sample is inverted as nurbs_invert does (precision FP64 or MIXED); each
 * then takes FP64 Newton steps from its two neighbours' answers and keeps such a minimum when it
 * is strictly closer (or when it had none); flags_dev[n] marks NURBS_PCURVE_JUMP (the parameter
 * step from the previous sample exceeds 4 |chord| / sigma_min(J): a seam, a fold, another
 * sheet), NURBS_PCURVE_AMBIGUOUS and NURBS_PCURVE_NOT_FOUND.  uv_dev[2n], status_dev[n],
 * residual_dev[n] as nurbs_invert.  Allocates and frees 48 n bytes of device scratch on
 * `stream`, from the library's stream-ordered pool (it keeps up to 512 MB of freed temporaries
 * per device between calls). */
#define NURBS_PCURVE_JUMP      1
#define NURBS_PCURVE_AMBIGUOUS 2
#define NURBS_PCURVE_NOT_FOUND 4
int nurbs_pcurve(nurbs_surface_t s, const double* C_dev, int64_t n, double* uv_dev, int* status_dev,
                 double* residual_dev, int* flags_dev, int precision, void* stream);

/* Diagnostic: the work one nurbs_invert of the same queries does, from a counting variant of
 * the kernel (same results, not timed): counts_host[0] = seed iterations (FP32 iterations for
 * NURBS_PREC_MIXED, FP64 for NURBS_PREC_FP64), counts_host[1] = final FP64 polishes (mixed).
 * No counterpart in the reference.  Waits for `stream`. */
int nurbs_invert_count(nurbs_surface_t s, const double* P_dev, int64_t n, int precision,
                       unsigned long long* counts_host, void* stream);
/* Same with host buffers: copies P in, runs, copies results out, waits.  Pinned host memory
 * gives the fastest copies; the 52 n bytes of device buffers come from the library's pool (as
 * nurbs_pcurve's scratch). */
int nurbs_invert_host(nurbs_surface_t s, const double* P_host, int64_t n, double* uv_host, int* status_host,
                      double* residual_host, int precision, void* stream);

/* ------------------------------------------------------------- surface pools */
/* Many surfaces resident in one device arena under a memory budget, inverted together in one
 * persistent launch.  No counterpart in the reference (one surface per process); the per
 * surface work is the same stages a-d as above. */
typedef struct nurbs_pool_s* nurbs_pool_t;
typedef struct nurbs_graph_s* nurbs_graph_t;

typedef struct {                   /* host arrays of one surface (layouts as in nurbs_surface_create) */
    int degree_u, degree_v, cp_u, cp_v;
    const double* knots_u;
    const double* knots_v;
    const double* cps;
    const double* weights;
} nurbs_surface_desc;

typedef struct {
    int64_t budget_bytes, used_bytes;
    int surfaces, max_surfaces;
    int tile_queries, ctas_per_sm;  /* current launch configuration */
} nurbs_pool_info_t;

/* Allocates the whole budget at once; surfaces and workspaces are carved from it. */
int nurbs_pool_create(int64_t budget_bytes, int max_surfaces, nurbs_pool_t* out);
int nurbs_pool_destroy(nurbs_pool_t pool);
/* Uploads and converts `count` surfaces in one batch (one copy, one launch per stage); returns
 * their ids.  NURBS_E_BUDGET when the budget (or max_surfaces) cannot hold them.  Synchronous. */
int nurbs_pool_add(nurbs_pool_t pool, int count, const nurbs_surface_desc* descs, void* stream, int* ids_out);
/* Frees a surface's memory.  Waits for `stream`; work queued on other streams must be done. */
int nurbs_pool_remove(nurbs_pool_t pool, int id, void* stream);
int nurbs_pool_info(nurbs_pool_t pool, nurbs_pool_info_t* info);
/* Device bytes one surface would take (for admission decisions before uploading it). */
int nurbs_pool_surface_bytes(int degree_u, int degree_v, int cp_u, int cp_v, const double* knots_u,
                             const double* knots_v, int64_t* bytes);
const char* nurbs_pool_last_error(void);
/* Launch configuration and persistent CTAs per SM.  tile_queries > 32 (a multiple of 32): each
 * CTA takes tiles of that many queries of one surface (throughput on large batches);
 * tile_queries <= 32: each warp takes chunks of that many queries on its own (small batches
 * spread over all SMs; fewer queries per warp lowers latency). */
int nurbs_pool_set_config(nurbs_pool_t pool, int tile_queries, int ctas_per_sm);
/* Batched inversion.  Queries are grouped by surface: surface ids_host[k] owns the queries
 * [offsets_host[k], offsets_host[k+1]) of P_dev (3 doubles each); outputs are indexed like P.
 * Asynchronous on `stream`. */
int nurbs_pool_invert(nurbs_pool_t pool, int nbatch, const int* ids_host, const int64_t* offsets_host,
                      const double* P_dev, double* uv_dev, int* status_dev, double* residual_dev, int precision,
                      void* stream);
/* Batched FP64 evaluation: surface ids_host[k] evaluates the (u,v) pairs [offsets[k], offsets[k+1])
 * of uv_dev; out_dev is SoA over all n pairs as in nurbs_eval.  Asynchronous on `stream`. */
int nurbs_pool_eval(nurbs_pool_t pool, int nbatch, const int* ids_host, const int64_t* offsets_host,
                    const double* uv_dev, int64_t n, unsigned mask, double* out_dev, void* stream);
/* Times tile size x CTAs per SM on the batch (or its prefix of at most max_queries queries, 0 =
 * all), keeps the fastest configuration in the pool and returns it.  With cache_path, a result
 * cached for the same GPU, precision and batch signature is reused, and new results appended. */
int nurbs_pool_autotune(nurbs_pool_t pool, int nbatch, const int* ids_host, const int64_t* offsets_host,
                        const double* P_dev, double* uv_dev, int* status_dev, double* residual_dev, int precision,
                        int64_t max_queries, const char* cache_path, void* stream, int* best_tile, int* best_ctas,
                        float* best_ms);
/* Captures the batched inversion of one batch layout as a CUDA graph (tile list uploaded once);
 * replay it with nurbs_graph_launch for new query values in the same buffers. */
int nurbs_pool_graph_create(nurbs_pool_t pool, int nbatch, const int* ids_host, const int64_t* offsets_host,
                            const double* P_dev, double* uv_dev, int* status_dev, double* residual_dev,
                            int precision, nurbs_graph_t* out);
int nurbs_graph_launch(nurbs_graph_t graph, void* stream);
/* Destroying the pool first releases the graph's device resources (launch then returns
 * NURBS_E_STATE); nurbs_graph_destroy must still be called once to free the handle. */
int nurbs_graph_destroy(nurbs_graph_t graph);

/* ------------------------------------------------------------------ serving */
/* A continuous-batching request loop over a pool.  No counterpart in the reference.
 * Requests are submitted from any host thread; a scheduler thread keeps up to `slots` batches
 * in flight (one CUDA stream each), forms every new batch from the requests that arrived while
 * the GPU was busy, and copies each request's results back to its host buffers.  Uploads are
 * converted on their own stream; when the budget is full, the least recently used surfaces
 * that no queued request references are evicted.  Host buffers passed to a submit call must
 * stay valid until the request completes. */
typedef struct nurbs_server_s* nurbs_server_t;
typedef struct {
    int slots;                   /* batches in flight (1..16) */
    int64_t max_batch_queries;   /* queries per batch; also the largest request accepted */
    int max_batch_requests;      /* requests per batch */
    int precision;               /* NURBS_PREC_MIXED or NURBS_PREC_FP64 */
} nurbs_server_config;
typedef struct {
    int64_t completed, batches, batch_queries;
    int in_flight;
    double gpu_ms;        /* sum over batches of stream time from H2D start to D2H end */
    double dispatch_us;   /* scheduler host time forming and enqueuing batches */
    double retire_us;     /* scheduler host time copying results back */
} nurbs_server_stats_t;

int nurbs_server_create(nurbs_pool_t pool, const nurbs_server_config* cfg, nurbs_server_t* out);
/* Stops the threads; batches in flight finish, requests not started complete with NURBS_E_STATE. */
int nurbs_server_destroy(nurbs_server_t server);
int nurbs_server_submit_invert(nurbs_server_t server, int surf_id, const double* P_host, int64_t n,
                               double* uv_host, int* status_host, double* residual_host,
                               double* latency_us_out, uint64_t* ticket);
int nurbs_server_submit_upload(nurbs_server_t server, const nurbs_surface_desc* desc, int* surf_id_out,
                               double* latency_us_out, uint64_t* ticket);
/* Bounded wait for one request (NURBS_E_TIMEOUT after timeout_ms); releases the ticket. */
int nurbs_server_wait(nurbs_server_t server, uint64_t ticket, int timeout_ms, int* result);
/* Completed requests since the last poll (tickets released). */
int nurbs_server_poll(nurbs_server_t server, uint64_t* tickets, int* results, int max, int* count);
/* Bounded wait until no request is queued or in flight. */
int nurbs_server_drain(nurbs_server_t server, int timeout_ms);
/* Holds (1) or resumes (0) the dispatch of new batches; batches in flight finish. */
int nurbs_server_pause(nurbs_server_t server, int paused);
int nurbs_server_stats(nurbs_server_t server, nurbs_server_stats_t* stats);
/* Native load generator: submits request i at arrival_us[i] after the start, then drains.
 * kind[i] 0 = inversion of queries [qoff[i], qoff[i+1]) of P against surf[i] (outputs at the
 * same offsets); 1 = upload of uploads[upload_index[i]] (its id written to upload_ids[...]).
 * latency_us[i] counts from the scheduled arrival; results[i] is the request's status. */
int nurbs_server_replay(nurbs_server_t server, int nreq, const double* arrival_us, const int* kind,
                        const int* surf, const int64_t* qoff, const double* P, double* uv, int* status,
                        double* residual, const nurbs_surface_desc* uploads, const int* upload_index,
                        int* upload_ids, double* latency_us, int* results, int timeout_ms);

/* ------------------------------------------------------------------ diagnostics */
/* Measured FMA throughput of the current GPU in TFLOP/s (bits = 64 or 32): independent FMA
 * chains over 8 CTAs per SM, timed with CUDA events.  No reference counterpart; used as the
 * roofline denominator for the FP64/FP32 pipes.  Synchronous. */
int nurbs_probe_fp_peak(int bits, double* tflops, void* stream);

#ifdef __cplusplus
}
#endif
#endif
