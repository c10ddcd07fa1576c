/* tbem_gpu.h -- C ABI of the GB300 BEM operator apply (KIFMM + direct + CSR).
 *
 * Drop-in for the reference's operator interface on the hot path
 * (tbenthompson/3bem):
 *   struct OperatorI { n_rows(); n_cols(); apply(x); clone(); }   cpp/operator.h:14-19
 *   FMMOperator<dim,R,C>(Kernel, NBodyData, FMMConfig)            cpp/fmm.h:131-147
 *     (dim 3: <3,1,1>, <3,3,3>; dim 2: <2,1,1>, <2,2,2>, cpp/fmm.cpp:651-654)
 *   FMMConfig(mac, order, min_pts_per_cell, d, account_for_small_cells)  cpp/fmm.h:73-96
 *   SparseOperator::apply (CSR SpMV)                              cpp/sparse_operator.cpp:19-28
 *   make_direct_nbody_operator / nbody_eval (direct sum)          cpp/nbody_operator.h:117-152
 *
 * Conventions (those of the reference):
 *   - points and normals are row-major float64 [n][dim] (dim = 3, or 2 for
 *     the 2D kernel ids); weights float64 [n];
 *   - densities are component-major per right-hand side: x[r][d][j] =
 *     x[(r*C + d)*n_src + j] (cpp/fmm.cpp:189-190); outputs likewise
 *     y[(r*R + d)*n_obs + i];
 *   - n_rows = R*n_obs, n_cols = C*n_src (cpp/fmm.h:235-236).
 * Pointers passed to the apply calls may be host or device memory (detected);
 * host buffers are copied in and out inside the call.  Every function returns
 * TBEM_OK or a negative status; tbem_last_error() gives the message.  Nothing
 * aborts.  Empty point sets are valid (the reference requires empty meshes
 * not to error, acceptance_tests/test_empty_operator.py:10-17).
 */
#ifndef TBEM_GPU_H
#define TBEM_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define TBEM_OK 0
#define TBEM_ERR_ARG (-1)      /* invalid argument / config            */
#define TBEM_ERR_CUDA (-2)     /* CUDA runtime or library failure      */
#define TBEM_ERR_ALLOC (-3)    /* device or host allocation failed     */
#define TBEM_ERR_STATE (-4)    /* call not valid for this handle state */
#define TBEM_ERR_TIMEOUT (-5)  /* a bounded device wait gave up        */

/* kernel ids: cpp/laplace_kernels.h:19-48, cpp/elastic_kernels.h:192-311,
 * cpp/identity_kernels.h:9-40 (IdentityScalar, a test kernel). */
#define TBEM_LAPLACE_SINGLE 0
#define TBEM_LAPLACE_DOUBLE 1
#define TBEM_ELASTIC_DISPLACEMENT 2
#define TBEM_ELASTIC_TRACTION 3
#define TBEM_ELASTIC_ADJOINT_TRACTION 4
#define TBEM_IDENTITY_SCALAR 5
#define TBEM_ELASTIC_HYPERSINGULAR 6  /* cpp/elastic_kernels.h:314-365 */
/* 2D kernels (cpp/laplace_kernels.h:66-110, cpp/elastic_kernels.h:21-189,
 * cpp/identity_kernels.h): points [n][2]; the plain FP64 form only (the
 * precision form is refused with TBEM_ERR_ARG); the gradient pass and the
 * allocation-free direct apply take 3D kernels only. */
#define TBEM_LAPLACE_SINGLE_2D 16          /* log(r) / (2 pi)                 */
#define TBEM_LAPLACE_DOUBLE_2D 17          /* n_src . d / (2 pi r^2)          */
#define TBEM_LAPLACE_HYPERSINGULAR_2D 18
#define TBEM_ELASTIC_DISPLACEMENT_2D 19    /* 2 x 2 tensors from here          */
#define TBEM_ELASTIC_TRACTION_2D 20
#define TBEM_ELASTIC_ADJOINT_TRACTION_2D 21
#define TBEM_ELASTIC_HYPERSINGULAR_2D 22
#define TBEM_IDENTITY_SCALAR_2D 23

/* precision forms */
#define TBEM_PRECISION_FP64 0   /* plain: reference surfaces and formulation, FP64 */
#define TBEM_PRECISION_MIXED 1  /* precision form: tensor-core M2L/M2M/L2L, FP32 P2P */
/* The precision form's operators (enclosing surfaces, single-layer
 * equivalent sources, the far field in the M2L SVD bases) applied in FP64 on
 * the SIMT FP64 pipes: the precision form's accuracy against the direct sum
 * (~1e-7 at the workload orders), but linear to FP64 rounding (its states
 * are well-conditioned check potentials, never the plain form's cancelling
 * equivalent densities) -- the O(N) FP64 residual operator of iterative
 * refinement.  3D kernels; the M2L operators must compress. */
#define TBEM_PRECISION_FP64_COMPRESSED 2

/* FMMConfig, cpp/fmm.h:73-96 (same five fields and meaning; `order` is the
 * requested number of translation-surface points, cpp/fmm.h:76-82). */
typedef struct {
    double mac;
    long order;
    long min_pts_per_cell;
    double d;
    int account_for_small_cells;
} TbemFmmConfig;

/* GPU-side options that have no reference counterpart. */
typedef struct {
    int precision;         /* TBEM_PRECISION_*                                   */
    int device;            /* CUDA device ordinal                                */
    double svd_threshold;  /* singular-value cutoff (reference: 1e-10, fmm.cpp:122) */
    int m2l_path;          /* precision form's dense translations:
                              0 auto (= 5 where the M2L operators are precomputed
                                and compress, = 2 where they are precomputed but
                                the compressed products, padded to the tensor-core
                                tiles, would not be cheaper; SIMT FP32 when the
                                M2L runs on the fly),
                              1 SIMT FP32 for all (uncompressed M2L),
                              2 tcgen05 3xBF16 for the uncompressed M2L only,
                              3 tcgen05 3xBF16 for M2L, M2M and L2L,
                              4 SVD-compressed far field on the SIMT FP32 pipes,
                              5 as 4 with the M2L products on tcgen05 3xBF16      */
    int p2p_block;         /* 0 auto; else threads per target in the P2P kernel (1,2,4,8) */
    int host_only;         /* 1: build trees and task lists only (no device use);
                              apply calls then fail with TBEM_ERR_STATE            */
    double m2l_rank_tol;   /* compressed M2L: singular values of the stacked M2L
                              operators kept down to this fraction of the largest
                              (0: 1e-7)                                           */
    int p2m_block;         /* 0 auto; else threads per target in the points-to-
                              check-surface kernel (1, 2, 4)                      */
    int tc_shape;          /* tensor-core tile: 0 auto (timed at creation); 1 N 128 x
                              K chunk 64, 2 N 64 x 64, 3 N 128 x 32, 4 N 256 x 32 */
} TbemGpuOptions;

typedef struct TbemFmm TbemFmm;

/* Fill *opt with defaults (FP64, device 0, threshold 1e-10, auto paths). */
void tbem_default_options(TbemGpuOptions* opt);

/* Replaces FMMOperator<dim,R,C>::FMMOperator(K, NBodyData, FMMConfig)
 * (cpp/fmm.cpp:72-101): builds both octrees (quadtrees for the 2D kernels,
 * with circle translation surfaces, cpp/fmm.cpp:7-20), the task lists, the translation
 * surfaces and the per-level check-to-equivalent operators, and uploads
 * everything to the device.  kernel_params = {shear_modulus, poisson_ratio}
 * for the elastic kernels (may be NULL for the scalar ones). */
int tbem_fmm_create(int kernel, const double* kernel_params,
                    const double* obs_locs, const double* obs_normals, long n_obs,
                    const double* src_locs, const double* src_normals,
                    const double* src_weights, long n_src,
                    const TbemFmmConfig* config, const TbemGpuOptions* options,
                    TbemFmm** out);

/* Batched form: one operator over n_meshes independent meshes (no reference
 * counterpart: the reference builds one FMMOperator per mesh,
 * cpp/fmm.cpp:72-101, and applies one right-hand side per call,
 * cpp/fmm.cpp:551-557).  Mesh m owns points [mesh_offsets[m],
 * mesh_offsets[m+1]) of locs / normals [N][3] and weights [N]; within a
 * mesh the observation points are its source points, and meshes do not
 * interact.  Each mesh is mapped into the cube [-1, 1]^3 (its bounding box's
 * centre to the origin, its largest half width to 1, the weights rescaled by
 * the kernel's homogeneity) and its octree is cut from that cube, so all
 * meshes share one set of translation operators and every pass of an apply
 * covers every mesh in one launch.  3D kernels (ids 0..6); either precision
 * form; no small-cell routing.  Apply with tbem_fmm_apply: x[r][d][j] over
 * all N points (meshes concatenated), y likewise; tbem_fmm_graph_create
 * captures it. */
int tbem_fmm_batch_create(int kernel, const double* kernel_params, int n_meshes,
                          const long* mesh_offsets, const double* locs, const double* normals,
                          const double* weights, const TbemFmmConfig* config,
                          const TbemGpuOptions* options, TbemFmm** out);
/* Number of meshes of an operator (1 for tbem_fmm_create's). */
long tbem_fmm_n_meshes(const TbemFmm* h);

/* Replaces FMMOperator::apply (cpp/fmm.cpp:551-557) for n_rhs right-hand
 * sides at once; stream is a cudaStream_t (NULL = the handle's stream).
 * With a host y the call is synchronous and a tensor-core pass that gave up
 * waiting (TBEM_ERR_TIMEOUT) is reported by this call.  With a device y the
 * call is asynchronous: such a timeout is only seen by the NEXT call on the
 * handle (the result of the failed apply is garbage), so a caller that keeps
 * its results on the device checks tbem_fmm_sync before using them.  Once
 * raised, the timeout stays: every later apply returns TBEM_ERR_TIMEOUT. */
int tbem_fmm_apply(TbemFmm* h, const double* x, double* y, int n_rhs, void* stream);

/* Waits for the handle's device work (its own stream and, when given, the
 * caller's stream) and returns TBEM_ERR_TIMEOUT if a tensor-core pass of any
 * earlier apply gave up waiting, else TBEM_OK.  No reference counterpart
 * (the reference's apply is synchronous). */
int tbem_fmm_sync(TbemFmm* h, void* stream);

/* Budget, in SM clock cycles, of every bounded wait in the tensor-core
 * kernels of this operator (0: the default of about two seconds).  A
 * smaller budget makes a slow wait give up sooner: the kernel then stops,
 * finishes the matrix products already issued, frees its tensor memory and
 * reports TBEM_ERR_TIMEOUT.  For tests of that error path; no reference
 * counterpart. */
int tbem_fmm_set_wait_cycles(TbemFmm* h, long long cycles);

/* Transpose apply: w = A^T z with A the operator tbem_fmm_apply applies
 * (the FMM passes run transposed and in reverse order).  No reference
 * counterpart; the reference's transpose partner kernel is
 * ElasticAdjointTraction (cpp/elastic_kernels.h:272-311). */
int tbem_fmm_apply_adjoint(TbemFmm* h, const double* z, double* w, int n_rhs, void* stream);

/* Source-side gradients of L = r^T A x (one right-hand side) through the
 * FMM: derivatives with respect to the source points' positions
 * (g_src_locs [n_src][3]), normals (g_src_normals [n_src][3]) and weights
 * (g_src_weights [n_src]); any output may be NULL.  One transposed apply of
 * r, then the three transposed passes that reach source points (near
 * field, points to up-check surfaces, points to down-check surfaces) again
 * with the kernel's exact derivatives (FP64 dual numbers), the far field
 * entering through the transposed check-surface states of that apply
 * (recomputed per call, nothing stored).  The O(N) counterpart of
 * tbem_direct_gradients' source outputs for the compressed forms (precision
 * and FP64 compressed; TBEM_ERR_STATE for the plain and batched forms).
 * Synchronous.  No reference counterpart. */
int tbem_fmm_source_gradients(TbemFmm* h, const double* x, const double* r, double* g_src_locs,
                              double* g_src_normals, double* g_src_weights, void* stream);

/* Observation-side gradients of L = r^T A x (one right-hand side) through
 * the FMM: derivatives with respect to the observation points' positions
 * (g_obs_locs [n_obs][3]) and normals (g_obs_normals [n_obs][3], nonzero
 * for the kernels with an observation normal); either output may be NULL.
 * One forward apply of x, then the three passes that reach observation
 * points (near field, M2P from the sources' up-equivalent surfaces, L2P from
 * the leaves' down-equivalent surfaces) again with the kernel's exact
 * derivatives (FP64 dual numbers); the down-equivalent densities are
 * rebuilt from the apply's compressed local coefficients.  The O(N)
 * counterpart of tbem_direct_gradients' observation outputs for the
 * compressed forms (TBEM_ERR_STATE for the plain and batched forms).
 * Synchronous.  No reference counterpart. */
int tbem_fmm_observation_gradients(TbemFmm* h, const double* x, const double* r,
                                   double* g_obs_locs, double* g_obs_normals, void* stream);

/* OperatorI::n_rows / n_cols (cpp/operator.h:15-16, cpp/fmm.h:235-236). */
long tbem_fmm_n_rows(const TbemFmm* h);
long tbem_fmm_n_cols(const TbemFmm* h);

/* OperatorI::clone (cpp/fmm.cpp:103-109): an independent operator. */
int tbem_fmm_clone(const TbemFmm* h, TbemFmm** out);

void tbem_fmm_destroy(TbemFmm* h);

/* Introspection for bit-exact checks against the reference octree
 * (cpp/octree.h:14-25) and task lists (FMMTasks, cpp/fmm.h:98-120).
 * which: 0 = source tree, 1 = observation tree.  Cells are reported in
 * pre-order with the reference's post-order `index`; center and half_width
 * are [n][3] (z = 0 for a 2D operator); any output pointer may be NULL;
 * returns the number of cells (or a negative status). */
long tbem_fmm_tree_cells(const TbemFmm* h, int which, long* level, long* index,
                         double* center, double* half_width, long* n_points,
                         long* n_children);
/* Point indices of every cell, concatenated in the same pre-order. */
long tbem_fmm_tree_indices(const TbemFmm* h, int which, long* out);
/* kind: 0 p2m, 1 m2m, 2 p2p, 3 m2p, 4 p2l, 5 m2l, 6 l2l, 7 l2p; pairs as
 * (obs cell index, src cell index), cell tasks with src = -1. */
long tbem_fmm_list(const TbemFmm* h, int kind, long* obs_index, long* src_index);
/* Number of translation-surface points actually used (cpp/fmm.cpp:22-45). */
long tbem_fmm_n_surface(const TbemFmm* h);
/* Number of check-to-equivalent levels (which: 0 up, 1 down). */
long tbem_fmm_n_c2e_levels(const TbemFmm* h, int which);
/* Read / replace the check-to-equivalent operator of one level (row-major,
 * (C n_s) x (R n_s), cpp/fmm.cpp:130-160).  Replacing is for the plain form
 * only: it lets a caller install operators from its own LAPACK. */
int tbem_fmm_get_c2e(const TbemFmm* h, int which, long level, double* out);
int tbem_fmm_set_c2e(TbemFmm* h, int which, long level, const double* op);

/* Per-phase device times: with timing enabled (tbem_fmm_set_timing) every
 * apply records CUDA events between its phases on its own stream, without
 * synchronizing.  tbem_fmm_phase_times waits for them and returns the mean
 * milliseconds per apply of every phase over the applies since the previous
 * call (the same numbers again when no apply ran since).  names/ms are
 * NULL-able; returns the number of phases. */
int tbem_fmm_set_timing(TbemFmm* h, int enabled);
int tbem_fmm_phase_times(const TbemFmm* h, const char** names, double* ms, int cap);

/* Wall seconds of the construction phases of this operator, in order
 * (trees_lists: octrees and task lists on the host; upload_tasks: device
 * geometry and work lists; c2e: check-to-equivalent pseudo-inverses; then
 * for the plain form operators: the translation tables, for the precision
 * forms translations: the translation tables, compression: the M2L SVD
 * bases and the compressed operators, leaf_operators: the per-leaf L2P
 * operators; autotune: launch shape choices), the device synchronized at
 * each phase end.  Replaces the
 * reference's construction inside FMMOperator's constructor
 * (cpp/fmm.cpp:71-101).  names/seconds are NULL-able; returns the number of
 * phases. */
int tbem_fmm_setup_times(const TbemFmm* h, const char** names, double* seconds, int cap);

/* Threads per target the point-to-point pass uses (chosen by timing the
 * candidates 2, 4, 8 at creation unless TbemGpuOptions.p2p_block fixed it). */
long tbem_fmm_p2p_block(const TbemFmm* h);
/* N tile (columns) of the precision form's tensor-core translations, chosen
 * by timing the 128- and 64-column shapes at creation (0 when unused). */
long tbem_fmm_tc_tile(const TbemFmm* h);

/* Ranks of the SVD-compressed M2L (input side, output side); both 0 when
 * the M2L is not compressed.  Returns 0 or a TBEM_ERR_* code. */
int tbem_fmm_m2l_ranks(const TbemFmm* h, long* r_in, long* r_out);

/* CUDA-graph capture (the batching form's single launch; no reference
 * counterpart: the reference applies one operator per call).  Captures the
 * applies (or, with adjoint != 0, the transposed applies) of n_ops operators
 * -- e.g. one per mesh of a batch -- from x[i] into y[i], n_rhs right-hand
 * sides each, spread over up to eight parallel branches.  x and y must be
 * device memory: the graph replays these addresses.  Each operator first
 * runs one ordinary apply (writing y[i]) that sizes its buffers; nothing is
 * allocated while capturing.  An operator's buffers are shared by its
 * applies and its graphs: do not run them concurrently.  Phase timing must be
 * off. */
typedef struct TbemGraph TbemGraph;
int tbem_fmm_graph_create(TbemFmm* const* ops, int n_ops, const double* const* x,
                          double* const* y, int n_rhs, int adjoint, TbemGraph** out);
/* Replays every captured apply with one graph launch on stream (NULL: the
 * graph's own stream); asynchronous.  Returns TBEM_ERR_TIMEOUT when a
 * tensor-core pass of an earlier replay gave up waiting. */
int tbem_fmm_graph_launch(TbemGraph* g, void* stream);
void tbem_fmm_graph_destroy(TbemGraph* g);

/* Number of kernel launches the last apply made on the device (no
 * reference counterpart; used to report the launch count of a timed run). */
long tbem_fmm_last_launches(const TbemFmm* h);

/* Direct N-body sum on the GPU in FP64 (nbody_eval over all pairs,
 * cpp/nbody_operator.h:117-141; the dense oracle make_direct_nbody_operator,
 * :143-152, matrix-free).  Same layouts as tbem_fmm_apply. */
int tbem_direct_apply(int kernel, const double* kernel_params,
                      const double* obs_locs, const double* obs_normals, long n_obs,
                      const double* src_locs, const double* src_normals,
                      const double* src_weights, long n_src,
                      const double* x, double* y, int n_rhs, void* stream);

/* Kernel-gradient pass of the direct FP64 operator (no reference
 * counterpart: the reference has no derivatives).  With A_ij =
 * w_j K(x_i, y_j; n_i, n_j) and L = r^T A x it writes dL/d(obs_locs) [n_obs][3],
 * dL/d(obs_normals), dL/d(src_locs) [n_src][3], dL/d(src_normals),
 * dL/d(src_weights) [n_src] and dL/dx = A^T r [C][n_src].  Kernel derivatives
 * are exact (forward-mode dual numbers on the device).  Any output may be
 * NULL; host or device memory. */
int tbem_direct_gradients(int kernel, const double* kernel_params,
                          const double* obs_locs, const double* obs_normals, long n_obs,
                          const double* src_locs, const double* src_normals,
                          const double* src_weights, long n_src,
                          const double* x, const double* r,
                          double* g_obs_locs, double* g_obs_normals,
                          double* g_src_locs, double* g_src_normals,
                          double* g_src_weights, double* g_x, void* stream);

/* The direct FP64 sum of tbem_direct_apply for callers that cannot allocate
 * device memory.  No counterpart in the reference.  3D kernel ids 0..6 only
 * (2D points would have to be widened into scratch).  Every point, weight,
 * density and output pointer must be device memory; kernel_params is read on
 * the host and must be host memory (or NULL for the defaults).  Nothing is
 * copied, allocated or freed.  Its scratch (weighted strengths and work
 * items) is a static 16 MiB device array kept by every GPU that loads the
 * library: R * n_src * n_rhs must not exceed 1,966,080 and n_obs must stay
 * below about 3 million, else TBEM_ERR_ARG.  Every call looks up the array's
 * device address on the current device (so a device reset is harmless); the
 * first call on a device loads the module there: make it before any stream
 * capture.  All calls share the array: calls that overlap on the GPU race.
 * Asynchronous on `stream`. */
int tbem_direct_apply_noalloc(int kernel, const double* kernel_params,
                              const double* obs_locs, const double* obs_normals, long n_obs,
                              const double* src_locs, const double* src_normals,
                              const double* src_weights, long n_src,
                              const double* x, double* y, int n_rhs, void* stream);

/* CSR operator (SparseOperator, cpp/sparse_operator.h:44-83):
 * y = A x for n_rhs right-hand sides (x[r*n_cols + j], y[r*n_rows + i]).
 * Column indices are int64 like the reference's size_t.  FP64. */
typedef struct TbemCsr TbemCsr;
int tbem_csr_create(long n_rows, long n_cols, const double* values,
                    const long* column_indices, const long* row_ptrs, TbemCsr** out);
int tbem_csr_apply(TbemCsr* h, const double* x, double* y, int n_rhs, void* stream);
long tbem_csr_nnz(const TbemCsr* h);
/* Shape and a host copy of the arrays (SparseOperator's n_rows / n_cols /
 * values / column_indices / row_ptrs, python_wrapper/linalg.cpp:15-38); any
 * output pointer may be NULL. */
int tbem_csr_shape(const TbemCsr* h, long* n_rows, long* n_cols);
int tbem_csr_download(const TbemCsr* h, double* values, long* column_indices, long* row_ptrs);
void tbem_csr_destroy(TbemCsr* h);

/* Replaces IntegralOperator::apply (cpp/integral_operator.h:55-63):
 * y = G (F (I x)) + N x + C x with the galerkin G, the farfield F (an FMM
 * operator), the interpolation I, the nearfield N and the farfield
 * correction C, chained on the device in one call (no host round trip between
 * the steps).  The operators are borrowed and must outlive the handle; the
 * shapes must chain (G: n x F.n_rows, I: F.n_cols x m, N and C: n x m), else
 * TBEM_ERR_ARG.  x: m * n_rhs, y: n * n_rhs values, host or device. */
typedef struct TbemIntegral TbemIntegral;
int tbem_integral_create(TbemCsr* nearfield, TbemCsr* correction, TbemCsr* galerkin,
                         TbemFmm* farfield, TbemCsr* interp, TbemIntegral** out);
int tbem_integral_apply(TbemIntegral* h, const double* x, double* y, int n_rhs, void* stream);
long tbem_integral_n_rows(const TbemIntegral* h);
long tbem_integral_n_cols(const TbemIntegral* h);
void tbem_integral_destroy(TbemIntegral* h);

/* Last error message of the calling thread ("" if none). */
const char* tbem_last_error(void);

/* Nearfield and farfield-correction matrices (make_nearfield_operator /
 * make_farfield_correction_operator, cpp/nearfield_operator.h:12-117, with
 * either integration strategy -- make_sinh_integrator or
 * make_adaptive_integrator, cpp/integral_term.h:53-150 -- and
 * IntegrationStrategy::compute_term, cpp/integral_term.cpp:33-92).  The host
 * finds every (Galerkin observation point, nearby source facet) term and the
 * point's Richardson direction; the GPU evaluates the quadratures (the
 * adaptive rule's subdivision is decided on the host, level by level, with
 * every level's points evaluated on the GPU).  Meshes share one vertex array [n_vertices][dim] (dim from the
 * kernel id); obs / src / all facets are [n][dim] vertex indices (the
 * reference's boundary_operator(obs_mesh, src_mesh, mthd, fmm_config,
 * all_mesh), cpp/integral_operator.h:66-99).  which: 0 the nearfield
 * operator (observation points from obs_near_order), 1 the farfield
 * correction (obs_far_order).  The result is a CSR operator with rows
 * R * n_obs_facets * n_obs_quad and columns C * dim * n_src_facets.  Runs
 * on the current CUDA device and synchronizes it before returning. */
#define TBEM_QUAD_SINH 0      /* make_sinh_integrator */
#define TBEM_QUAD_ADAPTIVE 1  /* make_adaptive_integrator (Gauss-Lobatto, near_tol) */

typedef struct {
    int strategy;          /* TBEM_QUAD_SINH or TBEM_QUAD_ADAPTIVE */
    double near_tol;       /* adaptive rule's tolerance */
    long sinh_order;       /* sinh rules: order + order * log(facet size / distance) points */
    long obs_near_order;   /* Gauss rule of the nearfield observation points */
    long obs_far_order;    /* Gauss rule of the farfield observation points */
    long src_far_order;    /* Gauss rule of far source facets */
    long n_singular_steps; /* Richardson steps (2..32) */
    double far_threshold;  /* facets nearer than far_threshold x facet size are "near" */
} TbemIntegrator;

/* Gauss rule on the reference facet (gauss_facet, cpp/gauss_quad.cpp:155-165):
 * points [n][dim - 1] on [-1, 1] (dim 2) or the triangle (0,0)-(1,0)-(0,1)
 * (dim 3), weights [n]; returns n (host only). */
long tbem_gauss_facet(int dim, long n, double* x, double* w);

/* Galerkin observation points of obs_facets with their Richardson (limit)
 * directions against all_facets (galerkin_obs_pts, cpp/nearfield_operator.h:
 * 12-40); outputs [n][dim] (NULL-able); returns n (host only). */
long tbem_galerkin_obs_points(int dim, const double* vertices, long n_vertices,
                              const long* obs_facets, long n_obs_facets, const long* all_facets,
                              long n_all_facets, long order, double* locs, double* normals,
                              double* dirs);

int tbem_nearfield_create(int kernel, const double* kernel_params, const double* vertices,
                          long n_vertices, const long* obs_facets, long n_obs_facets,
                          const long* src_facets, long n_src_facets, const long* all_facets,
                          long n_all_facets, const TbemIntegrator* mthd, int which,
                          TbemCsr** out);

/* The same matrices for given observation points (the reference's
 * interior_obs_pts, cpp/nearfield_operator.h:27-40, as dense_interior_operator
 * uses them, cpp/integral_operator.h:132-158): obs_locs / obs_normals
 * [n_obs][dim], their limit directions found against all_facets.  Rows
 * R * n_obs. */
int tbem_nearfield_points_create(int kernel, const double* kernel_params, const double* obs_locs,
                                 const double* obs_normals, long n_obs, const double* vertices,
                                 long n_vertices, const long* src_facets, long n_src_facets,
                                 const long* all_facets, long n_all_facets,
                                 const TbemIntegrator* mthd, int which, TbemCsr** out);

/* Limit (Richardson) directions of given points against all_facets
 * (decide_limit_dir, cpp/limit_direction.cpp:87-147, with the constants
 * interior_obs_pts passes); dirs [n][dim]; returns n (host only). */
long tbem_interior_obs_points(int dim, const double* locs, long n, const double* vertices,
                              long n_vertices, const long* all_facets, long n_all_facets,
                              double* dirs);

/* Measurement helper (no reference counterpart): the device's FMA rate in
 * TFLOP/s (FMA = 2 flops), FP32 (fp64 = 0) or FP64 (fp64 = 1), from a
 * microbenchmark of independent FMA chains filling every SM (2,048 threads
 * per SM, 8 chains per thread, ~10 ms per run, the best of 3 timed runs).
 * The denominator of the evaluation kernels' roofline. */
int tbem_fma_peak(int device, int fp64, double* tflops);

/* Setup cache (no reference counterpart): operator constructions in one
 * process reuse the check-to-equivalent pseudo-inverses and the M2L
 * compression's eigenbases of earlier constructions with the same kernel
 * parameters, surfaces and cell geometry (the displacement and traction
 * operators of one mesh factor once).  Host copies, at most 1 GB; this
 * empties the cache.  Returns TBEM_OK. */
int tbem_setup_cache_clear(void);

#ifdef __cplusplus
}
#endif
#endif /* TBEM_GPU_H */
