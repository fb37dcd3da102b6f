/*
 * grada_gpu.h -- C ABI of the GB300 (sm_103a) implementation of GraAda3D's
 * forward-modelling and inversion hot path.
 *
 * The reference has no FFI layer: its boundary is the C++ class interface of
 * Fwd (src/Forward_modelling/Fwd.h:14-94), AdaptiveInversion
 * (src/Inversion/AdaptiveInversion.h) and GaussNewtonInversion
 * (src/Inversion/GaussNewtonInversion.h:4-112).  Each entry point below names
 * the reference member it replaces.  Drop-in translation units that keep
 * those class headers unchanged and forward to these calls are in
 * graada3d_gb300/dropin/.
 *
 * Conventions
 *  - Every call returns an int status: GRADA_OK (0) or a negative GRADA_ERR_*.
 *    No C++ exception crosses the ABI.  grada_last_error() gives the message of
 *    the last failing call on that context.
 *  - A context owns one CUDA stream and all device buffers it allocates; they
 *    are released by grada_ctx_destroy().  Host arrays stay owned by the
 *    caller.  Calls taking host pointers are synchronous at return.  Calls
 *    whose name ends in _dev take device pointers, are enqueued on the context
 *    stream and return before the work finishes (grada_sync() waits).
 *  - One context is driven by one host thread at a time.
 *  - Geometry uses the reference conventions: metres, z positive downwards,
 *    prisms as (x0, x1, y0, y1, z0, z1) per cell in mesh leaf order
 *    (RectPrism._x/_y/_z, RectPrism.h:41-43), observation points as (x, y, z).
 *  - G is Nd x Nm with Nd = n_fields * n_obs; row i + k*n_obs holds the k-th
 *    requested component (ascending field bit) at observation i, column j is
 *    cell j (Fwd.cpp:47-78).  Field units follow GravFormula.h:6-14: V in
 *    m^2/s^2, g in mGal, T in Eotvos, for a density of 1 kg/m^3.
 */
#ifndef GRADA_GPU_H
#define GRADA_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
#define GRADA_OK 0
#define GRADA_ERR_INVALID_ARGUMENT (-1)
#define GRADA_ERR_CUDA (-2)
#define GRADA_ERR_OUT_OF_MEMORY (-3)
#define GRADA_ERR_STATE (-4)      /* call made before the data it needs was set */
#define GRADA_ERR_NONFINITE (-5)  /* NaN/Inf met in data or in a CG scalar */
#define GRADA_ERR_BREAKDOWN (-6)  /* CG scalar ||t||^2 == 0 */
#define GRADA_ERR_SCRATCH_LIMIT (-7) /* problem larger than a fixed scratch array */

/* Field bits, same layout as GS::ComputationOptions (gs.h:46-57). */
#define GRADA_FIELD_V 0x001u
#define GRADA_FIELD_GZ 0x002u
#define GRADA_FIELD_GX 0x004u
#define GRADA_FIELD_GY 0x008u
#define GRADA_FIELD_TZZ 0x010u
#define GRADA_FIELD_TXZ 0x020u
#define GRADA_FIELD_TYZ 0x040u
#define GRADA_FIELD_TXX 0x080u
#define GRADA_FIELD_TXY 0x100u
#define GRADA_FIELD_TYY 0x200u

/* Storage of the sensitivity matrix on the device. */
#define GRADA_G_FP64 0          /* Eigen::MatrixXd layout, bit-for-bit the FP64 entries */
#define GRADA_G_FP32 1          /* FP64 evaluation rounded to FP32 */
#define GRADA_G_BF16_ROWSCALE 2 /* bf16 entries times an FP32 scale per row */
#define GRADA_G_FP16_ROWSCALE 3 /* fp16 entries (|v| <= 1) times an FP32 scale per row */
#define GRADA_G_MATRIX_FREE 4   /* nothing stored: each product re-evaluates the prisms (FP64) */
#define GRADA_G_WAVELET 5       /* rows Daubechies-4 transformed and thresholded (grada_compute_G_wavelet) */

typedef struct grada_ctx grada_ctx;

/* Library version (major*10000 + minor*100 + patch). */
int grada_version(void);

/* Create a context on CUDA device `device`.  No reference counterpart (the
 * reference keeps all state in the Fwd/InversionBase objects). */
int grada_ctx_create(int device, grada_ctx **out);
int grada_ctx_destroy(grada_ctx *ctx);
const char *grada_last_error(const grada_ctx *ctx);
/* The context's cudaStream_t, as an opaque pointer. */
void *grada_ctx_stream(grada_ctx *ctx);
int grada_sync(grada_ctx *ctx);
/* Device bytes currently held by the context. */
int64_t grada_ctx_device_bytes(const grada_ctx *ctx);

/*
 * Replaces Fwd::set_mesh + Fwd::set_observation + the field_flag bitset
 * (Fwd.h:34-47, Fwd.cpp:18-45).  prisms: n_cells x 6 doubles, obs: n_obs x 3
 * doubles (host).  Drops any stored G.
 */
int grada_set_geometry(grada_ctx *ctx, const double *prisms, int64_t n_cells, const double *obs,
                       int64_t n_obs, uint32_t field_flag);

/* Dimensions of the current problem (any pointer may be NULL). */
int grada_get_dims(const grada_ctx *ctx, int64_t *n_cells, int64_t *n_obs, int *n_fields,
                   int64_t *nd, int64_t *ld);

/*
 * Replaces Fwd::compute_G (Fwd.cpp:47-78): assembles G on the device with
 * every entry evaluated in FP64, stored as `storage` (GRADA_G_*).
 */
int grada_compute_G(grada_ctx *ctx, int storage);

/* Storage kind of the current G, or -1 if none. */
int grada_G_storage(const grada_ctx *ctx);

/*
 * Replaces Fwd::get_G (Fwd.h:49): copies G to host, column-major, leading
 * dimension ld_host >= Nd, entries widened to double.
 */
int grada_get_G(grada_ctx *ctx, double *host, int64_t ld_host);
/*
 * Rows of the stored G (Fwd::get_G's matrix, Fwd.h:49, read row by row, as
 * the reference's own callers index G(i, :)): host[r * Nm + j] = G(rows[r], j)
 * for n_rows row indices in [0, Nd), widened to double.  For checking or
 * inspecting a G too large to copy whole.
 */
int grada_get_G_rows(grada_ctx *ctx, const int64_t *rows, int64_t n_rows, double *host);

/* Replaces Fwd::G_vec_mul, dense branch (Fwd.cpp:114-146): y[Nd] = G x[Nm]. */
int grada_G_vec_mul(grada_ctx *ctx, const double *x, double *y);
/* Replaces Fwd::GT_vec_mul, dense branch (Fwd.cpp:80-112): x[Nm] = G^T y[Nd]. */
int grada_GT_vec_mul(grada_ctx *ctx, const double *y, double *x);
/* Device-pointer forms of the two products, enqueued on the context stream. */
int grada_G_vec_mul_dev(grada_ctx *ctx, const double *d_x, double *d_y);
int grada_GT_vec_mul_dev(grada_ctx *ctx, const double *d_y, double *d_x);

/*
 * d_y[nd] = G d_x[nm] for an FP64 G that the caller owns (column-major,
 * leading dimension ld >= nd, ld even, 16-byte aligned), enqueued on `stream`
 * (a cudaStream_t; NULL = legacy default stream) of the current device,
 * without allocating anything: no context, no cudaMalloc/cudaFree.  No
 * counterpart in the reference; it exists for callers that cannot allocate
 * device memory at the point of the call (inside another library's stream
 * capture, under their own fixed device-memory budget, or on a path where
 * an allocation's device-wide synchronisation is not acceptable).  Its
 * scratch is an 8 MiB array built into the library (every GPU that loads the
 * library holds it until exit): ld above 1,048,576 returns
 * GRADA_ERR_SCRATCH_LIMIT.  The first call on a device looks up the array's
 * device address (make it before any stream capture that should contain
 * later calls); that address is cached for the process, so after a
 * cudaDeviceReset of that device the entry point must not be called there
 * again.  All calls on a device share the array: calls that may overlap on
 * the GPU race.  Only the status of its own two launches is returned; an
 * error pending from the caller's earlier work is left for the caller.
 */
int grada_G_vec_mul_noalloc(const double *d_G, int64_t nd, int64_t nm, int64_t ld,
                            const double *d_x, double *d_y, void *stream);

/*
 * Replaces AdaptiveInversion::expand_G (AdaptiveInversion.cpp:23-106) after
 * the host's Mesh::refinement split n_split leaf cells: parent_index[n_split]
 * (strictly ascending column indices of the current G) are each replaced, in
 * place, by the columns of their 8 children; child_prisms holds n_split x 8 x 6
 * doubles in Cell::child_cells order (x outer, y, z inner, Mesh.cpp:1579-1600),
 * or NULL to split every parent at its centre as Mesh::refinement does.  G
 * (FP64 or FP32 storage) and the context's cell list grow by 7 per split; the
 * other columns keep their order.  The regularisation operators must be set
 * again afterwards (the reference rebuilds them after a refinement,
 * GaussNewtonInversion.cpp:1160-1290).
 */
int grada_expand_G(grada_ctx *ctx, int64_t n_split, const int64_t *parent_index,
                   const double *child_prisms);

/*
 * Replaces the field sum of compute.cpp:246-260 (and Fwd::compute_gobs,
 * Fwd.h:25-29, without storing G): fields[i*n_fields + k] =
 * sum_j rho[j] * field_k(obs_i, cell_j), FP64 evaluation and accumulation.
 */
int grada_forward_field(grada_ctx *ctx, const double *rho, double *fields);
int grada_forward_field_dev(grada_ctx *ctx, const double *d_rho, double *d_fields);

/*
 * Replaces Fwd::compute_G_wavelet (Fwd.cpp:148-219, method_id 2 of
 * GaussNewtonInversion::invert): every row of G, its cells in `order`
 * (order[j] = Mesh::get_reordered_id(j), a permutation of the Nm cells),
 * zero-padded to the next power of two n_dy, is transformed with the periodic
 * Daubechies-4 pyramid (the algorithm of gsl_wavelet_daubechies, member 4)
 * and keeps the coefficients c with |c| > t or ||c| - t| < 1e-15,
 * t = relative_threshold x the row's largest |c| (Fwd::compress_vec,
 * :298-358).  Like the reference it never holds the dense G: rows are
 * assembled, transformed and thresholded a batch of points at a time.  Then
 * grada_G_vec_mul / grada_GT_vec_mul (and their
 * _dev forms), grada_solve_cg and grada_invert use the compressed rows, as
 * the reference's G_vec_mul / GT_vec_mul do (:80-146); other G readers answer
 * GRADA_ERR_STATE.  Needs 2 <= Nm <= 2^28.  The rows are assembled for batches of
 * points within about 8 GB of scratch (the environment variable
 * GRADA_WAVELET_BATCH_POINTS sets a smaller batch, for tests).
 */
int grada_compute_G_wavelet(grada_ctx *ctx, const int64_t *order, double relative_threshold);

/* As grada_compute_G_wavelet, the kept coefficients stored in value_storage:
 * GRADA_G_FP64 (the reference's) or GRADA_G_FP32 (rounded to nearest; 8 bytes
 * per coefficient with its index instead of 12).  The products stay FP64. */
int grada_compute_G_wavelet_ex(grada_ctx *ctx, const int64_t *order, double relative_threshold,
                               int value_storage);

/* The compressed rows: *n_dy and *nnz always; rowptr (Nd + 1), col and val
 * (nnz, widened to FP64 when stored in FP32) when not NULL.  GRADA_ERR_STATE
 * unless G is wavelet-compressed. */
int grada_get_wavelet_G(grada_ctx *ctx, int64_t *n_dy, int64_t *nnz, int64_t *rowptr, int32_t *col,
                        double *val);

/*
 * Measures the FP64 fused-multiply-add rate of the device (FLOP/s, FMA = 2
 * flops) with a register-resident DFMA loop, the denominator of the assembly
 * roofline.  No reference counterpart.
 */
int grada_measure_fp64_peak(grada_ctx *ctx, double *flops_per_s);

/* ------------------------------------------------------------------------
 * Inversion (GaussNewtonInversion on top of InversionBase / AdaptiveInversion)
 * ------------------------------------------------------------------------ */

/* Operator slots of grada_set_operator. */
#define GRADA_OP_WS 0 /* a_s*S_s*V*D_s*Z   (GaussNewtonInversion.cpp:711) */
#define GRADA_OP_WX 1 /* a_x*S_x*V*D_x1*Z  (:712) */
#define GRADA_OP_WY 2 /* a_y*S_y*V*D_y1*Z  (:713) */
#define GRADA_OP_WZ 3 /* a_z*S_z*V*D_z1*Z  (:714) */
#define GRADA_OP_TX 4 /* T_x of InversionBase::set_Tmatrix (InversionBase.cpp:468-495) */
#define GRADA_OP_TY 5 /* T_y */
#define GRADA_OP_TZ 6 /* T_z */

/*
 * Uploads one host-built regularisation operator (Nm x Nm), in the compressed
 * row storage of Eigen::SparseMatrix<double, RowMajor> (gs.h:29): rowptr[n+1]
 * = outerIndexPtr(), col[nnz] = innerIndexPtr(), val[nnz] = valuePtr().  The
 * construction of these operators stays on the host, as in the reference.
 */
int grada_set_operator(grada_ctx *ctx, int which, int64_t n, int64_t nnz, const int *rowptr,
                       const int *col, const double *val);

/*
 * Builds Ws, Wx, Wy, Wz on the device for the current cells, in place of the
 * host rebuild after a refinement (InversionBase::init_matrices,
 * InversionBase.cpp:146-187: set_Vmatrix :452-466, set_depth_weighting
 * :497-529, set_difference_matrix :189-434; W_* = a_* S_* V D_* Z with S_* = I,
 * GaussNewtonInversion.cpp:711-714), transposes included.
 *   faces: n_cells x 3 x 5 int32, per cell and axis (x, y, z) the face the
 *     reference differences against: [side, c0, c1, c2, c3].  side +1: the
 *     +axis face (-w on the diagonal, +w to the neighbour); -1: the -axis face,
 *     the +axis face being on the boundary (signs swapped); 0: no row.  One
 *     neighbour (c1 = c2 = c3 = -1), of the same or a coarser level, or four
 *     finer neighbours taking w/4 each.  w = 1 / (0.5 (h0 + h1)), h the sizes
 *     along the axis, h1 that of c0.  Checked on the host before any launch.
 *   depth_flag 0: Z_ii = 1 / |zp - zc_i|^(beta/2), zp the mean observation
 *     height; 1: Z_ii = sqrt(||G(:, i)|| / Nd) from the stored G.
 *   alphas: a_s, a_z, a_x, a_y.
 * The values follow the reference's operations in its order; Z's power may
 * differ from the host C library's in the last bits.
 */
int grada_build_operators(grada_ctx *ctx, const int32_t *faces, double beta, int depth_flag,
                          const double *alphas);

/* Reads an operator back (its rows as grada_set_operator takes them): *nnz
 * always, rowptr (Nm + 1), col and val (nnz) when not NULL.
 * GRADA_ERR_STATE if the slot is empty. */
int grada_get_operator(grada_ctx *ctx, int which, int64_t *nnz, int *rowptr, int *col,
                       double *val);

/*
 * Cross-gradient coupling (use_cross_gradient_constraint, InversionBase.h:125):
 * when enabled the CG system gains the rows a_crg*S_crg*T_{z,x,y}
 * (GaussNewtonInversion.cpp:1445-1450).  S_crg: Nm diagonal, NULL = identity.
 */
int grada_set_cross_gradient(grada_ctx *ctx, int enabled, double a_crg, const double *S_crg);

/* Replaces InversionBase::set_dobs (InversionBase.cpp:530-579): observed data
 * (Nd) and the diagonal of Wd (Nd). */
int grada_set_data(grada_ctx *ctx, const double *dobs, const double *wd);

/*
 * Replaces GaussNewtonInversion::solve_cg (GaussNewtonInversion.cpp:1417-1698),
 * with the reference's semantics: CGLS from dx = 0 on the stacked system
 * [Wd G P; sqrt(lambda) WL_s Ws P; sqrt(lambda) WL_z Wz P; ...], including the
 * operator choices of the reference (forward Ws row without WL_s; forward crg
 * rows weighted by WL_z/WL_x/WL_y; WL_y in the initial crg-y adjoint), and the
 * stopping test ||r||^2 / ||A^T b||^2 < tol.  WL[7] in the reference argument
 * order (WL_s, WL_x, WL_y, WL_z, WL_tx, WL_ty, WL_tz), Nm diagonals, NULL =
 * identity.  Host pointers; dx[Nm] out.  Returns GRADA_ERR_BREAKDOWN when
 * ||t||^2 becomes 0 (the reference would divide by zero).
 */
int grada_solve_cg(grada_ctx *ctx, double tol, int maxit, double lambda, const double *mk,
                   const double *mref, const double *P, const double *const WL[7], double *dx,
                   double *err, int *iterations);

typedef struct grada_invert_params {
  double max_lambda;             /* InversionBase::set_max_lambda */
  int n_lambda;                  /* set_n_lambda */
  double lambda_decreasing_rate; /* set_lambda_decreasing_rate */
  double target_misfit;          /* set_target_misfit */
  double stag_tol;               /* GaussNewtonInversion::set_stagnation_tolerance */
  double cg_tol;                 /* set_CG_parameter */
  double cg_iteration_factor;    /* set_CG_parameter: >= 1 iterations, < 1 fraction of Nm */
  int gn_iterations;             /* set_max_GN_iterations */
  int lp_s, lp_x, lp_y, lp_z, lp_t; /* set_Lp_inversion_parameter (p in {0,1,2}) */
  double epsilon2;
  int start_from_reference;      /* use_petrophysical_constraint: start from m0 */
  int fp64_refinement;           /* with FP32/bf16 G: FP64 matrix-free residual once per GN iteration */
} grada_invert_params;

typedef struct grada_invert_report {
  double final_misfit;      /* InversionBase::get_final_misfit */
  double final_lambda;      /* get_final_lambda */
  int gn_iterations;        /* Gauss-Newton iterations run */
  int n_trials;             /* lambda trials (lines of lambda_misfit_GN) */
  int64_t cg_iterations;    /* CG iterations over all trials */
  int64_t fp64_refinements; /* FP64 matrix-free residual evaluations */
  int64_t mesh_refinements; /* refinements of an adaptive inversion */
} grada_invert_report;

/*
 * Replaces GaussNewtonInversion::invert_with_own_CG on a fixed mesh
 * (GaussNewtonInversion.cpp:657-1103; the mesh-refinement branch stays with
 * the host's AdaptiveInversion): lambda search with cooling, IRLS reweighting
 * of the Ws/Wx/Wy/Wz (and crg) terms for p != 2, exponential bound transform,
 * stopping on the target misfit, stagnation, or increasing misfit.  Uses the
 * G assembled by grada_compute_G in whatever storage it has (FP64: the
 * reference arithmetic; FP32/bf16: the CG products in reduced precision).
 * m_ini, m_min, m_max, m0: Nm host vectors (m0 NULL = 0); m_out: Nm.
 */
int grada_invert(grada_ctx *ctx, const grada_invert_params *params, const double *m_ini,
                 const double *m_min, const double *m_max, const double *m0, double *m_out,
                 grada_invert_report *report);

/*
 * The adaptive inversion: invert_with_own_CG with its refinement branch
 * (GaussNewtonInversion.cpp:1098-1294).  After a Gauss-Newton iteration that
 * neither reaches the target nor is the last, with c refinements done so far:
 * if c >= max_refinement_number and the misfit stagnated, stop; else if
 * c < max_refinement_number and (interval_between_refinements iterations
 * passed since the last refinement, or the misfit stagnated), refine: the
 * library calls refine(user, ctx, m, Nm) with the current model on the host.
 * The callback is the host's AdaptiveInversion::refine_mesh
 * (AdaptiveInversion.cpp:637-735): it splits cells (mesh refinement stays on
 * the host), calls grada_expand_G, rebuilds Ws/Wx/Wy/Wz (grada_build_operators
 * or grada_set_operator; with the cross-gradient term also T and S_crg) and
 * hands back the model, bounds and reference model on the new cells with
 * grada_set_inversion_model; it returns GRADA_OK or a failure status.  The
 * library then resets the IRLS weights to one and recomputes those of the
 * p != 2 terms from the model, as the reference does, and continues.  FP64 or
 * FP32 G (not a kept FP64 G).  The final model has the final cell count:
 * read it with grada_get_model.
 */
typedef int (*grada_refine_fn)(void *user, grada_ctx *ctx, const double *m, int64_t nm);
typedef struct grada_adaptive_params {
  int max_refinement_number;        /* AdaptiveInversion::set_max_refinement_number */
  int interval_between_refinements; /* set_interval_between_refinements */
  grada_refine_fn refine;
  void *user;
} grada_adaptive_params;
int grada_invert_adaptive(grada_ctx *ctx, const grada_invert_params *params,
                          const grada_adaptive_params *adaptive, const double *m_ini,
                          const double *m_min, const double *m_max, const double *m0,
                          grada_invert_report *report);
/* Inside a refine callback only: m, m_min, m_max, m0 on the refined cells
 * (Nm each; m0 NULL = 0). */
int grada_set_inversion_model(grada_ctx *ctx, const double *m, const double *m_min,
                              const double *m_max, const double *m0);
/*
 * Trace of the persistent CG loop (no reference counterpart): the mean time per
 * CG iteration, in ns, of its four phases -- G p with the direction update,
 * the finish of G p with the regulariser rows and ||t||^2, the step, and G^T s
 * with the adjoint and ||r||^2 -- each up to the end of its team barrier, as
 * CTA 0 saw them, over the persistent solves since the last grada_invert (or
 * since the context was made); *iterations gets their iteration count.
 */
int grada_cg_phase_times(grada_ctx *ctx, double *mean_ns, int64_t *iterations);
/*
 * Host time in the CG loops of the solves since the last grada_invert (or since
 * the context was made), any G storage and loop (no reference counterpart):
 * seconds[0] from the first launch of each solve's loop to its last host
 * synchronisation, seconds[1] building the loops' CUDA graphs (capture and
 * instantiation; nothing for a solve that reuses a graph); *iterations gets
 * their CG iteration count.  Separates the loop's cost per iteration from the
 * set-up, predictions and lambda control around it.
 */
int grada_cg_loop_time(grada_ctx *ctx, double *seconds, int64_t *iterations);

/* The model of the last grada_invert / grada_invert_adaptive (Nm doubles). */
int grada_get_model(grada_ctx *ctx, double *m);

/*
 * Keep the FP64 G beside a reduced-precision one (no counterpart in the
 * reference, which has only FP64 G).  With keep != 0, the next
 * grada_compute_G with FP32 / bf16 / fp16 storage assembles G in FP64, keeps
 * it, and rounds the reduced entries from it (bitwise those of the direct
 * assembly).  grada_invert and grada_lambda_sweep with fp64_refinement then
 * predict the data with FP64 products of the kept G (CG right-hand sides and
 * every trial misfit exact in FP64; only the CG operator runs in reduced
 * precision) instead of one matrix-free FP64 residual per Gauss-Newton
 * iteration; report.fp64_refinements counts those products.  Costs the FP64
 * G's memory; dropped by grada_expand_G and grada_set_geometry.
 */
int grada_keep_fp64_G(grada_ctx *ctx, int keep);

/*
 * Column norms of the stored G: norms[j] = ||G(:, j)||_2 (Nm doubles, host),
 * FP64 sums of the stored entries (16-bit ones times their row scale).  Serves
 * InversionBase::set_depth_weighting with flag 1 (InversionBase.cpp:521-527,
 * Z_ii = sqrt(||G(:, i)|| / Nd)) without copying G to the host.
 * GRADA_ERR_STATE for matrix-free G.
 */
int grada_G_column_norms(grada_ctx *ctx, double *norms);

/* The records of the last grada_invert: trials as rows of 5 doubles
 * (gn_iteration, lambda, misfit, cg_iterations, cg_error) -- lambda_misfit_GN,
 * GaussNewtonInversion.cpp:921-923 -- and iterations as rows of 3 doubles
 * (gn_iteration, n_trials, misfit) -- Iteration_misfit_GN, :1046-1048.  At
 * most cap rows are written; *n gets the total. */
int grada_get_trials(const grada_ctx *ctx, double *rows, int64_t cap, int64_t *n);
int grada_get_iterations(const grada_ctx *ctx, double *rows, int64_t cap, int64_t *n);

/*
 * Many independent problems at once (no reference counterpart; the reference
 * runs one inversion per process).  Each context must be set up as for the
 * single calls; the batch runs them concurrently, one host thread per context
 * (at most max_threads, 0 = one per context) and each context on its own
 * stream, so small problems that cannot fill the GPU alone overlap on it.
 * statuses[n] gets each problem's status; the call returns GRADA_OK if all
 * succeeded, else the first failing status.
 *  grada_compute_G_batch: grada_compute_G(ctxs[k], storage) for every k.
 *  grada_invert_batch: grada_invert(ctxs[k], params[k], ...) for every k, the
 *  vectors given per problem (m0s[k] may be NULL, as may m0s itself).
 */
int grada_compute_G_batch(int n, grada_ctx *const *ctxs, int storage, int max_threads,
                          int *statuses);
int grada_invert_batch(int n, grada_ctx *const *ctxs, const grada_invert_params *params,
                       const double *const *m_ini, const double *const *m_min,
                       const double *const *m_max, const double *const *m0s,
                       double *const *m_out, grada_invert_report *reports, int max_threads,
                       int *statuses);

/*
 * The same batch as grada_invert_batch in ONE persistent cooperative launch
 * (captured in a CUDA graph) instead of host threads: the GPU's resident CTAs
 * are split into teams.  team_ctas > 0: teams of that many CTAs, each taking
 * the next problem from a device queue, largest first; -1: one team per
 * problem, its CTAs in proportion to the problem's G, all problems at once
 * (with more problems than resident CTAs, teams of 8 and the queue); 0: the
 * loaded tuning table's choice for the batch's largest G (8 without a table).
 * A team runs its problem's whole invert_with_own_CG
 * (GaussNewtonInversion.cpp:657-1103: lambda search, CG solves, bound
 * transform, misfits, IRLS, stopping tests) on the device, then the next.
 * Each problem's model, report and trial/iteration records are bitwise those
 * of grada_invert on the same context.  Needs every context on one device,
 * the same G storage for all, and either an FP64 G or a reduced-precision G
 * with the FP64 G kept (grada_keep_fp64_G) and params[k].fp64_refinement set;
 * otherwise GRADA_ERR_STATE (grada_invert_batch covers the rest).  Every
 * barrier wait of a team is bounded; an expiry returns GRADA_ERR_CUDA.
 * Messages go to grada_last_error(ctxs[0]).
 */
int grada_invert_batch_persistent(int n, grada_ctx *const *ctxs,
                                  const grada_invert_params *params,
                                  const double *const *m_ini, const double *const *m_min,
                                  const double *const *m_max, const double *const *m0s,
                                  double *const *m_out, grada_invert_report *reports,
                                  int team_ctas, int *statuses);
/*
 * The team-size table of grada_invert_batch_persistent, a text file of rows
 * "<largest G of the batch, entries> <CTAs per team, or -1>" ('#' starts a comment),
 * written by graada3d_gb300/autotune.py from measured batches.  Process-wide.
 */
int grada_load_batch_tuning(const char *path);
/* Shape of the last persistent batch run on ctx (the first context of the
 * batch): the number of teams and the CTAs per team. */
int grada_batch_shape(const grada_ctx *ctx, int *teams, int *team_ctas);

/*
 * Blocks of right-hand sides on one G (no single reference counterpart: each
 * column equals one call of the single entry point named).  Column-major host
 * arrays; n_rhs >= 1 columns are processed sixteen at a time, and each group
 * of sixteen reads G once per product (FP32 and 16-bit G on the tensor cores,
 * FP64 G on the FP64 pipe, matrix-free G with one prism evaluation per pair).
 *  grada_G_mat_mul:  Y[Nd x n] = G X[Nm x n]     (n x Fwd::G_vec_mul, Fwd.cpp:114-146)
 *  grada_GT_mat_mul: X[Nm x n] = G^T Y[Nd x n]   (n x Fwd::GT_vec_mul, Fwd.cpp:80-112)
 */
int grada_G_mat_mul(grada_ctx *ctx, int n_rhs, const double *X, double *Y);
int grada_GT_mat_mul(grada_ctx *ctx, int n_rhs, const double *Y, double *X);
/* Device-pointer forms for exactly 16 columns in the library's block layout
 * (element (i, c) at [i * 16 + c]): d_Y is Nd x 16, d_X is Nm x 16.  Enqueued
 * on the context stream; no synchronisation. */
int grada_G_block_mul_dev(grada_ctx *ctx, const double *d_X, double *d_Y);
int grada_GT_block_mul_dev(grada_ctx *ctx, const double *d_Y, double *d_X);

/*
 * n_rhs solve_cg systems that share G, the data and the operators
 * (GaussNewtonInversion::solve_cg, GaussNewtonInversion.cpp:1417-1698, once
 * per column): column c has its own lambda[c], model mk[:, c], P[:, c] and
 * weights WL[k][:, c] (WL[k] NULL = identity for every column); mref is
 * shared.  mk, P, WL[k], dx are Nm x n_rhs column-major.  Each column stops
 * on its own test; err[c] and iterations[c] are the single call's outputs.
 */
int grada_solve_cg_block(grada_ctx *ctx, double tol, int maxit, int n_rhs, const double *lambda,
                         const double *mk, const double *mref, const double *P,
                         const double *const WL[7], double *dx, double *err, int *iterations);

/*
 * Regularisation sweep: for each lambdas[c], the inversion grada_invert runs
 * with n_lambda = 1 and max_lambda = lambdas[c] (a fixed-lambda
 * Gauss-Newton run, invert_with_own_CG, GaussNewtonInversion.cpp:815-1103),
 * all lambda values advancing together so that their CG solves run as one
 * block per Gauss-Newton iteration.  prm->n_lambda and prm->max_lambda are
 * ignored.  m_out is Nm x n_lambda column-major; reports[c] as grada_invert's.
 * grada_get_sweep_trials gives column c's trial records (the rows of
 * grada_get_trials) of the last sweep.
 */
int grada_lambda_sweep(grada_ctx *ctx, const grada_invert_params *prm, int n_lambda,
                       const double *lambdas, const double *m_ini, const double *m_min,
                       const double *m_max, const double *m0, double *m_out,
                       grada_invert_report *reports);
int grada_get_sweep_trials(const grada_ctx *ctx, int column, double *rows, int64_t cap,
                           int64_t *n);

/*
 * Replaces AdaptiveInversion::indicator_calculator (AdaptiveInversion.cpp:
 * 108-204): indicator[i] = sum over k in [rowptr[i], rowptr[i+1]) of
 * (m[neighbour[k]] - m[i])^2 * area[k], in that order and with the
 * reference's rounding (bitwise equal).  The host builds each leaf cell's
 * (neighbour, area) list from its mesh faces in the reference's order: for
 * side j = 0, 1 the x, y, z faces; a leaf face with cells on both sides gives
 * the cell across it and the cell's own face area, a split face its four
 * child faces' cells and their face areas.  m, indicator: Nm; rowptr: Nm + 1.
 */
int grada_refinement_indicator(grada_ctx *ctx, const double *m, const int64_t *rowptr,
                               const int64_t *neighbour, const double *area, double *indicator);

/*
 * Fault injection for tests (no reference counterpart; nothing faults on the
 * GPU).  GRADA_FAULT_ALLOC: the context's next device allocation fails with
 * GRADA_ERR_OUT_OF_MEMORY.  GRADA_FAULT_TC_TIMEOUT: raises the flag a
 * tensor-core block product sets when one of its bounded waits expires, so
 * the next block product returns GRADA_ERR_CUDA.  GRADA_FAULT_CG_WAIT: the
 * next persistent CG solve (stored dense G) runs with a zero limit on its grid
 * barriers' waits, so a real device-side wait expires: every CTA returns, the
 * solve returns GRADA_ERR_CUDA.  GRADA_FAULT_TC_WAIT: the next tensor-core
 * block products run their main-loop mbarrier waits with no time at all, so a
 * real wait expires on the device: the CTA stops issuing, drains its own TMA
 * loads and MMAs (with the usual limit), frees its tensor memory and exits,
 * and the product returns GRADA_ERR_CUDA.  GRADA_FAULT_NONE clears pending
 * faults.  The context stays usable after each.
 */
#define GRADA_FAULT_NONE 0
#define GRADA_FAULT_ALLOC 1
#define GRADA_FAULT_TC_TIMEOUT 2
#define GRADA_FAULT_CG_WAIT 3
#define GRADA_FAULT_TC_WAIT 4
int grada_inject_fault(grada_ctx *ctx, int fault);

#ifdef __cplusplus
}
#endif

#endif /* GRADA_GPU_H */
