/*
 * grada_gpu.h -- C ABI of the GB300 (sm_103a) implementation of GraAda3D's
 * forward-modelling and inversion hot path.
 *
 * The reference has no FFI layer: its boundary is the C++ class interface of
 * Fwd (src/Forward_modelling/Fwd.h:14-94), AdaptiveInversion
 * (src/Inversion/AdaptiveInversion.h) and GaussNewtonInversion
 * (src/Inversion/GaussNewtonInversion.h:4-112).  Each entry point below names
 * the reference member it replaces.  A drop-in translation unit that keeps
 * those class headers unchanged and forwards to these calls is shown in
 * INTEGRATION.md.
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

/* Replaces Fwd::G_vec_mul, dense branch (Fwd.cpp:114-146): y[Nd] = G x[Nm]. */
int grada_G_vec_mul(grada_ctx *ctx, const double *x, double *y);
/* Replaces Fwd::GT_vec_mul, dense branch (Fwd.cpp:80-112): x[Nm] = G^T y[Nd]. */
int grada_GT_vec_mul(grada_ctx *ctx, const double *y, double *x);
/* Device-pointer forms of the two products, enqueued on the context stream. */
int grada_G_vec_mul_dev(grada_ctx *ctx, const double *d_x, double *d_y);
int grada_GT_vec_mul_dev(grada_ctx *ctx, const double *d_y, double *d_x);

/*
 * Replaces the field sum of compute.cpp:246-260 (and Fwd::compute_gobs,
 * Fwd.h:25-29, without storing G): fields[i*n_fields + k] =
 * sum_j rho[j] * field_k(obs_i, cell_j), FP64 evaluation and accumulation.
 */
int grada_forward_field(grada_ctx *ctx, const double *rho, double *fields);
int grada_forward_field_dev(grada_ctx *ctx, const double *d_rho, double *d_fields);

/*
 * Measures the FP64 fused-multiply-add rate of the device (FLOP/s, FMA = 2
 * flops) with a register-resident DFMA loop, the denominator of the assembly
 * roofline.  No reference counterpart.
 */
int grada_measure_fp64_peak(grada_ctx *ctx, double *flops_per_s);

#ifdef __cplusplus
}
#endif

#endif /* GRADA_GPU_H */
