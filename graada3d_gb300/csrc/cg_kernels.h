// Launchers of the inversion kernels (cg.cu).  Internal interface.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

namespace grada {

// CSR matrix on the device, Eigen RowMajor compressed layout (int indices).
struct DevCSR {
  int64_t n = 0;
  int64_t nnz = 0;
  const int *rowptr = nullptr;
  const int *col = nullptr;
  const double *val = nullptr;
};

// out = c * wl .* (A x)
struct ForwardTerm {
  DevCSR A;
  double c = 1.0;
  const double *wl = nullptr;
  double *out = nullptr;
};
struct ForwardTerms {
  ForwardTerm t[7];
  int count = 0;
};

// contribution c * A^T (wl .* s), with A^T stored as its own CSR
struct AdjointTerm {
  DevCSR AT;
  double c = 1.0;
  const double *wl = nullptr;
  const double *s = nullptr;
};
struct AdjointTerms {
  AdjointTerm t[7];
  int count = 0;
};

// Slots of the device scalar array of one CG solve.
enum : int {
  CG_R2 = 0,
  CG_T2 = 1,
  CG_ALPHA = 2,
  CG_BETA = 3,
  CG_RLAST2 = 4,
  CG_ERR = 5,
  CG_ATB2 = 6,
  CG_R2NEW = 7,
  CG_MISFIT2 = 8,
  CG_TOL = 9,
  CG_NSCALARS = 16
};

// Slots of the device control block of one CG solve (ints).
enum : int { CTL_DONE = 0, CTL_ITER = 1, CTL_MAXIT = 2, CTL_STATUS = 3, CTL_NINTS = 4 };
enum : int {
  CG_STATUS_RUNNING = 0,
  CG_STATUS_CONVERGED = 1,
  CG_STATUS_BREAKDOWN = 2,
  CG_STATUS_NONFINITE = 3
};

int dot_blocks(int64_t n, int sm_count);

void launch_csr_apply(const DevCSR &A, const double *x, const double *xs, double c, const double *wl,
                      double *y, cudaStream_t s);
// Kernels taking `skip` return at once while *skip != 0 (see CTL_DONE).
void launch_multi_forward(const ForwardTerms &T, int64_t n, const double *x, cudaStream_t s,
                          const int *skip = nullptr);
void launch_adjoint(const AdjointTerms &T, int64_t n, const double *P, const double *gtw,
                    double sign_g, double *r, cudaStream_t s, const int *skip = nullptr);
void launch_dot(const double *a, const double *b, int64_t n, double *partial, int nblocks,
                double *out, cudaStream_t s, const int *skip = nullptr);
void launch_misfit_sq(const double *g, const double *dobs, const double *wd, int64_t n,
                      double *partial, int nblocks, double *out, cudaStream_t s);
void launch_data_residual(const double *dobs, const double *g, const double *wd, int64_t n,
                          double *b0, double *s0, cudaStream_t s);
void launch_scale(const double *a, const double *w, int64_t n, double c, double *out,
                  cudaStream_t s, const int *skip = nullptr);
void launch_negate(const double *a, int64_t n, double *out, cudaStream_t s);
void launch_p_update(const double *r, const double *P, const double *scal, int64_t n, double *p,
                     double *pp, cudaStream_t s, const int *skip = nullptr);
void launch_axpy(const double *t, const double *p, const double *scal, int64_t nrow, int64_t n,
                 double *sv, double *dx, cudaStream_t s, const int *skip = nullptr);
// alpha = r2/t2 and beta/err with the stopping test; ctl may be null.
void launch_alpha(double *scal, int *ctl, cudaStream_t s);
void launch_beta(double *scal, int *ctl, cudaStream_t s);
void launch_bound_update(const double *m, const double *dx, const double *mmin, const double *mmax,
                         int64_t n, double *mt, const double *mt_old, int *guard, int *any_guard,
                         int *h_any_guard, cudaStream_t s);
void launch_p_diag(const double *m, const double *mmin, const double *mmax, int64_t n, double *P,
                   cudaStream_t s);
void launch_irls_weight(const double *v, int64_t n, double eps2, double expo, double *wl,
                        cudaStream_t s);
void launch_sub(const double *a, const double *b, int64_t n, double *out, cudaStream_t s);
void launch_add(const double *a, const double *b, int64_t n, double *out, cudaStream_t s);

// ---- block solves (cg_block.cu) ---------------------------------------------
// A block vector holds kBW right-hand sides row-interleaved: element (i, c) of
// an n x kBW block is at [i * kBW + c], so the kBW values of one row share a
// 128-byte line and every per-row kernel is coalesced across the columns.
constexpr int kBW = 16;

// Per-column scalar slots: column c's CG_* scalars at scal[c * CG_NSCALARS + slot].
// Control block of a block solve (ints): [CTLB_ALL] = every column stopped,
// column c's CTL_* slots at [CTLB_COL + c * CTL_NINTS + slot].
enum : int { CTLB_ALL = 0, CTLB_COL = 4, CTLB_NINTS = 4 + kBW * CTL_NINTS };

// out = c[col] * wl .* (A x)   for up to 7 terms; wl a block or null
struct BForwardTerms {
  DevCSR A[7];
  double c[7][kBW];
  const double *wl[7];
  double *out[7];
  int count = 0;
};
// contribution c[col] * A^T (wl .* s) per term, A^T given as CSR
struct BAdjointTerms {
  DevCSR AT[7];
  double c[7][kBW];
  const double *wl[7];
  const double *s[7];
  int count = 0;
};

// y = c[col] * wl .* (A (x - xs)); x and y blocks, xs a plain vector or null.
void launch_bcsr_apply(const DevCSR &A, const double *x, const double *xs, const double *c,
                       const double *wl, double *y, cudaStream_t s);
void launch_bmulti_forward(const BForwardTerms &T, int64_t n, const double *x, cudaStream_t s,
                           const int *skip);
void launch_badjoint(const BAdjointTerms &T, int64_t n, const double *P, const double *gtw,
                     double sign_g, double *r, cudaStream_t s, const int *skip);
// Per-column dot products of two blocks (b null: a.a) into scal[c*CG_NSCALARS + slot].
void launch_bdot(const double *a, const double *b, int64_t n, double *partial, int nblocks,
                 double *scal, int slot, cudaStream_t s, const int *skip);
void launch_bmisfit_sq(const double *g, const double *dobs, const double *wd, int64_t n,
                       double *partial, int nblocks, double *scal, int slot, cudaStream_t s);
void launch_bdata_residual(const double *dobs, const double *g, const double *wd, int64_t n,
                           double *b0, double *s0, cudaStream_t s);
// out(i, c) = w_i * a(i, c)
void launch_bscale_rows(const double *a, const double *w, int64_t n, double *out, cudaStream_t s);
void launch_bp_update(const double *r, const double *P, const double *scal, int64_t n, double *p,
                      double *pp, cudaStream_t s, const int *skip);
void launch_baxpy(const double *t, const double *p, const double *scal, int64_t nrow, int64_t n,
                  double *sv, double *dx, cudaStream_t s, const int *skip);
void launch_balpha(double *scal, int *ctl, cudaStream_t s);
void launch_bbeta(double *scal, int *ctl, cudaStream_t s);
// Bound transform per column; guard and mt_old are blocks, any_guard holds
// kBW ints (pinned host copy in h_any_guard).
void launch_bbound_update(const double *m, const double *dx, const double *mmin,
                          const double *mmax, int64_t n, double *mt, const double *mt_old,
                          int *guard, int *any_guard, int *h_any_guard, cudaStream_t s);
void launch_bp_diag(const double *m, const double *mmin, const double *mmax, int64_t n, double *P,
                    cudaStream_t s);
// dst(:, c) = src(:, c) for the columns whose bit is set in mask.
void launch_bcopy_columns(const double *src, int64_t n, uint32_t mask, double *dst, cudaStream_t s);
// Block <-> column-major host layout (n x ncol, leading dimension n) on the device.
void launch_bpack(const double *colmajor, int64_t n, int ncol, double *block, cudaStream_t s);
void launch_bunpack(const double *block, int64_t n, int ncol, double *colmajor, cudaStream_t s);

}  // namespace grada
