// Vector and sparse-operator kernels of a block of independent CG solves.
//
// A block solve runs kBW = 16 of the reference's solve_cg systems
// (src/Inversion/GaussNewtonInversion.cpp:1417-1698) side by side: the same
// G, data and operators, but per column its own lambda, model, P and WL
// weights.  Element (i, c) of a block vector sits at [i * kBW + c]; one
// thread owns one element, so the sixteen columns of a row are one 128-byte
// line and the sparse operators' index lists are read once per row for all
// columns.  Every column keeps its own CG scalars and stopping test; a column
// that has stopped keeps alpha = 0, so its dx and residuals stay frozen while
// the others continue.  Arithmetic is FP64 and every reduction has a fixed
// order (bit-reproducible), as in cg.cu.
#include "cg_kernels.h"
#include "common.cuh"

namespace grada {

namespace {

constexpr int BT = 256;               // threads per block
constexpr int ROWS = BT / kBW;        // rows per block in the reductions

unsigned bblocks(int64_t n) { return (unsigned)std::max<int64_t>(1, ceil_div(n * kBW, BT)); }

__global__ void bcsr_apply_kernel(DevCSR A, const double *__restrict__ x,
                                  const double *__restrict__ xs, const double *__restrict__ cvec,
                                  const double *__restrict__ wl, double *__restrict__ y) {
  const int64_t e = (int64_t)blockIdx.x * BT + threadIdx.x;
  if (e >= A.n * kBW) return;
  const int64_t i = e / kBW;
  const int c = (int)(e % kBW);
  double acc = 0.0;
  for (int k = A.rowptr[i]; k < A.rowptr[i + 1]; k++) {
    const int j = A.col[k];
    const double xv = xs ? (x[(int64_t)j * kBW + c] - xs[j]) : x[(int64_t)j * kBW + c];
    acc = fma(A.val[k], xv, acc);
  }
  double v = (cvec ? cvec[c] : 1.0) * acc;
  if (wl) v *= wl[e];
  y[e] = v;
}

__global__ void bmulti_forward_kernel(BForwardTerms T, const double *__restrict__ x,
                                      const int *__restrict__ skip) {
  if (skip && *skip) return;
  const int q = blockIdx.y;
  const DevCSR &A = T.A[q];
  const int64_t e = (int64_t)blockIdx.x * BT + threadIdx.x;
  if (e >= A.n * kBW) return;
  const int64_t i = e / kBW;
  const int c = (int)(e % kBW);
  double acc = 0.0;
  for (int k = A.rowptr[i]; k < A.rowptr[i + 1]; k++)
    acc = fma(A.val[k], x[(int64_t)A.col[k] * kBW + c], acc);
  double v = T.c[q][c] * acc;
  if (T.wl[q]) v *= T.wl[q][e];
  T.out[q][e] = v;
}

__global__ void badjoint_kernel(BAdjointTerms T, int64_t n, const double *__restrict__ P,
                                const double *__restrict__ gtw, double sign_g,
                                double *__restrict__ r, const int *__restrict__ skip) {
  if (skip && *skip) return;
  const int64_t e = (int64_t)blockIdx.x * BT + threadIdx.x;
  if (e >= n * kBW) return;
  const int64_t j = e / kBW;
  const int c = (int)(e % kBW);
  double acc = gtw ? sign_g * gtw[e] : 0.0;
  for (int q = 0; q < T.count; q++) {
    const DevCSR &AT = T.AT[q];
    const double *wl = T.wl[q];
    const double *sv = T.s[q];
    double s = 0.0;
    for (int k = AT.rowptr[j]; k < AT.rowptr[j + 1]; k++) {
      const int64_t f = (int64_t)AT.col[k] * kBW + c;
      const double w = wl ? wl[f] : 1.0;
      s = fma(AT.val[k], w * sv[f], s);
    }
    acc = fma(T.c[q][c], s, acc);
  }
  r[e] = P ? P[e] * acc : acc;
}

// Sum over the ROWS row-lanes of a block for each column, fixed order.
__device__ __forceinline__ double column_sum(double v, double (*red)[kBW]) {
  const int rl = threadIdx.x / kBW, c = threadIdx.x % kBW;
  red[rl][c] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x < kBW) {
    for (int k = 0; k < ROWS; k++) s += red[k][c];
  }
  __syncthreads();
  return s;  // valid in threads 0..kBW-1 (column = threadIdx.x)
}

__global__ void bdot_partial_kernel(const double *__restrict__ a, const double *__restrict__ b,
                                    int64_t n, double *__restrict__ partial,
                                    const int *__restrict__ skip) {
  if (skip && *skip) return;
  __shared__ double red[ROWS][kBW];
  const int rl = threadIdx.x / kBW, c = threadIdx.x % kBW;
  double v = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * ROWS + rl; i < n; i += (int64_t)gridDim.x * ROWS) {
    const int64_t e = i * kBW + c;
    v = fma(a[e], b ? b[e] : a[e], v);
  }
  v = column_sum(v, red);
  if (threadIdx.x < kBW) partial[(int64_t)blockIdx.x * kBW + threadIdx.x] = v;
}

__global__ void bmisfit_partial_kernel(const double *__restrict__ g, const double *__restrict__ dobs,
                                       const double *__restrict__ wd, int64_t n,
                                       double *__restrict__ partial) {
  __shared__ double red[ROWS][kBW];
  const int rl = threadIdx.x / kBW, c = threadIdx.x % kBW;
  double v = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * ROWS + rl; i < n; i += (int64_t)gridDim.x * ROWS) {
    const double e = wd[i] * (g[i * kBW + c] - dobs[i]);
    v = fma(e, e, v);
  }
  v = column_sum(v, red);
  if (threadIdx.x < kBW) partial[(int64_t)blockIdx.x * kBW + threadIdx.x] = v;
}

// scal[c * CG_NSCALARS + slot] = sum over blocks of partial[b][c], blocks in order.
__global__ void bsum_partials_kernel(const double *__restrict__ partial, int nblocks,
                                     double *__restrict__ scal, int slot,
                                     const int *__restrict__ skip) {
  if (skip && *skip) return;
  __shared__ double red[ROWS][kBW];
  const int rl = threadIdx.x / kBW, c = threadIdx.x % kBW;
  double v = 0.0;
  for (int b = rl; b < nblocks; b += ROWS) v += partial[(int64_t)b * kBW + c];
  v = column_sum(v, red);
  if (threadIdx.x < kBW) scal[threadIdx.x * CG_NSCALARS + slot] = v;
}

__global__ void bdata_residual_kernel(const double *__restrict__ dobs, const double *__restrict__ g,
                                      const double *__restrict__ wd, int64_t n,
                                      double *__restrict__ b0, double *__restrict__ s0) {
  const int64_t e = (int64_t)blockIdx.x * BT + threadIdx.x;
  if (e >= n * kBW) return;
  const int64_t i = e / kBW;
  const double v = wd[i] * (dobs[i] - g[e]);
  b0[e] = v;
  if (s0) s0[e] = -v;
}

__global__ void bscale_rows_kernel(const double *__restrict__ a, const double *__restrict__ w,
                                   int64_t n, double *__restrict__ out) {
  const int64_t e = (int64_t)blockIdx.x * BT + threadIdx.x;
  if (e >= n * kBW) return;
  out[e] = w[e / kBW] * a[e];
}

__global__ void bp_update_kernel(const double *__restrict__ r, const double *__restrict__ P,
                                 const double *__restrict__ scal, int64_t n,
                                 double *__restrict__ p, double *__restrict__ pp,
                                 const int *__restrict__ skip) {
  if (skip && *skip) return;
  const int64_t e = (int64_t)blockIdx.x * BT + threadIdx.x;
  if (e >= n * kBW) return;
  const double beta = scal[(e % kBW) * CG_NSCALARS + CG_BETA];
  const double v = -r[e] + beta * p[e];
  p[e] = v;
  pp[e] = P[e] * v;
}

__global__ void baxpy_kernel(const double *__restrict__ t, const double *__restrict__ p,
                             const double *__restrict__ scal, int64_t nrow, int64_t n,
                             double *__restrict__ s, double *__restrict__ dx,
                             const int *__restrict__ skip) {
  if (skip && *skip) return;
  const int64_t e = (int64_t)blockIdx.x * BT + threadIdx.x;
  const double alpha = scal[(e % kBW) * CG_NSCALARS + CG_ALPHA];
  if (e < nrow * kBW) s[e] = fma(alpha, t[e], s[e]);
  if (e < n * kBW) dx[e] = fma(alpha, p[e], dx[e]);
}

// Per column: alpha = r2 / t2 (GaussNewtonInversion.cpp:1601); a stopped
// column gets alpha = 0.  One thread per column.
__global__ void balpha_kernel(double *scal, int *ctl) {
  __shared__ int done[kBW];
  const int c = threadIdx.x;
  double *sc = scal + c * CG_NSCALARS;
  int *cc = ctl + CTLB_COL + c * CTL_NINTS;
  if (ctl[CTLB_ALL]) return;  // uniform over the block
  if (cc[CTL_DONE]) {
    sc[CG_ALPHA] = 0.0;
  } else {
    const double t2 = sc[CG_T2];
    const double a = sc[CG_R2] / t2;
    if (t2 == 0.0 || !isfinite(a)) {
      cc[CTL_STATUS] = (t2 == 0.0) ? CG_STATUS_BREAKDOWN : CG_STATUS_NONFINITE;
      cc[CTL_DONE] = 1;
      sc[CG_ALPHA] = 0.0;
    } else {
      sc[CG_ALPHA] = a;
    }
  }
  done[c] = cc[CTL_DONE];
  __syncthreads();
  if (c == 0) {
    int all = 1;
    for (int k = 0; k < kBW; k++) all &= done[k];
    ctl[CTLB_ALL] = all;
  }
}

// Per column: beta and err = ||r||^2 / ||A^T b||^2 with the stopping test
// (:1674-1691).  The iteration counter of a column advances only while it runs.
__global__ void bbeta_kernel(double *scal, int *ctl) {
  __shared__ int done[kBW];
  const int c = threadIdx.x;
  double *sc = scal + c * CG_NSCALARS;
  int *cc = ctl + CTLB_COL + c * CTL_NINTS;
  if (ctl[CTLB_ALL]) return;
  if (!cc[CTL_DONE]) {
    const double rlast2 = sc[CG_R2];
    const double r2 = sc[CG_R2NEW];
    sc[CG_RLAST2] = rlast2;
    sc[CG_R2] = r2;
    sc[CG_BETA] = r2 / rlast2;
    const double err = r2 / sc[CG_ATB2];
    sc[CG_ERR] = err;
    const int it = ++cc[CTL_ITER];
    if (!isfinite(err)) {
      cc[CTL_STATUS] = CG_STATUS_NONFINITE;
      cc[CTL_DONE] = 1;
    } else if (err < sc[CG_TOL]) {
      cc[CTL_STATUS] = CG_STATUS_CONVERGED;
      cc[CTL_DONE] = 1;
    } else if (it >= cc[CTL_MAXIT]) {
      cc[CTL_DONE] = 1;
    }
  }
  done[c] = cc[CTL_DONE];
  __syncthreads();
  if (c == 0) {
    int all = 1;
    for (int k = 0; k < kBW; k++) all &= done[k];
    ctl[CTLB_ALL] = all;
  }
}

// Bound transform (GaussNewtonInversion.cpp:877-911) per element; guarded
// cells are fixed per column by a sequential pass, as in cg.cu.
__global__ void bbound_update_kernel(const double *__restrict__ m, const double *__restrict__ dx,
                                     const double *__restrict__ mmin,
                                     const double *__restrict__ mmax, int64_t n,
                                     double *__restrict__ mt, int *__restrict__ guard,
                                     int *__restrict__ any_guard) {
  const int64_t e = (int64_t)blockIdx.x * BT + threadIdx.x;
  if (e >= n * kBW) return;
  const int64_t i = e / kBW;
  const double temp = exp(dx[e]);
  const double mi = m[e];
  const double temp2 = mmin[i] * (mmax[i] - mi) + mmax[i] * (mi - mmin[i]) * temp;
  const double temp3 = (mmax[i] - mi) + (mi - mmin[i]) * temp;
  int g = 0;
  if (isinf(temp) || isinf(temp2)) g = 1;
  else if (fabs(temp3) < 1e-10) g = 2;
  guard[e] = g;
  if (g) atomicOr(any_guard + (e % kBW), 1);
  else mt[e] = temp2 / temp3;
}

__global__ void bbound_fixup_kernel(const int *__restrict__ guard, const int *__restrict__ any_guard,
                                    const double *__restrict__ mmin,
                                    const double *__restrict__ mmax,
                                    const double *__restrict__ mt_old, int64_t n,
                                    double *__restrict__ mt) {
  const int c = threadIdx.x;
  if (c >= kBW || !any_guard[c]) return;
  for (int64_t id = 0; id < n; id++) {
    const int64_t e = id * kBW + c;
    const int g = guard[e];
    if (!g) continue;
    double v;
    if (g == 1) v = (mmax[id] - 1e-6 + mt_old[e]) / 2.0;
    else v = (mmin[id] + 1e-6 + mt_old[e]) / 2.0;
    if (id == 0) v = 0.5 * (v + (n > 1 ? mt_old[kBW + c] : v));
    else v = 0.5 * (v + mt[e - kBW]);
    mt[e] = v;
  }
}

__global__ void bp_diag_kernel(const double *__restrict__ m, const double *__restrict__ mmin,
                               const double *__restrict__ mmax, int64_t n, double *__restrict__ P) {
  const int64_t e = (int64_t)blockIdx.x * BT + threadIdx.x;
  if (e >= n * kBW) return;
  const int64_t i = e / kBW;
  const double nn = 1.0;
  P[e] = nn * (mmax[i] - m[e]) * (m[e] - mmin[i]) / (mmax[i] - mmin[i]);
}

__global__ void bcopy_columns_kernel(const double *__restrict__ src, int64_t n, uint32_t mask,
                                     double *__restrict__ dst) {
  const int64_t e = (int64_t)blockIdx.x * BT + threadIdx.x;
  if (e >= n * kBW) return;
  if (mask & (1u << (e % kBW))) dst[e] = src[e];
}

__global__ void bpack_kernel(const double *__restrict__ cm, int64_t n, int ncol,
                             double *__restrict__ blk) {
  const int64_t e = (int64_t)blockIdx.x * BT + threadIdx.x;
  if (e >= n * kBW) return;
  const int64_t i = e / kBW;
  const int c = (int)(e % kBW);
  blk[e] = c < ncol ? cm[(int64_t)c * n + i] : 0.0;
}

__global__ void bunpack_kernel(const double *__restrict__ blk, int64_t n, int ncol,
                               double *__restrict__ cm) {
  const int64_t f = (int64_t)blockIdx.x * BT + threadIdx.x;  // column-major index
  if (f >= n * ncol) return;
  const int64_t c = f / n, i = f % n;
  cm[f] = blk[i * kBW + c];
}

}  // namespace

void launch_bcsr_apply(const DevCSR &A, const double *x, const double *xs, const double *c,
                       const double *wl, double *y, cudaStream_t s) {
  if (A.n <= 0) return;
  bcsr_apply_kernel<<<bblocks(A.n), BT, 0, s>>>(A, x, xs, c, wl, y);
  GRADA_LAUNCH_CHECK();
}

void launch_bmulti_forward(const BForwardTerms &T, int64_t n, const double *x, cudaStream_t s,
                           const int *skip) {
  if (T.count <= 0 || n <= 0) return;
  dim3 grid(bblocks(n), (unsigned)T.count);
  bmulti_forward_kernel<<<grid, BT, 0, s>>>(T, x, skip);
  GRADA_LAUNCH_CHECK();
}

void launch_badjoint(const BAdjointTerms &T, int64_t n, const double *P, const double *gtw,
                     double sign_g, double *r, cudaStream_t s, const int *skip) {
  if (n <= 0) return;
  badjoint_kernel<<<bblocks(n), BT, 0, s>>>(T, n, P, gtw, sign_g, r, skip);
  GRADA_LAUNCH_CHECK();
}

void launch_bdot(const double *a, const double *b, int64_t n, double *partial, int nblocks,
                 double *scal, int slot, cudaStream_t s, const int *skip) {
  bdot_partial_kernel<<<nblocks, BT, 0, s>>>(a, b, n, partial, skip);
  GRADA_LAUNCH_CHECK();
  bsum_partials_kernel<<<1, BT, 0, s>>>(partial, nblocks, scal, slot, skip);
  GRADA_LAUNCH_CHECK();
}

void launch_bmisfit_sq(const double *g, const double *dobs, const double *wd, int64_t n,
                       double *partial, int nblocks, double *scal, int slot, cudaStream_t s) {
  bmisfit_partial_kernel<<<nblocks, BT, 0, s>>>(g, dobs, wd, n, partial);
  GRADA_LAUNCH_CHECK();
  bsum_partials_kernel<<<1, BT, 0, s>>>(partial, nblocks, scal, slot, nullptr);
  GRADA_LAUNCH_CHECK();
}

void launch_bdata_residual(const double *dobs, const double *g, const double *wd, int64_t n,
                           double *b0, double *s0, cudaStream_t s) {
  bdata_residual_kernel<<<bblocks(n), BT, 0, s>>>(dobs, g, wd, n, b0, s0);
  GRADA_LAUNCH_CHECK();
}

void launch_bscale_rows(const double *a, const double *w, int64_t n, double *out, cudaStream_t s) {
  bscale_rows_kernel<<<bblocks(n), BT, 0, s>>>(a, w, n, out);
  GRADA_LAUNCH_CHECK();
}

void launch_bp_update(const double *r, const double *P, const double *scal, int64_t n, double *p,
                      double *pp, cudaStream_t s, const int *skip) {
  bp_update_kernel<<<bblocks(n), BT, 0, s>>>(r, P, scal, n, p, pp, skip);
  GRADA_LAUNCH_CHECK();
}

void launch_baxpy(const double *t, const double *p, const double *scal, int64_t nrow, int64_t n,
                  double *sv, double *dx, cudaStream_t s, const int *skip) {
  baxpy_kernel<<<bblocks(std::max(nrow, n)), BT, 0, s>>>(t, p, scal, nrow, n, sv, dx, skip);
  GRADA_LAUNCH_CHECK();
}

void launch_balpha(double *scal, int *ctl, cudaStream_t s) {
  balpha_kernel<<<1, kBW, 0, s>>>(scal, ctl);
  GRADA_LAUNCH_CHECK();
}

void launch_bbeta(double *scal, int *ctl, cudaStream_t s) {
  bbeta_kernel<<<1, kBW, 0, s>>>(scal, ctl);
  GRADA_LAUNCH_CHECK();
}

void launch_bbound_update(const double *m, const double *dx, const double *mmin,
                          const double *mmax, int64_t n, double *mt, const double *mt_old,
                          int *guard, int *any_guard, int *h_any_guard, cudaStream_t s) {
  GRADA_CUDA_CHECK(cudaMemsetAsync(any_guard, 0, sizeof(int) * kBW, s));
  bbound_update_kernel<<<bblocks(n), BT, 0, s>>>(m, dx, mmin, mmax, n, mt, guard, any_guard);
  GRADA_LAUNCH_CHECK();
  GRADA_CUDA_CHECK(
      cudaMemcpyAsync(h_any_guard, any_guard, sizeof(int) * kBW, cudaMemcpyDeviceToHost, s));
  GRADA_CUDA_CHECK(cudaStreamSynchronize(s));
  int any = 0;
  for (int c = 0; c < kBW; c++) any |= h_any_guard[c];
  if (any) {
    bbound_fixup_kernel<<<1, kBW, 0, s>>>(guard, any_guard, mmin, mmax, mt_old, n, mt);
    GRADA_LAUNCH_CHECK();
  }
}

void launch_bp_diag(const double *m, const double *mmin, const double *mmax, int64_t n, double *P,
                    cudaStream_t s) {
  bp_diag_kernel<<<bblocks(n), BT, 0, s>>>(m, mmin, mmax, n, P);
  GRADA_LAUNCH_CHECK();
}

void launch_bcopy_columns(const double *src, int64_t n, uint32_t mask, double *dst, cudaStream_t s) {
  bcopy_columns_kernel<<<bblocks(n), BT, 0, s>>>(src, n, mask, dst);
  GRADA_LAUNCH_CHECK();
}

void launch_bpack(const double *colmajor, int64_t n, int ncol, double *block, cudaStream_t s) {
  bpack_kernel<<<bblocks(n), BT, 0, s>>>(colmajor, n, ncol, block);
  GRADA_LAUNCH_CHECK();
}

void launch_bunpack(const double *block, int64_t n, int ncol, double *colmajor, cudaStream_t s) {
  const int64_t tot = n * ncol;
  bunpack_kernel<<<(unsigned)std::max<int64_t>(1, ceil_div(tot, BT)), BT, 0, s>>>(block, n, ncol,
                                                                                  colmajor);
  GRADA_LAUNCH_CHECK();
}

}  // namespace grada
