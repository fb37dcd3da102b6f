// K4-K7: the vector and sparse-operator kernels of the Gauss-Newton + CG
// inversion (src/Inversion/GaussNewtonInversion.cpp:657-1698).
//
// All arithmetic is FP64.  Reductions are deterministic: each dot product is
// a fixed grid of block partial sums followed by one block that adds the
// partials in order, so repeated runs give bit-identical scalars.  The
// sparse operators are the host-built regularisation matrices (CSR, <= 9
// entries per row on the reference's meshes); one thread owns one row.
#include "cg_body.cuh"
#include "cg_kernels.h"
#include "common.cuh"

namespace grada {

namespace {

using cgb::block_sum;
using cgb::VT;

// y = c * wl .* (A (x - xs))    (wl, xs optional)
__global__ void csr_apply_kernel(DevCSR A, const double *x, const double *xs, double c,
                                 const double *wl, double *y) {
  const int64_t i = (int64_t)blockIdx.x * VT + threadIdx.x;
  if (i >= A.n) return;
  y[i] = cgb::csr_apply_value(A, x, xs, c, wl, i);
}

// Forward regulariser rows for up to 7 terms in one launch (blockIdx.y = term).
__global__ void multi_forward_kernel(ForwardTerms T, const double *x,
                                     const int *__restrict__ skip) {
  if (skip && *skip) return;
  cgb::forward_term_body(T.t[blockIdx.y], x, blockIdx.x);
}

// r = P .* (sign_g * gtw + sum_t c_t A_t^T (wl_t .* s_t)), A_t^T given as CSR.
__global__ void adjoint_kernel(AdjointTerms T, int64_t n, const double *__restrict__ P,
                               const double *gtw, double sign_g, double *r,
                               const int *__restrict__ skip) {
  if (skip && *skip) return;
  const int64_t j = (int64_t)blockIdx.x * VT + threadIdx.x;
  if (j >= n) return;
  r[j] = cgb::adjoint_column(T, j, P, gtw != nullptr, gtw ? __ldcg(gtw + j) : 0.0, sign_g);
}

__global__ void dot_partial_kernel(const double *a, const double *b, int64_t n, double *partial,
                                   const int *__restrict__ skip) {
  if (skip && *skip) return;
  const double v = cgb::dot_partial_body(a, b, n, blockIdx.x, gridDim.x);
  if (threadIdx.x == 0) partial[blockIdx.x] = v;
}

__global__ void sum_partials_kernel(const double *partial, int nblocks, double *out,
                                    const int *__restrict__ skip) {
  if (skip && *skip) return;
  const double v = cgb::sum_partials_body(partial, nblocks);
  if (threadIdx.x == 0) *out = v;
}

// b0 = wd .* (dobs - g);  s0 = -b0
__global__ void data_residual_kernel(const double *__restrict__ dobs, const double *g,
                                     const double *__restrict__ wd, int64_t n, double *b0,
                                     double *s0) {
  const int64_t i = (int64_t)blockIdx.x * VT + threadIdx.x;
  if (i >= n) return;
  const double v = cgb::data_residual_value(dobs, g, wd, i);
  b0[i] = v;
  if (s0) s0[i] = -v;
}

__global__ void scale_kernel(const double *__restrict__ a, const double *__restrict__ w, int64_t n,
                             double c, double *__restrict__ out, const int *__restrict__ skip) {
  if (skip && *skip) return;
  const int64_t i = (int64_t)blockIdx.x * VT + threadIdx.x;
  if (i >= n) return;
  out[i] = c * (w ? w[i] * a[i] : a[i]);
}

__global__ void negate_kernel(const double *__restrict__ a, int64_t n, double *__restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * VT + threadIdx.x;
  if (i < n) out[i] = -a[i];
}

// p = -r + beta p ;  pp = P .* p
__global__ void p_update_kernel(const double *r, const double *__restrict__ P,
                                const double *__restrict__ scal, int64_t n, double *p, double *pp,
                                const int *__restrict__ skip) {
  if (skip && *skip) return;
  cgb::p_update_body(r, P, scal[CG_BETA], n, p, pp, blockIdx.x);
}

// s += alpha t (nrow) ;  dx += alpha p (n)
__global__ void axpy_kernel(const double *t, const double *p, const double *__restrict__ scal,
                            int64_t nrow, int64_t n, double *s, double *dx,
                            const int *__restrict__ skip) {
  if (skip && *skip) return;
  cgb::axpy_body(t, p, scal[CG_ALPHA], nrow, n, s, dx, blockIdx.x);
}

// ctl[CTL_DONE] != 0 turns every later kernel of the iteration (and of later
// iterations) into a no-op; ctl[CTL_STATUS] says why the solve stopped early.
__global__ void alpha_kernel(double *scal, int *ctl) {
  if (ctl && ctl[CTL_DONE]) return;
  // alpha = r2 / t2   (GaussNewtonInversion.cpp:1601)
  const double t2 = scal[CG_T2];
  const double a = scal[CG_R2] / t2;
  scal[CG_ALPHA] = a;
  if (ctl && (t2 == 0.0 || !isfinite(a))) {
    ctl[CTL_STATUS] = (t2 == 0.0) ? CG_STATUS_BREAKDOWN : CG_STATUS_NONFINITE;
    ctl[CTL_DONE] = 1;
  }
}

__global__ void beta_kernel(double *scal, int *ctl) {
  if (ctl && ctl[CTL_DONE]) return;
  // rlast2 = r2 ; r2 = ||r||^2 ; beta = r2/rlast2 ; err = r2/ATb2   (:1674-1684)
  const double rlast2 = scal[CG_R2];
  const double r2 = scal[CG_R2NEW];
  scal[CG_RLAST2] = rlast2;
  scal[CG_R2] = r2;
  scal[CG_BETA] = r2 / rlast2;
  const double err = r2 / scal[CG_ATB2];
  scal[CG_ERR] = err;
  if (ctl) {
    const int it = ++ctl[CTL_ITER];
    if (!isfinite(err)) {
      ctl[CTL_STATUS] = CG_STATUS_NONFINITE;
      ctl[CTL_DONE] = 1;
    } else if (err < scal[CG_TOL]) {  // iterations = i + 1 (:1685-1691)
      ctl[CTL_STATUS] = CG_STATUS_CONVERGED;
      ctl[CTL_DONE] = 1;
    } else if (it >= ctl[CTL_MAXIT]) {
      ctl[CTL_DONE] = 1;
    }
  }
}

// Bound transform, GaussNewtonInversion.cpp:877-911.  Cells that hit the
// infinity / zero-denominator guards are flagged; their values depend on a
// neighbour updated earlier in the same sweep and are fixed sequentially.
__global__ void bound_update_kernel(const double *m, const double *dx,
                                    const double *__restrict__ mmin, const double *__restrict__ mmax,
                                    int64_t n, double *mt, int *guard, int *any_guard) {
  const int64_t i = (int64_t)blockIdx.x * VT + threadIdx.x;
  if (i >= n) return;
  const int g = cgb::bound_update_cell(m, dx, mmin, mmax, mt, i);
  guard[i] = g;
  if (g) atomicOr(any_guard, 1);
}

// Sequential pass over guarded cells in index order (one thread).  mt_old is
// m_trial before this sweep (the id == 0 branch reads the not-yet-updated
// neighbour 1).
__global__ void bound_fixup_kernel(const int *guard, const double *__restrict__ mmin,
                                   const double *__restrict__ mmax, const double *mt_old, int64_t n,
                                   double *mt) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  cgb::bound_fixup_seq(guard, mmin, mmax, mt_old, n, mt);
}

// P_ii = (mmax - m)(m - mmin)/(mmax - mmin)   (GaussNewtonInversion.cpp:856-861)
__global__ void p_diag_kernel(const double *m, const double *__restrict__ mmin,
                              const double *__restrict__ mmax, int64_t n, double *P) {
  const int64_t i = (int64_t)blockIdx.x * VT + threadIdx.x;
  if (i >= n) return;
  P[i] = cgb::p_diag_value(m, mmin, mmax, i);
}

// WL_ii = (v_i^2 + eps2)^(-(2-p)/4)   (GaussNewtonInversion.cpp:962-1022)
__global__ void irls_weight_kernel(const double *v, int64_t n, double eps2, double expo,
                                   double *wl) {
  const int64_t i = (int64_t)blockIdx.x * VT + threadIdx.x;
  if (i >= n) return;
  wl[i] = cgb::irls_value(__ldcg(v + i), eps2, expo);
}

__global__ void sub_kernel(const double *__restrict__ a, const double *__restrict__ b, int64_t n,
                           double *__restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * VT + threadIdx.x;
  if (i < n) out[i] = a[i] - b[i];
}

__global__ void add_kernel(const double *__restrict__ a, const double *__restrict__ b, int64_t n,
                           double *__restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * VT + threadIdx.x;
  if (i < n) out[i] = a[i] + b[i];
}

// misfit partials: sum (wd (g - dobs))^2
__global__ void misfit_partial_kernel(const double *g, const double *__restrict__ dobs,
                                      const double *__restrict__ wd, int64_t n, double *partial) {
  const double v = cgb::misfit_partial_body(g, dobs, wd, n, blockIdx.x, gridDim.x);
  if (threadIdx.x == 0) partial[blockIdx.x] = v;
}

unsigned blocks_for(int64_t n) { return (unsigned)std::max<int64_t>(1, ceil_div(n, VT)); }

}  // namespace

int dot_blocks(int64_t n, int sm_count) {
  int64_t b = ceil_div(n, VT);
  const int64_t cap = (int64_t)sm_count * 4;
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return (int)b;
}

void launch_csr_apply(const DevCSR &A, const double *x, const double *xs, double c, const double *wl,
                      double *y, cudaStream_t s) {
  if (A.n <= 0) return;
  csr_apply_kernel<<<blocks_for(A.n), VT, 0, s>>>(A, x, xs, c, wl, y);
  GRADA_LAUNCH_CHECK();
}

void launch_multi_forward(const ForwardTerms &T, int64_t n, const double *x, cudaStream_t s,
                          const int *skip) {
  if (T.count <= 0 || n <= 0) return;
  dim3 grid(blocks_for(n), (unsigned)T.count);
  multi_forward_kernel<<<grid, VT, 0, s>>>(T, x, skip);
  GRADA_LAUNCH_CHECK();
}

void launch_adjoint(const AdjointTerms &T, int64_t n, const double *P, const double *gtw,
                    double sign_g, double *r, cudaStream_t s, const int *skip) {
  if (n <= 0) return;
  adjoint_kernel<<<blocks_for(n), VT, 0, s>>>(T, n, P, gtw, sign_g, r, skip);
  GRADA_LAUNCH_CHECK();
}

void launch_dot(const double *a, const double *b, int64_t n, double *partial, int nblocks,
                double *out, cudaStream_t s, const int *skip) {
  dot_partial_kernel<<<nblocks, VT, 0, s>>>(a, b, n, partial, skip);
  GRADA_LAUNCH_CHECK();
  sum_partials_kernel<<<1, VT, 0, s>>>(partial, nblocks, out, skip);
  GRADA_LAUNCH_CHECK();
}

void launch_misfit_sq(const double *g, const double *dobs, const double *wd, int64_t n,
                      double *partial, int nblocks, double *out, cudaStream_t s) {
  misfit_partial_kernel<<<nblocks, VT, 0, s>>>(g, dobs, wd, n, partial);
  GRADA_LAUNCH_CHECK();
  sum_partials_kernel<<<1, VT, 0, s>>>(partial, nblocks, out, nullptr);
  GRADA_LAUNCH_CHECK();
}

void launch_data_residual(const double *dobs, const double *g, const double *wd, int64_t n,
                          double *b0, double *s0, cudaStream_t s) {
  data_residual_kernel<<<blocks_for(n), VT, 0, s>>>(dobs, g, wd, n, b0, s0);
  GRADA_LAUNCH_CHECK();
}

void launch_scale(const double *a, const double *w, int64_t n, double c, double *out,
                  cudaStream_t s, const int *skip) {
  scale_kernel<<<blocks_for(n), VT, 0, s>>>(a, w, n, c, out, skip);
  GRADA_LAUNCH_CHECK();
}

void launch_negate(const double *a, int64_t n, double *out, cudaStream_t s) {
  negate_kernel<<<blocks_for(n), VT, 0, s>>>(a, n, out);
  GRADA_LAUNCH_CHECK();
}

void launch_p_update(const double *r, const double *P, const double *scal, int64_t n, double *p,
                     double *pp, cudaStream_t s, const int *skip) {
  p_update_kernel<<<blocks_for(n), VT, 0, s>>>(r, P, scal, n, p, pp, skip);
  GRADA_LAUNCH_CHECK();
}

void launch_axpy(const double *t, const double *p, const double *scal, int64_t nrow, int64_t n,
                 double *sv, double *dx, cudaStream_t s, const int *skip) {
  axpy_kernel<<<blocks_for(std::max(nrow, n)), VT, 0, s>>>(t, p, scal, nrow, n, sv, dx, skip);
  GRADA_LAUNCH_CHECK();
}

void launch_alpha(double *scal, int *ctl, cudaStream_t s) {
  alpha_kernel<<<1, 1, 0, s>>>(scal, ctl);
  GRADA_LAUNCH_CHECK();
}

void launch_beta(double *scal, int *ctl, cudaStream_t s) {
  beta_kernel<<<1, 1, 0, s>>>(scal, ctl);
  GRADA_LAUNCH_CHECK();
}

void launch_bound_update(const double *m, const double *dx, const double *mmin, const double *mmax,
                         int64_t n, double *mt, const double *mt_old, int *guard, int *any_guard,
                         int *h_any_guard, cudaStream_t s) {
  GRADA_CUDA_CHECK(cudaMemsetAsync(any_guard, 0, sizeof(int), s));
  bound_update_kernel<<<blocks_for(n), VT, 0, s>>>(m, dx, mmin, mmax, n, mt, guard, any_guard);
  GRADA_LAUNCH_CHECK();
  GRADA_CUDA_CHECK(cudaMemcpyAsync(h_any_guard, any_guard, sizeof(int), cudaMemcpyDeviceToHost, s));
  GRADA_CUDA_CHECK(cudaStreamSynchronize(s));
  if (*h_any_guard) {
    bound_fixup_kernel<<<1, 1, 0, s>>>(guard, mmin, mmax, mt_old, n, mt);
    GRADA_LAUNCH_CHECK();
  }
}

void launch_p_diag(const double *m, const double *mmin, const double *mmax, int64_t n, double *P,
                   cudaStream_t s) {
  p_diag_kernel<<<blocks_for(n), VT, 0, s>>>(m, mmin, mmax, n, P);
  GRADA_LAUNCH_CHECK();
}

void launch_irls_weight(const double *v, int64_t n, double eps2, double expo, double *wl,
                        cudaStream_t s) {
  irls_weight_kernel<<<blocks_for(n), VT, 0, s>>>(v, n, eps2, expo, wl);
  GRADA_LAUNCH_CHECK();
}

void launch_sub(const double *a, const double *b, int64_t n, double *out, cudaStream_t s) {
  sub_kernel<<<blocks_for(n), VT, 0, s>>>(a, b, n, out);
  GRADA_LAUNCH_CHECK();
}

void launch_add(const double *a, const double *b, int64_t n, double *out, cudaStream_t s) {
  add_kernel<<<blocks_for(n), VT, 0, s>>>(a, b, n, out);
  GRADA_LAUNCH_CHECK();
}

}  // namespace grada
