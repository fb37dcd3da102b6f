// Per-block bodies of the CG iteration's vector and sparse-operator kernels
// (cg.cu), shared by those kernels and the persistent CG kernel
// (cg_fused.cu).  A body takes its block index as an argument, so the
// persistent kernel runs the same blocks with the same arithmetic and
// summation order: bitwise the results of the stand-alone kernels.
//
// Reference: GaussNewtonInversion::solve_cg
// (src/Inversion/GaussNewtonInversion.cpp:1556-1692).  Vectors rewritten
// within a solve (r, p, pp, s, t, dx and the partial sums) are read with
// ld.global.cg; the operators, weights and P are fixed during a solve.
#pragma once

#include <stdint.h>

#include "cg_kernels.h"

namespace grada {
namespace cgb {

constexpr int VT = 256;  // threads per block of every vector kernel

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sum over the block, in a fixed tree; valid in thread 0.
__device__ __forceinline__ double block_sum(double v) {
  __shared__ double red[VT / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  v = warp_sum(v);
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double s = 0.0;
  if (warp == 0) {
    s = (lane < VT / 32) ? red[lane] : 0.0;
    s = warp_sum(s);
  }
  __syncthreads();
  return s;
}

// p = -r + beta p ;  pp = P .* p   (block b of 256 entries)
__device__ __forceinline__ void p_update_body(const double *r, const double *__restrict__ P,
                                              double beta, int64_t n, double *p, double *pp,
                                              int64_t b) {
  const int64_t i = b * VT + threadIdx.x;
  if (i >= n) return;
  const double v = -__ldcg(r + i) + beta * __ldcg(p + i);
  p[i] = v;
  pp[i] = P[i] * v;
}

// Forward regulariser rows of one term: out = c * wl .* (A x)   (block b)
__device__ __forceinline__ void forward_term_body(const ForwardTerm &t, const double *x,
                                                  int64_t b) {
  const int64_t i = b * VT + threadIdx.x;
  if (i >= t.A.n) return;
  double acc = 0.0;
  for (int k = t.A.rowptr[i]; k < t.A.rowptr[i + 1]; k++)
    acc = fma(t.A.val[k], __ldcg(x + t.A.col[k]), acc);
  double v = t.c * acc;
  if (t.wl) v *= t.wl[i];
  t.out[i] = v;
}

// Column j of the adjoint: P_j (sign_g gtw_j + sum_t c_t (A_t^T (wl_t .* s_t))_j)
// with A_t^T given as CSR; gtw_j passed in.
__device__ __forceinline__ double adjoint_column(const AdjointTerms &T, int64_t j,
                                                 const double *__restrict__ P, bool has_g,
                                                 double gtw_j, double sign_g) {
  double acc = has_g ? sign_g * gtw_j : 0.0;
  for (int q = 0; q < T.count; q++) {
    const AdjointTerm &t = T.t[q];
    double s = 0.0;
    for (int k = t.AT.rowptr[j]; k < t.AT.rowptr[j + 1]; k++) {
      const int i = t.AT.col[k];
      const double w = t.wl ? t.wl[i] : 1.0;
      s = fma(t.AT.val[k], w * __ldcg(t.s + i), s);
    }
    acc = fma(t.c, s, acc);
  }
  return P ? P[j] * acc : acc;
}

// Block b's partial of sum a_i b_i (b null: a_i^2), grid-stride over nb blocks;
// valid in thread 0.
__device__ __forceinline__ double dot_partial_body(const double *a, const double *bv, int64_t n,
                                                   int64_t b, int64_t nb) {
  double v = 0.0;
  for (int64_t i = b * VT + threadIdx.x; i < n; i += nb * VT) {
    const double x = __ldcg(a + i);
    v = fma(x, bv ? __ldcg(bv + i) : x, v);
  }
  return block_sum(v);
}

// Sum of nblocks partials in a fixed order; valid in thread 0.
__device__ __forceinline__ double sum_partials_body(const double *partial, int nblocks) {
  double v = 0.0;
  for (int i = threadIdx.x; i < nblocks; i += VT) v += __ldcg(partial + i);
  return block_sum(v);
}

// s += alpha t (nrow) ;  dx += alpha p (n)   (block b)
__device__ __forceinline__ void axpy_body(const double *t, const double *p, double alpha,
                                          int64_t nrow, int64_t n, double *s, double *dx,
                                          int64_t b) {
  const int64_t i = b * VT + threadIdx.x;
  if (i < nrow) s[i] = fma(alpha, __ldcg(t + i), __ldcg(s + i));
  if (i < n) dx[i] = fma(alpha, __ldcg(p + i), __ldcg(dx + i));
}


// y = c * wl .* (A (x - xs))  (wl, xs optional), block b of rows
__device__ __forceinline__ double csr_row(const DevCSR &A, const double *x, const double *xs,
                                          int64_t i) {
  double acc = 0.0;
  for (int k = A.rowptr[i]; k < A.rowptr[i + 1]; k++) {
    const int j = A.col[k];
    const double xv = xs ? (__ldcg(x + j) - __ldcg(xs + j)) : __ldcg(x + j);
    acc = fma(A.val[k], xv, acc);
  }
  return acc;
}

__device__ __forceinline__ double csr_apply_value(const DevCSR &A, const double *x,
                                                  const double *xs, double c,
                                                  const double *wl, int64_t i) {
  double v = c * csr_row(A, x, xs, i);
  if (wl) v *= __ldcg(wl + i);
  return v;
}

// b0 = wd .* (dobs - g) ; s0 = -b0 (s0 optional)
__device__ __forceinline__ double data_residual_value(const double *__restrict__ dobs,
                                                      const double *g,
                                                      const double *__restrict__ wd, int64_t i) {
  return wd[i] * (dobs[i] - __ldcg(g + i));
}

// misfit partial of block b over nb blocks: sum (wd (g - dobs))^2; valid in thread 0
__device__ __forceinline__ double misfit_partial_body(const double *g,
                                                      const double *__restrict__ dobs,
                                                      const double *__restrict__ wd, int64_t n,
                                                      int64_t b, int64_t nb) {
  double v = 0.0;
  for (int64_t i = b * VT + threadIdx.x; i < n; i += nb * VT) {
    const double e = wd[i] * (__ldcg(g + i) - dobs[i]);
    v = fma(e, e, v);
  }
  return block_sum(v);
}

// Bound transform of one cell (GaussNewtonInversion.cpp:877-911): writes mt[i]
// unless a guard applies; returns the guard (0 none, 1 infinity, 2 zero
// denominator).
__device__ __forceinline__ int bound_update_cell(const double *m, const double *dx,
                                                 const double *__restrict__ mmin,
                                                 const double *__restrict__ mmax, double *mt,
                                                 int64_t i) {
  const double mi = __ldcg(m + i);
  const double temp = exp(__ldcg(dx + i));
  const double temp2 = mmin[i] * (mmax[i] - mi) + mmax[i] * (mi - mmin[i]) * temp;
  const double temp3 = (mmax[i] - mi) + (mi - mmin[i]) * temp;
  int g = 0;
  if (isinf(temp) || isinf(temp2)) g = 1;
  else if (fabs(temp3) < 1e-10) g = 2;
  if (!g) mt[i] = temp2 / temp3;
  return g;
}

// The guarded cells in index order, one thread: their values depend on a
// neighbour updated earlier in the same sweep.  mt_old is m_trial before the
// sweep (the id == 0 branch reads the not-yet-updated neighbour 1).
__device__ __forceinline__ void bound_fixup_seq(const int *guard, const double *__restrict__ mmin,
                                                const double *__restrict__ mmax,
                                                const double *mt_old, int64_t n, double *mt) {
  for (int64_t id = 0; id < n; id++) {
    const int g = __ldcg(guard + id);
    if (!g) continue;
    double v;
    if (g == 1) v = (mmax[id] - 1e-6 + __ldcg(mt_old + id)) / 2.0;
    else v = (mmin[id] + 1e-6 + __ldcg(mt_old + id)) / 2.0;
    if (id == 0) {
      v = 0.5 * (v + (n > 1 ? __ldcg(mt_old + 1) : v));
    } else {
      v = 0.5 * (v + __ldcg(mt + id - 1));
    }
    mt[id] = v;
  }
}

// P_ii = (mmax - m)(m - mmin)/(mmax - mmin)   (GaussNewtonInversion.cpp:856-861)
__device__ __forceinline__ double p_diag_value(const double *m, const double *__restrict__ mmin,
                                               const double *__restrict__ mmax, int64_t i) {
  const double nn = 1.0;
  const double mi = __ldcg(m + i);
  return nn * (mmax[i] - mi) * (mi - mmin[i]) / (mmax[i] - mmin[i]);
}

// WL_ii = (v_i^2 + eps2)^(-(2-p)/4)   (GaussNewtonInversion.cpp:962-1022)
__device__ __forceinline__ double irls_value(double v, double eps2, double expo) {
  return pow(v * v + eps2, expo);
}

}  // namespace cgb
}  // namespace grada
