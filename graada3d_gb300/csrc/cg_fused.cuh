// The persistent CG loop (one solve's CGLS iterations run by a team of
// co-resident CTAs with bounded barriers) and its building blocks, shared by
// the single-solve kernel (cg_fused.cu) and the batched inversion kernel
// (invert_batch.cu).  See cg_fused.cu for the phases.
#pragma once

#include "cg_body.cuh"
#include "cg_fused.h"
#include "common.cuh"
#include "gemv_body.cuh"

namespace grada {

namespace fused {

__device__ __forceinline__ unsigned long long global_timer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ unsigned ld_relaxed_u32(const unsigned *p) {
  unsigned v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Barrier over the n CTAs of a team.  word[0] counts arrivals (it only grows:
// barrier k of a launch completes at n * k), word[1] is the error word.  Both
// start at zero (the host clears them before the launch).
struct TeamBarrier {
  unsigned *word;
  unsigned n;
  unsigned target;
  unsigned long long limit_ns;

  __device__ bool sync() {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
      target += n;
      int ok = 1;
      __threadfence();
      atomicAdd(word, 1u);
      const unsigned long long t0 = global_timer_ns();
      while ((int)(ld_acquire_u32(word) - target) < 0) {
        if (ld_relaxed_u32(word + 1)) {
          ok = 0;
          break;
        }
        if (global_timer_ns() - t0 > limit_ns) {
          atomicExch(word + 1, 1u);
          ok = 0;
          break;
        }
        __nanosleep(32);
      }
      __threadfence();
      if (ld_relaxed_u32(word + 1)) ok = 0;
      s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
  }
};

// Broadcast thread 0's value to the block.
__device__ __forceinline__ double bcast(double v) {
  __shared__ double s_v;
  if (threadIdx.x == 0) s_v = v;
  __syncthreads();
  const double out = s_v;
  __syncthreads();
  return out;
}

// Scalars a solve's loop starts from (the setup's) and ends with.
struct CgIn {
  double R2 = 0.0, ATB2 = 0.0, tol = 0.0, rlast2 = 0.0, err = 0.0;
  int maxit = 0;
};
struct CgOut {
  double R2 = 0.0, T2 = 0.0, alpha = 0.0, beta = 0.0, rlast2 = 0.0, err = 0.0;
  int iterations = 0, status = CG_STATUS_RUNNING;
  bool ok = true;  // false: a barrier wait expired (the team abandons its work)
};

// The loop of one solve, run by CTA `cta` of the nct CTAs of its team, from
// r (set up), p = dx = 0 and beta = 0.  Every CTA returns the same CgOut.
template <class L>
__device__ CgOut cg_loop(const FusedCgArgs &a, const CgIn &in, unsigned cta, unsigned nct,
                         TeamBarrier &bar) {
  using Acc = typename L::Acc;
  const int64_t Nm = a.nm, nd = a.nd, ld = a.ld, nrow = a.nrow;
  const int64_t nb_vec = ceil_div_d(Nm, cgb::VT);  // blocks of an Nm-long vector kernel
  const int64_t nb_fin = ceil_div_d(nd, 256);
  const int64_t nb_axpy = ceil_div_d(nrow > Nm ? nrow : Nm, cgb::VT);
  const int64_t nb_prep = ceil_div_d(ld, 256);
  const int64_t nb_gt = ceil_div_d(Nm, gemv::kGtCols);
  const int64_t n_gx = (int64_t)a.tiles * a.splits;
  const int64_t n_g2 = nb_fin + (int64_t)a.FT.count * nb_vec;
  Acc *y = reinterpret_cast<Acc *>(a.scratch);

  CgOut o;
  double R2 = in.R2, beta = 0.0, rlast2 = in.rlast2, err = in.err;
  double T2 = 0.0, alpha = 0.0;
  const double ATB2 = in.ATB2, tol = in.tol;
  int it = 0;
  const int maxit = in.maxit;
  int status = CG_STATUS_RUNNING;
  bool ok = true;
  while (true) {
    // P
    for (int64_t b = cta; b < nb_vec; b += nct) cgb::p_update_body(a.r, a.P, beta, Nm, a.p, a.pp, b);
    if (!(ok = bar.sync())) break;
    // G1
    for (int64_t b = cta; b < n_gx; b += nct)
      gemv::gx_partial_body<L>(a.G, ld, Nm, a.per, a.pp, a.scratch, b % a.tiles, b / a.tiles);
    if (!(ok = bar.sync())) break;
    // G2
    for (int64_t b = cta; b < n_g2; b += nct) {
      if (b < nb_fin) {
        gemv::gx_finish_body(a.scratch, a.splits, ld, nd, a.row_scale, a.wd, a.t, b);
      } else {
        const int64_t k = b - nb_fin;
        cgb::forward_term_body(a.FT.t[k / nb_vec], a.pp, k % nb_vec);
      }
    }
    if (!(ok = bar.sync())) break;
    // D1
    for (int64_t b = cta; b < a.nb_row; b += nct) {
      const double v = cgb::dot_partial_body(a.t, nullptr, nrow, b, a.nb_row);
      if (threadIdx.x == 0) a.part[b] = v;
    }
    if (!(ok = bar.sync())) break;
    T2 = bcast(cgb::sum_partials_body(a.part, a.nb_row));
    alpha = R2 / T2;  // GaussNewtonInversion.cpp:1601
    if (T2 == 0.0 || !isfinite(alpha)) {
      status = (T2 == 0.0) ? CG_STATUS_BREAKDOWN : CG_STATUS_NONFINITE;
      break;
    }
    // S
    for (int64_t b = cta; b < nb_axpy; b += nct) {
      cgb::axpy_body(a.t, a.p, alpha, nrow, Nm, a.s, a.dx, b);
      if (b < nb_prep) gemv::prep_y_body<Acc>(a.s, nd, ld, a.row_scale, a.wd, y, b);
    }
    if (!(ok = bar.sync())) break;
    // GT
    for (int64_t b = cta; b < nb_gt; b += nct) {
      int ncol = 0;
      const double g = gemv::gty_body<L>(a.G, ld, Nm, y, b, &ncol);
      if ((int)threadIdx.x < ncol) {
        const int64_t j = b * gemv::kGtCols + threadIdx.x;
        a.gtw[j] = g;
        a.r[j] = cgb::adjoint_column(a.AT, j, a.P, true, g, 1.0);
      }
    }
    if (!(ok = bar.sync())) break;
    // D2
    for (int64_t b = cta; b < a.nb_m; b += nct) {
      const double v = cgb::dot_partial_body(a.r, nullptr, Nm, b, a.nb_m);
      if (threadIdx.x == 0) a.part[b] = v;
    }
    if (!(ok = bar.sync())) break;
    const double r2 = bcast(cgb::sum_partials_body(a.part, a.nb_m));
    // :1674-1691
    rlast2 = R2;
    R2 = r2;
    beta = r2 / rlast2;
    err = r2 / ATB2;
    it++;
    if (!isfinite(err)) {
      status = CG_STATUS_NONFINITE;
      break;
    }
    if (err < tol) {
      status = CG_STATUS_CONVERGED;
      break;
    }
    if (it >= maxit) break;
  }
  o.R2 = R2;
  o.T2 = T2;
  o.alpha = alpha;
  o.beta = beta;
  o.rlast2 = rlast2;
  o.err = err;
  o.iterations = it;
  o.status = status;
  o.ok = ok;
  return o;
}

}  // namespace fused
}  // namespace grada
