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

// Broadcast thread 0's value to the block.
__device__ __forceinline__ double bcast(double v) {
  __shared__ double s_v;
  if (threadIdx.x == 0) s_v = v;
  __syncthreads();
  const double out = s_v;
  __syncthreads();
  return out;
}

// Block sum (fixed tree) broadcast to every thread.
__device__ __forceinline__ double bcast_sum(double v) { return bcast(cgb::block_sum(v)); }

__device__ __forceinline__ void st_release_u32(unsigned *p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Barrier over the n CTAs of a team, a two-level arrival tree: CTA c arrives
// on counter c % G (G = min(16, n) counters, 32 bytes apart), the last arrival
// of each counter arrives on the top counter, and the last top arrival
// publishes the barrier's number on the release word, which every CTA polls.
// Counters only grow (barrier k completes when counter g reaches size_g * k),
// so nothing is reset.  The team's words (kBarrierWords, zeroed before the
// launch): counters at 8 g, top at 160, release at 192, error at 224.  A wait
// longer than limit_ns raises the error word; every CTA then leaves at its
// next barrier.
constexpr int kBarrierWords = 256;

struct TeamBarrier {
  unsigned *word;
  unsigned n;
  unsigned cta;
  unsigned long long limit_ns;
  unsigned epoch = 0;

  __device__ TeamBarrier(unsigned *w, unsigned n_ctas, unsigned my_cta, unsigned long long limit)
      : word(w), n(n_ctas), cta(my_cta), limit_ns(limit) {}

  __device__ bool sync() {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
      const unsigned groups = n < 16u ? n : 16u;
      const unsigned g = cta % groups;
      const unsigned gsize = n / groups + (g < n % groups ? 1u : 0u);
      epoch++;
      int ok = 1;
      __threadfence();
      if (atomicAdd(word + 8 * g, 1u) + 1u == gsize * epoch) {
        __threadfence();
        if (atomicAdd(word + 160, 1u) + 1u == groups * epoch) {
          __threadfence();
          st_release_u32(word + 192, epoch);
        }
      }
      const unsigned long long t0 = global_timer_ns();
      while ((int)(ld_acquire_u32(word + 192) - epoch) < 0) {
        if (ld_relaxed_u32(word + 224)) {
          ok = 0;
          break;
        }
        if (global_timer_ns() - t0 > limit_ns) {
          atomicExch(word + 224, 1u);
          ok = 0;
          break;
        }
        __nanosleep(20);
      }
      __threadfence();
      if (ld_relaxed_u32(word + 224)) ok = 0;
      s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
  }
};

// Sum of the n per-block partials in index order (each thread a fixed stride,
// then the block's fixed tree); every thread of every CTA gets the same value.
__device__ __forceinline__ double sum_partials_all(const double *partial, int64_t n) {
  double v = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += cgb::VT) v += __ldcg(partial + i);
  return bcast_sum(v);
}

// Rows per finish block of the persistent loop.
constexpr int kFinRows = 16;

// G pp's rows r0 .. r0 + 15 (block b): the 16 half-warps each add the split
// partials k = g, g + 16, ... (g = 2 warp + half) of the 16 rows, loads eight
// deep, and the 16 sums are added in g order; times the row scale and Wd.
// Returns t_r^2 for the block's rows, summed (valid in every thread).
__device__ __forceinline__ double finish_rows(const double *partial, int n_split, int64_t ld,
                                             int64_t nd, const float *__restrict__ row_scale,
                                             const double *__restrict__ wd, double *t,
                                             int64_t b) {
  constexpr int kGroups = 2 * (cgb::VT / 32);
  __shared__ double part[kGroups][kFinRows];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int row_in = lane & (kFinRows - 1), g = 2 * warp + (lane >> 4);
  const int64_t r = b * kFinRows + row_in;
  double s = 0.0;
  if (r < nd) {
#pragma unroll 8
    for (int k = g; k < n_split; k += kGroups) s += __ldcg(partial + (int64_t)k * ld + r);
  }
  __syncthreads();
  part[g][row_in] = s;
  __syncthreads();
  double sq = 0.0;
  if (threadIdx.x < kFinRows) {
    const int64_t rr = b * kFinRows + threadIdx.x;
    double v = 0.0;
#pragma unroll
    for (int w = 0; w < kGroups; w++) v += part[w][threadIdx.x];
    if (rr < nd) {
      if (row_scale) v *= (double)row_scale[rr];
      v *= wd[rr];
      t[rr] = v;
      sq = v * v;
    }
  }
  return bcast_sum(sq);
}

// G^T y for the 32 columns of block b (warp w takes columns 4w .. 4w + 3,
// lanes striding the rows), then r_j for those columns (the adjoint of the
// regulariser rows and P), y staged in shared memory (gemv::gty_body; read
// from L2 by every warp instead, the same sums took 70 against 47 us for FP32
// and 103 against 29 us for bf16 at 3,392 x 16,384).  The regulariser terms of the warp's 4 columns run on one lane per
// (column, term), their dependent CSR loads in parallel; the lane holding a
// column adds them to its G^T sum in term order (cgb::adjoint_column's
// arithmetic).  Writes gtw and r; returns the block's sum of r_j^2 (valid in
// every thread).
template <class L, int U = gemv::kGtUnroll>
__device__ __forceinline__ double gty_adjoint_block(const FusedCgArgs &a, const typename L::Acc *y,
                                                    int64_t b) {
  static_assert(gemv::kGtWarpCols * 8 <= 32, "one lane per (column, term)");
  __shared__ double wsum[cgb::VT / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int64_t j = -1;
  const double g = gemv::gty_body<L, U>(a.G, a.ld, a.nm, y, b, &j);
  // lane 8c + q: term q of the warp's column c
  const int tc = lane >> 3, tq = lane & 7;
  const int64_t tj = b * gemv::kGtBlockCols + (int64_t)warp * gemv::kGtWarpCols + tc;
  double ts = 0.0;
  if (tc < gemv::kGtWarpCols && tq < a.AT.count && tj < a.nm) {
    const AdjointTerm &t = a.AT.t[tq];
    for (int k = t.AT.rowptr[tj]; k < t.AT.rowptr[tj + 1]; k++) {
      const int i = t.AT.col[k];
      const double w = t.wl ? t.wl[i] : 1.0;
      ts = fma(t.AT.val[k], w * __ldcg(t.s + i), ts);
    }
  }
  double acc = g;  // lanes c < 4: P_j (gtw_j + sum_q c_q s_q), terms in order
  for (int q = 0; q < a.AT.count; q++) {
    const double sq_term = __shfl_sync(0xffffffffu, ts, (lane & 3) * 8 + q);
    acc = fma(a.AT.t[q].c, sq_term, acc);
  }
  double sq = 0.0;
  if (j >= 0) {
    a.gtw[j] = g;
    const double rj = a.P ? a.P[j] * acc : acc;
    a.r[j] = rj;
    sq = rj * rj;
  }
  sq = cgb::warp_sum(sq);
  __syncthreads();
  if (lane == 0) wsum[warp] = sq;
  __syncthreads();
  double tot = 0.0;
#pragma unroll
  for (int w = 0; w < cgb::VT / 32; w++) tot += wsum[w];
  return tot;
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

// Layout of a.red for a loop: per-block partials of ||t||^2 over the finish
// and forward-row blocks, then of ||r||^2 over the G^T blocks.
struct RedLayout {
  int64_t nb_fin, nb_t, nb_r;
  __host__ __device__ RedLayout(int64_t nd, int64_t nm, int nterms) {
    nb_fin = ceil_div_d(nd, kFinRows);
    nb_t = nb_fin + (int64_t)nterms * ceil_div_d(nm, 256);
    nb_r = ceil_div_d(nm, gemv::kGtBlockCols);
  }
  __host__ __device__ int64_t doubles() const { return nb_t + nb_r; }
  __host__ __device__ int64_t counters() const { return 1; }
};

// The loop of one solve, run by CTA `cta` of the nct CTAs of its team, from
// r (set up), p = dx = 0 and beta = 0.  Every CTA returns the same CgOut.
// Four team barriers per iteration:
//   A  p_new = -r + beta p_old and pp = P p_new folded into the partial row
//      sums of G pp (row tiles of 64 VEC rows x column ranges, the block's
//      four warp pairs splitting a range)
//   B  t_data = Wd (sum of the partials, 16 rows per block, the splits shared
//      by 16 half-warps), the forward regulariser rows of t, per-block ||t||^2
//   C  alpha = r2 / t2; s += alpha t, dx += alpha p_new, y = Wd s_data in G's
//      accumulation type
//   D  G^T y for 32 columns per block (4 per warp), r for those columns (the
//      adjoint of the regulariser rows, P), per-block ||r||^2; then beta, err
//      and the stopping test
// Every CTA adds the per-block partials in index order, so the sums do not
// depend on the team size or on which CTA ran which block.
template <class L>
__device__ CgOut cg_loop(const FusedCgArgs &a, const CgIn &in, unsigned cta, unsigned nct,
                         TeamBarrier &bar) {
  using Acc = typename L::Acc;
  const int64_t Nm = a.nm, nd = a.nd, ld = a.ld, nrow = a.nrow;
  const int64_t nb_vec = ceil_div_d(Nm, cgb::VT);  // blocks of an Nm-long vector
  const int64_t nb_axpy = ceil_div_d(nrow > Nm ? nrow : Nm, cgb::VT);
  const int64_t nb_prep = ceil_div_d(ld, 256);
  const int64_t n_gx = (int64_t)a.tiles * a.splits;
  const RedLayout rl(nd, Nm, a.FT.count);
  double *part_t = a.red, *part_r = a.red + rl.nb_t;
  Acc *y = reinterpret_cast<Acc *>(a.scratch);

  CgOut o;
  double R2 = in.R2, beta = 0.0, rlast2 = in.rlast2, err = in.err;
  double T2 = 0.0, alpha = 0.0;
  const double ATB2 = in.ATB2, tol = in.tol;
  int it = 0;
  const int maxit = in.maxit;
  int status = CG_STATUS_RUNNING;
  bool ok = true;
  // phase trace: CTA 0's thread 0 sums the spans in shared memory (no
  // registers held across the loop but the last stamp)
  __shared__ unsigned long long s_span[4];
  const bool tracing = a.trace && cta == 0 && threadIdx.x == 0;
  unsigned long long t_last = 0;
  if (tracing) {
    for (int q = 0; q < 4; q++) s_span[q] = 0;
    t_last = global_timer_ns();
  }
  auto stamp = [&](int phase) {
    if (tracing) {
      const unsigned long long t = global_timer_ns();
      s_span[phase] += t - t_last;
      t_last = t;
    }
  };
  while (true) {
    double *p_old = (it & 1) ? a.p2 : a.p;
    double *p_new = (it & 1) ? a.p : a.p2;
    // A
    for (int64_t b = cta; b < n_gx; b += nct)
      gemv::gx_partial_fold_body<L>(a.G, ld, Nm, a.per, a.r, p_old, a.P, beta, p_new, a.pp,
                                    a.scratch, b % a.tiles, b / a.tiles);
    if (!(ok = bar.sync())) break;
    stamp(0);
    // B
    for (int64_t b = cta; b < rl.nb_t; b += nct) {
      double v;
      if (b < rl.nb_fin) {
        v = finish_rows(a.scratch, a.splits, ld, nd, a.row_scale, a.wd, a.t, b);
      } else {
        const int64_t k = b - rl.nb_fin;
        const ForwardTerm &ft = a.FT.t[k / nb_vec];
        cgb::forward_term_body(ft, a.pp, k % nb_vec);
        const int64_t i = (k % nb_vec) * cgb::VT + threadIdx.x;
        double q = 0.0;
        if (i < Nm) {
          const double tv = __ldcg(ft.out + i);
          q = tv * tv;
        }
        v = bcast_sum(q);
      }
      if (threadIdx.x == 0) part_t[b] = v;
    }
    if (!(ok = bar.sync())) break;
    stamp(1);
    // C
    T2 = sum_partials_all(part_t, rl.nb_t);
    alpha = R2 / T2;  // GaussNewtonInversion.cpp:1601
    if (T2 == 0.0 || !isfinite(alpha)) {
      status = (T2 == 0.0) ? CG_STATUS_BREAKDOWN : CG_STATUS_NONFINITE;
      break;
    }
    for (int64_t b = cta; b < nb_axpy; b += nct) {
      cgb::axpy_body(a.t, p_new, alpha, nrow, Nm, a.s, a.dx, b);
      if (b < nb_prep) gemv::prep_y_body<Acc>(a.s, nd, ld, a.row_scale, a.wd, y, b);
    }
    if (!(ok = bar.sync())) break;
    stamp(2);
    // D
    for (int64_t b = cta; b < rl.nb_r; b += nct) {
      const double v = gty_adjoint_block<L>(a, y, b);
      if (threadIdx.x == 0) part_r[b] = v;
    }
    if (!(ok = bar.sync())) break;
    stamp(3);
    const double r2 = sum_partials_all(part_r, rl.nb_r);
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
  if (tracing) {
    for (int q = 0; q < 4; q++) a.trace[q] += s_span[q];
    a.trace[4] += (unsigned long long)it;
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
