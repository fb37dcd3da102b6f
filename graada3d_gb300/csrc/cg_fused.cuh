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

// Forward regulariser row block k of phase A: term k / nb_vec, rows
// (k % nb_vec) * VT + thread: t_out = c (A pp) (x wl), with pp_j computed from
// r, p_old and beta by gemv::cg_direction (the bits G pp's staging uses), so
// the rows need no stored pp.  Returns the block's sum of t^2 (every thread).
__device__ __forceinline__ double forward_rows_block(const FusedCgArgs &a, const double *p_old,
                                                     double beta, int64_t k, int64_t nb_vec) {
  const ForwardTerm &t = a.FT.t[k / nb_vec];
  const int64_t i = (k % nb_vec) * cgb::VT + threadIdx.x;
  double q = 0.0;
  if (i < t.A.n) {
    double acc = 0.0;
    for (int e = t.A.rowptr[i]; e < t.A.rowptr[i + 1]; e++)
      acc = fma(t.A.val[e], gemv::cg_direction(a.r, p_old, a.P, beta, t.A.col[e], nullptr), acc);
    double v = t.c * acc;
    if (t.wl) v *= t.wl[i];
    t.out[i] = v;
    q = v * v;
  }
  return bcast_sum(q);
}

// y of phase C for rows r0 .. r0 + n - 1: Wd (s_old + alpha t) on the data
// rows (times the 16-bit row scale), zero in the padding, in G's
// accumulation type -- the bits of the step s += alpha t followed by the
// scaling of y.
template <typename Acc>
struct StepY {
  const double *s_old, *t, *wd;
  const float *row_scale;
  double alpha;
  int64_t nd;
  __device__ __forceinline__ void operator()(int64_t r0, int n, Acc *ys) const {
    for (int k = threadIdx.x; k < n; k += cgb::VT) {
      const int64_t r = r0 + k;
      double v = 0.0;
      if (r < nd) {
        v = fma(alpha, __ldcg(t + r), __ldcg(s_old + r));
        v = wd[r] * v;
        if (row_scale) v *= (double)row_scale[r];
      }
      ys[k] = (Acc)v;
    }
  }
};

// Phase C block b of nb: the step s_new = s_old + alpha t and dx += alpha
// p_new over the indices b * VT + thread + m nb VT; then G^T y for the 32
// columns of block b (warp w takes columns 4w .. 4w + 3, lanes striding the
// rows, y = StepY staged in shared memory) and r_j for those columns: the
// regulariser adjoint terms on one lane per (column, term), their dependent
// CSR loads in parallel and s_new formed on the fly from s_old and t, added
// by the lane holding the column to its G^T sum in term order
// (cgb::adjoint_column's arithmetic), then P.  Writes s_new, dx, gtw and r;
// returns the block's sum of r_j^2 (valid in every thread).
template <class L>
__device__ __forceinline__ double step_gty_adjoint_block(const FusedCgArgs &a, double alpha,
                                                         const double *s_old, double *s_new,
                                                         const double *p_new, int64_t b,
                                                         int64_t nb) {
  static_assert(gemv::kGtWarpCols * 8 <= 32, "one lane per (column, term)");
  using Acc = typename L::Acc;
  __shared__ double wsum[cgb::VT / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t top = a.nrow > a.nm ? a.nrow : a.nm;
  for (int64_t i = b * cgb::VT + threadIdx.x; i < top; i += nb * cgb::VT) {
    if (i < a.nrow) s_new[i] = fma(alpha, __ldcg(a.t + i), __ldcg(s_old + i));
    if (i < a.nm) a.dx[i] = fma(alpha, __ldcg(p_new + i), __ldcg(a.dx + i));
  }
  int64_t j = -1;
  const StepY<Acc> fill{s_old, a.t, a.wd, a.row_scale, alpha, a.nd};
  const double g = gemv::gty_body_f<L>(a.G, a.ld, a.nm, fill, b, &j);
  // lane 8c + q: term q of the warp's column c
  const int tc = lane >> 3, tq = lane & 7;
  const int64_t tj = b * gemv::kGtBlockCols + (int64_t)warp * gemv::kGtWarpCols + tc;
  double ts = 0.0;
  if (tc < gemv::kGtWarpCols && tq < a.AT.count && tj < a.nm) {
    const AdjointTerm &t = a.AT.t[tq];
    const int64_t off = t.s - a.s;  // the term's segment of s (and of t)
    for (int k = t.AT.rowptr[tj]; k < t.AT.rowptr[tj + 1]; k++) {
      const int64_t i = off + t.AT.col[k];
      const double w = t.wl ? t.wl[t.AT.col[k]] : 1.0;
      const double sv = fma(alpha, __ldcg(a.t + i), __ldcg(s_old + i));
      ts = fma(t.AT.val[k], w * sv, ts);
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
// blocks (phase B) and the forward-row blocks (phase A), then of ||r||^2 over
// the G^T blocks.
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
// Three team barriers per iteration:
//   A  p_new = -r + beta p_old folded into the partial row sums of G pp (row
//      tiles of 32 VEC rows x column ranges, the block's 8 warps splitting a
//      range), and the forward regulariser rows of t from pp formed on the
//      fly, with their per-block ||t||^2
//   B  t_data = Wd (sum of the partials, 16 rows per block, the splits shared
//      by 16 half-warps), per-block ||t||^2; then alpha = r2 / t2
//   C  s += alpha t (s and s2 alternate), dx += alpha p_new, and G^T y with
//      y = Wd s_data staged per block, for 32 columns per block (4 per warp),
//      r for those columns (the adjoint of the regulariser rows, P), per-block
//      ||r||^2; then beta, err and the stopping test
// Every CTA adds the per-block partials in index order, so the sums do not
// depend on the team size or on which CTA ran which block.
template <class L>
__device__ CgOut cg_loop(const FusedCgArgs &a, const CgIn &in, unsigned cta, unsigned nct,
                         TeamBarrier &bar) {
  const int64_t Nm = a.nm, nd = a.nd;
  const int64_t nb_vec = ceil_div_d(Nm, cgb::VT);  // blocks of an Nm-long vector
  const int64_t n_gx = (int64_t)a.tiles * a.splits;
  const RedLayout rl(nd, Nm, a.FT.count);
  const int64_t n_a = n_gx + (rl.nb_t - rl.nb_fin);  // G pp units, then forward-row blocks
  double *part_t = a.red, *part_r = a.red + rl.nb_t;

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
    const double *p_old = (it & 1) ? a.p2 : a.p;
    double *p_new = (it & 1) ? a.p : a.p2;
    const double *s_old = (it & 1) ? a.s2 : a.s;
    double *s_new = (it & 1) ? a.s : a.s2;
    // A
    for (int64_t b = cta; b < n_a; b += nct) {
      if (b < n_gx) {
        gemv::gx_partial_fold_body<L>(a.G, a.ld, Nm, a.per, a.r, p_old, a.P, beta, p_new, nullptr,
                                      a.scratch, b % a.tiles, b / a.tiles);
      } else {
        const double v = forward_rows_block(a, p_old, beta, b - n_gx, nb_vec);
        if (threadIdx.x == 0) part_t[rl.nb_fin + (b - n_gx)] = v;
      }
    }
    if (!(ok = bar.sync())) break;
    stamp(0);
    // B
    for (int64_t b = cta; b < rl.nb_fin; b += nct) {
      const double v = finish_rows(a.scratch, a.splits, a.ld, nd, a.row_scale, a.wd, a.t, b);
      if (threadIdx.x == 0) part_t[b] = v;
    }
    if (!(ok = bar.sync())) break;
    stamp(1);
    T2 = sum_partials_all(part_t, rl.nb_t);
    alpha = R2 / T2;  // GaussNewtonInversion.cpp:1601
    if (T2 == 0.0 || !isfinite(alpha)) {
      status = (T2 == 0.0) ? CG_STATUS_BREAKDOWN : CG_STATUS_NONFINITE;
      break;
    }
    // C
    for (int64_t b = cta; b < rl.nb_r; b += nct) {
      const double v = step_gty_adjoint_block<L>(a, alpha, s_old, s_new, p_new, b, rl.nb_r);
      if (threadIdx.x == 0) part_r[b] = v;
    }
    if (!(ok = bar.sync())) break;
    stamp(2);
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
