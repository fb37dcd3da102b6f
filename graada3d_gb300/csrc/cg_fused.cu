// Persistent CG: the whole CGLS loop of one solve in one cooperative launch.
//
// Reference: GaussNewtonInversion::solve_cg, the iteration loop
// (src/Inversion/GaussNewtonInversion.cpp:1556-1692).  The graph-replayed
// iteration (inversion.cu) launches 13 kernels per iteration; at the sizes of
// small inversions those launches, not the two reads of G, set the time.
// Here every CTA of a cooperative grid (all co-resident) runs the iteration's
// phases in turn, separated by grid barriers, and decides the stopping test
// itself from the same reduced scalars, so no host round trip or launch
// happens until the solve ends.  Each phase runs the blocks of the
// corresponding stand-alone kernel (gemv_body.cuh, cg_body.cuh) with the same
// arithmetic and summation orders, so the iterates are bitwise those of the
// graph path.  Phases per iteration:
//   P    p = -r + beta p, pp = P p
//   G1   partial row sums of G pp over column ranges
//   G2   t_data = Wd (sum of partials) and the forward regulariser rows of t
//   D1   block partials of ||t||^2
//   S    alpha = r2 / t2; s += alpha t, dx += alpha p, and y = Wd s_data in
//        G's accumulation type (each thread converts the entries it updated)
//   GT   G^T y for 4 columns per block, then r for those columns (the adjoint
//        of the regulariser rows and P) in the same block
//   D2   block partials of ||r||^2; beta, err and the stopping test
// Seven grid barriers per iteration.  Every barrier wait is bounded (a
// globaltimer limit): a CTA whose wait expires raises the barrier's error word
// and returns, every other CTA returns at its next barrier, and the host turns
// the word into GRADA_ERR_CUDA with the context still usable.
#include <algorithm>

#include "cg_body.cuh"
#include "cg_fused.h"
#include "common.cuh"
#include "gemv_body.cuh"

namespace grada {

namespace {

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

}  // namespace

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

namespace {

// Broadcast thread 0's value to the block.
__device__ __forceinline__ double bcast(double v) {
  __shared__ double s_v;
  if (threadIdx.x == 0) s_v = v;
  __syncthreads();
  const double out = s_v;
  __syncthreads();
  return out;
}

}  // namespace

// The loop of one solve, run by CTA `cta` of the nct CTAs of its team.
template <class L>
__device__ void cg_fused_team(const FusedCgArgs &a, unsigned cta, unsigned nct) {
  using Acc = typename L::Acc;
  TeamBarrier bar{a.barrier, nct, 0u, a.wait_limit_ns};
  const int64_t Nm = a.nm, nd = a.nd, ld = a.ld, nrow = a.nrow;
  const int64_t nb_vec = ceil_div_d(Nm, cgb::VT);  // blocks of an Nm-long vector kernel
  const int64_t nb_fin = ceil_div_d(nd, 256);
  const int64_t nb_axpy = ceil_div_d(nrow > Nm ? nrow : Nm, cgb::VT);
  const int64_t nb_prep = ceil_div_d(ld, 256);
  const int64_t nb_gt = ceil_div_d(Nm, gemv::kGtCols);
  const int64_t n_gx = (int64_t)a.tiles * a.splits;
  const int64_t n_g2 = nb_fin + (int64_t)a.FT.count * nb_vec;
  Acc *y = reinterpret_cast<Acc *>(a.scratch);

  double R2 = __ldcg(a.scal + CG_R2), beta = __ldcg(a.scal + CG_BETA);
  double rlast2 = __ldcg(a.scal + CG_RLAST2), err = __ldcg(a.scal + CG_ERR);
  double T2 = 0.0, alpha = 0.0;
  const double ATB2 = __ldcg(a.scal + CG_ATB2), tol = __ldcg(a.scal + CG_TOL);
  int it = __ldcg(a.ctl + CTL_ITER);
  const int maxit = __ldcg(a.ctl + CTL_MAXIT);
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
  if (cta == 0 && threadIdx.x == 0 && ok) {
    a.scal[CG_R2] = R2;
    a.scal[CG_T2] = T2;
    a.scal[CG_ALPHA] = alpha;
    a.scal[CG_BETA] = beta;
    a.scal[CG_RLAST2] = rlast2;
    a.scal[CG_ERR] = err;
    a.ctl[CTL_ITER] = it;
    a.ctl[CTL_STATUS] = status;
    a.ctl[CTL_DONE] = 1;
  }
}

namespace {

template <class L>
__global__ void __launch_bounds__(256) cg_fused_kernel(FusedCgArgs a) {
  cg_fused_team<L>(a, blockIdx.x, gridDim.x);
}

template <class L>
const void *kernel_of() {
  return reinterpret_cast<const void *>(&cg_fused_kernel<L>);
}

const void *fused_kernel_for(GKind k) {
  switch (k) {
    case GKind::FP64: return kernel_of<gemv::LoadF64>();
    case GKind::FP32: return kernel_of<gemv::LoadF32>();
    case GKind::BF16: return kernel_of<gemv::LoadBF16>();
    case GKind::FP16: return kernel_of<gemv::LoadF16>();
  }
  return nullptr;
}

}  // namespace

int fused_cg_grid(GKind kind, int sm_count) {
  int per_sm = 0;
  GRADA_CUDA_CHECK(
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fused_kernel_for(kind), 256, 0));
  return std::max(1, per_sm) * sm_count;
}

void launch_cg_fused(const FusedCgArgs &a, GKind kind, int grid, cudaStream_t s) {
  GRADA_CUDA_CHECK(cudaMemsetAsync(a.barrier, 0, 2 * sizeof(unsigned), s));
  FusedCgArgs copy = a;
  void *args[] = {&copy};
  GRADA_CUDA_CHECK(cudaLaunchCooperativeKernel(fused_kernel_for(kind), dim3((unsigned)grid),
                                               dim3(256), args, 0, s));
}

}  // namespace grada
