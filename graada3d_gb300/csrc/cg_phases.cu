// The CG loop's four phases as separate kernels, replayed from a CUDA graph.
//
// Reference: GaussNewtonInversion::solve_cg, the iteration loop
// (src/Inversion/GaussNewtonInversion.cpp:1556-1692).  The phase bodies are
// the persistent loop's (cg_fused.cuh), on its partition of G pp
// (fused_gx_partition), so both paths compute the same sums in the same order
// and give bitwise the same solve.  What the
// persistent loop does at a team barrier happens here at a kernel boundary,
// and the two reductions that end a phase (||t||^2 -> alpha, ||r||^2 -> beta
// and the stopping test) run in the phase's last block: every block stores
// its partial, fences and counts itself in; the block that counts last adds
// the partials in index order (nothing waits on another block).  Each kernel
// returns at once while ctl[CTL_DONE] is raised, so a graph of K iterations
// can be replayed until the solve ends, one host synchronisation per replay.
// Each phase kernel runs at its own occupancy, which the products need: the
// persistent launch holds three CTAs per SM throughout.  (Launching the
// phases as programmatic dependents, each block waiting in griddepcontrol.wait,
// measured slower at 3,392 x 16,384: 0.165 against 0.158 ms per FP32 iteration.)
#include "cg_fused.cuh"

namespace grada {

namespace {

using fused::RedLayout;

// True in every thread of the block that counted last on *count (which it
// resets for the next phase), after this block's thread 0 stored its partial.
__device__ __forceinline__ bool last_block(unsigned *count, unsigned nblocks) {
  __shared__ int s_last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned prev = atomicAdd(count, 1u);
    s_last = (prev + 1u == nblocks);
    if (s_last) {
      __threadfence();
      *count = 0u;
    }
  }
  __syncthreads();
  return s_last != 0;
}

__device__ __forceinline__ bool done(const FusedCgArgs &a) {
  return *reinterpret_cast<volatile const int *>(a.ctl + CTL_DONE) != 0;
}

// A: p_new = -r + beta p_old, pp = P p_new, folded into G pp's partial sums.
template <class L>
__global__ void __launch_bounds__(256)
    phase_a_kernel(const FusedCgArgs *__restrict__ ap, int parity) {
  const FusedCgArgs &a = *ap;
  if (done(a)) return;
  const double *p_old = parity ? a.p2 : a.p;
  double *p_new = parity ? a.p : a.p2;
  const double beta = __ldcg(a.scal + CG_BETA);
  const int64_t b = blockIdx.x;
  gemv::gx_partial_fold_body<L>(a.G, a.ld, a.nm, a.per, a.r, p_old, a.P, beta, p_new, a.pp,
                                a.scratch, b % a.tiles, b / a.tiles);
}

// B: t_data = Wd (sum of the partials), the forward regulariser rows, the
// per-block ||t||^2; the last block: t2, alpha = r2 / t2 (:1601) and the
// breakdown / non-finite checks.
__global__ void __launch_bounds__(256) phase_b_kernel(const FusedCgArgs *__restrict__ ap) {
  const FusedCgArgs &a = *ap;
  if (done(a)) return;
  const RedLayout rl(a.nd, a.nm, a.FT.count);
  const int64_t nb_vec = ceil_div_d(a.nm, cgb::VT);
  const int64_t b = blockIdx.x;
  double v;
  if (b < rl.nb_fin) {
    v = fused::finish_rows(a.scratch, a.splits, a.ld, a.nd, a.row_scale, a.wd, a.t, b);
  } else {
    const int64_t k = b - rl.nb_fin;
    const ForwardTerm &ft = a.FT.t[k / nb_vec];
    cgb::forward_term_body(ft, a.pp, k % nb_vec);
    const int64_t i = (k % nb_vec) * cgb::VT + threadIdx.x;
    double q = 0.0;
    if (i < a.nm) {
      const double tv = __ldcg(ft.out + i);
      q = tv * tv;
    }
    v = fused::bcast_sum(q);
  }
  if (threadIdx.x == 0) a.red[b] = v;
  if (!last_block(a.red_count, (unsigned)rl.nb_t)) return;
  const double T2 = fused::sum_partials_all(a.red, rl.nb_t);
  if (threadIdx.x == 0) {
    const double alpha = __ldcg(a.scal + CG_R2) / T2;
    a.scal[CG_T2] = T2;
    a.scal[CG_ALPHA] = alpha;
    if (T2 == 0.0 || !isfinite(alpha)) {
      a.ctl[CTL_STATUS] = (T2 == 0.0) ? CG_STATUS_BREAKDOWN : CG_STATUS_NONFINITE;
      a.ctl[CTL_DONE] = 1;
    }
  }
}

// C: s += alpha t, dx += alpha p_new, y = Wd s_data in G's accumulation type.
template <class L>
__global__ void __launch_bounds__(256)
    phase_c_kernel(const FusedCgArgs *__restrict__ ap, int parity) {
  const FusedCgArgs &a = *ap;
  if (done(a)) return;
  using Acc = typename L::Acc;
  const double *p_new = parity ? a.p : a.p2;
  const double alpha = __ldcg(a.scal + CG_ALPHA);
  const int64_t b = blockIdx.x;
  cgb::axpy_body(a.t, p_new, alpha, a.nrow, a.nm, a.s, a.dx, b);
  if (b < ceil_div_d(a.ld, 256))
    gemv::prep_y_body<Acc>(a.s, a.nd, a.ld, a.row_scale, a.wd, reinterpret_cast<Acc *>(a.scratch),
                           b);
}

// D: G^T y and r for 32 columns per block, the per-block ||r||^2; the last
// block: r2, beta = r2 / rlast2, err = r2 / ||A^T b||^2, the iteration count
// and the stopping tests (:1674-1691).
template <class L, int U>
__global__ void __launch_bounds__(256) phase_d_kernel(const FusedCgArgs *__restrict__ ap) {
  const FusedCgArgs &a = *ap;
  if (done(a)) return;
  using Acc = typename L::Acc;
  const RedLayout rl(a.nd, a.nm, a.FT.count);
  double *part_r = a.red + rl.nb_t;
  const double v =
      fused::gty_adjoint_block<L, U>(a, reinterpret_cast<const Acc *>(a.scratch), blockIdx.x);
  if (threadIdx.x == 0) part_r[blockIdx.x] = v;
  if (!last_block(a.red_count, (unsigned)rl.nb_r)) return;
  const double r2 = fused::sum_partials_all(part_r, rl.nb_r);
  if (threadIdx.x == 0) {
    const double rlast2 = __ldcg(a.scal + CG_R2);
    const double err = r2 / __ldcg(a.scal + CG_ATB2);
    a.scal[CG_RLAST2] = rlast2;
    a.scal[CG_R2] = r2;
    a.scal[CG_BETA] = r2 / rlast2;
    a.scal[CG_ERR] = err;
    const int it = a.ctl[CTL_ITER] + 1;
    a.ctl[CTL_ITER] = it;
    if (!isfinite(err)) {
      a.ctl[CTL_STATUS] = CG_STATUS_NONFINITE;
      a.ctl[CTL_DONE] = 1;
    } else if (err < __ldcg(a.scal + CG_TOL)) {
      a.ctl[CTL_STATUS] = CG_STATUS_CONVERGED;
      a.ctl[CTL_DONE] = 1;
    } else if (it >= a.ctl[CTL_MAXIT]) {
      a.ctl[CTL_DONE] = 1;
    }
  }
}

template <class L>
void launch_iteration(const FusedCgArgs &a, const FusedCgArgs *ap, int parity, cudaStream_t s) {
  int64_t g[4];
  cg_phase_grids(a, g);
  phase_a_kernel<L><<<(unsigned)g[0], 256, 0, s>>>(ap, parity);
  GRADA_LAUNCH_CHECK();
  phase_b_kernel<<<(unsigned)g[1], 256, 0, s>>>(ap);
  GRADA_LAUNCH_CHECK();
  phase_c_kernel<L><<<(unsigned)g[2], 256, 0, s>>>(ap, parity);
  GRADA_LAUNCH_CHECK();
  if constexpr (L::VEC >= 4) {  // FP64 G stays FP64-pipe bound
    if (a.ld >= gemv::kGtTallRows) {
      phase_d_kernel<L, gemv::kGtUnrollTall><<<(unsigned)g[3], 256, 0, s>>>(ap);
      GRADA_LAUNCH_CHECK();
      return;
    }
  }
  phase_d_kernel<L, gemv::kGtUnroll><<<(unsigned)g[3], 256, 0, s>>>(ap);
  GRADA_LAUNCH_CHECK();
}

}  // namespace

int cg_phase_a_blocks_per_sm(GKind kind) {
  const void *k = nullptr;
  switch (kind) {
    case GKind::FP64: k = reinterpret_cast<const void *>(&phase_a_kernel<gemv::LoadF64>); break;
    case GKind::FP32: k = reinterpret_cast<const void *>(&phase_a_kernel<gemv::LoadF32>); break;
    case GKind::BF16: k = reinterpret_cast<const void *>(&phase_a_kernel<gemv::LoadBF16>); break;
    case GKind::FP16: k = reinterpret_cast<const void *>(&phase_a_kernel<gemv::LoadF16>); break;
  }
  int n = 0;
  GRADA_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, 256, 0));
  return n > 0 ? n : 1;
}

void cg_phase_grids(const FusedCgArgs &a, int64_t grids[4]) {
  const RedLayout rl(a.nd, a.nm, a.FT.count);
  grids[0] = (int64_t)a.tiles * a.splits;
  grids[1] = rl.nb_t;
  grids[2] = ceil_div_d(a.nrow > a.nm ? a.nrow : a.nm, cgb::VT);
  grids[3] = rl.nb_r;
}

void launch_cg_phase_iteration(const FusedCgArgs &a, const FusedCgArgs *dev_args, GKind kind,
                               int parity, cudaStream_t s) {
  switch (kind) {
    case GKind::FP64: launch_iteration<gemv::LoadF64>(a, dev_args, parity, s); break;
    case GKind::FP32: launch_iteration<gemv::LoadF32>(a, dev_args, parity, s); break;
    case GKind::BF16: launch_iteration<gemv::LoadBF16>(a, dev_args, parity, s); break;
    case GKind::FP16: launch_iteration<gemv::LoadF16>(a, dev_args, parity, s); break;
  }
}

}  // namespace grada
