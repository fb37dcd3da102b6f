// Persistent CG: the whole CGLS loop of one solve in one cooperative launch.
//
// Reference: GaussNewtonInversion::solve_cg, the iteration loop
// (src/Inversion/GaussNewtonInversion.cpp:1556-1692).  The graph-replayed
// iteration (inversion.cu) launches 13 kernels per iteration.  Here every CTA
// of a cooperative grid (all co-resident) runs the iteration's phases in turn
// (cg_fused.cuh: four team barriers per iteration) and decides the stopping
// test itself from the same reduced scalars, so no host round trip or launch
// happens until the solve ends.  The sums are fixed-order and independent of
// the grid, so a solve is deterministic and gives what the batched kernel
// (invert_batch.cu) and the phase kernels (cg_phases.cu) give for the same
// problem; against the generic graph path it agrees to rounding (different
// summation orders).  Every barrier wait is
// bounded (a globaltimer limit): a CTA whose wait expires raises the barrier's
// error word and returns, every other CTA returns at its next barrier, and the
// host turns the word into GRADA_ERR_CUDA with the context still usable.
#include <algorithm>
#include <cstdlib>

#include "cg_fused.cuh"

namespace grada {

namespace {

// One solve on the whole cooperative grid: the loop starts from the scalars
// and control block the host setup left in a.scal / a.ctl and writes them back.
template <class L>
__global__ void __launch_bounds__(256, 3) cg_fused_kernel(FusedCgArgs a) {
  fused::TeamBarrier bar(a.barrier, gridDim.x, blockIdx.x, a.wait_limit_ns);
  fused::CgIn in;
  in.R2 = __ldcg(a.scal + CG_R2);
  in.ATB2 = __ldcg(a.scal + CG_ATB2);
  in.tol = __ldcg(a.scal + CG_TOL);
  in.rlast2 = __ldcg(a.scal + CG_RLAST2);
  in.err = __ldcg(a.scal + CG_ERR);
  in.maxit = __ldcg(a.ctl + CTL_MAXIT);
  const fused::CgOut o = fused::cg_loop<L>(a, in, blockIdx.x, gridDim.x, bar);
  if (blockIdx.x == 0 && threadIdx.x == 0 && o.ok) {
    a.scal[CG_R2] = o.R2;
    a.scal[CG_T2] = o.T2;
    a.scal[CG_ALPHA] = o.alpha;
    a.scal[CG_BETA] = o.beta;
    a.scal[CG_RLAST2] = o.rlast2;
    a.scal[CG_ERR] = o.err;
    a.ctl[CTL_ITER] = o.iterations;
    a.ctl[CTL_STATUS] = o.status;
    a.ctl[CTL_DONE] = 1;
  }
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

void fused_gx_partition(const DevG &G, int sm_count, int &tiles, int &splits, int64_t &per) {
  const int vec = vec_of(G.kind);
  const int64_t rows = gemv::fold_tile_rows_for_vec(vec);
  const int64_t esize = G.kind == GKind::FP64 ? 8 : (G.kind == GKind::FP32 ? 4 : 2);
  const int64_t t = ceil_div(G.ld, rows);
  const int64_t slots = (int64_t)cg_phase_a_blocks_per_sm(G.kind) * sm_count;
  const int64_t max_s = std::max<int64_t>(1, std::min<int64_t>(ceil_div(G.nm, 64), 65535));
  // at least one full round of the phase kernel's resident blocks where the
  // columns allow; among those, the split count with the fewest bytes per
  // round times whole rounds (a last, partly filled round streams at the rate
  // of its few blocks), plus the partial rows' write and read
  const int64_t min_s = std::min<int64_t>(max_s, std::max<int64_t>(1, ceil_div(slots, t)));
  int64_t best_s = min_s;
  double best = -1.0;
  for (int64_t sp = min_s; sp <= max_s; sp++) {
    const double unit_bytes = (double)(rows * esize) * (double)ceil_div(G.nm, sp);
    const double cost = (double)ceil_div(t * sp, slots) * (double)slots * unit_bytes +
                        (double)sp * (double)G.ld * 16.0;
    if (best < 0.0 || cost < best) {
      best = cost;
      best_s = sp;
    }
  }
  if (const char *e = std::getenv("GRADA_GX_SPLITS")) {  // a fixed split count, for tuning
    const long v = std::atol(e);
    if (v >= 1) best_s = std::min<int64_t>(v, max_s);
  }
  tiles = (int)t;
  splits = (int)best_s;
  per = ceil_div(G.nm, best_s);
}

void fused_red_sizes(int64_t nd, int64_t nm, int nterms, int64_t &doubles, int64_t &counters) {
  const fused::RedLayout rl(nd, nm, nterms);
  doubles = rl.doubles();
  counters = rl.counters();
}

void launch_cg_fused(const FusedCgArgs &a, GKind kind, int grid, cudaStream_t s) {
  GRADA_CUDA_CHECK(
      cudaMemsetAsync(a.barrier, 0, fused::kBarrierWords * sizeof(unsigned), s));
  FusedCgArgs copy = a;
  void *args[] = {&copy};
  GRADA_CUDA_CHECK(cudaLaunchCooperativeKernel(fused_kernel_for(kind), dim3((unsigned)grid),
                                               dim3(256), args, 0, s));
}

}  // namespace grada
