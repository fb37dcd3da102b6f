// Persistent CG (cg_fused.cu): arguments of one solve's loop and its launch.
// Internal interface.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "cg_kernels.h"
#include "kernels.h"

namespace grada {

__host__ __device__ inline int64_t ceil_div_d(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Everything the CG loop touches.  The loop starts from the state the setup
// left on the device (r, p = 0, dx = 0, s, the scalars R2, ATB2, TOL, BETA = 0
// and the control block) and leaves the same state the graph path leaves.
struct FusedCgArgs {
  // stored G and the G x partition (gx_splits)
  const void *G = nullptr;
  const float *row_scale = nullptr;
  int64_t nd = 0, nm = 0, ld = 0;
  int tiles = 0, splits = 0;
  int64_t per = 0;
  double *scratch = nullptr;  // splits * ld doubles: G x partials, then y
  const double *wd = nullptr;  // Wd: post-scale of G pp, pre-scale of G^T s
  // CG vectors (GaussNewtonInversion.cpp:1556-1692)
  double *r = nullptr, *p = nullptr, *pp = nullptr, *dx = nullptr, *t = nullptr, *s = nullptr,
         *gtw = nullptr;
  const double *P = nullptr;
  int64_t nrow = 0;
  ForwardTerms FT;
  AdjointTerms AT;
  double *p2 = nullptr;        // second direction buffer (p and p2 alternate)
  double *part = nullptr;      // set-up dot products (dot_blocks partition)
  int nb_m = 0, nb_row = 0;    // dot-product block counts of the set-up
  double *red = nullptr;       // per-block partials and group sums of ||t||^2, ||r||^2
  unsigned *red_count = nullptr;  // group counts (zero at the start, reset by their last block)
  double *scal = nullptr;
  int *ctl = nullptr;
  unsigned *barrier = nullptr;  // the team barrier's words
  // phase trace (CTA 0 of the team): summed globaltimer spans of phases A-D,
  // each up to the end of its barrier, and the iteration count; null: none
  unsigned long long *trace = nullptr;
  unsigned long long wait_limit_ns = 2000000000ull;
};

// CTAs of a persistent CG launch for this storage (all co-resident).
int fused_cg_grid(GKind kind, int sm_count);
// G pp's partition in the persistent loop and its phase kernels: row tiles of
// 64 * vec rows x column ranges, the split count chosen for whole rounds of
// the phase-A kernel's resident blocks and few partial rows.  It depends on
// G's shape, the SM count and that kernel's occupancy only, so the sums of a
// solve do not depend on the launch.  GRADA_GX_SPLITS fixes the split count
// (for tuning).
void fused_gx_partition(const DevG &G, int sm_count, int &tiles, int &splits, int64_t &per);
// Doubles and counters of a.red / a.red_count for a loop over Nm cells, Nd
// rows and nterms regulariser terms.
void fused_red_sizes(int64_t nd, int64_t nm, int nterms, int64_t &doubles, int64_t &counters);
// Clears the barrier words and launches the cooperative kernel.
void launch_cg_fused(const FusedCgArgs &a, GKind kind, int grid, cudaStream_t s);
// Resident blocks per SM of the phase-A kernel (G pp) for this storage.
int cg_phase_a_blocks_per_sm(GKind kind);
// One iteration of the same loop as four kernels (cg_phases.cu) reading their
// arguments from dev_args (a device copy of a, which sizes the grids); parity
// alternates p and p2 as the persistent loop's iteration count does.
void launch_cg_phase_iteration(const FusedCgArgs &a, const FusedCgArgs *dev_args, GKind kind,
                               int parity, cudaStream_t s);
// The four phase kernels' grid sizes for a (what a captured iteration bakes in
// besides the storage and the argument pointer).
void cg_phase_grids(const FusedCgArgs &a, int64_t grids[4]);

}  // namespace grada
