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
// Work units of G pp in the persistent loop and its phase kernels: 12 per SM
// (GRADA_GX_UNITS_PER_SM overrides), a whole number of rounds at 1, 2, 3, 4
// or 6 resident blocks per SM.
int fused_gx_units(int sm_count);
// G pp's partition: row tiles of 256 * vec rows and column ranges, about
// `units` of them.  The sums of a solve depend on it, not on the launch.
void fused_gx_partition(const DevG &G, int units, int &tiles, int &splits, int64_t &per);
// Doubles and counters of a.red / a.red_count for a loop over Nm cells, Nd
// rows and nterms regulariser terms.
void fused_red_sizes(int64_t nd, int64_t nm, int nterms, int64_t &doubles, int64_t &counters);
// Clears the barrier words and launches the cooperative kernel.
void launch_cg_fused(const FusedCgArgs &a, GKind kind, int grid, cudaStream_t s);
// One iteration of the same loop as four kernels (cg_phases.cu); parity
// alternates p and p2 as the persistent loop's iteration count does.
void launch_cg_phase_iteration(const FusedCgArgs &a, GKind kind, int parity, cudaStream_t s);

}  // namespace grada
