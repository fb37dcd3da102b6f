// Batched inversions in one persistent launch (invert_batch.cu): the device
// description of one problem.  Internal interface.
#pragma once

#include <stdint.h>

#include "../../include/grada_gpu.h"
#include "cg_fused.h"

namespace grada {

// One inversion problem, as invert_with_own_CG (GaussNewtonInversion.cpp:
// 657-1103) runs it on a fixed mesh, with every device buffer it touches.
// Built on the host from the problem's context after the same set-up that
// Context::invert does; the kernel runs the rest.
struct alignas(16) BatchProblem {
  FusedCgArgs cg;  // G, CG vectors, forward/adjoint terms (c of terms 0-3 = sqrt(lambda))
  // solve_cg set-up (GaussNewtonInversion.cpp:1458-1551)
  const double *dobs = nullptr;
  double *b = nullptr, *atb = nullptr, *gx = nullptr, *tmpd = nullptr, *part2 = nullptr;
  DevCSR seg_A[7];           // row-segment operators s, z, x, y, tz, tx, ty
  const double *seg_wl[7];   // their weights
  AdjointTerms AT_b, AT_s0;  // adjoints of b and of s0 (crg-y weighted by WL_y)
  int nterms = 4;
  // FP64 predictions G m (the kept FP64 G, or G itself when it is FP64)
  const double *Gp = nullptr;
  int p_tiles = 0, p_splits = 0;
  int64_t p_per = 0;
  int nb_d = 0;  // dot blocks of an Nd-long vector (misfit)
  // inversion state
  double *m = nullptr, *mt = nullptr, *mt_old = nullptr, *mopt = nullptr, *P = nullptr,
         *dpre = nullptr, *wl = nullptr;
  const double *mmin = nullptr, *mmax = nullptr, *m0 = nullptr;
  int *guard = nullptr, *flag = nullptr;
  DevCSR irls_A[7];  // Ws, Wx, Wy, Wz, Tx, Ty, Tz (the T ones unscaled)
  // parameters, with the powers the host computes (so both paths round alike)
  grada_invert_params prm;
  double lambda_up = 1.0;   // (1/rate)^min(3, n_lambda-2)
  double min_lambda = 0.0;  // min(max_lambda rate^20, 1e-5)
  double p_expo[5];
  int crg = 0;
  int cg_maxit = 0;
  // records: trials (gn, lambda, misfit, cg_iterations, cg_err) and iterations
  // (gn, n_trials, misfit), the report (final misfit, final lambda,
  // gn_iterations, n_trials, cg_iterations, predictions), status
  double *trials = nullptr;
  int max_trials = 0;
  double *iters = nullptr;
  int max_iters = 0;
  double *report = nullptr;  // 8 doubles
};
// The kernel copies a problem to shared memory in 16-byte words.
static_assert(sizeof(BatchProblem) % 16 == 0, "BatchProblem is copied in 16-byte words");

// Runs problems[0..n) (device array) on the teams of one cooperative launch.
// map (device ints): team of each CTA [grid], its rank in the team [grid], the
// size of each team [n_teams], each team's first problem [n_teams] (-1: take
// it from the queue); queue[0] (zeroed) counts the problems the queue has
// handed out after the first queue_base (those handed out in advance), in
// index order; bar_words holds the teams' barrier words (zeroed); team_slot
// 32 ints per team.  kind: storage of the CG G (the same for every problem).
int invert_batch_resident(GKind kind, int sm_count);
void launch_invert_batch(const BatchProblem *problems, int n, int *queue, int queue_base,
                         unsigned *bar_words, int *team_slot, const int *map, int n_teams,
                         int grid, GKind kind, unsigned long long wait_ns, cudaStream_t s);

}  // namespace grada
