// Many independent inversions in one persistent cooperative launch.
//
// Reference: GaussNewtonInversion::invert_with_own_CG on a fixed mesh
// (src/Inversion/GaussNewtonInversion.cpp:657-1103) with solve_cg
// (:1417-1698), once per problem.  The grid is split into teams of
// team_ctas co-resident CTAs; a team takes the next problem from a device
// queue (problems ordered by size, largest first), runs that problem's whole
// inversion -- lambda search, the CG solves, the bound transform, the misfits,
// the IRLS reweighting and the stopping tests -- with team barriers between
// its phases, then takes the next.  The control flow is the host loop of
// Context::invert, executed by every CTA of the team on the same reduced
// scalars; every vector step runs the blocks of the stand-alone kernels
// (cg_body.cuh, gemv_body.cuh) in the same summation orders, so each problem's
// model and lambda/misfit record are bitwise those of grada_invert.  The
// powers of the lambda schedule and the IRLS exponents come from the host,
// where grada_invert computes them.
//
// Scope: G stored FP64, or a reduced-precision G with the FP64 G kept (every
// prediction an FP64 product); other storages run through grada_invert_batch.
#include <algorithm>

#include "cg_fused.cuh"
#include "invert_batch.h"

namespace grada {

namespace {

using fused::TeamBarrier;

// Everything below runs in every CTA of the team with the same arguments.
template <class L>
struct TeamInversion {
  using Acc = typename L::Acc;
  BatchProblem &P;
  unsigned cta, nct;
  TeamBarrier &bar;
  int64_t Nm, Nd, ld, nbv;
  double predictions = 0.0;

  __device__ TeamInversion(BatchProblem &p, unsigned c, unsigned n, TeamBarrier &b)
      : P(p), cta(c), nct(n), bar(b) {
    Nm = P.cg.nm;
    Nd = P.cg.nd;
    ld = P.cg.ld;
    nbv = ceil_div_d(Nm, cgb::VT);
  }

  // out = G_fp64 mv  (Context::data_prediction with an FP64 product)
  __device__ bool predict(const double *mv, double *out) {
    const int64_t n_gx = (int64_t)P.p_tiles * P.p_splits;
    for (int64_t b = cta; b < n_gx; b += nct)
      gemv::gx_partial_body<gemv::LoadF64>(P.Gp, ld, Nm, P.p_per, mv, P.cg.scratch,
                                           b % P.p_tiles, b / P.p_tiles);
    if (!bar.sync()) return false;
    const int64_t nb = ceil_div_d(Nd, gemv::kFinishRows);
    for (int64_t b = cta; b < nb; b += nct)
      gemv::gx_finish_body(P.cg.scratch, P.p_splits, ld, Nd, nullptr, nullptr, out, b);
    if (!bar.sync()) return false;
    predictions += 1.0;
    return true;
  }

  // sqrt(||Wd (G mv - dobs)||^2 / Nd)   (GaussNewtonInversion.cpp:784, :916)
  __device__ bool misfit_of(const double *mv, double &misfit) {
    if (!predict(mv, P.dpre)) return false;
    for (int64_t b = cta; b < P.nb_d; b += nct) {
      const double v = cgb::misfit_partial_body(P.dpre, P.dobs, P.cg.wd, Nd, b, P.nb_d);
      if (threadIdx.x == 0) P.cg.part[b] = v;
    }
    if (!bar.sync()) return false;
    const double s = fused::bcast(cgb::sum_partials_body(P.cg.part, P.nb_d));
    misfit = sqrt(s / (double)Nd);
    return true;
  }

  // dst = src (and dst2 = src when dst2 is given)
  __device__ bool copy(const double *src, double *dst, double *dst2) {
    for (int64_t b = cta; b < nbv; b += nct) {
      const int64_t i = b * cgb::VT + threadIdx.x;
      if (i < Nm) {
        const double v = __ldcg(src + i);
        dst[i] = v;
        if (dst2) dst2[i] = v;
      }
    }
    return bar.sync();
  }

  // GaussNewtonInversion::solve_cg (:1417-1698) from mk, mref = m0, P, WL.
  __device__ bool solve(double lambda, double tol, int maxit, const double *mk,
                        const double *mref, int &iterations, double &err, int &status) {
    FusedCgArgs &a = P.cg;
    const double sl = sqrt(lambda);
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int k = 0; k < 4 && k < P.nterms; k++) {
        a.FT.t[k].c = sl;
        a.AT.t[k].c = sl;
        P.AT_b.t[k].c = sl;
        P.AT_s0.t[k].c = sl;
      }
    }
    __syncthreads();
    iterations = 0;
    err = 0.0;
    status = CG_STATUS_RUNNING;
    // b and s = -b (:1458-1472), Wd b, and the zero start of p, dx, t
    if (!predict(mk, P.gx)) return false;
    const int64_t nrow = a.nrow;
    const int64_t nb_data = ceil_div_d(Nd, cgb::VT);
    const int64_t n_seg = (int64_t)P.nterms * nbv;
    const int64_t nb_t = ceil_div_d(nrow, cgb::VT);
    if (cta == 0 && threadIdx.x == 0) *P.flag = 0;
    for (int64_t b = cta; b < nb_data + n_seg + nb_t; b += nct) {
      if (b < nb_data) {
        const int64_t i = b * cgb::VT + threadIdx.x;
        if (i < Nd) {
          const double v = cgb::data_residual_value(P.dobs, P.gx, a.wd, i);
          P.b[i] = v;
          a.s[i] = -v;
          P.tmpd[i] = 1.0 * (a.wd[i] * v);
        }
      } else if (b < nb_data + n_seg) {
        const int64_t k = (b - nb_data) / nbv;
        const int64_t i = ((b - nb_data) % nbv) * cgb::VT + threadIdx.x;
        if (i < Nm) {
          const double c = k < 4 ? -sl : -1.0;
          const double v =
              cgb::csr_apply_value(P.seg_A[k], mk, k == 0 ? mref : nullptr, c, P.seg_wl[k], i);
          P.b[Nd + k * Nm + i] = v;
          a.s[Nd + k * Nm + i] = -v;
        }
      } else {
        const int64_t i = (b - nb_data - n_seg) * cgb::VT + threadIdx.x;
        if (i < nrow) a.t[i] = 0.0;
        if (i < Nm) {
          a.p[i] = 0.0;
          a.dx[i] = 0.0;
        }
      }
    }
    if (!bar.sync()) return false;
    // A^T b and r = A^T s0 (:1485-1551): one G^T (Wd b) serves both
    Acc *y = reinterpret_cast<Acc *>(a.scratch);
    const int64_t nb_prep = ceil_div_d(ld, 256);
    for (int64_t b = cta; b < nb_prep; b += nct)
      gemv::prep_y_body<Acc>(P.tmpd, Nd, ld, a.row_scale, nullptr, y, b);
    if (!bar.sync()) return false;
    const int64_t nb_gt = ceil_div_d(Nm, gemv::kGtBlockCols);
    for (int64_t b = cta; b < nb_gt; b += nct) {
      int64_t j = -1;
      const double g = gemv::gty_body<L>(a.G, ld, Nm, y, b, &j);
      if (j >= 0) {
        a.gtw[j] = g;
        P.atb[j] = cgb::adjoint_column(P.AT_b, j, a.P, true, g, 1.0);
        a.r[j] = cgb::adjoint_column(P.AT_s0, j, a.P, true, g, -1.0);
      }
    }
    if (!bar.sync()) return false;
    for (int64_t b = cta; b < a.nb_m; b += nct) {
      const double v1 = cgb::dot_partial_body(P.atb, nullptr, Nm, b, a.nb_m);
      const double v2 = cgb::dot_partial_body(a.r, nullptr, Nm, b, a.nb_m);
      if (threadIdx.x == 0) {
        a.part[b] = v1;
        P.part2[b] = v2;
      }
    }
    if (!bar.sync()) return false;
    fused::CgIn in;
    in.ATB2 = fused::bcast(cgb::sum_partials_body(a.part, a.nb_m));
    in.R2 = fused::bcast(cgb::sum_partials_body(P.part2, a.nb_m));
    in.tol = tol;
    in.maxit = maxit;
    if (maxit <= 0) return true;       // iterations = maxit (:1693-1696)
    if (in.R2 == 0.0) return true;     // a zero right-hand side: dx = 0
    const fused::CgOut o = fused::cg_loop<L>(a, in, cta, nct, bar);
    if (!o.ok) return false;
    iterations = o.iterations;
    err = o.err;
    status = o.status;
    return true;
  }

  // m_trial from m and dx with the bounds (:877-911); mt_old = the previous m_trial
  __device__ bool bound_update() {
    for (int64_t b = cta; b < nbv; b += nct) {
      const int64_t i = b * cgb::VT + threadIdx.x;
      if (i < Nm) {
        P.mt_old[i] = __ldcg(P.mt + i);
        const int g = cgb::bound_update_cell(P.m, P.cg.dx, P.mmin, P.mmax, P.mt, i);
        P.guard[i] = g;
        if (g) atomicOr(P.flag, 1);
      }
    }
    if (!bar.sync()) return false;
    if (*(volatile int *)P.flag) {
      if (cta == 0 && threadIdx.x == 0)
        cgb::bound_fixup_seq(P.guard, P.mmin, P.mmax, P.mt_old, Nm, P.mt);
      if (!bar.sync()) return false;
    }
    return true;
  }

  // IRLS weights from m_opt (:962-1022)
  __device__ bool irls() {
    const grada_invert_params &prm = P.prm;
    const int lp[7] = {prm.lp_s, prm.lp_x, prm.lp_y, prm.lp_z, prm.lp_t, prm.lp_t, prm.lp_t};
    for (int64_t b = cta; b < 7 * nbv; b += nct) {
      const int q = (int)(b / nbv);
      if (lp[q] == 2 || (q >= 4 && !P.crg)) continue;
      const int64_t i = (b % nbv) * cgb::VT + threadIdx.x;
      if (i < Nm) {
        const double v = cgb::csr_apply_value(P.irls_A[q], P.mopt, q == 0 ? P.m0 : nullptr, 1.0,
                                              nullptr, i);
        P.wl[q * Nm + i] = cgb::irls_value(v, prm.epsilon2, P.p_expo[q < 4 ? q : 4]);
      }
    }
    return bar.sync();
  }

  __device__ void record_trial(int n, int gn, double lambda, double misfit, int cg_it, double cg_err) {
    if (cta == 0 && threadIdx.x == 0 && n < P.max_trials) {
      double *o = P.trials + 5 * n;
      o[0] = gn;
      o[1] = lambda;
      o[2] = misfit;
      o[3] = cg_it;
      o[4] = cg_err;
    }
  }

  // invert_with_own_CG (:657-1103) on a fixed mesh; returns false when a
  // barrier wait expired, and sets status != 0 on a CG breakdown.
  __device__ bool run(int &status_out) {
    const grada_invert_params &prm = P.prm;
    status_out = 0;
    double misfit = 0.0;
    if (!misfit_of(P.m, misfit)) return false;
    double lambda = prm.max_lambda, lambda_opt = lambda, misfit_opt = misfit;
    if (!copy(P.m, P.mopt, nullptr)) return false;
    const double rate = prm.lambda_decreasing_rate;
    int n_trials = 0, n_iters = 0;
    double cg_total = 0.0;
    int i = 0, j = 0;
    for (i = 0; i < prm.gn_iterations; i++) {
      double misfit_last1 = 10 * misfit;
      double misfit_last2 = 100 * misfit;
      const double misfit_last_iteration = misfit;
      if (i == 0 || prm.n_lambda == 1 || fabs(rate - 1) < 1e-6) {
        lambda = prm.max_lambda;
      } else {
        lambda = lambda_opt * P.lambda_up;
        if (lambda < P.min_lambda) lambda = 1.0;
      }
      // m_trial = m and P (:856-861)
      for (int64_t b = cta; b < nbv; b += nct) {
        const int64_t k = b * cgb::VT + threadIdx.x;
        if (k < Nm) {
          P.mt[k] = __ldcg(P.m + k);
          P.P[k] = cgb::p_diag_value(P.m, P.mmin, P.mmax, k);
        }
      }
      if (!bar.sync()) return false;
      for (j = 0; j < prm.n_lambda; j++) {
        int cg_it = 0, cg_status = 0;
        double cg_err = 0.0;
        if (!solve(lambda, prm.cg_tol, P.cg_maxit, P.m, P.m0, cg_it, cg_err, cg_status))
          return false;
        if (cg_status == CG_STATUS_BREAKDOWN || cg_status == CG_STATUS_NONFINITE) {
          status_out = cg_status == CG_STATUS_BREAKDOWN ? GRADA_ERR_BREAKDOWN : GRADA_ERR_NONFINITE;
          break;
        }
        cg_total += cg_it;
        if (!bound_update()) return false;
        misfit_last2 = misfit_last1;
        misfit_last1 = misfit;
        if (!misfit_of(P.mt, misfit)) return false;
        record_trial(n_trials++, i + 1, lambda, misfit, cg_it, cg_err);
        if (j == 0 || misfit < misfit_opt) {
          misfit_opt = misfit;
          if (!copy(P.mt, P.mopt, i > 0 ? P.m : nullptr)) return false;
          lambda_opt = lambda;
        }
        if ((fabs(misfit - misfit_last1) / fmin(misfit, misfit_last1) < prm.stag_tol) &&
            (fabs(misfit_last1 - misfit_last2) / fmin(misfit_last1, misfit_last2) < prm.stag_tol) &&
            j > 1)
          break;
        if (misfit > misfit_last1 && misfit_last1 > misfit_last2 && j > 1) {
          break;
        } else {
          lambda = lambda * rate;
          if (!irls()) return false;
        }
        if (misfit < prm.target_misfit) break;
      }
      if (status_out) break;
      if (!copy(P.mopt, P.m, nullptr)) return false;
      misfit = misfit_opt;
      if (cta == 0 && threadIdx.x == 0 && n_iters < P.max_iters) {
        double *o = P.iters + 3 * n_iters;
        o[0] = i + 1;
        o[1] = (j == prm.n_lambda) ? prm.n_lambda : (j + 1);
        o[2] = misfit;
      }
      n_iters++;
      if (misfit < prm.target_misfit || i == prm.gn_iterations - 1) break;
      const bool flag1 = fabs(misfit - misfit_last_iteration) /
                             fmin(misfit, misfit_last_iteration) < prm.stag_tol;
      if (flag1) break;
    }
    if (cta == 0 && threadIdx.x == 0) {
      P.report[0] = misfit;
      P.report[1] = lambda;
      P.report[2] = n_iters;
      P.report[3] = n_trials;
      P.report[4] = cg_total;
      P.report[5] = predictions;
      P.report[6] = status_out;
      P.report[7] = 1.0;  // done
    }
    return true;
  }
};

// Team layout of a launch: CTA c belongs to team team_of[c] as its
// rank_of[c]-th CTA; team t has size_of[t] CTAs and starts with problem
// first_of[t] (-1: it takes its first problem from the queue too).
struct TeamMap {
  const int *team_of, *rank_of, *size_of, *first_of;
};

template <class L>
__global__ void __launch_bounds__(256, 2)
    invert_batch_kernel(const BatchProblem *problems, int n, int *queue, int queue_base,
                        unsigned *bar_words, int *team_slot, TeamMap map,
                        unsigned long long wait_ns) {
  __shared__ __align__(16) unsigned char sp_raw[sizeof(BatchProblem)];
  BatchProblem &sp = *reinterpret_cast<BatchProblem *>(sp_raw);
  const unsigned team = (unsigned)map.team_of[blockIdx.x];
  const unsigned cta = (unsigned)map.rank_of[blockIdx.x];
  const unsigned team_ctas = (unsigned)map.size_of[team];
  TeamBarrier bar(bar_words + (size_t)fused::kBarrierWords * team, team_ctas, cta, wait_ns);
  int next = map.first_of[team];
  while (true) {
    int k = next;
    next = -1;
    if (k < 0) {
      if (cta == 0 && threadIdx.x == 0) {
        team_slot[32 * team] = queue_base + atomicAdd(queue, 1);
        __threadfence();
      }
      if (!bar.sync()) return;
      k = __ldcg(team_slot + 32 * team);
    }
    if (k >= n) return;
    // this CTA's copy of the problem (its lambda-dependent coefficients change)
    const uint4 *src = reinterpret_cast<const uint4 *>(problems + k);
    uint4 *dst = reinterpret_cast<uint4 *>(sp_raw);
    for (int w = threadIdx.x; w < (int)(sizeof(BatchProblem) / 16); w += blockDim.x) dst[w] = src[w];
    __syncthreads();
    TeamInversion<L> inv(sp, cta, team_ctas, bar);
    int status = 0;
    if (!inv.run(status)) return;
  }
}

const void *batch_kernel_for(GKind k) {
  switch (k) {
    case GKind::FP64: return reinterpret_cast<const void *>(&invert_batch_kernel<gemv::LoadF64>);
    case GKind::FP32: return reinterpret_cast<const void *>(&invert_batch_kernel<gemv::LoadF32>);
    case GKind::BF16: return reinterpret_cast<const void *>(&invert_batch_kernel<gemv::LoadBF16>);
    case GKind::FP16: return reinterpret_cast<const void *>(&invert_batch_kernel<gemv::LoadF16>);
  }
  return nullptr;
}

}  // namespace

int invert_batch_resident(GKind kind, int sm_count) {
  int per_sm = 0;
  GRADA_CUDA_CHECK(
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_kernel_for(kind), 256, 0));
  return std::max(1, per_sm) * sm_count;
}

void launch_invert_batch(const BatchProblem *problems, int n, int *queue, int queue_base,
                         unsigned *bar_words, int *team_slot, const int *map, int n_teams,
                         int grid, GKind kind, unsigned long long wait_ns, cudaStream_t s) {
  TeamMap tm{map, map + grid, map + 2 * grid, map + 2 * grid + n_teams};
  void *args[] = {(void *)&problems,  (void *)&n,  (void *)&queue,  (void *)&queue_base,
                  (void *)&bar_words, (void *)&team_slot, (void *)&tm, (void *)&wait_ns};
  GRADA_CUDA_CHECK(cudaLaunchCooperativeKernel(batch_kernel_for(kind), dim3((unsigned)grid),
                                               dim3(256), args, 0, s));
}

}  // namespace grada

// ---- host side ---------------------------------------------------------------

#include <dlfcn.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <mutex>
#include <numeric>
#include <string>
#include <vector>

#include "context.h"

namespace grada {

namespace {
double *dbuf(const DevBuf &b) { return b.as<double>(); }
}  // namespace

// This context's inversion as a BatchProblem, after invert_setup.
void Context::batch_problem(const grada_invert_params &prm, BatchProblem &bp) {
  const bool fp64 = g_storage == GRADA_G_FP64;
  const bool stored = fp64 || g_storage == GRADA_G_FP32 || g_storage == GRADA_G_BF16_ROWSCALE ||
                      g_storage == GRADA_G_FP16_ROWSCALE;
  if (!stored || (!fp64 && !predict_fp64))
    throw Error(GRADA_ERR_STATE,
                "the persistent batch runs an FP64 G, or a reduced-precision G with the FP64 G "
                "kept (grada_keep_fp64_G) and fp64_refinement set; use grada_invert_batch");
  for (int t = 0; t < 4; t++)
    if (!ops[t].set) throw Error(GRADA_ERR_STATE, "regularisation operators Ws/Wx/Wy/Wz not set");
  const int nterms = crg_enabled ? 7 : 4;
  const int64_t Nm = n_cells, Nd = nd, nrow = Nd + (int64_t)nterms * Nm;
  ensure_cg_workspace(nterms);
  const DevG g = devG();
  int64_t need = product_scratch_doubles();
  if (predict_fp64) need = std::max(need, gemv_scratch_doubles(devG64(), sm_count));
  double *scr = scratch_doubles(need);
  bt_part2.alloc(this, sizeof(double) * (size_t)sm_count * 4);
  const int max_trials = prm.gn_iterations * prm.n_lambda;
  bt_trials.alloc(this, sizeof(double) * 5 * (size_t)max_trials);
  bt_iters.alloc(this, sizeof(double) * 3 * (size_t)prm.gn_iterations);
  bt_report.alloc(this, sizeof(double) * 8);
  GRADA_CUDA_CHECK(cudaMemsetAsync(bt_report.ptr, 0, sizeof(double) * 8, stream));

  double *wlv = dbuf(iv_wl);
  const double *WL[7] = {wlv, wlv + Nm, wlv + 2 * Nm, wlv + 3 * Nm, wlv + 4 * Nm, wlv + 5 * Nm,
                         wlv + 6 * Nm};
  const CgTerms T = cg_terms(1.0, WL, dbuf(cg_b), dbuf(cg_s), dbuf(cg_t));  // c of terms 0-3 set per trial

  bp = BatchProblem();
  FusedCgArgs &a = bp.cg;
  a.G = g.data;
  a.row_scale = g.row_scale;
  a.nd = g.nd;
  a.nm = g.nm;
  a.ld = g.ld;
  // the single solve's partition, so both paths sum alike
  if (fused_grid[(int)g.kind] <= 0) fused_grid[(int)g.kind] = fused_cg_grid(g.kind, sm_count);
  fused_gx_partition(g, sm_count, a.tiles, a.splits, a.per);
  if ((int64_t)a.splits * g.ld > need) scr = scratch_doubles((int64_t)a.splits * g.ld);
  a.scratch = scr;
  a.wd = dbuf(wd);
  a.r = dbuf(cg_r);
  a.p = dbuf(cg_p);
  cg_p2.alloc(this, sizeof(double) * (size_t)Nm);
  a.p2 = dbuf(cg_p2);
  a.pp = dbuf(cg_pp);
  a.dx = dbuf(iv_dx);
  a.t = dbuf(cg_t);
  a.s = dbuf(cg_s);
  a.gtw = dbuf(cg_gtw);
  a.P = dbuf(iv_P);
  a.nrow = nrow;
  a.FT = T.FT;
  a.AT = T.AT_s;
  a.part = dbuf(cg_part);
  a.nb_m = dot_blocks(Nm, sm_count);
  a.nb_row = dot_blocks(nrow, sm_count);
  a.scal = dbuf(cg_scal);
  int64_t red_d = 0, red_c = 0;
  fused_red_sizes(Nd, Nm, nterms, red_d, red_c);
  cg_red.alloc(this, sizeof(double) * (size_t)red_d);
  cg_redc.alloc(this, sizeof(unsigned) * (size_t)red_c);
  GRADA_CUDA_CHECK(cudaMemsetAsync(cg_redc.ptr, 0, sizeof(unsigned) * (size_t)red_c, stream));
  a.red = dbuf(cg_red);
  a.red_count = cg_redc.as<unsigned>();

  bp.dobs = dbuf(dobs);
  bp.b = dbuf(cg_b);
  bp.atb = dbuf(cg_atb);
  bp.gx = dbuf(cg_gx);
  bp.tmpd = dbuf(cg_tmpd);
  bp.part2 = dbuf(bt_part2);
  for (int k = 0; k < 7; k++) {
    bp.seg_A[k] = T.seg_A[k];
    bp.seg_wl[k] = T.seg_wl[k];
  }
  bp.AT_b = T.AT_b;
  bp.AT_s0 = T.AT_s0;
  bp.nterms = nterms;
  const DevG gp = predict_fp64 ? devG64() : g;
  bp.Gp = static_cast<const double *>(gp.data);
  bp.p_splits = gx_splits(gp, sm_count, 2);
  bp.p_tiles = (int)ceil_div(gp.ld, (int64_t)256 * 2);
  bp.p_per = ceil_div(gp.nm, bp.p_splits);
  bp.nb_d = dot_blocks(Nd, sm_count);
  bp.m = dbuf(iv_m);
  bp.mt = dbuf(iv_mt);
  bp.mt_old = dbuf(iv_mt_old);
  bp.mopt = dbuf(iv_mopt);
  bp.P = dbuf(iv_P);
  bp.dpre = dbuf(iv_dpre);
  bp.wl = wlv;
  bp.mmin = dbuf(iv_mmin);
  bp.mmax = dbuf(iv_mmax);
  bp.m0 = dbuf(iv_m0);
  bp.guard = iv_guard.as<int>();
  bp.flag = iv_flag.as<int>();
  for (int q = 0; q < 7; q++) bp.irls_A[q] = ops[q].A();
  bp.prm = prm;
  const double rate = prm.lambda_decreasing_rate;
  // the powers Context::invert evaluates on the host (same calls, same values)
  bp.lambda_up = std::pow(1 / rate, std::min(3, prm.n_lambda - 2));
  bp.min_lambda = std::min(prm.max_lambda * std::pow(rate, 20), 1.0e-5);
  const double p_expo[5] = {-(2 - prm.lp_s) / 4.0, -(2 - prm.lp_x) / 4.0, -(2 - prm.lp_y) / 4.0,
                            -(2 - prm.lp_z) / 4.0, -(2 - prm.lp_t) / 4.0};
  for (int q = 0; q < 5; q++) bp.p_expo[q] = p_expo[q];
  bp.crg = crg_enabled ? 1 : 0;
  if (prm.cg_iteration_factor < 1) bp.cg_maxit = (int)(prm.cg_iteration_factor * Nm);
  else bp.cg_maxit = (int)prm.cg_iteration_factor;
  bp.trials = dbuf(bt_trials);
  bp.max_trials = max_trials;
  bp.iters = dbuf(bt_iters);
  bp.max_iters = prm.gn_iterations;
  bp.report = dbuf(bt_report);
}

// The model and records of this context's problem after the batch launch.
void Context::batch_results(const grada_invert_params &prm, double *h_m_out,
                            grada_invert_report &rep) {
  double r[8];
  download(r, bt_report.ptr, sizeof(r));
  sync();
  std::memset(&rep, 0, sizeof(rep));
  if (r[7] != 1.0) throw Error(GRADA_ERR_CUDA, "persistent batch: the problem did not finish");
  if (r[6] != 0.0)
    throw Error((int)r[6], (int)r[6] == GRADA_ERR_BREAKDOWN ? "CG breakdown: ||t||^2 = 0"
                                                            : "non-finite CG scalar");
  rep.final_misfit = r[0];
  rep.final_lambda = r[1];
  rep.gn_iterations = (int)r[2];
  rep.n_trials = (int)r[3];
  rep.cg_iterations = (int64_t)r[4];
  rep.fp64_refinements = predict_fp64 ? (int64_t)r[5] : 0;
  std::vector<double> t(5 * (size_t)std::max(rep.n_trials, 1)), it(3 * (size_t)std::max(rep.gn_iterations, 1));
  download(t.data(), bt_trials.ptr, sizeof(double) * 5 * (size_t)rep.n_trials);
  download(it.data(), bt_iters.ptr, sizeof(double) * 3 * (size_t)rep.gn_iterations);
  download(h_m_out, iv_m.ptr, sizeof(double) * (size_t)n_cells);
  sync();
  trials.clear();
  iterations.clear();
  for (int k = 0; k < rep.n_trials; k++)
    trials.push_back({(int)t[5 * k], t[5 * k + 1], t[5 * k + 2], (int)t[5 * k + 3], t[5 * k + 4]});
  for (int k = 0; k < rep.gn_iterations; k++)
    iterations.push_back({(int)it[3 * k], (int)it[3 * k + 1], it[3 * k + 2]});
  (void)prm;
}

// ---- team sizes: the tuning table ----------------------------------------------

namespace {

// Rows (largest G of the batch in entries, CTAs per team, -1 for one team per
// problem sized by its G), ascending; the batch takes the first row whose
// bound holds its largest problem.  Loaded
// from the file grada_load_batch_tuning names or, on first use, from
// tuning/batch_teams.tsv beside the library (graada3d_gb300/autotune.py
// writes it); without a table, a team of 8.
std::mutex g_tune_mutex;
std::vector<std::pair<double, int>> g_tune_rows;
bool g_tune_tried = false;

std::vector<std::pair<double, int>> read_table(const char *path) {
  std::vector<std::pair<double, int>> rows;
  std::ifstream f(path);
  if (!f) return rows;
  std::string line;
  while (std::getline(f, line)) {
    if (line.empty() || line[0] == '#') continue;
    double bound = 0;
    int team = 0;
    if (std::sscanf(line.c_str(), "%lf %d", &bound, &team) == 2 && team >= -1 && team != 0 &&
        team <= 1024)
      rows.push_back({bound, team});
  }
  std::sort(rows.begin(), rows.end());
  return rows;
}

// The default table beside this library (once per process).
void load_default_table_locked() {
  if (g_tune_tried) return;
  g_tune_tried = true;
  Dl_info info;
  if (!dladdr(reinterpret_cast<void *>(&read_table), &info) || !info.dli_fname) return;
  std::string dir(info.dli_fname);
  const size_t slash = dir.find_last_of('/');
  dir = (slash == std::string::npos) ? std::string(".") : dir.substr(0, slash);
  auto rows = read_table((dir + "/tuning/batch_teams.tsv").c_str());
  if (!rows.empty()) g_tune_rows = rows;
}

}  // namespace

int load_batch_tuning(const char *path) {
  std::ifstream f(path);
  if (!f) return GRADA_ERR_INVALID_ARGUMENT;
  f.close();
  auto rows = read_table(path);
  if (rows.empty()) return GRADA_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(g_tune_mutex);
  g_tune_rows = rows;
  g_tune_tried = true;
  return GRADA_OK;
}

int tuned_team_ctas(double max_entries) {
  std::lock_guard<std::mutex> lock(g_tune_mutex);
  load_default_table_locked();
  for (const auto &r : g_tune_rows)
    if (max_entries <= r.first) return r.second;
  return g_tune_rows.empty() ? 8 : g_tune_rows.back().second;
}


// grada_invert_batch_persistent: see include/grada_gpu.h.
int invert_batch_persistent(int n, Context *const *ctxs, const grada_invert_params *params,
                            const double *const *m_ini, const double *const *m_min,
                            const double *const *m_max, const double *const *m0s,
                            double *const *m_out, grada_invert_report *reports, int team_ctas,
                            int *statuses, std::string &err) {
  if (n <= 0) return GRADA_OK;
  Context *c0 = ctxs[0];
  std::vector<BatchProblem> probs(n);
  std::vector<int> order(n);
  std::iota(order.begin(), order.end(), 0);
  double max_entries = 0;
  struct PredictReset {
    Context *const *c;
    int n;
    ~PredictReset() {
      for (int k = 0; k < n; k++) c[k]->predict_fp64 = false;
    }
  } reset{ctxs, n};
  for (int k = 0; k < n; k++) {
    Context *c = ctxs[k];
    if (c->device != c0->device) {
      err = "every context of a persistent batch must be on the same device";
      return GRADA_ERR_INVALID_ARGUMENT;
    }
    if (c->g_storage != c0->g_storage) {
      err = "every problem of a persistent batch must store G the same way";
      return GRADA_ERR_INVALID_ARGUMENT;
    }
    try {
      c->invert_setup(params[k], m_ini[k], m_min[k], m_max[k], m0s ? m0s[k] : nullptr);
      c->batch_problem(params[k], probs[k]);
      c->sync();
    } catch (const Error &e) {
      err = "problem " + std::to_string(k) + ": " + e.what();
      if (statuses) statuses[k] = e.status;
      return e.status;
    }
    max_entries = std::max(max_entries, (double)c->nd * (double)c->n_cells);
  }
  // largest problems first: the last ones a team takes are the short ones
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
    return (double)ctxs[x]->nd * ctxs[x]->n_cells > (double)ctxs[y]->nd * ctxs[y]->n_cells;
  });
  std::vector<BatchProblem> sorted(n);
  for (int k = 0; k < n; k++) sorted[k] = probs[order[k]];
  try {
    const GKind kind = (GKind)c0->g_storage;
    const int resident = invert_batch_resident(kind, c0->sm_count);
    // team_ctas > 0: teams of that size take problems from the queue; 0: the
    // tuning table's choice; a table value (or team_ctas) of -1: one team per
    // problem, sized in proportion to its G, all problems at once
    int team = team_ctas != 0 ? team_ctas : tuned_team_ctas(max_entries);
    if (team < 0 && n > resident) team = 8;  // more problems than CTAs: queue
    std::vector<int> team_of, rank_of, size_of, first_of;
    int grid = 0;
    if (team > 0) {
      if (team > resident) throw Error(GRADA_ERR_INVALID_ARGUMENT, "team larger than the resident grid");
      const int nt = resident / team;
      grid = nt * team;
      for (int c = 0; c < grid; c++) {
        team_of.push_back(c / team);
        rank_of.push_back(c % team);
      }
      size_of.assign(nt, team);
      first_of.assign(nt, -1);
    } else {
      // sizes in proportion to each problem's G entries, at least one CTA each,
      // the resident CTAs left over by the rounding given to the largest
      std::vector<double> w(n);
      double W = 0;
      for (int k = 0; k < n; k++) {
        w[k] = (double)ctxs[order[k]]->nd * (double)ctxs[order[k]]->n_cells;
        W += w[k];
      }
      size_of.assign(n, 1);
      int used = n;
      for (int k = 0; k < n; k++) {
        const int extra = std::max(0, (int)std::floor(resident * w[k] / W) - 1);
        const int take = std::min(extra, resident - used);
        size_of[k] += take;
        used += take;
      }
      for (int k = 0; used < resident; k = (k + 1) % n, used++) size_of[k]++;
      for (int t = 0; t < n; t++) {
        for (int r = 0; r < size_of[t]; r++) {
          team_of.push_back(t);
          rank_of.push_back(r);
        }
        first_of.push_back(t);
      }
      grid = (int)team_of.size();
    }
    const int n_teams = (int)size_of.size();
    DevBuf d_probs, d_words, d_map;
    d_probs.alloc(c0, sizeof(BatchProblem) * (size_t)n);
    // queue (1 int), then per team its barrier words, then a 32-int problem slot per team
    const size_t bw = fused::kBarrierWords;
    const size_t words = 32 + (bw + 32) * (size_t)n_teams;
    d_words.alloc(c0, sizeof(unsigned) * words);
    std::vector<int> map;
    map.insert(map.end(), team_of.begin(), team_of.end());
    map.insert(map.end(), rank_of.begin(), rank_of.end());
    map.insert(map.end(), size_of.begin(), size_of.end());
    map.insert(map.end(), first_of.begin(), first_of.end());
    d_map.alloc(c0, sizeof(int) * map.size());
    c0->upload(d_map.ptr, map.data(), sizeof(int) * map.size());
    c0->upload(d_probs.ptr, sorted.data(), sizeof(BatchProblem) * (size_t)n);
    int *queue = d_words.as<int>();
    unsigned *bars = d_words.as<unsigned>() + 32;
    int *slots = d_words.as<int>() + 32 + bw * (size_t)n_teams;
    // problems handed out in advance (one per team in the proportional layout)
    int handed = 0;
    for (int f : first_of) handed += (f >= 0) ? 1 : 0;
    unsigned long long wait_ns = 2000000000ull;
    if (c0->inject_cg_wait) {
      c0->inject_cg_wait = false;
      wait_ns = 0;
    }
    // one CUDA graph: clear the queue and barrier words, the cooperative launch
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    GRADA_CUDA_CHECK(cudaStreamBeginCapture(c0->stream, cudaStreamCaptureModeThreadLocal));
    try {
      GRADA_CUDA_CHECK(cudaMemsetAsync(d_words.ptr, 0, sizeof(unsigned) * words, c0->stream));
      launch_invert_batch(d_probs.as<BatchProblem>(), n, queue, handed, bars, slots,
                          d_map.as<int>(), n_teams, grid, kind, wait_ns, c0->stream);
    } catch (...) {
      cudaGraph_t gph = nullptr;
      cudaStreamEndCapture(c0->stream, &gph);
      if (gph) cudaGraphDestroy(gph);
      throw;
    }
    GRADA_CUDA_CHECK(cudaStreamEndCapture(c0->stream, &graph));
    const cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    GRADA_CUDA_CHECK(ie);
    const cudaError_t le = cudaGraphLaunch(exec, c0->stream);
    const cudaError_t se = cudaStreamSynchronize(c0->stream);
    cudaGraphExecDestroy(exec);
    GRADA_CUDA_CHECK(le);
    GRADA_CUDA_CHECK(se);
    std::vector<unsigned> h_words(words);
    c0->download(h_words.data(), d_words.ptr, sizeof(unsigned) * words);
    c0->sync();
    for (int t = 0; t < n_teams; t++)
      if (h_words[32 + bw * (size_t)t + 224])
        throw Error(GRADA_ERR_CUDA, "persistent batch: a team barrier wait expired");
    c0->last_batch_teams = n_teams;
    c0->last_batch_team_ctas = team > 0 ? team : -1;
  } catch (const Error &e) {
    err = e.what();
    return e.status;
  }
  int first = GRADA_OK;
  for (int k = 0; k < n; k++) {
    int st = GRADA_OK;
    try {
      grada_invert_report rep;
      ctxs[k]->batch_results(params[k], m_out[k], rep);
      if (reports) reports[k] = rep;
    } catch (const Error &e) {
      st = e.status;
      if (first == GRADA_OK) err = "problem " + std::to_string(k) + ": " + e.what();
    }
    if (statuses) statuses[k] = st;
    if (first == GRADA_OK) first = st;
  }
  return first;
}

}  // namespace grada
