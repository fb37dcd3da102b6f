// Blocks of right-hand sides on one G: block products, the block CG solve
// and the fixed-lambda regularisation sweep.
//
// Reference: GaussNewtonInversion::solve_cg (src/Inversion/
// GaussNewtonInversion.cpp:1417-1698) and invert_with_own_CG (:657-1103).
// solve_cg_block_dev is solve_cg_dev (inversion.cu) for kBW = 16 systems at
// once: the same stacked rows, the same quirks, every column with its own
// lambda, model, P, weights, scalars and stopping test.  One CG iteration
// reads G twice for all sixteen columns (tensor-core GEMMs for FP32 and
// 16-bit G) instead of twice per column.
//
// The sweep runs, for each lambda of a list, the reference's Gauss-Newton
// loop with a single lambda trial per iteration (n_lambda = 1, max_lambda =
// that lambda: lambda is then max_lambda at every iteration, :833-836), all
// columns in lockstep; a column whose run has stopped (target misfit, last
// iteration, stagnation) is frozen and drops out of later block solves.
#include <cmath>
#include <cstring>

#include "common.cuh"
#include "context.h"

namespace grada {

namespace {

double *dptr(const DevBuf &b) { return b.as<double>(); }

}  // namespace

void Context::ensure_block_scratch(bool fp64_forward) {
  require_G();
  int64_t bytes = 0;
  if (g_storage == GRADA_G_MATRIX_FREE || fp64_forward)
    bytes = mf_block_scratch_doubles(geometry(), sm_count) * (int64_t)sizeof(double);
  if (g_storage != GRADA_G_MATRIX_FREE)
    bytes = std::max(bytes, block_scratch_bytes(devG(), sm_count));
  if (fp64_resident()) bytes = std::max(bytes, block_scratch_bytes(devG64(), sm_count));
  bscratch.alloc(this, (size_t)std::max<int64_t>(bytes, 256));
  if (!tc_err.ptr) {
    tc_err.alloc(this, sizeof(int) * 4);
    GRADA_CUDA_CHECK(cudaMemsetAsync(tc_err.ptr, 0, sizeof(int) * 4, stream));
  }
  if (!h_bflag) GRADA_CUDA_CHECK(cudaMallocHost(&h_bflag, sizeof(int) * (kBW + 1)));
}

void Context::apply_G_block(const double *X, double *Y, const GemvOpts &o) {
  if (g_storage == GRADA_G_MATRIX_FREE)
    launch_forward_field_block(geometry(), X, Y, dptr(bscratch), sm_count, stream, o);
  else
    launch_G_mat_mul(devG(), X, Y, bscratch.ptr, sm_count, stream, o, tc_err.as<int>());
}

void Context::apply_GT_block(const double *Y, double *X, const GemvOpts &o) {
  if (g_storage == GRADA_G_MATRIX_FREE)
    launch_adjoint_field_block(geometry(), Y, X, dptr(bscratch), sm_count, stream, o);
  else
    launch_GT_mat_mul(devG(), Y, X, bscratch.ptr, sm_count, stream, o, tc_err.as<int>());
}

// Reads the tensor-core wait flags (after a synchronisation point of the
// caller's stream order) and turns a raised flag into an error.
void Context::check_tc_error() {
  if (!tc_err.ptr) return;
  GRADA_CUDA_CHECK(cudaMemcpyAsync(h_bflag + kBW, tc_err.ptr, sizeof(int), cudaMemcpyDeviceToHost,
                                   stream));
  sync();
  const int e = h_bflag[kBW];
  if (e) {
    GRADA_CUDA_CHECK(cudaMemsetAsync(tc_err.ptr, 0, sizeof(int) * 2, stream));  // flags, test arm
    sync();
    throw Error(GRADA_ERR_CUDA, "tensor-core block product: a bounded wait expired (flags " +
                                    std::to_string(e) + ")");
  }
}

void Context::ensure_block_workspace(int nterms) {
  const int64_t Nm = n_cells;
  const int64_t nrow = nd + (int64_t)nterms * Nm;
  const size_t W = sizeof(double) * kBW;
  bk_b.alloc(this, W * nrow);
  bk_s.alloc(this, W * nrow);
  bk_t.alloc(this, W * nrow);
  bk_p.alloc(this, W * Nm);
  bk_pp.alloc(this, W * Nm);
  bk_r.alloc(this, W * Nm);
  bk_atb.alloc(this, W * Nm);
  bk_gtw.alloc(this, W * Nm);
  bk_gx.alloc(this, W * ld);
  bk_tmpd.alloc(this, W * ld);
  bk_scal.alloc(this, sizeof(double) * kBW * CG_NSCALARS);
  bk_part.alloc(this, W * (size_t)sm_count * 4);
  bk_ctl.alloc(this, sizeof(int) * CTLB_NINTS);
  if (!h_bscal) GRADA_CUDA_CHECK(cudaMallocHost(&h_bscal, sizeof(double) * kBW * CG_NSCALARS));
  if (!h_bctl) GRADA_CUDA_CHECK(cudaMallocHost(&h_bctl, sizeof(int) * CTLB_NINTS));
  ensure_cg_workspace(nterms);  // crg operators, pinned scalars
}

// out = G m (block) in the precision of G; with d64: d64 + G (m - m_start).
void Context::block_prediction(const double *m, const double *m_start, const double *d64,
                               double *out) {
  if (predict_fp64) {  // FP64 block product with the kept FP64 G
    launch_G_mat_mul(devG64(), m, out, bscratch.ptr, sm_count, stream, GemvOpts(),
                     tc_err.as<int>());
    fp64_products++;
  } else if (d64) {
    double *dm = dptr(sw_tmp2);
    launch_sub(m, m_start, n_cells * kBW, dm, stream);
    apply_G_block(dm, out, GemvOpts());
    launch_add(out, d64, nd * kBW, out, stream);
  } else {
    apply_G_block(m, out, GemvOpts());
  }
}

// Per-column misfit sqrt(||Wd (G m - dobs)||^2 / Nd)  (GaussNewtonInversion.cpp:916).
void Context::block_misfits(const double *m, const double *m_start, const double *d64,
                            double *out) {
  double *g = dptr(sw_dpre);
  block_prediction(m, m_start, d64, g);
  double *scal = dptr(bk_scal);
  launch_bmisfit_sq(g, dptr(dobs), dptr(wd), nd, dptr(bk_part), dot_blocks(nd, sm_count), scal,
                    CG_MISFIT2, stream);
  GRADA_CUDA_CHECK(cudaMemcpyAsync(h_bscal, scal, sizeof(double) * kBW * CG_NSCALARS,
                                   cudaMemcpyDeviceToHost, stream));
  sync();
  check_tc_error();
  for (int c = 0; c < kBW; c++) out[c] = std::sqrt(h_bscal[c * CG_NSCALARS + CG_MISFIT2] / (double)nd);
}

void Context::solve_cg_block_dev(const double *lambda, uint32_t active, double tol, int maxit,
                                 const double *mk, const double *mref, const double *P,
                                 const double *const WL[7], double *dx, const double *d64,
                                 const double *m_start, CgResult *res) {
  NvtxRange nvtx("grada solve_cg_block");
  require_G();
  if (!data_set) throw Error(GRADA_ERR_STATE, "observed data not set (grada_set_data)");
  for (int t = 0; t < 4; t++)
    if (!ops[t].set) throw Error(GRADA_ERR_STATE, "regularisation operators Ws/Wx/Wy/Wz not set");
  const int nterms = crg_enabled ? 7 : 4;
  ensure_block_workspace(nterms);
  ensure_block_scratch(false);
  const int64_t Nm = n_cells, Nd = nd, nrow = Nd + (int64_t)nterms * Nm;
  double sl[kBW];
  for (int c = 0; c < kBW; c++) sl[c] = ((active >> c) & 1u) ? std::sqrt(lambda[c]) : 0.0;
  const double *WL_s = WL[0], *WL_x = WL[1], *WL_y = WL[2], *WL_z = WL[3];
  const double *WL_tx = WL[4], *WL_ty = WL[5], *WL_tz = WL[6];
  const DevOperator *seg_op[7] = {&ops[GRADA_OP_WS], &ops[GRADA_OP_WZ], &ops[GRADA_OP_WX],
                                  &ops[GRADA_OP_WY], &crg[2], &crg[0], &crg[1]};
  double *b = dptr(bk_b), *s = dptr(bk_s), *t = dptr(bk_t);
  double *p = dptr(bk_p), *pp = dptr(bk_pp), *r = dptr(bk_r), *atb = dptr(bk_atb);
  double *gtw = dptr(bk_gtw), *gx = dptr(bk_gx), *tmpd = dptr(bk_tmpd);
  double *scal = dptr(bk_scal), *part = dptr(bk_part);
  auto seg = [&](double *base, int k) { return base + (Nd + (int64_t)k * Nm) * kBW; };
  const int nb_m = dot_blocks(Nm, sm_count), nb_row = dot_blocks(nrow, sm_count);
  for (int c = 0; c < kBW; c++) res[c] = CgResult();

  // per-column coefficient arrays on the device: -sqrt(lambda), -1
  double hc[2][kBW];
  for (int c = 0; c < kBW; c++) {
    hc[0][c] = -sl[c];
    hc[1][c] = -1.0;
  }
  bk_coef.alloc(this, sizeof(hc));
  double *dcoef = dptr(bk_coef);
  upload(dcoef, hc, sizeof(hc));

  // b and s = -b   (GaussNewtonInversion.cpp:1458-1472)
  block_prediction(mk, m_start, d64, gx);
  launch_bdata_residual(dptr(dobs), gx, dptr(wd), Nd, b, s, stream);
  launch_bcsr_apply(seg_op[0]->A(), mk, mref, dcoef, WL_s, seg(b, 0), stream);
  launch_bcsr_apply(seg_op[1]->A(), mk, nullptr, dcoef, WL_z, seg(b, 1), stream);
  launch_bcsr_apply(seg_op[2]->A(), mk, nullptr, dcoef, WL_x, seg(b, 2), stream);
  launch_bcsr_apply(seg_op[3]->A(), mk, nullptr, dcoef, WL_y, seg(b, 3), stream);
  if (crg_enabled) {
    launch_bcsr_apply(seg_op[4]->A(), mk, nullptr, dcoef + kBW, WL_tz, seg(b, 4), stream);
    launch_bcsr_apply(seg_op[5]->A(), mk, nullptr, dcoef + kBW, WL_tx, seg(b, 5), stream);
    launch_bcsr_apply(seg_op[6]->A(), mk, nullptr, dcoef + kBW, WL_ty, seg(b, 6), stream);
  }
  launch_negate(b + Nd * kBW, (nrow - Nd) * kBW, s + Nd * kBW, stream);

  // A^T b and the initial r (:1485-1551)
  launch_bscale_rows(b, dptr(wd), Nd, tmpd, stream);
  apply_GT_block(tmpd, gtw, GemvOpts());
  BAdjointTerms AT_b, AT_s0, AT_s;
  const double *adj_wl[7] = {WL_s, WL_z, WL_x, WL_y, WL_tz, WL_tx, WL_ty};
  for (int k = 0; k < nterms; k++) {
    for (int c = 0; c < kBW; c++) AT_b.c[k][c] = (k < 4) ? sl[c] : 1.0;
    AT_b.AT[k] = seg_op[k]->AT();
    AT_b.wl[k] = adj_wl[k];
    AT_b.s[k] = seg(b, k);
  }
  AT_b.count = nterms;
  AT_s = AT_b;
  for (int k = 0; k < nterms; k++) AT_s.s[k] = seg(s, k);
  AT_s0 = AT_s;
  if (nterms == 7) AT_s0.wl[6] = WL_y;  // the initial adjoint weights the crg-y rows by WL_y (:1508)
  launch_badjoint(AT_b, Nm, P, gtw, 1.0, atb, stream, nullptr);
  launch_badjoint(AT_s0, Nm, P, gtw, -1.0, r, stream, nullptr);
  GRADA_CUDA_CHECK(cudaMemsetAsync(scal, 0, sizeof(double) * kBW * CG_NSCALARS, stream));
  launch_bdot(atb, nullptr, Nm, part, nb_m, scal, CG_ATB2, stream, nullptr);
  GRADA_CUDA_CHECK(cudaMemsetAsync(p, 0, sizeof(double) * kBW * Nm, stream));
  GRADA_CUDA_CHECK(cudaMemsetAsync(dx, 0, sizeof(double) * kBW * Nm, stream));
  GRADA_CUDA_CHECK(cudaMemsetAsync(t, 0, sizeof(double) * kBW * nrow, stream));
  launch_bdot(r, nullptr, Nm, part, nb_m, scal, CG_R2, stream, nullptr);

  // forward rows of t = A p (:1569-1586)
  BForwardTerms FT;
  const double *fwd_wl[7] = {nullptr, WL_z, WL_x, WL_y, WL_z, WL_x, WL_y};
  for (int k = 0; k < nterms; k++) {
    FT.A[k] = seg_op[k]->A();
    for (int c = 0; c < kBW; c++) FT.c[k][c] = (k < 4) ? sl[c] : 1.0;
    FT.wl[k] = fwd_wl[k];
    FT.out[k] = seg(t, k);
  }
  FT.count = nterms;

  GRADA_CUDA_CHECK(cudaMemcpyAsync(h_bscal, scal, sizeof(double) * kBW * CG_NSCALARS,
                                   cudaMemcpyDeviceToHost, stream));
  sync();
  check_tc_error();
  if (maxit <= 0) return;
  // Columns that run: active ones with a non-zero right-hand side (a zero one
  // is solved by dx = 0, as in solve_cg_dev).
  uint32_t running = 0;
  for (int c = 0; c < kBW; c++)
    if (((active >> c) & 1u) && h_bscal[c * CG_NSCALARS + CG_R2] != 0.0) running |= 1u << c;
  if (!running) return;
  for (int i = 0; i < CTLB_NINTS; i++) h_bctl[i] = 0;
  for (int c = 0; c < kBW; c++) {
    int *cc = h_bctl + CTLB_COL + c * CTL_NINTS;
    cc[CTL_DONE] = ((running >> c) & 1u) ? 0 : 1;
    cc[CTL_MAXIT] = maxit;
    cc[CTL_STATUS] = CG_STATUS_RUNNING;
    h_bscal[c * CG_NSCALARS + CG_TOL] = tol;
  }
  int *ctl = bk_ctl.as<int>();
  upload(ctl, h_bctl, sizeof(int) * CTLB_NINTS);
  upload(scal, h_bscal, sizeof(double) * kBW * CG_NSCALARS);
  const double *wdp = dptr(wd);
  auto iteration = [&]() {
    launch_bp_update(r, P, scal, Nm, p, pp, stream, ctl);
    GemvOpts o;
    o.skip = ctl;
    o.scale = wdp;
    apply_G_block(pp, t, o);
    launch_bmulti_forward(FT, Nm, pp, stream, ctl);
    launch_bdot(t, nullptr, nrow, part, nb_row, scal, CG_T2, stream, ctl);
    launch_balpha(scal, ctl, stream);
    launch_baxpy(t, p, scal, nrow, Nm, s, dx, stream, ctl);
    apply_GT_block(s, gtw, o);
    launch_badjoint(AT_s, Nm, P, gtw, 1.0, r, stream, ctl);
    launch_bdot(r, nullptr, Nm, part, nb_m, scal, CG_R2NEW, stream, ctl);
    launch_bbeta(scal, ctl, stream);
  };
  const int K = std::min(maxit, kCgGraphIters);
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  GRADA_CUDA_CHECK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
  try {
    for (int k = 0; k < K; k++) iteration();
  } catch (...) {
    cudaGraph_t g = nullptr;
    cudaStreamEndCapture(stream, &g);
    if (g) cudaGraphDestroy(g);
    throw;
  }
  GRADA_CUDA_CHECK(cudaStreamEndCapture(stream, &graph));
  cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  GRADA_CUDA_CHECK(ie);
  int launched = 0;
  try {
    while (true) {
      GRADA_CUDA_CHECK(cudaGraphLaunch(exec, stream));
      launched += K;
      GRADA_CUDA_CHECK(cudaMemcpyAsync(h_bctl, ctl, sizeof(int) * CTLB_NINTS,
                                       cudaMemcpyDeviceToHost, stream));
      GRADA_CUDA_CHECK(cudaMemcpyAsync(h_bscal, scal, sizeof(double) * kBW * CG_NSCALARS,
                                       cudaMemcpyDeviceToHost, stream));
      sync();
      check_tc_error();
      if (h_bctl[CTLB_ALL] || launched >= maxit) break;
    }
  } catch (...) {
    cudaGraphExecDestroy(exec);
    throw;
  }
  cudaGraphExecDestroy(exec);
  for (int c = 0; c < kBW; c++) {
    if (!((running >> c) & 1u)) continue;
    const int *cc = h_bctl + CTLB_COL + c * CTL_NINTS;
    res[c].iterations = cc[CTL_ITER];
    res[c].err = h_bscal[c * CG_NSCALARS + CG_ERR];
    if (cc[CTL_STATUS] == CG_STATUS_BREAKDOWN)
      throw Error(GRADA_ERR_BREAKDOWN, "CG breakdown in column " + std::to_string(c) +
                                           ": ||t||^2 = 0 at iteration " +
                                           std::to_string(res[c].iterations));
    if (cc[CTL_STATUS] == CG_STATUS_NONFINITE)
      throw Error(GRADA_ERR_NONFINITE, "non-finite CG scalar in column " + std::to_string(c) +
                                           " at iteration " + std::to_string(res[c].iterations));
  }
}

// ---- host-array entry points ----------------------------------------------

void Context::G_mat_mul_host(int n, const double *X, double *Y, bool transpose) {
  require_G();
  if (n < 1 || !X || !Y) throw Error(GRADA_ERR_INVALID_ARGUMENT, "bad block product arguments");
  ensure_block_scratch(false);
  const int64_t rin = transpose ? nd : n_cells, rout = transpose ? n_cells : nd;
  sw_in.alloc(this, sizeof(double) * kBW * std::max(rin, rout));
  sw_out.alloc(this, sizeof(double) * kBW * std::max(ld, n_cells));
  sw_tmp.alloc(this, sizeof(double) * kBW * std::max(rin, rout));
  for (int c0 = 0; c0 < n; c0 += kBW) {
    const int nc = std::min(kBW, n - c0);
    double *tmp = dptr(sw_tmp);
    upload(tmp, X + (int64_t)c0 * rin, sizeof(double) * rin * nc);
    launch_bpack(tmp, rin, nc, dptr(sw_in), stream);
    if (transpose) apply_GT_block(dptr(sw_in), dptr(sw_out), GemvOpts());
    else apply_G_block(dptr(sw_in), dptr(sw_out), GemvOpts());
    launch_bunpack(dptr(sw_out), rout, nc, tmp, stream);
    download(Y + (int64_t)c0 * rout, tmp, sizeof(double) * rout * nc);
    sync();
    check_tc_error();
  }
}

void Context::solve_cg_block_host(double tol, int maxit, int n, const double *lambda,
                                  const double *mk, const double *mref, const double *P,
                                  const double *const WL[7], double *dx, double *err, int *iters) {
  require_G();
  if (n < 1 || !lambda || !mk || !mref || !P || !dx || !err || !iters)
    throw Error(GRADA_ERR_INVALID_ARGUMENT, "null argument to the block solve");
  const int64_t Nm = n_cells;
  const size_t bb = sizeof(double) * kBW * Nm;
  sw_m.alloc(this, bb);
  sw_P.alloc(this, bb);
  sw_dx.alloc(this, bb);
  sw_m0.alloc(this, sizeof(double) * Nm);
  sw_wl.alloc(this, bb * 7);
  sw_tmp.alloc(this, bb);
  upload(sw_m0.ptr, mref, sizeof(double) * Nm);
  double *tmp = dptr(sw_tmp);
  for (int c0 = 0; c0 < n; c0 += kBW) {
    const int nc = std::min(kBW, n - c0);
    auto put = [&](const double *h, double *blk) {
      upload(tmp, h + (int64_t)c0 * Nm, sizeof(double) * Nm * nc);
      launch_bpack(tmp, Nm, nc, blk, stream);
    };
    put(mk, dptr(sw_m));
    put(P, dptr(sw_P));
    const double *wl[7];
    for (int k = 0; k < 7; k++) {
      wl[k] = nullptr;
      if (WL && WL[k]) {
        double *blk = dptr(sw_wl) + (int64_t)k * kBW * Nm;
        put(WL[k], blk);
        wl[k] = blk;
      }
    }
    double lam[kBW] = {0};
    for (int c = 0; c < nc; c++) lam[c] = lambda[c0 + c];
    const uint32_t active = (nc == 32) ? 0xffffffffu : ((1u << nc) - 1u);
    CgResult res[kBW];
    solve_cg_block_dev(lam, active, tol, maxit, dptr(sw_m), dptr(sw_m0), dptr(sw_P), wl,
                       dptr(sw_dx), nullptr, nullptr, res);
    launch_bunpack(dptr(sw_dx), Nm, nc, tmp, stream);
    download(dx + (int64_t)c0 * Nm, tmp, sizeof(double) * Nm * nc);
    sync();
    for (int c = 0; c < nc; c++) {
      err[c0 + c] = res[c].err;
      iters[c0 + c] = (maxit <= 0) ? maxit : res[c].iterations;
    }
  }
}

// ---- the lambda sweep -------------------------------------------------------

void Context::lambda_sweep(const grada_invert_params &prm, int n, const double *lambdas,
                           const double *h_m_ini, const double *h_mmin, const double *h_mmax,
                           const double *h_m0, double *h_m_out, grada_invert_report *reps) {
  NvtxRange nvtx("grada lambda_sweep");
  require_G();
  if (!data_set) throw Error(GRADA_ERR_STATE, "observed data not set (grada_set_data)");
  if (n < 1 || !lambdas || !h_m_ini || !h_mmin || !h_mmax || !h_m_out || !reps)
    throw Error(GRADA_ERR_INVALID_ARGUMENT, "null or empty sweep argument");
  if (prm.gn_iterations < 1) throw Error(GRADA_ERR_INVALID_ARGUMENT, "gn_iterations must be >= 1");
  for (int c = 0; c < n; c++)
    if (!(lambdas[c] >= 0.0) || !std::isfinite(lambdas[c]))
      throw Error(GRADA_ERR_INVALID_ARGUMENT, "lambda values must be finite and >= 0");
  const int64_t Nm = n_cells;
  sweep_trials.assign(n, {});

  // starting model (GaussNewtonInversion.cpp:757-786), the same for every column
  std::vector<double> m(Nm), mmin(h_mmin, h_mmin + Nm), mmax(h_mmax, h_mmax + Nm);
  std::vector<double> m0(Nm, 0.0);
  if (h_m0) m0.assign(h_m0, h_m0 + Nm);
  for (int64_t i = 0; i < Nm; i++) {
    if (!(mmin[i] < mmax[i])) throw Error(GRADA_ERR_INVALID_ARGUMENT, "m_min must be < m_max");
    if (prm.start_from_reference) {
      m[i] = m0[i];
      if (m[i] > mmax[i] || std::abs(m[i] - mmax[i]) < 1e-7) m[i] = mmax[i] - 0.01;
      if (m[i] < mmin[i] || std::abs(m[i] - mmin[i]) < 1e-7) m[i] = mmin[i] + 0.01;
    } else {
      m[i] = h_m_ini[i];
      if (m[i] > mmax[i] || std::abs(m[i] - mmax[i]) < 1e-7) m[i] = 0.5 * (mmax[i] + mmin[i]);
      if (m[i] < mmin[i] || std::abs(m[i] - mmin[i]) < 1e-7) m[i] = 0.5 * (mmax[i] + mmin[i]);
    }
  }
  const bool refine =
      prm.fp64_refinement && g_storage != GRADA_G_FP64 && g_storage != GRADA_G_MATRIX_FREE;
  // with a kept FP64 G every prediction is an FP64 block product instead
  struct PredictGuard {
    Context *c;
    ~PredictGuard() { c->predict_fp64 = false; }
  } predict_guard{this};
  predict_fp64 = refine && fp64_resident();
  const size_t bb = sizeof(double) * kBW * Nm;
  DevBuf *blocks[] = {&sw_m, &sw_mt, &sw_mt_old, &sw_mopt, &sw_dx, &sw_P, &sw_tmp, &sw_tmp2};
  for (DevBuf *b : blocks) b->alloc(this, bb);
  sw_mmin.alloc(this, sizeof(double) * Nm);
  sw_mmax.alloc(this, sizeof(double) * Nm);
  sw_m0.alloc(this, sizeof(double) * Nm);
  sw_wl.alloc(this, bb * 7);
  sw_dpre.alloc(this, sizeof(double) * kBW * ld);
  sw_guard.alloc(this, sizeof(int) * kBW * Nm);
  sw_flag.alloc(this, sizeof(int) * kBW);
  if (refine) {
    sw_d64.alloc(this, sizeof(double) * kBW * ld);
    sw_mstart.alloc(this, bb);
  }
  const int nterms = crg_enabled ? 7 : 4;
  ensure_block_workspace(nterms);
  ensure_block_scratch(refine && !predict_fp64);
  upload(sw_mmin.ptr, mmin.data(), sizeof(double) * Nm);
  upload(sw_mmax.ptr, mmax.data(), sizeof(double) * Nm);
  upload(sw_m0.ptr, m0.data(), sizeof(double) * Nm);
  {
    std::vector<double> mb((size_t)kBW * Nm), ones((size_t)kBW * Nm * 7, 1.0);
    for (int64_t i = 0; i < Nm; i++)
      for (int c = 0; c < kBW; c++) mb[(size_t)i * kBW + c] = m[i];
    upload(sw_m.ptr, mb.data(), bb);
    upload(sw_wl.ptr, ones.data(), bb * 7);
    sync();
  }
  double *dm = dptr(sw_m), *dmt = dptr(sw_mt), *dmt_old = dptr(sw_mt_old), *dmopt = dptr(sw_mopt);
  double *ddx = dptr(sw_dx), *dP = dptr(sw_P), *dtmp = dptr(sw_tmp);
  double *wlv = dptr(sw_wl);
  const int64_t wstride = (int64_t)kBW * Nm;
  double *WLs = wlv, *WLx = wlv + wstride, *WLy = wlv + 2 * wstride, *WLz = wlv + 3 * wstride;
  double *WLtx = wlv + 4 * wstride, *WLty = wlv + 5 * wstride, *WLtz = wlv + 6 * wstride;
  const double *WL[7] = {WLs, WLx, WLy, WLz, WLtx, WLty, WLtz};
  double *d64 = refine ? dptr(sw_d64) : nullptr;
  double *mstart = refine ? dptr(sw_mstart) : nullptr;
  const double p_expo[5] = {-(2 - prm.lp_s) / 4.0, -(2 - prm.lp_x) / 4.0, -(2 - prm.lp_y) / 4.0,
                            -(2 - prm.lp_z) / 4.0, -(2 - prm.lp_t) / 4.0};
  const double rate = prm.lambda_decreasing_rate;

  for (int g0 = 0; g0 < n; g0 += kBW) {
    const int nc = std::min(kBW, n - g0);
    if (g0 > 0) {  // fresh start model and weights for the next group
      std::vector<double> mb((size_t)kBW * Nm), ones((size_t)kBW * Nm * 7, 1.0);
      for (int64_t i = 0; i < Nm; i++)
        for (int c = 0; c < kBW; c++) mb[(size_t)i * kBW + c] = m[i];
      upload(sw_m.ptr, mb.data(), bb);
      upload(sw_wl.ptr, ones.data(), bb * 7);
      sync();
    }
    double lam[kBW] = {0};
    for (int c = 0; c < nc; c++) lam[c] = lambdas[g0 + c];
    grada_invert_report *rp = reps + g0;
    for (int c = 0; c < nc; c++) std::memset(&rp[c], 0, sizeof(grada_invert_report));
    auto refresh_fp64 = [&]() {
      launch_forward_field_block(geometry(), dm, d64, dptr(bscratch), sm_count, stream, GemvOpts());
      GRADA_CUDA_CHECK(cudaMemcpyAsync(mstart, dm, bb, cudaMemcpyDeviceToDevice, stream));
      for (int c = 0; c < nc; c++) rp[c].fp64_refinements++;
    };
    fp64_products = 0;
    if (refine && !predict_fp64) refresh_fp64();
    double misfit[kBW], mli[kBW], trial_misfit[kBW];
    block_misfits(dm, mstart, d64, misfit);
    uint32_t active = (1u << nc) - 1u;
    int cg_maxit = 0;
    if (prm.cg_iteration_factor < 1) cg_maxit = (int)(prm.cg_iteration_factor * Nm);
    else cg_maxit = (int)prm.cg_iteration_factor;
    for (int i = 0; i < prm.gn_iterations && active; i++) {
      for (int c = 0; c < nc; c++) mli[c] = misfit[c];
      if (refine && !predict_fp64 && i > 0) refresh_fp64();
      launch_bp_diag(dm, dptr(sw_mmin), dptr(sw_mmax), Nm, dP, stream);
      CgResult res[kBW];
      solve_cg_block_dev(lam, active, prm.cg_tol, cg_maxit, dm, dptr(sw_m0), dP, WL, ddx, d64,
                         mstart, res);
      // m_trial = m at the start of the iteration; bound transform (:877-911)
      GRADA_CUDA_CHECK(cudaMemcpyAsync(dmt, dm, bb, cudaMemcpyDeviceToDevice, stream));
      GRADA_CUDA_CHECK(cudaMemcpyAsync(dmt_old, dm, bb, cudaMemcpyDeviceToDevice, stream));
      launch_bbound_update(dm, ddx, dptr(sw_mmin), dptr(sw_mmax), Nm, dmt, dmt_old,
                           sw_guard.as<int>(), sw_flag.as<int>(), h_bflag, stream);
      block_misfits(dmt, mstart, d64, trial_misfit);
      launch_bcopy_columns(dmt, Nm, active, dmopt, stream);
      // IRLS weights from m_opt (:962-1022)
      if (prm.lp_s != 2) {
        launch_bcsr_apply(ops[GRADA_OP_WS].A(), dmopt, dptr(sw_m0), nullptr, nullptr, dtmp, stream);
        launch_irls_weight(dtmp, Nm * kBW, prm.epsilon2, p_expo[0], WLs, stream);
      }
      if (prm.lp_x != 2) {
        launch_bcsr_apply(ops[GRADA_OP_WX].A(), dmopt, nullptr, nullptr, nullptr, dtmp, stream);
        launch_irls_weight(dtmp, Nm * kBW, prm.epsilon2, p_expo[1], WLx, stream);
      }
      if (prm.lp_y != 2) {
        launch_bcsr_apply(ops[GRADA_OP_WY].A(), dmopt, nullptr, nullptr, nullptr, dtmp, stream);
        launch_irls_weight(dtmp, Nm * kBW, prm.epsilon2, p_expo[2], WLy, stream);
      }
      if (prm.lp_z != 2) {
        launch_bcsr_apply(ops[GRADA_OP_WZ].A(), dmopt, nullptr, nullptr, nullptr, dtmp, stream);
        launch_irls_weight(dtmp, Nm * kBW, prm.epsilon2, p_expo[3], WLz, stream);
      }
      if (prm.lp_t != 2 && crg_enabled) {
        double *wt[3] = {WLtx, WLty, WLtz};
        for (int q = 0; q < 3; q++) {
          launch_bcsr_apply(ops[GRADA_OP_TX + q].A(), dmopt, nullptr, nullptr, nullptr, dtmp,
                            stream);
          launch_irls_weight(dtmp, Nm * kBW, prm.epsilon2, p_expo[4], wt[q], stream);
        }
      }
      launch_bcopy_columns(dmopt, Nm, active, dm, stream);
      uint32_t next = active;
      for (int c = 0; c < nc; c++) {
        if (!((active >> c) & 1u)) continue;
        sweep_trials[g0 + c].push_back({i + 1, lam[c], trial_misfit[c], res[c].iterations, res[c].err});
        rp[c].cg_iterations += res[c].iterations;
        rp[c].n_trials++;
        rp[c].gn_iterations = i + 1;
        misfit[c] = trial_misfit[c];
        rp[c].final_misfit = misfit[c];
        rp[c].final_lambda = lam[c] * rate;
        const bool stag = std::abs(misfit[c] - mli[c]) / std::min(misfit[c], mli[c]) < prm.stag_tol;
        if (misfit[c] < prm.target_misfit || i == prm.gn_iterations - 1 || stag)
          next &= ~(1u << c);
      }
      active = next;
    }
    if (predict_fp64)
      for (int c = 0; c < nc; c++) rp[c].fp64_refinements = fp64_products;
    launch_bunpack(dm, Nm, nc, dtmp, stream);
    download(h_m_out + (int64_t)g0 * Nm, dtmp, sizeof(double) * Nm * nc);
    sync();
  }
}

}  // namespace grada
