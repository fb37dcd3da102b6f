// Host orchestration of the Gauss-Newton + CG inversion on the device.
//
// Reference: GaussNewtonInversion::solve_cg (src/Inversion/
// GaussNewtonInversion.cpp:1417-1698) and invert_with_own_CG (:657-1103).
// The control flow (lambda search, stopping tests, IRLS updates) is the
// reference's, line for line, on host scalars; every vector operation runs on
// the device (cg.cu, gemv.cu) and only a few scalars per CG iteration cross to
// the host (the stopping test needs ||r||^2 / ||A^T b||^2 there).
//
// Row segments of the stacked CG system, in the reference's order
// (GaussNewtonInversion.cpp:1461-1471): data (Nd), Ws, Wz, Wx, Wy and, with
// the cross-gradient constraint, Tz, Tx, Ty (Nm each).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <numeric>

#include "cg_fused.h"
#include "common.cuh"
#include "context.h"

namespace grada {

DevCSR DevOperator::A() const {
  DevCSR c;
  c.n = n;
  c.nnz = nnz;
  c.rowptr = rowptr.as<int>();
  c.col = col.as<int>();
  c.val = val.as<double>();
  return c;
}

DevCSR DevOperator::AT() const {
  DevCSR c;
  c.n = n;
  c.nnz = nnz;
  c.rowptr = t_rowptr.as<int>();
  c.col = t_col.as<int>();
  c.val = t_val.as<double>();
  return c;
}

void Context::release_all() {
  prisms.release();
  obs.release();
  math_tables.release();
  G.release();
  row_scale.release();
  G64.release();
  g64_valid = false;
  scratch.release();
  vx.release();
  vy.release();
  for (auto &o : ops) {
    o.rowptr.release(); o.col.release(); o.val.release();
    o.t_rowptr.release(); o.t_col.release(); o.t_val.release();
  }
  for (auto &o : crg) {
    o.rowptr.release(); o.col.release(); o.val.release();
    o.t_rowptr.release(); o.t_col.release(); o.t_val.release();
  }
  for (DevBuf *b : {&wv_order, &wv_rowptr, &wv_col, &wv_val, &wv_part, &wv_segptr})
    b->release();
  DevBuf *bufs[] = {&dobs, &wd, &cg_b, &cg_s, &cg_t, &cg_p, &cg_pp, &cg_r, &cg_atb, &cg_gtw,
                    &cg_gx, &cg_tmpd, &cg_scal, &cg_part, &cg_wl_ones, &cg_ctl, &cg_bar, &cg_p2, &cg_red,
                    &cg_trace,
                    &cg_redc, &bt_part2, &bt_trials,
                    &bt_iters, &bt_report, &iv_m, &iv_mt, &iv_mt_old,
                    &iv_mopt, &iv_dx, &iv_P, &iv_mmin, &iv_mmax, &iv_m0, &iv_wl, &iv_tmp, &iv_tmp2,
                    &iv_dpre, &iv_d64, &iv_mstart, &iv_guard, &iv_flag,
                    &bscratch, &tc_err, &bk_b, &bk_s, &bk_t, &bk_p, &bk_pp, &bk_r, &bk_atb,
                    &bk_gtw, &bk_gx, &bk_tmpd, &bk_scal, &bk_part, &bk_ctl, &bk_coef, &sw_m, &sw_mt,
                    &sw_mt_old, &sw_mopt, &sw_dx, &sw_P, &sw_mmin, &sw_mmax, &sw_m0, &sw_wl,
                    &sw_tmp, &sw_tmp2, &sw_dpre, &sw_d64, &sw_mstart, &sw_guard, &sw_flag, &sw_in,
                    &sw_out, &cg_args};
  for (DevBuf *b : bufs) b->release();
  if (phase_exec) cudaGraphExecDestroy(phase_exec);
  phase_exec = nullptr;
  for (auto &k : phase_key) k = -1;
  if (h_cg_args) cudaFreeHost(h_cg_args);
  h_cg_args = nullptr;
  if (h_scal) cudaFreeHost(h_scal);
  if (h_flag) cudaFreeHost(h_flag);
  if (h_ctl) cudaFreeHost(h_ctl);
  if (h_bscal) cudaFreeHost(h_bscal);
  if (h_bctl) cudaFreeHost(h_bctl);
  if (h_bflag) cudaFreeHost(h_bflag);
  h_scal = nullptr;
  h_flag = nullptr;
  h_ctl = nullptr;
  h_bscal = nullptr;
  h_bctl = nullptr;
  h_bflag = nullptr;
}

namespace {

// CSR (n x n) -> CSR of its transpose, by counting sort over columns (entries
// of a transposed row come out in increasing original-row order).
void transpose_csr(int64_t n, const int *rp, const int *ci, const double *v, std::vector<int> &trp,
                   std::vector<int> &tci, std::vector<double> &tv) {
  const int64_t nnz = rp[n];
  trp.assign(n + 1, 0);
  for (int64_t k = 0; k < nnz; k++) trp[ci[k] + 1]++;
  for (int64_t i = 0; i < n; i++) trp[i + 1] += trp[i];
  std::vector<int> pos(trp.begin(), trp.end() - 1);
  tci.resize(nnz);
  tv.resize(nnz);
  for (int64_t r = 0; r < n; r++)
    for (int k = rp[r]; k < rp[r + 1]; k++) {
      const int c = ci[k];
      tci[pos[c]] = (int)r;
      tv[pos[c]] = v[k];
      pos[c]++;
    }
}

void upload_operator(Context *ctx, DevOperator &op, int64_t n, const int *rp, const int *ci,
                     const double *v) {
  const int64_t nnz = rp[n];
  std::vector<int> trp, tci;
  std::vector<double> tv;
  transpose_csr(n, rp, ci, v, trp, tci, tv);
  op.rowptr.alloc(ctx, sizeof(int) * (n + 1));
  op.col.alloc(ctx, sizeof(int) * std::max<int64_t>(nnz, 1));
  op.val.alloc(ctx, sizeof(double) * std::max<int64_t>(nnz, 1));
  op.t_rowptr.alloc(ctx, sizeof(int) * (n + 1));
  op.t_col.alloc(ctx, sizeof(int) * std::max<int64_t>(nnz, 1));
  op.t_val.alloc(ctx, sizeof(double) * std::max<int64_t>(nnz, 1));
  ctx->upload(op.rowptr.ptr, rp, sizeof(int) * (n + 1));
  ctx->upload(op.col.ptr, ci, sizeof(int) * nnz);
  ctx->upload(op.val.ptr, v, sizeof(double) * nnz);
  ctx->upload(op.t_rowptr.ptr, trp.data(), sizeof(int) * (n + 1));
  ctx->upload(op.t_col.ptr, tci.data(), sizeof(int) * nnz);
  ctx->upload(op.t_val.ptr, tv.data(), sizeof(double) * nnz);
  ctx->sync();  // host vectors go out of scope
  op.n = n;
  op.nnz = nnz;
  op.set = true;
}

double *dptr(const DevBuf &b) { return b.as<double>(); }

}  // namespace

void Context::set_operator(int which, int64_t n, int64_t nnz, const int *rp, const int *ci,
                           const double *v) {
  require_geometry();
  if (which < GRADA_OP_WS || which > GRADA_OP_TZ)
    throw Error(GRADA_ERR_INVALID_ARGUMENT, "unknown operator slot");
  if (n != n_cells) throw Error(GRADA_ERR_INVALID_ARGUMENT, "operator size differs from the cell count");
  if (!rp || (nnz > 0 && (!ci || !v))) throw Error(GRADA_ERR_INVALID_ARGUMENT, "null operator array");
  if (rp[0] != 0 || rp[n] != nnz) throw Error(GRADA_ERR_INVALID_ARGUMENT, "rowptr does not match nnz");
  for (int64_t r = 0; r < n; r++)
    if (rp[r + 1] < rp[r]) throw Error(GRADA_ERR_INVALID_ARGUMENT, "rowptr not monotone");
  for (int64_t k = 0; k < nnz; k++) {
    if (ci[k] < 0 || ci[k] >= n) throw Error(GRADA_ERR_INVALID_ARGUMENT, "column index out of range");
    if (!std::isfinite(v[k])) throw Error(GRADA_ERR_NONFINITE, "non-finite operator entry");
  }
  upload_operator(this, ops[which], n, rp, ci, v);
  if (which >= GRADA_OP_TX) {
    const int t = which - GRADA_OP_TX;
    host_T_rowptr[t].assign(rp, rp + n + 1);
    host_T_col[t].assign(ci, ci + nnz);
    host_T_val[t].assign(v, v + nnz);
    crg[t].set = false;  // rescaled on next use
  }
}

void Context::set_cross_gradient(int enabled, double a, const double *S) {
  require_geometry();
  crg_enabled = enabled != 0;
  a_crg = a;
  if (S) s_crg.assign(S, S + n_cells);
  else s_crg.clear();
  for (auto &c : crg) c.set = false;
}

void Context::set_data(const double *h_dobs, const double *h_wd) {
  require_geometry();
  if (!h_dobs || !h_wd) throw Error(GRADA_ERR_INVALID_ARGUMENT, "null data vector");
  for (int64_t i = 0; i < nd; i++)
    if (!std::isfinite(h_dobs[i]) || !std::isfinite(h_wd[i]))
      throw Error(GRADA_ERR_NONFINITE, "non-finite observed datum or weight at row " + std::to_string(i));
  dobs.alloc(this, sizeof(double) * nd);
  wd.alloc(this, sizeof(double) * nd);
  upload(dobs.ptr, h_dobs, sizeof(double) * nd);
  upload(wd.ptr, h_wd, sizeof(double) * nd);
  sync();
  data_set = true;
}

void Context::ensure_cg_workspace(int nterms) {
  const int64_t Nm = n_cells;
  const int64_t nrow = nd + (int64_t)nterms * Nm;
  cg_b.alloc(this, sizeof(double) * nrow);
  cg_s.alloc(this, sizeof(double) * nrow);
  cg_t.alloc(this, sizeof(double) * nrow);
  cg_p.alloc(this, sizeof(double) * Nm);
  cg_pp.alloc(this, sizeof(double) * Nm);
  cg_r.alloc(this, sizeof(double) * Nm);
  cg_atb.alloc(this, sizeof(double) * Nm);
  cg_gtw.alloc(this, sizeof(double) * Nm);
  cg_gx.alloc(this, sizeof(double) * ld);
  cg_tmpd.alloc(this, sizeof(double) * ld);
  cg_scal.alloc(this, sizeof(double) * CG_NSCALARS);
  cg_part.alloc(this, sizeof(double) * (size_t)sm_count * 4);
  if (!h_scal) GRADA_CUDA_CHECK(cudaMallocHost(&h_scal, sizeof(double) * CG_NSCALARS));
  if (!h_flag) GRADA_CUDA_CHECK(cudaMallocHost(&h_flag, sizeof(int) * 4));
  if (!h_ctl) GRADA_CUDA_CHECK(cudaMallocHost(&h_ctl, sizeof(int) * CTL_NINTS));
  if (crg_enabled) {
    for (int t = 0; t < 3; t++) {
      if (crg[t].set) continue;
      if (!ops[GRADA_OP_TX + t].set)
        throw Error(GRADA_ERR_STATE, "cross-gradient constraint enabled but T operators not set");
      // a_crg * S_crg * T0 (GaussNewtonInversion.cpp:1447-1449): row i scaled by a_crg*S_ii
      std::vector<double> v = host_T_val[t];
      const std::vector<int> &rp = host_T_rowptr[t];
      for (int64_t r = 0; r < Nm; r++) {
        const double sc = a_crg * (s_crg.empty() ? 1.0 : s_crg[r]);
        for (int k = rp[r]; k < rp[r + 1]; k++) v[k] = sc * host_T_val[t][k];
      }
      upload_operator(this, crg[t], Nm, rp.data(), host_T_col[t].data(), v.data());
    }
  }
}

// d = G m in the precision of the stored G; with an FP64 reference prediction
// d64 = G m_start: d = d64 + G (m - m_start) (the low-precision product only
// carries the increment).
void Context::data_prediction(const double *m, const double *m_start, const double *d64,
                              double *out) {
  if (predict_fp64) {  // FP64 product with the kept FP64 G
    launch_G_vec_mul(devG64(), m, out, scratch_doubles(gemv_scratch_doubles(devG64(), sm_count)),
                     sm_count, stream);
    fp64_products++;
  } else if (d64) {
    double *dm = dptr(iv_tmp2);
    launch_sub(m, m_start, n_cells, dm, stream);
    G_vec_mul_dev(dm, out);
    launch_add(out, d64, nd, out, stream);
  } else {
    G_vec_mul_dev(m, out);
  }
}

double Context::misfit_of(const double *m, const double *m_start, const double *d64) {
  double *g = dptr(iv_dpre);
  data_prediction(m, m_start, d64, g);
  double *scal = dptr(cg_scal);
  launch_misfit_sq(g, dptr(dobs), dptr(wd), nd, dptr(cg_part), dot_blocks(nd, sm_count),
                   scal + CG_MISFIT2, stream);
  GRADA_CUDA_CHECK(cudaMemcpyAsync(h_scal + CG_MISFIT2, scal + CG_MISFIT2, sizeof(double),
                                   cudaMemcpyDeviceToHost, stream));
  sync();
  return std::sqrt(h_scal[CG_MISFIT2] / (double)nd);  // GaussNewtonInversion.cpp:784, :916
}

// The stacked system's operators for one solve (GaussNewtonInversion.cpp:
// 1458-1586): row segments s, z, x, y (and tz, tx, ty) with their weights for
// b, and the forward and adjoint terms of the iteration.  The forward Ws row
// has no WL_s, the forward crg rows take WL_z / WL_x / WL_y, and the initial
// adjoint of s0 weights the crg-y rows by WL_y -- the reference's choices.
CgTerms Context::cg_terms(double sl, const double *const WL[7], double *b, double *s, double *t) {
  const int nterms = crg_enabled ? 7 : 4;
  const int64_t Nm = n_cells, Nd = nd;
  const double *WL_s = WL[0], *WL_x = WL[1], *WL_y = WL[2], *WL_z = WL[3];
  const double *WL_tx = WL[4], *WL_ty = WL[5], *WL_tz = WL[6];
  const DevOperator *seg_op[7] = {&ops[GRADA_OP_WS], &ops[GRADA_OP_WZ], &ops[GRADA_OP_WX],
                                  &ops[GRADA_OP_WY], &crg[2], &crg[0], &crg[1]};
  auto seg = [&](double *base, int k) { return base + Nd + (int64_t)k * Nm; };
  CgTerms T;
  T.nterms = nterms;
  const double *b_wl[7] = {WL_s, WL_z, WL_x, WL_y, WL_tz, WL_tx, WL_ty};
  const double adj_c[7] = {sl, sl, sl, sl, 1.0, 1.0, 1.0};
  const double fwd_c[7] = {sl, sl, sl, sl, 1.0, 1.0, 1.0};
  const double *fwd_wl[7] = {nullptr, WL_z, WL_x, WL_y, WL_z, WL_x, WL_y};
  for (int k = 0; k < nterms; k++) {
    T.seg_A[k] = seg_op[k]->A();
    T.seg_wl[k] = b_wl[k];
    AdjointTerm a;
    a.AT = seg_op[k]->AT();
    a.c = adj_c[k];
    a.wl = b_wl[k];
    a.s = seg(b, k);
    T.AT_b.t[k] = a;
    a.s = seg(s, k);
    T.AT_s.t[k] = a;
    if (k == 6) a.wl = WL_y;  // the initial adjoint weights the crg-y rows by WL_y (:1508)
    T.AT_s0.t[k] = a;
    T.FT.t[k].A = seg_op[k]->A();
    T.FT.t[k].c = fwd_c[k];
    T.FT.t[k].wl = fwd_wl[k];
    T.FT.t[k].out = seg(t, k);
  }
  T.AT_b.count = T.AT_s.count = T.AT_s0.count = T.FT.count = nterms;
  return T;
}

CgResult Context::solve_cg_dev(double lambda, double tol, int maxit, const double *mk,
                               const double *mref, const double *P, const double *const WL[7],
                               double *dx, const double *d64, const double *m_start) {
  NvtxRange nvtx("grada solve_cg");
  require_G();
  if (!data_set) throw Error(GRADA_ERR_STATE, "observed data not set (grada_set_data)");
  for (int t = 0; t < 4; t++)
    if (!ops[t].set) throw Error(GRADA_ERR_STATE, "regularisation operators Ws/Wx/Wy/Wz not set");
  const int nterms = crg_enabled ? 7 : 4;
  ensure_cg_workspace(nterms);
  const int64_t Nm = n_cells, Nd = nd, nrow = Nd + (int64_t)nterms * Nm;
  const double sl = std::sqrt(lambda);
  double *b = dptr(cg_b), *s = dptr(cg_s), *t = dptr(cg_t);
  // WL in the reference argument order s, x, y, z, tx, ty, tz; segments in
  // row order s, z, x, y, tz, tx, ty
  const CgTerms T = cg_terms(sl, WL, b, s, t);
  double *p = dptr(cg_p), *pp = dptr(cg_pp), *r = dptr(cg_r), *atb = dptr(cg_atb);
  double *gtw = dptr(cg_gtw), *gx = dptr(cg_gx), *tmpd = dptr(cg_tmpd);
  double *scal = dptr(cg_scal), *part = dptr(cg_part);
  auto seg = [&](double *base, int k) { return base + Nd + (int64_t)k * Nm; };
  const int nb_m = dot_blocks(Nm, sm_count), nb_row = dot_blocks(nrow, sm_count);

  // b and s = -b   (GaussNewtonInversion.cpp:1458-1472)
  data_prediction(mk, m_start, d64, gx);
  launch_data_residual(dptr(dobs), gx, dptr(wd), Nd, b, s, stream);
  for (int k = 0; k < nterms; k++)
    launch_csr_apply(T.seg_A[k], mk, k == 0 ? mref : nullptr, k < 4 ? -sl : -1.0, T.seg_wl[k],
                     seg(b, k), stream);
  launch_negate(b + Nd, nrow - Nd, s + Nd, stream);

  // A^T b and the initial r = A^T s (:1485-1551).  G^T(Wd s0) = -G^T(Wd b0)
  // exactly, so one product serves both.
  launch_scale(b, dptr(wd), Nd, 1.0, tmpd, stream);
  GT_vec_mul_dev(tmpd, gtw);
  const AdjointTerms &AT_b = T.AT_b, &AT_s0 = T.AT_s0, &AT_s = T.AT_s;
  launch_adjoint(AT_b, Nm, P, gtw, 1.0, atb, stream);
  launch_adjoint(AT_s0, Nm, P, gtw, -1.0, r, stream);
  launch_dot(atb, nullptr, Nm, part, nb_m, scal + CG_ATB2, stream);

  GRADA_CUDA_CHECK(cudaMemsetAsync(p, 0, sizeof(double) * Nm, stream));
  GRADA_CUDA_CHECK(cudaMemsetAsync(dx, 0, sizeof(double) * Nm, stream));
  GRADA_CUDA_CHECK(cudaMemsetAsync(t, 0, sizeof(double) * nrow, stream));
  GRADA_CUDA_CHECK(cudaMemsetAsync(scal + CG_BETA, 0, sizeof(double), stream));
  launch_dot(r, nullptr, Nm, part, nb_m, scal + CG_R2, stream);

  // forward rows of t = A p (:1569-1586): Ws row without WL_s, crg rows
  // weighted by WL_z / WL_x / WL_y
  const ForwardTerms &FT = T.FT;

  CgResult res;
  if (maxit <= 0) {  // the loop never runs: iterations = maxit (:1693-1696)
    sync();
    return res;
  }
  // A zero right-hand side (A^T s = 0 already, e.g. no data signal and m at the
  // reference) is solved by dx = 0; the reference would divide 0 by 0 in its
  // first step.  Return the exact solution instead of a breakdown.
  GRADA_CUDA_CHECK(cudaMemcpyAsync(h_scal, scal, sizeof(double) * CG_NSCALARS,
                                   cudaMemcpyDeviceToHost, stream));
  sync();
  if (h_scal[CG_R2] == 0.0) return res;
  const CgLoop loop = cg_loop_kind();
  if (loop != kCgGeneric)
    return solve_cg_fused(tol, maxit, P, dx, FT, AT_s, nrow, nb_m, nb_row, loop == kCgPersistent);
  // Device-side stopping: the beta kernel counts iterations and raises
  // ctl[CTL_DONE] on err < tol (or maxit, breakdown, non-finite scalar);
  // every kernel of an iteration returns at once while it is raised, so a
  // CUDA graph of CG_GRAPH_ITERS iterations can be replayed until done with
  // one host synchronisation per replay.
  cg_ctl.alloc(this, sizeof(int) * CTL_NINTS);
  int *ctl = cg_ctl.as<int>();
  h_ctl[CTL_DONE] = 0;
  h_ctl[CTL_ITER] = 0;
  h_ctl[CTL_MAXIT] = maxit;
  h_ctl[CTL_STATUS] = CG_STATUS_RUNNING;
  upload(ctl, h_ctl, sizeof(int) * CTL_NINTS);
  h_scal[CG_TOL] = tol;
  upload(scal + CG_TOL, h_scal + CG_TOL, sizeof(double));
  scratch_doubles(product_scratch_doubles());  // allocate before capture
  const double *wdp = dptr(wd);
  auto iteration = [&]() {
    launch_p_update(r, P, scal, Nm, p, pp, stream, ctl);
    GemvOpts o;
    o.skip = ctl;
    o.scale = wdp;  // t0 = Wd (G P p)
    apply_G(pp, t, o);
    launch_multi_forward(FT, Nm, pp, stream, ctl);
    launch_dot(t, nullptr, nrow, part, nb_row, scal + CG_T2, stream, ctl);
    launch_alpha(scal, ctl, stream);
    launch_axpy(t, p, scal, nrow, Nm, s, dx, stream, ctl);
    apply_GT(s, gtw, o);  // G^T (Wd s0)
    launch_adjoint(AT_s, Nm, P, gtw, 1.0, r, stream, ctl);
    launch_dot(r, nullptr, Nm, part, nb_m, scal + CG_R2NEW, stream, ctl);
    launch_beta(scal, ctl, stream);
  };
  const int K = std::min(maxit, kCgGraphIters);
  const auto t_build = std::chrono::steady_clock::now();
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
  const auto t_loop = std::chrono::steady_clock::now();
  int launched = 0;
  try {
    while (true) {
      GRADA_CUDA_CHECK(cudaGraphLaunch(exec, stream));
      launched += K;
      GRADA_CUDA_CHECK(cudaMemcpyAsync(h_ctl, ctl, sizeof(int) * CTL_NINTS,
                                       cudaMemcpyDeviceToHost, stream));
      GRADA_CUDA_CHECK(cudaMemcpyAsync(h_scal, scal, sizeof(double) * CG_NSCALARS,
                                       cudaMemcpyDeviceToHost, stream));
      sync();
      if (h_ctl[CTL_DONE] || launched >= maxit) break;
    }
  } catch (...) {
    cudaGraphExecDestroy(exec);
    throw;
  }
  cudaGraphExecDestroy(exec);
  count_cg_loop(t_build, t_loop, h_ctl[CTL_ITER]);
  res.iterations = h_ctl[CTL_ITER];
  res.err = h_scal[CG_ERR];
  if (h_ctl[CTL_STATUS] == CG_STATUS_BREAKDOWN)
    throw Error(GRADA_ERR_BREAKDOWN,
                "CG breakdown: ||t||^2 = 0 at iteration " + std::to_string(res.iterations));
  if (h_ctl[CTL_STATUS] == CG_STATUS_NONFINITE)
    throw Error(GRADA_ERR_NONFINITE,
                "non-finite CG scalar at iteration " + std::to_string(res.iterations));
  return res;
}

void Context::count_cg_loop(std::chrono::steady_clock::time_point t_build,
                            std::chrono::steady_clock::time_point t_loop, int iterations) {
  const auto t_end = std::chrono::steady_clock::now();
  cg_graph_ns += (double)std::chrono::duration_cast<std::chrono::nanoseconds>(t_loop - t_build).count();
  cg_loop_ns += (double)std::chrono::duration_cast<std::chrono::nanoseconds>(t_end - t_loop).count();
  cg_loop_iters += iterations;
}

Context::CgLoop Context::cg_loop_kind() const {
  // Stored dense G runs the persistent loop's phase bodies: by default as a
  // graph of four kernels per iteration (cg_phases.cu), each at its own
  // occupancy; GRADA_CG_FUSED=1 takes the one-launch persistent loop (the
  // batched inversion's engine, bitwise the same solve).  The matrix-free and
  // wavelet products, and GRADA_CG_FUSED=0, take the graph of the generic
  // product kernels (13 per iteration, other summation orders).
  if (g_storage != GRADA_G_FP64 && g_storage != GRADA_G_FP32 && g_storage != GRADA_G_BF16_ROWSCALE &&
      g_storage != GRADA_G_FP16_ROWSCALE)
    return kCgGeneric;
  const char *e = std::getenv("GRADA_CG_FUSED");
  if (e && e[0] == '0') return kCgGeneric;
  if (e && e[0] == '1') return kCgPersistent;
  return kCgPhases;
}

// The CG loop as one persistent cooperative launch (cg_fused.cu), from the
// state the setup of solve_cg_dev left on the device.
CgResult Context::solve_cg_fused(double tol, int maxit, const double *P, double *dx,
                                 const ForwardTerms &FT, const AdjointTerms &AT, int64_t nrow,
                                 int nb_m, int nb_row, bool persistent) {
  const DevG g = devG();
  FusedCgArgs a;
  a.G = g.data;
  a.row_scale = g.row_scale;
  a.nd = g.nd;
  a.nm = g.nm;
  a.ld = g.ld;
  if (fused_grid[(int)g.kind] <= 0) fused_grid[(int)g.kind] = fused_cg_grid(g.kind, sm_count);
  const int grid = fused_grid[(int)g.kind];
  fused_gx_partition(g, sm_count, a.tiles, a.splits, a.per);
  a.scratch = scratch_doubles(std::max(product_scratch_doubles(), (int64_t)a.splits * g.ld));
  a.wd = dptr(wd);
  a.r = dptr(cg_r);
  a.p = dptr(cg_p);
  cg_p2.alloc(this, sizeof(double) * (size_t)n_cells);
  a.p2 = dptr(cg_p2);
  a.pp = dptr(cg_pp);
  a.dx = dx;
  a.t = dptr(cg_t);
  a.s = dptr(cg_s);
  a.gtw = dptr(cg_gtw);
  a.P = P;
  a.nrow = nrow;
  a.FT = FT;
  a.AT = AT;
  a.part = dptr(cg_part);
  a.nb_m = nb_m;
  a.nb_row = nb_row;
  a.scal = dptr(cg_scal);
  cg_ctl.alloc(this, sizeof(int) * CTL_NINTS);
  a.ctl = cg_ctl.as<int>();
  cg_bar.alloc(this, sizeof(unsigned) * 256);
  a.barrier = cg_bar.as<unsigned>();
  int64_t red_d = 0, red_c = 0;
  fused_red_sizes(nd, n_cells, FT.count, red_d, red_c);
  cg_red.alloc(this, sizeof(double) * (size_t)red_d);
  cg_redc.alloc(this, sizeof(unsigned) * (size_t)red_c);
  GRADA_CUDA_CHECK(cudaMemsetAsync(cg_redc.ptr, 0, sizeof(unsigned) * (size_t)red_c, stream));
  a.red = dptr(cg_red);
  a.red_count = cg_redc.as<unsigned>();
  if (inject_cg_wait) {  // grada_inject_fault(GRADA_FAULT_CG_WAIT): every barrier wait expires
    inject_cg_wait = false;
    a.wait_limit_ns = 0;
  }
  h_ctl[CTL_DONE] = 0;
  h_ctl[CTL_ITER] = 0;
  h_ctl[CTL_MAXIT] = maxit;
  h_ctl[CTL_STATUS] = CG_STATUS_RUNNING;
  upload(a.ctl, h_ctl, sizeof(int) * CTL_NINTS);
  h_scal[CG_TOL] = tol;
  upload(a.scal + CG_TOL, h_scal + CG_TOL, sizeof(double));
  if (!persistent) return solve_cg_phases(a, g.kind, maxit);
  cg_trace.alloc(this, sizeof(unsigned long long) * 5);
  a.trace = cg_trace.as<unsigned long long>();
  GRADA_CUDA_CHECK(cudaMemsetAsync(a.trace, 0, sizeof(unsigned long long) * 5, stream));
  // CTAs of the launch: all resident ones, or fewer with GRADA_CG_CTAS (the
  // partition above does not depend on the launch, so the sums do not change)
  int launch_grid = grid;
  if (const char *e = std::getenv("GRADA_CG_CTAS")) {
    const int c = std::atoi(e);
    if (c >= 1 && c < grid) launch_grid = c;
  }
  const auto t_loop = std::chrono::steady_clock::now();
  launch_cg_fused(a, g.kind, launch_grid, stream);
  unsigned bar_words[256];
  unsigned long long trace[5];
  download(trace, a.trace, sizeof(trace));
  download(bar_words, a.barrier, sizeof(bar_words));
  download(h_ctl, a.ctl, sizeof(int) * CTL_NINTS);
  download(h_scal, a.scal, sizeof(double) * CG_NSCALARS);
  sync();
  if (bar_words[224])
    throw Error(GRADA_ERR_CUDA, "persistent CG: a grid barrier wait expired; the solve was abandoned");
  for (int q = 0; q < 5; q++) trace_sum[q] += trace[q];
  count_cg_loop(t_loop, t_loop, h_ctl[CTL_ITER]);
  CgResult res;
  res.iterations = h_ctl[CTL_ITER];
  res.err = h_scal[CG_ERR];
  if (h_ctl[CTL_STATUS] == CG_STATUS_BREAKDOWN)
    throw Error(GRADA_ERR_BREAKDOWN,
                "CG breakdown: ||t||^2 = 0 at iteration " + std::to_string(res.iterations));
  if (h_ctl[CTL_STATUS] == CG_STATUS_NONFINITE)
    throw Error(GRADA_ERR_NONFINITE,
                "non-finite CG scalar at iteration " + std::to_string(res.iterations));
  return res;
}

// The persistent loop's phases as a graph of four kernels per iteration
// (cg_phases.cu), replayed until the device raises ctl[CTL_DONE]; a holds the
// state solve_cg_fused set up.  K iterations per graph, K even (or maxit), so
// the p / p2 parity of a captured iteration is that of the solve's count.  The
// kernels take their arguments from cg_args, so a graph built for one solve
// serves every later solve of the same shape (the arguments are rewritten,
// nothing is captured or instantiated again).
CgResult Context::solve_cg_phases(const FusedCgArgs &a, GKind kind, int maxit) {
  const int K = std::min(maxit, kCgGraphIters);
  const auto t_build = std::chrono::steady_clock::now();
  cg_args.alloc(this, sizeof(FusedCgArgs));
  if (!h_cg_args) {
    void *hp = nullptr;
    GRADA_CUDA_CHECK(cudaMallocHost(&hp, sizeof(FusedCgArgs)));
    h_cg_args = static_cast<FusedCgArgs *>(hp);
  }
  // the previous solve's upload has completed (every solve ends synchronised)
  *h_cg_args = a;
  const FusedCgArgs *dev_args = cg_args.as<FusedCgArgs>();
  GRADA_CUDA_CHECK(cudaMemcpyAsync(cg_args.ptr, h_cg_args, sizeof(FusedCgArgs),
                                   cudaMemcpyHostToDevice, stream));
  int64_t key[7];
  cg_phase_grids(a, key);
  key[4] = (int64_t)kind;
  key[5] = K;
  key[6] = (int64_t)(uintptr_t)dev_args;
  if (!phase_exec || !std::equal(key, key + 7, phase_key)) {
    if (phase_exec) cudaGraphExecDestroy(phase_exec);
    phase_exec = nullptr;
    cudaGraph_t graph = nullptr;
    GRADA_CUDA_CHECK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    try {
      for (int k = 0; k < K; k++) launch_cg_phase_iteration(a, dev_args, kind, k & 1, stream);
    } catch (...) {
      cudaGraph_t g = nullptr;
      cudaStreamEndCapture(stream, &g);
      if (g) cudaGraphDestroy(g);
      throw;
    }
    GRADA_CUDA_CHECK(cudaStreamEndCapture(stream, &graph));
    cudaError_t ie = cudaGraphInstantiate(&phase_exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ie != cudaSuccess) phase_exec = nullptr;
    GRADA_CUDA_CHECK(ie);
    std::copy(key, key + 7, phase_key);
  }
  const auto t_loop = std::chrono::steady_clock::now();
  int launched = 0;
  while (true) {
    GRADA_CUDA_CHECK(cudaGraphLaunch(phase_exec, stream));
    launched += K;
    GRADA_CUDA_CHECK(cudaMemcpyAsync(h_ctl, a.ctl, sizeof(int) * CTL_NINTS,
                                     cudaMemcpyDeviceToHost, stream));
    GRADA_CUDA_CHECK(cudaMemcpyAsync(h_scal, a.scal, sizeof(double) * CG_NSCALARS,
                                     cudaMemcpyDeviceToHost, stream));
    sync();
    if (h_ctl[CTL_DONE] || launched >= maxit) break;
  }
  count_cg_loop(t_build, t_loop, h_ctl[CTL_ITER]);
  CgResult res;
  res.iterations = h_ctl[CTL_ITER];
  res.err = h_scal[CG_ERR];
  if (h_ctl[CTL_STATUS] == CG_STATUS_BREAKDOWN)
    throw Error(GRADA_ERR_BREAKDOWN,
                "CG breakdown: ||t||^2 = 0 at iteration " + std::to_string(res.iterations));
  if (h_ctl[CTL_STATUS] == CG_STATUS_NONFINITE)
    throw Error(GRADA_ERR_NONFINITE,
                "non-finite CG scalar at iteration " + std::to_string(res.iterations));
  return res;
}

// The set-up of invert_with_own_CG (GaussNewtonInversion.cpp:757-786): input
// checks, the starting model, the device vectors, IRLS weights of one, and
// the mixed-precision mode (refine: FP64 residual refinement; predict_fp64:
// every prediction an FP64 product of the kept G).  Shared by invert and the
// batched persistent inversion.
bool Context::invert_setup(const grada_invert_params &prm, const double *h_m_ini,
                           const double *h_mmin, const double *h_mmax, const double *h_m0) {
  require_G();
  if (!data_set) throw Error(GRADA_ERR_STATE, "observed data not set (grada_set_data)");
  if (!h_m_ini || !h_mmin || !h_mmax)
    throw Error(GRADA_ERR_INVALID_ARGUMENT, "null model vector");
  if (prm.n_lambda < 1 || prm.gn_iterations < 1)
    throw Error(GRADA_ERR_INVALID_ARGUMENT, "n_lambda and gn_iterations must be >= 1");
  const int64_t Nm = n_cells;
  trials.clear();
  iterations.clear();

  // starting model (GaussNewtonInversion.cpp:757-786)
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
  const size_t vb = sizeof(double) * Nm;
  DevBuf *vecs[] = {&iv_m, &iv_mt, &iv_mt_old, &iv_mopt, &iv_dx, &iv_P, &iv_mmin, &iv_mmax,
                    &iv_m0, &iv_tmp, &iv_tmp2, &iv_mstart};
  for (DevBuf *b : vecs) b->alloc(this, vb);
  iv_wl.alloc(this, vb * 7);
  iv_dpre.alloc(this, sizeof(double) * ld);
  iv_guard.alloc(this, sizeof(int) * Nm);
  iv_flag.alloc(this, sizeof(int) * 4);
  const bool refine =
      prm.fp64_refinement && g_storage != GRADA_G_FP64 && g_storage != GRADA_G_MATRIX_FREE;
  // with a kept FP64 G every prediction is an FP64 product instead
  predict_fp64 = refine && fp64_resident();
  fp64_products = 0;
  if (predict_fp64) scratch_doubles(std::max(product_scratch_doubles(),
                                             gemv_scratch_doubles(devG64(), sm_count)));
  if (refine) iv_d64.alloc(this, sizeof(double) * ld);
  ensure_cg_workspace(crg_enabled ? 7 : 4);
  upload(iv_m.ptr, m.data(), vb);
  upload(iv_mmin.ptr, mmin.data(), vb);
  upload(iv_mmax.ptr, mmax.data(), vb);
  upload(iv_m0.ptr, m0.data(), vb);
  {
    std::vector<double> ones(7 * Nm, 1.0);
    upload(iv_wl.ptr, ones.data(), vb * 7);
    sync();
  }
  return refine;
}

void Context::invert(const grada_invert_params &prm, const double *h_m_ini, const double *h_mmin,
                     const double *h_mmax, const double *h_m0, double *h_m_out,
                     grada_invert_report &rep, const grada_adaptive_params *adapt) {
  NvtxRange nvtx("grada invert");
  if (!h_m_out && !adapt) throw Error(GRADA_ERR_INVALID_ARGUMENT, "null model vector");
  if (adapt && (!adapt->refine || adapt->interval_between_refinements < 1))
    throw Error(GRADA_ERR_INVALID_ARGUMENT, "adaptive inversion needs a refine callback and an interval >= 1");
  std::memset(&rep, 0, sizeof(rep));
  struct PredictGuard {
    Context *c;
    ~PredictGuard() { c->predict_fp64 = false; }
  } predict_guard{this};
  const bool refine = invert_setup(prm, h_m_ini, h_mmin, h_mmax, h_m0);
  for (auto &t : trace_sum) t = 0;
  cg_loop_ns = cg_graph_ns = 0.0;
  cg_loop_iters = 0;
  if (adapt && predict_fp64)
    throw Error(GRADA_ERR_STATE, "adaptive inversion: a kept FP64 G is not expanded by refinement");
  int64_t Nm = n_cells;
  size_t vb = sizeof(double) * Nm;
  double *dm, *dmt, *dmt_old, *dmopt, *ddx, *dP, *dmin, *dmax, *dm0, *dtmp, *wlv;
  // WL slots in the reference argument order s, x, y, z, tx, ty, tz
  double *WLs, *WLx, *WLy, *WLz, *WLtx, *WLty, *WLtz;
  const double *WL[7];
  double *d64, *mstart;
  // device pointers of the inversion vectors (again after a refinement)
  auto bind = [&]() {
    dm = dptr(iv_m), dmt = dptr(iv_mt), dmt_old = dptr(iv_mt_old), dmopt = dptr(iv_mopt);
    ddx = dptr(iv_dx), dP = dptr(iv_P), dmin = dptr(iv_mmin), dmax = dptr(iv_mmax);
    dm0 = dptr(iv_m0), dtmp = dptr(iv_tmp);
    wlv = dptr(iv_wl);
    WLs = wlv, WLx = wlv + Nm, WLy = wlv + 2 * Nm, WLz = wlv + 3 * Nm;
    WLtx = wlv + 4 * Nm, WLty = wlv + 5 * Nm, WLtz = wlv + 6 * Nm;
    WL[0] = WLs, WL[1] = WLx, WL[2] = WLy, WL[3] = WLz, WL[4] = WLtx, WL[5] = WLty,
    WL[6] = WLtz;
    d64 = refine ? dptr(iv_d64) : nullptr;
    mstart = dptr(iv_mstart);
  };
  bind();

  auto refresh_fp64 = [&](const double *mref_point) {
    // FP64 matrix-free prediction at the current model: the residual
    // refinement step of the mixed-precision path
    const DevGeometry g = geometry();
    const int splits = forward_field_splits(g, sm_count);
    double *partial = scratch_doubles((int64_t)splits * n_obs * n_fields);
    launch_forward_field(g, mref_point, splits, partial, d64, true, stream);
    GRADA_CUDA_CHECK(cudaMemcpyAsync(mstart, mref_point, vb, cudaMemcpyDeviceToDevice, stream));
    rep.fp64_refinements++;
  };
  if (refine && !predict_fp64) refresh_fp64(dm);

  double misfit = misfit_of(dm, mstart, d64);
  double misfit_last_iteration = 5 * misfit;
  (void)misfit_last_iteration;
  double lambda = prm.max_lambda;
  double lambda_opt = lambda;
  double misfit_opt = misfit;
  GRADA_CUDA_CHECK(cudaMemcpyAsync(dmopt, dm, vb, cudaMemcpyDeviceToDevice, stream));
  const double rate = prm.lambda_decreasing_rate;
  int i = 0, j = 0;
  const double p_expo[5] = {-(2 - prm.lp_s) / 4.0, -(2 - prm.lp_x) / 4.0, -(2 - prm.lp_y) / 4.0,
                            -(2 - prm.lp_z) / 4.0, -(2 - prm.lp_t) / 4.0};
  // IRLS weights of the terms with p != 2 from the model mv (:962-1022; after
  // a refinement from m itself, :1228-1281)
  auto irls_from = [&](const double *mv) {
    if (prm.lp_s != 2) {
      launch_csr_apply(ops[GRADA_OP_WS].A(), mv, dm0, 1.0, nullptr, dtmp, stream);
      launch_irls_weight(dtmp, Nm, prm.epsilon2, p_expo[0], WLs, stream);
    }
    if (prm.lp_x != 2) {
      launch_csr_apply(ops[GRADA_OP_WX].A(), mv, nullptr, 1.0, nullptr, dtmp, stream);
      launch_irls_weight(dtmp, Nm, prm.epsilon2, p_expo[1], WLx, stream);
    }
    if (prm.lp_y != 2) {
      launch_csr_apply(ops[GRADA_OP_WY].A(), mv, nullptr, 1.0, nullptr, dtmp, stream);
      launch_irls_weight(dtmp, Nm, prm.epsilon2, p_expo[2], WLy, stream);
    }
    if (prm.lp_z != 2) {
      launch_csr_apply(ops[GRADA_OP_WZ].A(), mv, nullptr, 1.0, nullptr, dtmp, stream);
      launch_irls_weight(dtmp, Nm, prm.epsilon2, p_expo[3], WLz, stream);
    }
    if (prm.lp_t != 2 && crg_enabled) {
      double *wt[3] = {WLtx, WLty, WLtz};
      for (int q = 0; q < 3; q++) {
        launch_csr_apply(ops[GRADA_OP_TX + q].A(), mv, nullptr, 1.0, nullptr, dtmp, stream);
        launch_irls_weight(dtmp, Nm, prm.epsilon2, p_expo[4], wt[q], stream);
      }
    }
  };
  int c_refinement = 0, i_between_refinement = 0;
  const int max_refinements = adapt ? adapt->max_refinement_number : 0;
  for (i = 0; i < prm.gn_iterations; i++) {
    GRADA_CUDA_CHECK(cudaMemcpyAsync(dmt, dm, vb, cudaMemcpyDeviceToDevice, stream));
    double misfit_last1 = 10 * misfit;
    double misfit_last2 = 100 * misfit;
    misfit_last_iteration = misfit;
    if (i == 0 || prm.n_lambda == 1 || std::abs(rate - 1) < 1e-6) {
      lambda = prm.max_lambda;
    } else {
      lambda = lambda_opt * std::pow(1 / rate, std::min(3, prm.n_lambda - 2));
      const double min_lambda = std::min(prm.max_lambda * std::pow(rate, 20), 1.0e-5);
      if (lambda < min_lambda) lambda = 1.0;
    }
    int cg_maxit = 0;
    if (prm.cg_iteration_factor < 1) cg_maxit = (int)(prm.cg_iteration_factor * Nm);
    else cg_maxit = (int)prm.cg_iteration_factor;
    if (refine && !predict_fp64 && i > 0) refresh_fp64(dm);
    launch_p_diag(dm, dmin, dmax, Nm, dP, stream);
    for (j = 0; j < prm.n_lambda; j++) {
      CgResult cg = solve_cg_dev(lambda, prm.cg_tol, cg_maxit, dm, dm0, dP, WL, ddx, d64, mstart);
      rep.cg_iterations += cg.iterations;
      GRADA_CUDA_CHECK(cudaMemcpyAsync(dmt_old, dmt, vb, cudaMemcpyDeviceToDevice, stream));
      launch_bound_update(dm, ddx, dmin, dmax, Nm, dmt, dmt_old, iv_guard.as<int>(),
                          iv_flag.as<int>(), h_flag, stream);
      misfit_last2 = misfit_last1;
      misfit_last1 = misfit;
      misfit = misfit_of(dmt, mstart, d64);
      trials.push_back({i + 1, lambda, misfit, cg.iterations, cg.err});
      if (j == 0 || misfit < misfit_opt) {
        misfit_opt = misfit;
        GRADA_CUDA_CHECK(cudaMemcpyAsync(dmopt, dmt, vb, cudaMemcpyDeviceToDevice, stream));
        if (i > 0) GRADA_CUDA_CHECK(cudaMemcpyAsync(dm, dmopt, vb, cudaMemcpyDeviceToDevice, stream));
        lambda_opt = lambda;
      }
      if ((std::abs(misfit - misfit_last1) / std::min(misfit, misfit_last1) < prm.stag_tol) &&
          (std::abs(misfit_last1 - misfit_last2) / std::min(misfit_last1, misfit_last2) < prm.stag_tol) &&
          j > 1)
        break;
      if (misfit > misfit_last1 && misfit_last1 > misfit_last2 && j > 1) {
        break;
      } else {
        lambda = lambda * rate;
        irls_from(dmopt);  // IRLS (:962-1022)
      }
      if (misfit < prm.target_misfit) break;
    }
    GRADA_CUDA_CHECK(cudaMemcpyAsync(dm, dmopt, vb, cudaMemcpyDeviceToDevice, stream));
    misfit = misfit_opt;
    iterations.push_back({i + 1, (j == prm.n_lambda) ? prm.n_lambda : (j + 1), misfit});
    if (misfit < prm.target_misfit || i == prm.gn_iterations - 1) break;
    const bool flag1 = std::abs(misfit - misfit_last_iteration) /
                           std::min(misfit, misfit_last_iteration) < prm.stag_tol;
    // the refinement branch (GaussNewtonInversion.cpp:1098-1294); on a fixed
    // mesh max_refinement_number is 0 and a stagnation ends the inversion
    if (c_refinement >= max_refinements && flag1) break;
    if (c_refinement < max_refinements &&
        (++i_between_refinement % adapt->interval_between_refinements == 0 || flag1)) {
      i_between_refinement = 0;
      ++c_refinement;
      // the host's refine_mesh (AdaptiveInversion.cpp:637-735): it splits the
      // mesh, expands G (grada_expand_G), rebuilds Ws/Wx/Wy/Wz (and T) and
      // hands back the model, bounds and reference model on the new cells
      std::vector<double> hm((size_t)Nm);
      download(hm.data(), dm, vb);
      sync();
      refine_pending = true;
      refine_model.clear();
      const int st = adapt->refine(adapt->user, static_cast<grada_ctx *>(this), hm.data(), Nm);
      refine_pending = false;
      if (st != GRADA_OK)
        throw Error(st, "refine callback failed: " + last_error);
      if (refine_model.size() != (size_t)(4 * n_cells))
        throw Error(GRADA_ERR_STATE,
                    "the refine callback must hand back the model on the refined mesh "
                    "(grada_set_inversion_model)");
      for (int t = 0; t < 4; t++)
        if (!ops[t].set || ops[t].n != n_cells)
          throw Error(GRADA_ERR_STATE,
                      "the refine callback must rebuild Ws/Wx/Wy/Wz for the refined mesh");
      if (crg_enabled) {
        // the constrained refine_mesh(a, interpolator, "crg") re-interpolates the
        // structure model and set_Tmatrix rebuilds T_x, T_y, T_z from it
        // (AdaptiveInversion.cpp:206-386, GaussNewtonInversion.cpp:1266-1279)
        for (int t = GRADA_OP_TX; t <= GRADA_OP_TZ; t++)
          if (!ops[t].set || ops[t].n != n_cells)
            throw Error(GRADA_ERR_STATE,
                        "the refine callback must rebuild Tx/Ty/Tz for the refined mesh");
        // init_matrices resets S_crg to the identity (InversionBase.cpp:113-130)
        if (!s_crg.empty() && s_crg.size() != (size_t)n_cells) {
          s_crg.clear();
          for (auto &c : crg) c.set = false;
        }
      }
      Nm = n_cells;
      vb = sizeof(double) * Nm;
      DevBuf *vecs[] = {&iv_m, &iv_mt, &iv_mt_old, &iv_mopt, &iv_dx, &iv_P, &iv_mmin, &iv_mmax,
                        &iv_m0, &iv_tmp, &iv_tmp2, &iv_mstart};
      for (DevBuf *b : vecs) b->alloc(this, vb);
      iv_wl.alloc(this, vb * 7);
      iv_guard.alloc(this, sizeof(int) * Nm);
      ensure_cg_workspace(crg_enabled ? 7 : 4);
      bind();
      upload(dm, refine_model.data(), vb);
      upload(dmin, refine_model.data() + Nm, vb);
      upload(dmax, refine_model.data() + 2 * Nm, vb);
      upload(dm0, refine_model.data() + 3 * Nm, vb);
      {
        std::vector<double> ones(7 * (size_t)Nm, 1.0);  // WL = I (:1185-1199)
        upload(wlv, ones.data(), vb * 7);
        sync();
      }
      irls_from(dm);
      rep.mesh_refinements++;
    }
  }
  if (h_m_out) download(h_m_out, dm, vb);
  sync();
  rep.final_misfit = misfit;
  rep.final_lambda = lambda;
  rep.gn_iterations = (int)iterations.size();
  rep.n_trials = (int)trials.size();
  if (predict_fp64) rep.fp64_refinements = fp64_products;
}

}  // namespace grada
