// Host-side state of one library context: the device copies of the reference
// Fwd object's data (mesh leaf cells, observation points, field flag, dense G)
// plus the inversion operators and work vectors.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <chrono>
#include <string>
#include <vector>

#include "../../include/grada_gpu.h"
#include "cg_kernels.h"
#include "kernels.h"

namespace grada {

struct Context;

// Owning device allocation, accounted against its context.
struct DevBuf {
  void *ptr = nullptr;
  size_t bytes = 0;
  Context *owner = nullptr;
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  ~DevBuf();
  void alloc(Context *ctx, size_t nbytes);  // keeps the buffer if already large enough
  void release();
  template <typename T>
  T *as() const {
    return static_cast<T *>(ptr);
  }
};

// A host-built sparse operator and its transpose on the device.
struct DevOperator {
  DevBuf rowptr, col, val, t_rowptr, t_col, t_val;
  int64_t n = 0, nnz = 0;
  bool set = false;
  DevCSR A() const;
  DevCSR AT() const;
};

// One lambda trial of the Gauss-Newton loop (a line of lambda_misfit_GN).
struct TrialRecord {
  int gn_iteration;
  double lambda;
  double misfit;
  int cg_iterations;
  double cg_error;
};

// One Gauss-Newton iteration (a line of Iteration_misfit_GN).
struct IterationRecord {
  int gn_iteration;
  int n_trials;
  double misfit;
};

// CG iterations captured per CUDA graph replay.
constexpr int kCgGraphIters = 16;

struct CgResult {
  double err = 0.0;
  int iterations = 0;
};

// The operators of one solve's stacked system (Context::cg_terms).
struct CgTerms {
  int nterms = 4;
  DevCSR seg_A[7];
  const double *seg_wl[7] = {};
  ForwardTerms FT;
  AdjointTerms AT_b, AT_s0, AT_s;
};

struct BatchProblem;
struct FusedCgArgs;

struct Context {
  int device = 0;
  int sm_count = 0;
  cudaStream_t stream = nullptr;
  std::string last_error;
  int64_t bytes_held = 0;
  bool inject_alloc_failure = false;  // grada_inject_fault

  // Geometry (Fwd::mesh leaf cells, Fwd::ob, Fwd::field_flag) and the
  // prism kernels' math tables.
  DevBuf prisms, obs, math_tables;
  std::vector<double> host_prisms;  // the cell list, kept for expand_G
  int64_t n_cells = 0, n_obs = 0, nd = 0, ld = 0;
  uint32_t mask = 0;
  int n_fields = 0;

  // Dense sensitivity matrix (Fwd::G), column-major, leading dimension ld.
  int g_storage = -1;
  DevBuf G, row_scale;
  // FP64 G kept beside a reduced-precision G (grada_keep_fp64_G): the reduced
  // entries are rounded from it, and while an inversion runs with
  // predict_fp64 every data prediction (CG right-hand side, trial misfit) is
  // an FP64 product with it instead of d64 + G_lp (m - m_start).
  DevBuf G64;
  bool keep_fp64 = false, g64_valid = false, predict_fp64 = false;
  int64_t fp64_products = 0;
  // Tile plan of the cell list for the assembly (built from host_prisms).
  DevBuf plan_tiles, plan_cells;
  int64_t plan_n_tiles = 0;
  bool plan_valid = false;

  // Work space.
  DevBuf scratch, vx, vy;

  // Inversion data (InversionBase / GaussNewtonInversion members).
  // Operator slots follow GRADA_OP_*: Ws, Wx, Wy, Wz, Tx, Ty, Tz (the T slots
  // hold the unscaled set_Tmatrix() operators; crg[] the a_crg*S_crg*T ones).
  DevOperator ops[7];
  DevOperator crg[3];
  std::vector<int> host_T_rowptr[3], host_T_col[3];
  std::vector<double> host_T_val[3];
  bool crg_enabled = false;
  double a_crg = 1.0;
  std::vector<double> s_crg;
  DevBuf dobs, wd;
  bool data_set = false;

  // CG work vectors.
  DevBuf cg_b, cg_s, cg_t, cg_p, cg_pp, cg_r, cg_atb, cg_gtw, cg_gx, cg_tmpd, cg_scal, cg_part;
  DevBuf cg_wl_ones, cg_ctl, cg_bar, cg_p2, cg_red, cg_redc;
  int fused_grid[4] = {0, 0, 0, 0};  // persistent CG grid per G storage kind
  DevBuf cg_trace;                    // phase trace of a persistent solve (5 u64)
  unsigned long long trace_sum[5] = {0, 0, 0, 0, 0};  // since the last invert / reset
  // The graph of the CG loop's phase kernels (cg_phases.cu), kept across the
  // solves of one shape: its kernels read their arguments from cg_args, which
  // each solve rewrites from the pinned h_cg_args.  phase_key: what the graph
  // bakes in (storage, iterations, grids, the argument buffer).
  DevBuf cg_args;
  FusedCgArgs *h_cg_args = nullptr;
  cudaGraphExec_t phase_exec = nullptr;
  int64_t phase_key[7] = {-1, -1, -1, -1, -1, -1, -1};
  // CG loops since the last invert / reset: host wall ns from the first launch
  // of a solve's loop to its last synchronisation, ns building their graphs,
  // their iterations
  double cg_loop_ns = 0.0, cg_graph_ns = 0.0;
  int64_t cg_loop_iters = 0;
  bool inject_cg_wait = false;       // grada_inject_fault(GRADA_FAULT_CG_WAIT)
  double *h_scal = nullptr;  // pinned
  int *h_flag = nullptr;     // pinned
  int *h_ctl = nullptr;      // pinned

  // Inversion work vectors and records.
  DevBuf iv_m, iv_mt, iv_mt_old, iv_mopt, iv_dx, iv_P, iv_mmin, iv_mmax, iv_m0, iv_wl, iv_tmp,
      iv_tmp2, iv_dpre, iv_d64, iv_mstart, iv_guard, iv_flag;
  std::vector<TrialRecord> trials;
  std::vector<IterationRecord> iterations;

  // Block solves and the lambda sweep (sweep.cu).  Block vectors hold kBW
  // columns row-interleaved (cg_kernels.h).
  DevBuf bscratch, tc_err;
  DevBuf bk_b, bk_s, bk_t, bk_p, bk_pp, bk_r, bk_atb, bk_gtw, bk_gx, bk_tmpd, bk_scal, bk_part,
      bk_ctl, bk_coef;
  DevBuf sw_m, sw_mt, sw_mt_old, sw_mopt, sw_dx, sw_P, sw_mmin, sw_mmax, sw_m0, sw_wl, sw_tmp,
      sw_tmp2, sw_dpre, sw_d64, sw_mstart, sw_guard, sw_flag, sw_in, sw_out;
  double *h_bscal = nullptr;  // pinned, kBW * CG_NSCALARS
  int *h_bctl = nullptr;      // pinned, CTLB_NINTS
  int *h_bflag = nullptr;     // pinned, kBW + 1
  std::vector<std::vector<TrialRecord>> sweep_trials;

  void release_all();

  // inversion.cu
  void set_operator(int which, int64_t n, int64_t nnz, const int *rowptr, const int *col,
                    const double *val);
  void set_cross_gradient(int enabled, double a, const double *S);
  // wavelet.cu: the wavelet-compressed G (g_storage == GRADA_G_WAVELET): rows
  // (CSR, coefficient index ascending), the cell order the rows run along and
  // the partial vectors of G^T y's row blocks
  DevBuf wv_order, wv_rowptr, wv_col, wv_val, wv_part, wv_segptr;
  int64_t wv_ndy = 0, wv_nnz = 0, wv_rows_per_block = 1, wv_blocks = 0, wv_seg_len = 1,
          wv_nseg = 0;
  bool wv_fp32 = false;
  void compute_G_wavelet(const int64_t *order, double rel, int value_storage);
  void apply_G_wavelet(const double *x, double *y, const GemvOpts &o);
  void apply_GT_wavelet(const double *y, double *x, const GemvOpts &o);
  void get_wavelet_G(int64_t *n_dy, int64_t *nnz, int64_t *rowptr, int *col, double *val);
  // operators.cu
  void build_operators(const int *faces, double beta, int depth_flag, const double *alphas);
  void get_operator(int which, int64_t *nnz, int *rowptr, int *col, double *val);
  void set_data(const double *h_dobs, const double *h_wd);
  void ensure_cg_workspace(int nterms);
  void data_prediction(const double *m, const double *m_start, const double *d64, double *out);
  CgTerms cg_terms(double sl, const double *const WL[7], double *b, double *s, double *t);
  bool invert_setup(const grada_invert_params &prm, const double *h_m_ini, const double *h_mmin,
                    const double *h_mmax, const double *h_m0);
  // invert_batch.cu host side: the device description of this context's
  // inversion (after invert_setup), and the records read back after the launch
  DevBuf bt_part2, bt_trials, bt_iters, bt_report;
  int last_batch_teams = 0, last_batch_team_ctas = 0;  // shape of the last persistent batch
  void batch_problem(const grada_invert_params &prm, BatchProblem &bp);
  void batch_results(const grada_invert_params &prm, double *h_m_out, grada_invert_report &rep);
  // CG loop of a single solve: kCgGeneric (graph of the generic product
  // kernels), kCgPhases (graph of the persistent loop's four phases), kCgPersistent
  enum CgLoop { kCgGeneric = 0, kCgPersistent = 1, kCgPhases = 2 };
  CgLoop cg_loop_kind() const;
  CgResult solve_cg_fused(double tol, int maxit, const double *P, double *dx,
                          const ForwardTerms &FT, const AdjointTerms &AT, int64_t nrow, int nb_m,
                          int nb_row, bool persistent);
  CgResult solve_cg_phases(const FusedCgArgs &a, GKind kind, int maxit);
  void count_cg_loop(std::chrono::steady_clock::time_point t_build,
                     std::chrono::steady_clock::time_point t_loop, int iterations);
  CgResult solve_cg_dev(double lambda, double tol, int maxit, const double *mk, const double *mref,
                        const double *P, const double *const WL[7], double *dx,
                        const double *d64, const double *m_start);
  double misfit_of(const double *m, const double *m_start, const double *d64);
  void invert(const grada_invert_params &prm, const double *h_m_ini, const double *h_mmin,
              const double *h_mmax, const double *h_m0, double *h_m_out, grada_invert_report &rep,
              const grada_adaptive_params *adapt = nullptr);
  // adaptive inversion: set while the host's refine callback runs; the model,
  // bounds and reference model on the refined mesh it hands back (4 x Nm)
  bool refine_pending = false;
  std::vector<double> refine_model;

  void upload(void *dst, const void *src, size_t nbytes);
  void download(void *dst, const void *src, size_t nbytes);
  void sync();
  DevGeometry geometry() const;
  DevG devG() const;
  DevG devG64() const;          // the kept FP64 G
  bool fp64_resident() const;   // a kept FP64 G beside a reduced-precision G
  double *scratch_doubles(int64_t n);
  void require_G() const;
  void require_geometry() const;

  void set_geometry(const double *h_prisms, int64_t nc, const double *h_obs, int64_t no,
                    uint32_t fmask);
  void compute_G(int storage);
  void zero_padding_rows(void *base, size_t esz);
  TilePlan tile_plan();
  void G_vec_mul_dev(const double *d_x, double *d_y);
  void GT_vec_mul_dev(const double *d_y, double *d_x);
  // y = G x and x = G^T y for every storage, matrix-free included (GemvOpts
  // scale: G x result / G^T y input; skip: CG stop flag).  Scratch must be
  // sized first with product_scratch_doubles().
  int64_t product_scratch_doubles();
  void apply_G(const double *x, double *y, const GemvOpts &o);
  void apply_GT(const double *y, double *x, const GemvOpts &o);
  void forward_field_dev(const double *d_rho, double *d_fields);
  void expand_G(int64_t n_split, const int64_t *parent, const double *children);  // expand.cu
  void refinement_indicator(const double *m, const int64_t *rowptr, const int64_t *nb,
                            const double *area, double *out);  // refine.cu

  // sweep.cu: block products (kBW columns) for every storage, the block CG
  // solve and the fixed-lambda sweep.
  void ensure_block_scratch(bool fp64_forward);
  void apply_G_block(const double *X, double *Y, const GemvOpts &o);
  void apply_GT_block(const double *Y, double *X, const GemvOpts &o);
  void check_tc_error();
  void ensure_block_workspace(int nterms);
  void block_prediction(const double *m, const double *m_start, const double *d64, double *out);
  void block_misfits(const double *m, const double *m_start, const double *d64, double *out);
  void solve_cg_block_dev(const double *lambda, uint32_t active, double tol, int maxit,
                          const double *mk, const double *mref, const double *P,
                          const double *const WL[7], double *dx, const double *d64,
                          const double *m_start, CgResult *res);
  void G_mat_mul_host(int n, const double *X, double *Y, bool transpose);
  void solve_cg_block_host(double tol, int maxit, int n, const double *lambda, const double *mk,
                           const double *mref, const double *P, const double *const WL[7],
                           double *dx, double *err, int *iters);
  void lambda_sweep(const grada_invert_params &prm, int n, const double *lambdas,
                    const double *m_ini, const double *mmin, const double *mmax, const double *m0,
                    double *m_out, grada_invert_report *reps);
};

// invert_batch.cu: the batched persistent inversion and its tuning table.
int invert_batch_persistent(int n, Context *const *ctxs, const grada_invert_params *params,
                            const double *const *m_ini, const double *const *m_min,
                            const double *const *m_max, const double *const *m0s,
                            double *const *m_out, grada_invert_report *reports, int team_ctas,
                            int *statuses, std::string &err);
int load_batch_tuning(const char *path);
int tuned_team_ctas(double max_entries);

}  // namespace grada

// The C ABI's opaque context is the internal one (every context the ABI
// creates is a grada_ctx, so a Context inside the library may be handed to a
// host callback as one).
struct grada_ctx : public grada::Context {};
