// C ABI of the library (include/grada_gpu.h) and the host-side context that
// mirrors the reference's Fwd object: the geometry it is bound to, the field
// flag, and the dense sensitivity matrix it owns (src/Forward_modelling/Fwd.h:14-94).
// Every entry point converts internal errors into a status code and keeps
// the message for grada_last_error().
#include <atomic>
#include <cmath>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/grada_gpu.h"
#include "common.cuh"
#include "context.h"
#include "kernels.h"

using grada::Error;

namespace grada {

DevBuf::~DevBuf() { release(); }

void DevBuf::release() {
  if (ptr) {
    cudaFree(ptr);
    if (owner) owner->bytes_held -= (int64_t)bytes;
  }
  ptr = nullptr;
  bytes = 0;
}

void DevBuf::alloc(Context *ctx, size_t nbytes) {
  if (ptr && bytes >= nbytes) return;
  release();
  owner = ctx;
  if (nbytes == 0) return;
  if (ctx->inject_alloc_failure) {  // grada_inject_fault(GRADA_FAULT_ALLOC)
    ctx->inject_alloc_failure = false;
    throw Error(GRADA_ERR_OUT_OF_MEMORY,
                "cudaMalloc of " + std::to_string(nbytes) + " bytes: injected failure");
  }
  cudaError_t e = cudaMalloc(&ptr, nbytes);
  if (e != cudaSuccess) {
    ptr = nullptr;
    cudaGetLastError();
    throw Error(e == cudaErrorMemoryAllocation ? GRADA_ERR_OUT_OF_MEMORY : GRADA_ERR_CUDA,
                "cudaMalloc of " + std::to_string(nbytes) + " bytes: " + cudaGetErrorString(e));
  }
  bytes = nbytes;
  ctx->bytes_held += (int64_t)nbytes;
}

void Context::upload(void *dst, const void *src, size_t nbytes) {
  if (nbytes == 0) return;
  GRADA_CUDA_CHECK(cudaMemcpyAsync(dst, src, nbytes, cudaMemcpyHostToDevice, stream));
}

void Context::download(void *dst, const void *src, size_t nbytes) {
  if (nbytes == 0) return;
  GRADA_CUDA_CHECK(cudaMemcpyAsync(dst, src, nbytes, cudaMemcpyDeviceToHost, stream));
}

void Context::sync() { GRADA_CUDA_CHECK(cudaStreamSynchronize(stream)); }

DevGeometry Context::geometry() const {
  DevGeometry g;
  g.prisms = prisms.as<double>();
  g.obs = obs.as<double>();
  g.n_cells = n_cells;
  g.n_obs = n_obs;
  g.mask = mask;
  g.n_fields = n_fields;
  g.tables = math_tables.as<double>();
  g.plan.tiles = plan_tiles.as<int32_t>();
  g.plan.cells = plan_cells.as<int64_t>();
  g.plan.n_tiles = plan_n_tiles;
  return g;
}

DevG Context::devG() const {
  if (g_storage == GRADA_G_WAVELET)
    throw Error(GRADA_ERR_STATE,
                "not available for the wavelet-compressed G (products and solve_cg/invert only)");
  DevG d;
  d.kind = (GKind)g_storage;
  d.data = G.ptr;
  // The scale buffer may be left over from an earlier 16-bit G; only those use it.
  const bool scaled = g_storage == GRADA_G_BF16_ROWSCALE || g_storage == GRADA_G_FP16_ROWSCALE;
  d.row_scale = scaled ? row_scale.as<float>() : nullptr;
  d.nd = nd;
  d.nm = n_cells;
  d.ld = ld;
  return d;
}

double *Context::scratch_doubles(int64_t n) {
  scratch.alloc(this, sizeof(double) * (size_t)n);
  return scratch.as<double>();
}

void Context::require_G() const {
  if (g_storage < 0) throw Error(GRADA_ERR_STATE, "G has not been assembled (call grada_compute_G)");
}

void Context::require_geometry() const {
  if (n_cells <= 0 || n_obs <= 0) throw Error(GRADA_ERR_STATE, "geometry has not been set");
}

void Context::set_geometry(const double *h_prisms, int64_t nc, const double *h_obs, int64_t no,
                           uint32_t fmask) {
  if (!h_prisms || !h_obs) throw Error(GRADA_ERR_INVALID_ARGUMENT, "null geometry pointer");
  if (nc <= 0 || no <= 0) throw Error(GRADA_ERR_INVALID_ARGUMENT, "empty mesh or observation set");
  if (fmask == 0 || (fmask & ~0x3FFu)) throw Error(GRADA_ERR_INVALID_ARGUMENT, "bad field flag");
  for (int64_t c = 0; c < nc; c++) {
    const double *p = h_prisms + 6 * c;
    for (int k = 0; k < 6; k++)
      if (!std::isfinite(p[k])) throw Error(GRADA_ERR_NONFINITE, "non-finite prism coordinate");
    if (!(p[0] < p[1] && p[2] < p[3] && p[4] < p[5]))
      throw Error(GRADA_ERR_INVALID_ARGUMENT,
                  "prism " + std::to_string(c) + " is not (x0<x1, y0<y1, z0<z1)");
  }
  for (int64_t i = 0; i < 3 * no; i++)
    if (!std::isfinite(h_obs[i])) throw Error(GRADA_ERR_NONFINITE, "non-finite observation point");
  // The old G is invalid from here on; its allocation is kept for reuse by the
  // next compute_G when large enough.  Data and operators belong to the old
  // mesh/observation set and must be set again (InversionBase::set_mesh and
  // set_observation reinitialise them the same way).
  g_storage = -1;
  g64_valid = false;
  data_set = false;
  for (auto &o : ops) o.set = false;
  for (auto &o : crg) o.set = false;
  crg_enabled = false;
  n_cells = nc;
  n_obs = no;
  mask = fmask;
  n_fields = __builtin_popcount(fmask);
  nd = (int64_t)n_fields * no;
  // columns start on 128-byte boundaries for 16-bit entries (and 256/512 B for
  // FP32/FP64), so tile loads of a column never straddle an extra sector
  ld = round_up(nd, 64);
  if (!math_tables.ptr) {
    std::vector<double> tab(math_table_size());
    build_math_tables_host(tab.data());
    math_tables.alloc(this, sizeof(double) * tab.size());
    upload(math_tables.ptr, tab.data(), sizeof(double) * tab.size());
    sync();
  }
  prisms.alloc(this, sizeof(double) * 6 * nc);
  obs.alloc(this, sizeof(double) * 3 * no);
  upload(prisms.ptr, h_prisms, sizeof(double) * 6 * nc);
  host_prisms.assign(h_prisms, h_prisms + 6 * nc);
  plan_valid = false;
  upload(obs.ptr, h_obs, sizeof(double) * 3 * no);
  sync();
  tile_plan();  // every kernel walking the cells uses it
}

// The assembly's tile plan for the current cell list (rebuilt after a change
// of the cells).
TilePlan Context::tile_plan() {
  if (!plan_valid) {
    std::vector<int32_t> tiles;
    std::vector<int64_t> cl;
    build_tile_plan(host_prisms.data(), n_cells, tiles, cl);
    plan_tiles.alloc(this, sizeof(int32_t) * tiles.size());
    plan_cells.alloc(this, sizeof(int64_t) * cl.size());
    upload(plan_tiles.ptr, tiles.data(), sizeof(int32_t) * tiles.size());
    upload(plan_cells.ptr, cl.data(), sizeof(int64_t) * cl.size());
    sync();
    plan_n_tiles = (int64_t)tiles.size() / 4;
    plan_valid = true;
  }
  TilePlan p;
  p.tiles = plan_tiles.as<int32_t>();
  p.cells = plan_cells.as<int64_t>();
  p.n_tiles = plan_n_tiles;
  return p;
}

// Rows nd..ld-1 of every column (the padding) set to zero: one 2-D memset.
void Context::zero_padding_rows(void *base, size_t esz) {
  if (ld <= nd) return;
  GRADA_CUDA_CHECK(cudaMemset2DAsync(static_cast<char *>(base) + esz * nd, esz * ld, 0,
                                     esz * (ld - nd), n_cells, stream));
}

void Context::compute_G(int storage) {
  NvtxRange nvtx("grada compute_G");
  require_geometry();
  if (storage < GRADA_G_FP64 || storage > GRADA_G_MATRIX_FREE)
    throw Error(GRADA_ERR_INVALID_ARGUMENT, "unknown G storage");
  const DevGeometry g = geometry();
  const size_t n_entries = (size_t)ld * (size_t)n_cells;
  g_storage = -1;
  g64_valid = false;
  const bool derive = keep_fp64 && storage != GRADA_G_FP64 && storage != GRADA_G_MATRIX_FREE;
  if (derive) {
    // FP64 G kept; the reduced entries are rounded from it below, bitwise what
    // the FP32 assembly writes (it rounds the same FP64 values at the store)
    G64.alloc(this, n_entries * sizeof(double));
    zero_padding_rows(G64.ptr, sizeof(double));
    launch_assemble_tiled_fp64(g, tile_plan(), G64.as<double>(), ld, stream);
  } else if (G64.ptr) {
    G64.release();
  }
  if (storage == GRADA_G_MATRIX_FREE) {
    // nothing to assemble: products re-evaluate the prisms (cfg-5-sized G
    // does not fit in HBM)
  } else if (storage == GRADA_G_FP64) {
    G.alloc(this, n_entries * sizeof(double));
    zero_padding_rows(G.ptr, sizeof(double));
    launch_assemble_tiled_fp64(g, tile_plan(), G.as<double>(), ld, stream);
  } else if (storage == GRADA_G_FP32) {
    G.alloc(this, n_entries * sizeof(float));
    if (derive) {
      launch_round_to_fp32(G64.as<double>(), G.as<float>(), n_entries, stream);
    } else {
      zero_padding_rows(G.ptr, sizeof(float));
      launch_assemble_tiled_fp32(g, tile_plan(), G.as<float>(), ld, stream);
    }
  } else {
    // FP32 staging copy; the quantiser reads its rows < nd and writes zero
    // padding rows itself
    DevBuf tmp;
    tmp.alloc(this, n_entries * sizeof(float));
    if (derive)
      launch_round_to_fp32(G64.as<double>(), tmp.as<float>(), n_entries, stream);
    else
      launch_assemble_tiled_fp32(g, tile_plan(), tmp.as<float>(), ld, stream);
    G.alloc(this, n_entries * sizeof(uint16_t));
    row_scale.alloc(this, sizeof(float) * (size_t)nd);
    launch_rowscale_16(tmp.as<float>(), nd, n_cells, ld, row_scale.as<float>(),
                       G.as<uint16_t>(), storage == GRADA_G_FP16_ROWSCALE, stream);
    sync();
  }
  g_storage = storage;
  g64_valid = derive;
}

DevG Context::devG64() const {
  DevG d;
  d.kind = GKind::FP64;
  d.data = G64.ptr;
  d.nd = nd;
  d.nm = n_cells;
  d.ld = ld;
  return d;
}

bool Context::fp64_resident() const {
  return g64_valid && G64.ptr && g_storage != GRADA_G_FP64 && g_storage != GRADA_G_MATRIX_FREE;
}

int64_t Context::product_scratch_doubles() {
  require_G();
  if (g_storage == GRADA_G_WAVELET) return 3 * wv_ndy;
  if (g_storage == GRADA_G_MATRIX_FREE) {
    const DevGeometry g = geometry();
    const int64_t f = (int64_t)forward_field_splits(g, sm_count) * n_obs * n_fields;
    const int64_t a = (int64_t)adjoint_field_splits(g, sm_count) * n_cells;
    return f > a ? f : a;
  }
  return gemv_scratch_doubles(devG(), sm_count);
}

void Context::apply_G(const double *x, double *y, const GemvOpts &o) {
  double *sc = scratch.as<double>();
  if (g_storage == GRADA_G_WAVELET) {
    apply_G_wavelet(x, y, o);
  } else if (g_storage == GRADA_G_MATRIX_FREE) {
    const DevGeometry g = geometry();
    launch_forward_field(g, x, forward_field_splits(g, sm_count), sc, y, true, stream, o.scale,
                         o.skip);
  } else {
    launch_G_vec_mul(devG(), x, y, sc, sm_count, stream, o);
  }
}

void Context::apply_GT(const double *y, double *x, const GemvOpts &o) {
  double *sc = scratch.as<double>();
  if (g_storage == GRADA_G_WAVELET) {
    apply_GT_wavelet(y, x, o);
  } else if (g_storage == GRADA_G_MATRIX_FREE) {
    const DevGeometry g = geometry();
    launch_adjoint_field(g, y, o.scale, adjoint_field_splits(g, sm_count), sc, x, stream, o.skip);
  } else {
    launch_GT_vec_mul(devG(), y, x, sc, sm_count, stream, o);
  }
}

void Context::G_vec_mul_dev(const double *d_x, double *d_y) {
  require_G();
  scratch_doubles(product_scratch_doubles());
  apply_G(d_x, d_y, GemvOpts());
}

void Context::GT_vec_mul_dev(const double *d_y, double *d_x) {
  require_G();
  scratch_doubles(product_scratch_doubles());
  apply_GT(d_y, d_x, GemvOpts());
}

void Context::forward_field_dev(const double *d_rho, double *d_fields) {
  require_geometry();
  const DevGeometry g = geometry();
  const int splits = forward_field_splits(g, sm_count);
  double *partial = scratch_doubles((int64_t)splits * n_obs * n_fields);
  launch_forward_field(g, d_rho, splits, partial, d_fields, false, stream);
}

}  // namespace grada

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------


namespace {

template <class F>
int guarded(grada_ctx *ctx, F &&f) {
  if (!ctx) return GRADA_ERR_INVALID_ARGUMENT;
  try {
    GRADA_CUDA_CHECK(cudaSetDevice(ctx->device));
    f();
    ctx->last_error.clear();
    return GRADA_OK;
  } catch (const Error &e) {
    ctx->last_error = e.what();
    return e.status;
  } catch (const std::exception &e) {
    ctx->last_error = e.what();
    return GRADA_ERR_CUDA;
  }
}

}  // namespace

namespace {

// Runs job(k) for k in [0, n) on up to max_threads host threads; each k is
// taken by exactly one thread, so each context is driven by one thread.
template <class F>
int run_batch(int n, int max_threads, int *statuses, F &&job) {
  if (n <= 0) return GRADA_OK;
  int nt = (max_threads <= 0 || max_threads > n) ? n : max_threads;
  std::atomic<int> next(0);
  std::vector<int> st(n, GRADA_OK);
  auto worker = [&]() {
    for (int k = next++; k < n; k = next++) st[k] = job(k);
  };
  std::vector<std::thread> pool;
  for (int t = 1; t < nt; t++) pool.emplace_back(worker);
  worker();
  for (auto &th : pool) th.join();
  int first = GRADA_OK;
  for (int k = 0; k < n; k++) {
    if (statuses) statuses[k] = st[k];
    if (first == GRADA_OK && st[k] != GRADA_OK) first = st[k];
  }
  return first;
}

}  // namespace

extern "C" {

int grada_version(void) { return 100; }

int grada_ctx_create(int device, grada_ctx **out) {
  if (!out) return GRADA_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) {
    cudaGetLastError();
    return GRADA_ERR_CUDA;
  }
  grada_ctx *c = new grada_ctx();
  c->device = device;
  if (cudaSetDevice(device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) {
    cudaGetLastError();
    delete c;
    return GRADA_ERR_CUDA;
  }
  *out = c;
  return GRADA_OK;
}

int grada_ctx_destroy(grada_ctx *ctx) {
  if (!ctx) return GRADA_OK;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  ctx->release_all();
  cudaStreamDestroy(ctx->stream);
  delete ctx;
  return GRADA_OK;
}

const char *grada_last_error(const grada_ctx *ctx) {
  return ctx ? ctx->last_error.c_str() : "null context";
}

void *grada_ctx_stream(grada_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

int grada_sync(grada_ctx *ctx) {
  return guarded(ctx, [&] { ctx->sync(); });
}

int64_t grada_ctx_device_bytes(const grada_ctx *ctx) { return ctx ? ctx->bytes_held : 0; }

int grada_set_geometry(grada_ctx *ctx, const double *prisms, int64_t n_cells, const double *obs,
                       int64_t n_obs, uint32_t field_flag) {
  return guarded(ctx, [&] { ctx->set_geometry(prisms, n_cells, obs, n_obs, field_flag); });
}

int grada_get_dims(const grada_ctx *ctx, int64_t *n_cells, int64_t *n_obs, int *n_fields,
                   int64_t *nd, int64_t *ld) {
  if (!ctx) return GRADA_ERR_INVALID_ARGUMENT;
  if (n_cells) *n_cells = ctx->n_cells;
  if (n_obs) *n_obs = ctx->n_obs;
  if (n_fields) *n_fields = ctx->n_fields;
  if (nd) *nd = ctx->nd;
  if (ld) *ld = ctx->ld;
  return GRADA_OK;
}

int grada_compute_G(grada_ctx *ctx, int storage) {
  return guarded(ctx, [&] {
    ctx->compute_G(storage);
    ctx->sync();
  });
}

int grada_G_storage(const grada_ctx *ctx) { return ctx ? ctx->g_storage : -1; }

int grada_get_G(grada_ctx *ctx, double *host, int64_t ld_host) {
  return guarded(ctx, [&] {
    ctx->require_G();
    if (ctx->g_storage == GRADA_G_MATRIX_FREE)
      throw Error(GRADA_ERR_STATE, "matrix-free mode stores no G");
    if (!host || ld_host < ctx->nd) throw Error(GRADA_ERR_INVALID_ARGUMENT, "bad host buffer");
    // Widen column blocks to FP64 on the device, then copy them out.
    const int64_t cols_per_block = 256;
    grada::DevBuf stage;
    stage.alloc(ctx, sizeof(double) * (size_t)ctx->ld * cols_per_block);
    std::vector<double> tmp;
    for (int64_t c0 = 0; c0 < ctx->n_cells; c0 += cols_per_block) {
      const int64_t nc = std::min(cols_per_block, ctx->n_cells - c0);
      grada::launch_widen_columns(ctx->devG(), c0, nc, stage.as<double>(), ctx->stream);
      if (ld_host == ctx->ld) {
        ctx->download(host + c0 * ld_host, stage.ptr, sizeof(double) * (size_t)(ctx->ld * nc));
      } else {
        GRADA_CUDA_CHECK(cudaMemcpy2DAsync(host + c0 * ld_host, sizeof(double) * ld_host,
                                           stage.ptr, sizeof(double) * ctx->ld,
                                           sizeof(double) * ctx->nd, nc, cudaMemcpyDeviceToHost,
                                           ctx->stream));
      }
      ctx->sync();
    }
  });
}

int grada_get_G_rows(grada_ctx *ctx, const int64_t *rows, int64_t n_rows, double *host) {
  return guarded(ctx, [&] {
    ctx->require_G();
    if (ctx->g_storage == GRADA_G_MATRIX_FREE || ctx->g_storage == GRADA_G_WAVELET)
      throw Error(GRADA_ERR_STATE, "no stored dense G to read rows from");
    if (n_rows < 0 || (n_rows > 0 && (!rows || !host)))
      throw Error(GRADA_ERR_INVALID_ARGUMENT, "bad row list or host buffer");
    for (int64_t r = 0; r < n_rows; r++)
      if (rows[r] < 0 || rows[r] >= ctx->nd)
        throw Error(GRADA_ERR_INVALID_ARGUMENT, "row index " + std::to_string(rows[r]) +
                                                    " outside G's " + std::to_string(ctx->nd) + " rows");
    const int64_t nm = ctx->n_cells;
    // rows in chunks whose FP64 copies take at most ~256 MB of device memory
    const int64_t chunk = std::max<int64_t>(1, std::min<int64_t>(65535, ((int64_t)1 << 25) / nm));
    grada::DevBuf d_rows, stage;
    d_rows.alloc(ctx, sizeof(int64_t) * (size_t)std::min(chunk, n_rows));
    stage.alloc(ctx, sizeof(double) * (size_t)(std::min(chunk, n_rows) * nm));
    for (int64_t r0 = 0; r0 < n_rows; r0 += chunk) {
      const int64_t nr = std::min(chunk, n_rows - r0);
      ctx->upload(d_rows.ptr, rows + r0, sizeof(int64_t) * (size_t)nr);
      grada::launch_gather_rows(ctx->devG(), d_rows.as<int64_t>(), nr, stage.as<double>(),
                                ctx->stream);
      ctx->download(host + r0 * nm, stage.ptr, sizeof(double) * (size_t)(nr * nm));
      ctx->sync();
    }
  });
}

int grada_G_vec_mul(grada_ctx *ctx, const double *x, double *y) {
  return guarded(ctx, [&] {
    ctx->require_G();
    if (!x || !y) throw Error(GRADA_ERR_INVALID_ARGUMENT, "null vector");
    ctx->vx.alloc(ctx, sizeof(double) * ctx->n_cells);
    ctx->vy.alloc(ctx, sizeof(double) * ctx->ld);
    ctx->upload(ctx->vx.ptr, x, sizeof(double) * ctx->n_cells);
    ctx->G_vec_mul_dev(ctx->vx.as<double>(), ctx->vy.as<double>());
    ctx->download(y, ctx->vy.ptr, sizeof(double) * ctx->nd);
    ctx->sync();
  });
}

int grada_GT_vec_mul(grada_ctx *ctx, const double *y, double *x) {
  return guarded(ctx, [&] {
    ctx->require_G();
    if (!x || !y) throw Error(GRADA_ERR_INVALID_ARGUMENT, "null vector");
    ctx->vx.alloc(ctx, sizeof(double) * ctx->n_cells);
    ctx->vy.alloc(ctx, sizeof(double) * ctx->ld);
    ctx->upload(ctx->vy.ptr, y, sizeof(double) * ctx->nd);
    ctx->GT_vec_mul_dev(ctx->vy.as<double>(), ctx->vx.as<double>());
    ctx->download(x, ctx->vx.ptr, sizeof(double) * ctx->n_cells);
    ctx->sync();
  });
}

int grada_G_vec_mul_dev(grada_ctx *ctx, const double *d_x, double *d_y) {
  return guarded(ctx, [&] { ctx->G_vec_mul_dev(d_x, d_y); });
}

int grada_GT_vec_mul_dev(grada_ctx *ctx, const double *d_y, double *d_x) {
  return guarded(ctx, [&] { ctx->GT_vec_mul_dev(d_y, d_x); });
}

int grada_expand_G(grada_ctx *ctx, int64_t n_split, const int64_t *parent_index,
                   const double *child_prisms) {
  return guarded(ctx, [&] { ctx->expand_G(n_split, parent_index, child_prisms); });
}

int grada_forward_field(grada_ctx *ctx, const double *rho, double *fields) {
  return guarded(ctx, [&] {
    ctx->require_geometry();
    if (!rho || !fields) throw Error(GRADA_ERR_INVALID_ARGUMENT, "null vector");
    ctx->vx.alloc(ctx, sizeof(double) * ctx->n_cells);
    ctx->vy.alloc(ctx, sizeof(double) * ctx->ld);
    ctx->upload(ctx->vx.ptr, rho, sizeof(double) * ctx->n_cells);
    ctx->forward_field_dev(ctx->vx.as<double>(), ctx->vy.as<double>());
    ctx->download(fields, ctx->vy.ptr, sizeof(double) * ctx->nd);
    ctx->sync();
  });
}

int grada_forward_field_dev(grada_ctx *ctx, const double *d_rho, double *d_fields) {
  return guarded(ctx, [&] { ctx->forward_field_dev(d_rho, d_fields); });
}

int grada_measure_fp64_peak(grada_ctx *ctx, double *flops_per_s) {
  return guarded(ctx, [&] {
    if (!flops_per_s) throw Error(GRADA_ERR_INVALID_ARGUMENT, "null output");
    *flops_per_s = grada::measure_fp64_fma_rate(ctx->sm_count, ctx->stream);
  });
}

int grada_set_operator(grada_ctx *ctx, int which, int64_t n, int64_t nnz, const int *rowptr,
                       const int *col, const double *val) {
  return guarded(ctx, [&] { ctx->set_operator(which, n, nnz, rowptr, col, val); });
}

int grada_set_cross_gradient(grada_ctx *ctx, int enabled, double a_crg, const double *S_crg) {
  return guarded(ctx, [&] { ctx->set_cross_gradient(enabled, a_crg, S_crg); });
}

int grada_set_data(grada_ctx *ctx, const double *dobs, const double *wd) {
  return guarded(ctx, [&] { ctx->set_data(dobs, wd); });
}

int grada_solve_cg(grada_ctx *ctx, double tol, int maxit, double lambda, const double *mk,
                   const double *mref, const double *P, const double *const WL[7], double *dx,
                   double *err, int *iterations) {
  return guarded(ctx, [&] {
    ctx->require_G();
    if (!mk || !mref || !P || !dx) throw Error(GRADA_ERR_INVALID_ARGUMENT, "null vector");
    if (!(lambda >= 0.0) || !std::isfinite(lambda))
      throw Error(GRADA_ERR_INVALID_ARGUMENT, "lambda must be finite and >= 0");
    const int64_t Nm = ctx->n_cells;
    const size_t vb = sizeof(double) * Nm;
    ctx->iv_m.alloc(ctx, vb);
    ctx->iv_m0.alloc(ctx, vb);
    ctx->iv_P.alloc(ctx, vb);
    ctx->iv_dx.alloc(ctx, vb);
    ctx->iv_wl.alloc(ctx, vb * 7);
    ctx->upload(ctx->iv_m.ptr, mk, vb);
    ctx->upload(ctx->iv_m0.ptr, mref, vb);
    ctx->upload(ctx->iv_P.ptr, P, vb);
    const double *wl_dev[7];
    for (int k = 0; k < 7; k++) {
      if (WL && WL[k]) {
        double *d = ctx->iv_wl.as<double>() + k * Nm;
        ctx->upload(d, WL[k], vb);
        wl_dev[k] = d;
      } else {
        wl_dev[k] = nullptr;
      }
    }
    grada::CgResult r = ctx->solve_cg_dev(lambda, tol, maxit, ctx->iv_m.as<double>(),
                                          ctx->iv_m0.as<double>(), ctx->iv_P.as<double>(), wl_dev,
                                          ctx->iv_dx.as<double>(), nullptr, nullptr);
    ctx->download(dx, ctx->iv_dx.ptr, vb);
    ctx->sync();
    if (err) *err = r.err;
    if (iterations) *iterations = r.iterations;
  });
}

int grada_G_column_norms(grada_ctx *ctx, double *norms) {
  return guarded(ctx, [&] {
    ctx->require_G();
    if (!norms) throw grada::Error(GRADA_ERR_INVALID_ARGUMENT, "null output");
    if (ctx->g_storage == GRADA_G_MATRIX_FREE)
      throw grada::Error(GRADA_ERR_STATE, "column norms need a stored G (not matrix-free)");
    grada::DevBuf d;
    d.alloc(ctx, sizeof(double) * (size_t)ctx->n_cells);
    grada::launch_column_norms(ctx->devG(), d.as<double>(), ctx->stream);
    ctx->download(norms, d.ptr, sizeof(double) * (size_t)ctx->n_cells);
    ctx->sync();
  });
}

int grada_build_operators(grada_ctx *ctx, const int32_t *faces, double beta, int depth_flag,
                          const double *alphas) {
  return guarded(ctx, [&] { ctx->build_operators(faces, beta, depth_flag, alphas); });
}

int grada_get_operator(grada_ctx *ctx, int which, int64_t *nnz, int *rowptr, int *col,
                       double *val) {
  return guarded(ctx, [&] { ctx->get_operator(which, nnz, rowptr, col, val); });
}

int grada_compute_G_wavelet(grada_ctx *ctx, const int64_t *order, double relative_threshold) {
  return guarded(ctx, [&] { ctx->compute_G_wavelet(order, relative_threshold, GRADA_G_FP64); });
}

int grada_compute_G_wavelet_ex(grada_ctx *ctx, const int64_t *order, double relative_threshold,
                               int value_storage) {
  return guarded(ctx,
                 [&] { ctx->compute_G_wavelet(order, relative_threshold, value_storage); });
}

int grada_get_wavelet_G(grada_ctx *ctx, int64_t *n_dy, int64_t *nnz, int64_t *rowptr, int32_t *col,
                        double *val) {
  return guarded(ctx, [&] { ctx->get_wavelet_G(n_dy, nnz, rowptr, col, val); });
}

int grada_keep_fp64_G(grada_ctx *ctx, int keep) {
  return guarded(ctx, [&] { ctx->keep_fp64 = keep != 0; });
}

int grada_invert(grada_ctx *ctx, const grada_invert_params *params, const double *m_ini,
                 const double *m_min, const double *m_max, const double *m0, double *m_out,
                 grada_invert_report *report) {
  return guarded(ctx, [&] {
    if (!params) throw Error(GRADA_ERR_INVALID_ARGUMENT, "null parameters");
    grada_invert_report rep;
    ctx->invert(*params, m_ini, m_min, m_max, m0, m_out, rep);
    if (report) *report = rep;
  });
}

int grada_invert_adaptive(grada_ctx *ctx, const grada_invert_params *params,
                          const grada_adaptive_params *adaptive, const double *m_ini,
                          const double *m_min, const double *m_max, const double *m0,
                          grada_invert_report *report) {
  return guarded(ctx, [&] {
    if (!params || !adaptive) throw Error(GRADA_ERR_INVALID_ARGUMENT, "null parameters");
    grada_invert_report rep;
    ctx->invert(*params, m_ini, m_min, m_max, m0, nullptr, rep, adaptive);
    if (report) *report = rep;
  });
}

int grada_set_inversion_model(grada_ctx *ctx, const double *m, const double *m_min,
                              const double *m_max, const double *m0) {
  return guarded(ctx, [&] {
    if (!ctx->refine_pending)
      throw Error(GRADA_ERR_STATE, "grada_set_inversion_model is for refine callbacks");
    if (!m || !m_min || !m_max) throw Error(GRADA_ERR_INVALID_ARGUMENT, "null model vector");
    const size_t n = (size_t)ctx->n_cells;
    std::vector<double> v(4 * n, 0.0);
    std::memcpy(v.data(), m, sizeof(double) * n);
    std::memcpy(v.data() + n, m_min, sizeof(double) * n);
    std::memcpy(v.data() + 2 * n, m_max, sizeof(double) * n);
    if (m0) std::memcpy(v.data() + 3 * n, m0, sizeof(double) * n);
    for (size_t i = 0; i < n; i++)
      if (!(v[n + i] < v[2 * n + i]))
        throw Error(GRADA_ERR_INVALID_ARGUMENT, "m_min must be < m_max");
    ctx->refine_model.swap(v);
  });
}

int grada_cg_phase_times(grada_ctx *ctx, double *mean_ns, int64_t *iterations) {
  return guarded(ctx, [&] {
    const unsigned long long it = ctx->trace_sum[4];
    if (iterations) *iterations = (int64_t)it;
    if (mean_ns)
      for (int q = 0; q < 4; q++) mean_ns[q] = it ? (double)ctx->trace_sum[q] / (double)it : 0.0;
  });
}

int grada_cg_loop_time(grada_ctx *ctx, double *seconds, int64_t *iterations) {
  return guarded(ctx, [&] {
    if (iterations) *iterations = ctx->cg_loop_iters;
    if (seconds) {
      seconds[0] = ctx->cg_loop_ns * 1e-9;
      seconds[1] = ctx->cg_graph_ns * 1e-9;
    }
  });
}

int grada_get_model(grada_ctx *ctx, double *m) {
  return guarded(ctx, [&] {
    if (!m) throw Error(GRADA_ERR_INVALID_ARGUMENT, "null model vector");
    if (!ctx->iv_m.ptr || ctx->iv_m.bytes < sizeof(double) * (size_t)ctx->n_cells)
      throw Error(GRADA_ERR_STATE, "no inversion has run");
    ctx->download(m, ctx->iv_m.ptr, sizeof(double) * (size_t)ctx->n_cells);
    ctx->sync();
  });
}

int grada_get_trials(const grada_ctx *ctx, double *rows, int64_t cap, int64_t *n) {
  if (!ctx) return GRADA_ERR_INVALID_ARGUMENT;
  const int64_t total = (int64_t)ctx->trials.size();
  if (n) *n = total;
  for (int64_t k = 0; k < total && k < cap && rows; k++) {
    const grada::TrialRecord &t = ctx->trials[k];
    double *o = rows + 5 * k;
    o[0] = t.gn_iteration;
    o[1] = t.lambda;
    o[2] = t.misfit;
    o[3] = t.cg_iterations;
    o[4] = t.cg_error;
  }
  return GRADA_OK;
}

int grada_compute_G_batch(int n, grada_ctx *const *ctxs, int storage, int max_threads,
                          int *statuses) {
  if (n < 0 || (n > 0 && !ctxs)) return GRADA_ERR_INVALID_ARGUMENT;
  return run_batch(n, max_threads, statuses,
                   [&](int k) { return grada_compute_G(ctxs[k], storage); });
}

int grada_invert_batch(int n, grada_ctx *const *ctxs, const grada_invert_params *params,
                       const double *const *m_ini, const double *const *m_min,
                       const double *const *m_max, const double *const *m0s,
                       double *const *m_out, grada_invert_report *reports, int max_threads,
                       int *statuses) {
  if (n < 0 || (n > 0 && (!ctxs || !params || !m_ini || !m_min || !m_max || !m_out)))
    return GRADA_ERR_INVALID_ARGUMENT;
  return run_batch(n, max_threads, statuses, [&](int k) {
    return grada_invert(ctxs[k], &params[k], m_ini[k], m_min[k], m_max[k], m0s ? m0s[k] : nullptr,
                        m_out[k], reports ? &reports[k] : nullptr);
  });
}

int grada_invert_batch_persistent(int n, grada_ctx *const *ctxs, const grada_invert_params *params,
                                  const double *const *m_ini, const double *const *m_min,
                                  const double *const *m_max, const double *const *m0s,
                                  double *const *m_out, grada_invert_report *reports,
                                  int team_ctas, int *statuses) {
  if (n < 0 || (n > 0 && (!ctxs || !params || !m_ini || !m_min || !m_max || !m_out)))
    return GRADA_ERR_INVALID_ARGUMENT;
  if (n == 0) return GRADA_OK;
  for (int k = 0; k < n; k++)
    if (!ctxs[k] || !m_ini[k] || !m_min[k] || !m_max[k] || !m_out[k])
      return GRADA_ERR_INVALID_ARGUMENT;
  std::vector<grada::Context *> cs(ctxs, ctxs + n);
  std::string err;
  int st = GRADA_OK;
  try {
    if (cudaSetDevice(ctxs[0]->device) != cudaSuccess) return GRADA_ERR_CUDA;
    st = grada::invert_batch_persistent(n, cs.data(), params, m_ini, m_min, m_max, m0s, m_out,
                                        reports, team_ctas, statuses, err);
  } catch (const std::exception &e) {
    err = e.what();
    st = GRADA_ERR_CUDA;
  }
  ctxs[0]->last_error = (st == GRADA_OK) ? std::string() : err;
  return st;
}

int grada_load_batch_tuning(const char *path) {
  if (!path) return GRADA_ERR_INVALID_ARGUMENT;
  return grada::load_batch_tuning(path);
}

int grada_batch_shape(const grada_ctx *ctx, int *teams, int *team_ctas) {
  if (!ctx) return GRADA_ERR_INVALID_ARGUMENT;
  if (teams) *teams = ctx->last_batch_teams;
  if (team_ctas) *team_ctas = ctx->last_batch_team_ctas;
  return GRADA_OK;
}

int grada_get_iterations(const grada_ctx *ctx, double *rows, int64_t cap, int64_t *n) {
  if (!ctx) return GRADA_ERR_INVALID_ARGUMENT;
  const int64_t total = (int64_t)ctx->iterations.size();
  if (n) *n = total;
  for (int64_t k = 0; k < total && k < cap && rows; k++) {
    const grada::IterationRecord &t = ctx->iterations[k];
    double *o = rows + 3 * k;
    o[0] = t.gn_iteration;
    o[1] = t.n_trials;
    o[2] = t.misfit;
  }
  return GRADA_OK;
}

int grada_G_mat_mul(grada_ctx *ctx, int n_rhs, const double *X, double *Y) {
  return guarded(ctx, [&] { ctx->G_mat_mul_host(n_rhs, X, Y, false); });
}

int grada_GT_mat_mul(grada_ctx *ctx, int n_rhs, const double *Y, double *X) {
  return guarded(ctx, [&] { ctx->G_mat_mul_host(n_rhs, Y, X, true); });
}

int grada_G_block_mul_dev(grada_ctx *ctx, const double *d_X, double *d_Y) {
  return guarded(ctx, [&] {
    ctx->ensure_block_scratch(false);
    ctx->apply_G_block(d_X, d_Y, grada::GemvOpts());
  });
}

int grada_GT_block_mul_dev(grada_ctx *ctx, const double *d_Y, double *d_X) {
  return guarded(ctx, [&] {
    ctx->ensure_block_scratch(false);
    ctx->apply_GT_block(d_Y, d_X, grada::GemvOpts());
  });
}

int grada_solve_cg_block(grada_ctx *ctx, double tol, int maxit, int n_rhs, const double *lambda,
                         const double *mk, const double *mref, const double *P,
                         const double *const WL[7], double *dx, double *err, int *iterations) {
  return guarded(ctx, [&] {
    ctx->solve_cg_block_host(tol, maxit, n_rhs, lambda, mk, mref, P, WL, dx, err, iterations);
  });
}

int grada_lambda_sweep(grada_ctx *ctx, const grada_invert_params *prm, int n_lambda,
                       const double *lambdas, const double *m_ini, const double *m_min,
                       const double *m_max, const double *m0, double *m_out,
                       grada_invert_report *reports) {
  if (!prm) return GRADA_ERR_INVALID_ARGUMENT;
  return guarded(ctx, [&] {
    ctx->lambda_sweep(*prm, n_lambda, lambdas, m_ini, m_min, m_max, m0, m_out, reports);
  });
}

int grada_get_sweep_trials(const grada_ctx *ctx, int column, double *rows, int64_t cap,
                           int64_t *n) {
  if (!ctx || column < 0 || column >= (int)ctx->sweep_trials.size())
    return GRADA_ERR_INVALID_ARGUMENT;
  const std::vector<grada::TrialRecord> &tr = ctx->sweep_trials[column];
  const int64_t total = (int64_t)tr.size();
  if (n) *n = total;
  for (int64_t k = 0; k < total && k < cap && rows; k++) {
    double *o = rows + 5 * k;
    o[0] = tr[k].gn_iteration;
    o[1] = tr[k].lambda;
    o[2] = tr[k].misfit;
    o[3] = tr[k].cg_iterations;
    o[4] = tr[k].cg_error;
  }
  return GRADA_OK;
}

int grada_refinement_indicator(grada_ctx *ctx, const double *m, const int64_t *rowptr,
                               const int64_t *neighbour, const double *area, double *indicator) {
  return guarded(ctx, [&] { ctx->refinement_indicator(m, rowptr, neighbour, area, indicator); });
}

int grada_inject_fault(grada_ctx *ctx, int fault) {
  return guarded(ctx, [&] {
    if (fault == GRADA_FAULT_ALLOC) {
      ctx->inject_alloc_failure = true;
    } else if (fault == GRADA_FAULT_TC_TIMEOUT) {
      // the flag a tensor-core product raises when one of its bounded waits
      // expires; the next block product's host check reports it
      ctx->tc_err.alloc(ctx, sizeof(int) * 4);
      const int flag = 1;
      ctx->upload(ctx->tc_err.ptr, &flag, sizeof(int));
      ctx->sync();
    } else if (fault == GRADA_FAULT_CG_WAIT) {
      ctx->inject_cg_wait = true;
    } else if (fault == GRADA_FAULT_TC_WAIT) {
      // arms the tensor-core kernels' expiry test (word 1 of their flag
      // block); the host check that reports the expiry disarms it
      ctx->tc_err.alloc(ctx, sizeof(int) * 4);
      const int arm[2] = {0, 1};
      ctx->upload(ctx->tc_err.ptr, arm, sizeof(arm));
      ctx->sync();
    } else if (fault != GRADA_FAULT_NONE) {
      throw grada::Error(GRADA_ERR_INVALID_ARGUMENT, "unknown fault kind");
    } else {
      ctx->inject_alloc_failure = false;
      ctx->inject_cg_wait = false;
      if (ctx->tc_err.ptr) {
        GRADA_CUDA_CHECK(cudaMemsetAsync(ctx->tc_err.ptr, 0, sizeof(int) * 4, ctx->stream));
        ctx->sync();
      }
    }
  });
}

}  // extern "C"
