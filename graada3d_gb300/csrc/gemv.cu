// K2/K3: dense products with the stored sensitivity matrix.
//
// Reference: Fwd::G_vec_mul / Fwd::GT_vec_mul, dense branches
// (src/Forward_modelling/Fwd.cpp:145 `product = G * vec`, :111
// `product = G.transpose() * vec`), i.e. Eigen GEMV on a column-major
// MatrixXd.
//
// Both products stream G once from HBM with 16-byte vector loads and are
// bound by HBM bandwidth.  G is column-major with leading dimension ld (a
// multiple of 64, padding rows zero), so:
//  * G^T y: a block owns 32 consecutive columns, 4 per warp; the lanes walk
//    the rows with 16-byte loads, multiply by y (staged per row chunk in
//    shared memory and reused for the warp's 4 columns) and each column is
//    summed with a warp butterfly.  Deterministic: fixed per-lane row order
//    and tree.
//  * G x: a block owns a tile of 256*VEC rows and a range of columns; threads
//    accumulate VEC rows each over that range; the column ranges' partial rows
//    go to scratch and a second pass sums them (32 rows per block, the ranges
//    shared by the block's 8 warps, then added in warp order; deterministic,
//    no atomics).
// FP64 G accumulates in FP64.  FP32 / bf16 G multiply and accumulate in FP32
// (the vector is rounded to FP32 once); partial sums across blocks are added
// in FP64.  bf16 rows carry an FP32 scale applied after the row sum (G x) or
// folded into y (G^T y).
#include "common.cuh"
#include "gemv_body.cuh"
#include "kernels.h"

namespace grada {

namespace {

using gemv::LoadBF16;
using gemv::LoadF16;
using gemv::LoadF32;
using gemv::LoadF64;
constexpr int GV_THREADS = gemv::kThreads;

// ---- G x ----------------------------------------------------------------------

template <class L>
__global__ void __launch_bounds__(GV_THREADS)
    gx_partial_kernel(const void *__restrict__ G, int64_t ld, int64_t nm, int64_t cols_per_split,
                      const double *x, double *partial, const int *__restrict__ skip) {
  if (skip && *skip) return;
  gemv::gx_partial_body<L>(G, ld, nm, cols_per_split, x, partial, blockIdx.x, blockIdx.y);
}

__global__ void gx_finish_kernel(const double *partial, int n_split, int64_t ld, int64_t nd,
                                 const float *__restrict__ row_scale,
                                 const double *__restrict__ post_scale, double *y,
                                 const int *__restrict__ skip) {
  if (skip && *skip) return;
  gemv::gx_finish_body(partial, n_split, ld, nd, row_scale, post_scale, y, blockIdx.x);
}

// ---- G^T y --------------------------------------------------------------------

template <class L>
__global__ void __launch_bounds__(GV_THREADS)
    gty_kernel(const void *__restrict__ G, int64_t ld, int64_t nm, const typename L::Acc *y,
               double *x, const int *__restrict__ skip) {
  if (skip && *skip) return;
  int64_t col = -1;
  const double s = gemv::gty_body<L>(G, ld, nm, y, blockIdx.x, &col);
  if (col >= 0) x[col] = s;
}

// y (FP64, nd entries) -> padded vector of the accumulation type, times the
// row scale for bf16, zero in the padding rows.
template <typename Acc>
__global__ void prep_y_kernel(const double *y, int64_t nd, int64_t ld,
                              const float *__restrict__ row_scale,
                              const double *__restrict__ pre_scale, Acc *out,
                              const int *__restrict__ skip) {
  if (skip && *skip) return;
  gemv::prep_y_body<Acc>(y, nd, ld, row_scale, pre_scale, out, blockIdx.x);
}

__global__ void widen_kernel(const void *__restrict__ G, int kind, const float *__restrict__ scale,
                             int64_t nd, int64_t ld, int64_t c0, double *__restrict__ out) {
  const int64_t r = (int64_t)blockIdx.y * blockDim.x + threadIdx.x;
  const int64_t c = blockIdx.x;
  if (r >= ld) return;
  const int64_t src = r + (c0 + c) * ld;
  double v;
  if (kind == 0) {
    v = static_cast<const double *>(G)[src];
  } else if (kind == 1) {
    v = (double)static_cast<const float *>(G)[src];
  } else if (kind == 2) {
    const uint32_t bits = (uint32_t) static_cast<const uint16_t *>(G)[src] << 16;
    v = (double)__uint_as_float(bits) * (r < nd ? (double)scale[r] : 0.0);
  } else {
    const __half h = __ushort_as_half(static_cast<const uint16_t *>(G)[src]);
    v = (double)__half2float(h) * (r < nd ? (double)scale[r] : 0.0);
  }
  out[r + c * ld] = v;
}

template <class L>
void run_gx(const DevG &G, const double *x, double *y, double *scratch, int sm_count,
            const GemvOpts &o, cudaStream_t s) {
  const int splits = gx_splits(G, sm_count, L::VEC);
  const int64_t per = ceil_div(G.nm, splits);
  dim3 grid((unsigned)ceil_div(G.ld, (int64_t)GV_THREADS * L::VEC), (unsigned)splits);
  gx_partial_kernel<L><<<grid, GV_THREADS, 0, s>>>(G.data, G.ld, G.nm, per, x, scratch, o.skip);
  GRADA_LAUNCH_CHECK();
  gx_finish_kernel<<<(unsigned)ceil_div(G.nd, gemv::kFinishRows), GV_THREADS, 0, s>>>(
      scratch, splits, G.ld, G.nd, G.row_scale, o.scale, y, o.skip);
  GRADA_LAUNCH_CHECK();
}

}  // namespace

int gx_splits(const DevG &G, int sm_count, int vec) {
  const int64_t tiles = ceil_div(G.ld, (int64_t)GV_THREADS * vec);
  int64_t splits = ceil_div((int64_t)sm_count * 8, tiles);
  const int64_t max_splits = ceil_div(G.nm, 64);
  if (splits > max_splits) splits = max_splits;
  if (splits < 1) splits = 1;
  if (splits > 65535) splits = 65535;
  return (int)splits;
}

int vec_of(GKind k) { return k == GKind::FP64 ? 2 : (k == GKind::FP32 ? 4 : 8); }

int64_t gemv_scratch_doubles(const DevG &G, int sm_count) {
  const int splits = gx_splits(G, sm_count, vec_of(G.kind));
  const int64_t gx = (int64_t)splits * G.ld;
  const int64_t gty = G.ld;  // converted y (FP32 uses half of it)
  return gx > gty ? gx : gty;
}

void launch_G_vec_mul(const DevG &G, const double *x, double *y, double *scratch, int sm_count,
                      cudaStream_t s, const GemvOpts &o) {
  if (G.nd <= 0 || G.nm <= 0) return;
  switch (G.kind) {
    case GKind::FP64: run_gx<LoadF64>(G, x, y, scratch, sm_count, o, s); break;
    case GKind::FP32: run_gx<LoadF32>(G, x, y, scratch, sm_count, o, s); break;
    case GKind::BF16: run_gx<LoadBF16>(G, x, y, scratch, sm_count, o, s); break;
    case GKind::FP16: run_gx<LoadF16>(G, x, y, scratch, sm_count, o, s); break;
  }
}

namespace {

// out[r * nm + j] = G(rows[r], j) widened to FP64 (16-bit entries times their
// row scale); one thread per (row, column), blockIdx.y = the row.
__global__ void gather_rows_kernel(const void *__restrict__ G, int kind,
                                   const float *__restrict__ scale, int64_t nm, int64_t ld,
                                   const int64_t *__restrict__ rows, double *__restrict__ out) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nm) return;
  const int64_t r = rows[blockIdx.y];
  const int64_t src = r + j * ld;
  double v;
  if (kind == 0) {
    v = static_cast<const double *>(G)[src];
  } else if (kind == 1) {
    v = (double)static_cast<const float *>(G)[src];
  } else if (kind == 2) {
    const uint32_t bits = (uint32_t) static_cast<const uint16_t *>(G)[src] << 16;
    v = (double)__uint_as_float(bits) * (double)scale[r];
  } else {
    const __half h = __ushort_as_half(static_cast<const uint16_t *>(G)[src]);
    v = (double)__half2float(h) * (double)scale[r];
  }
  out[(int64_t)blockIdx.y * nm + j] = v;
}

}  // namespace

void launch_gather_rows(const DevG &G, const int64_t *rows, int64_t n_rows, double *out,
                        cudaStream_t s) {
  if (n_rows <= 0 || G.nm <= 0) return;
  dim3 grid((unsigned)ceil_div(G.nm, 256), (unsigned)n_rows);
  gather_rows_kernel<<<grid, 256, 0, s>>>(G.data, (int)G.kind, G.row_scale, G.nm, G.ld, rows, out);
  GRADA_LAUNCH_CHECK();
}

void launch_widen_columns(const DevG &G, int64_t c0, int64_t nc, double *out, cudaStream_t s) {
  if (nc <= 0) return;
  dim3 grid((unsigned)nc, (unsigned)ceil_div(G.ld, 256));
  widen_kernel<<<grid, 256, 0, s>>>(G.data, (int)G.kind, G.row_scale, G.nd, G.ld, c0, out);
  GRADA_LAUNCH_CHECK();
}

void launch_GT_vec_mul(const DevG &G, const double *y, double *x, double *scratch, int sm_count,
                       cudaStream_t s, const GemvOpts &o) {
  (void)sm_count;
  if (G.nd <= 0 || G.nm <= 0) return;
  const unsigned prep_blocks = (unsigned)ceil_div(G.ld, 256);
  switch (G.kind) {
    case GKind::FP64: {
      prep_y_kernel<double><<<prep_blocks, 256, 0, s>>>(y, G.nd, G.ld, nullptr, o.scale, scratch,
                                                        o.skip);
      GRADA_LAUNCH_CHECK();
      gty_kernel<LoadF64><<<(unsigned)ceil_div(G.nm, gemv::kGtBlockCols), GV_THREADS, 0, s>>>(
          G.data, G.ld, G.nm, scratch, x, o.skip);
      break;
    }
    case GKind::FP32: {
      float *y32 = reinterpret_cast<float *>(scratch);
      prep_y_kernel<float><<<prep_blocks, 256, 0, s>>>(y, G.nd, G.ld, nullptr, o.scale, y32,
                                                       o.skip);
      GRADA_LAUNCH_CHECK();
      gty_kernel<LoadF32><<<(unsigned)ceil_div(G.nm, gemv::kGtBlockCols), GV_THREADS, 0, s>>>(
          G.data, G.ld, G.nm, y32, x, o.skip);
      break;
    }
    case GKind::BF16: {
      float *y32 = reinterpret_cast<float *>(scratch);
      prep_y_kernel<float><<<prep_blocks, 256, 0, s>>>(y, G.nd, G.ld, G.row_scale, o.scale, y32,
                                                       o.skip);
      GRADA_LAUNCH_CHECK();
      gty_kernel<LoadBF16><<<(unsigned)ceil_div(G.nm, gemv::kGtBlockCols), GV_THREADS, 0, s>>>(
          G.data, G.ld, G.nm, y32, x, o.skip);
      break;
    }
    case GKind::FP16: {
      float *y32 = reinterpret_cast<float *>(scratch);
      prep_y_kernel<float><<<prep_blocks, 256, 0, s>>>(y, G.nd, G.ld, G.row_scale, o.scale, y32,
                                                       o.skip);
      GRADA_LAUNCH_CHECK();
      gty_kernel<LoadF16><<<(unsigned)ceil_div(G.nm, gemv::kGtBlockCols), GV_THREADS, 0, s>>>(
          G.data, G.ld, G.nm, y32, x, o.skip);
      break;
    }
  }
  GRADA_LAUNCH_CHECK();
}

// ---- column norms ---------------------------------------------------------------

namespace {

// norms[j] = ||G(:, j)||_2 of the stored entries (16-bit ones times their row
// scale), one warp per column, squares summed in FP64 in a fixed order.
template <class L>
__global__ void __launch_bounds__(GV_THREADS)
    column_norms_kernel(const void *__restrict__ G, const float *__restrict__ row_scale, int64_t nd,
                        int64_t nm, int64_t ld, double *__restrict__ norms) {
  const int64_t col = (int64_t)blockIdx.x * (GV_THREADS / 32) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (col >= nm) return;
  double s = 0.0;
  for (int64_t r = (int64_t)lane * L::VEC; r < ld; r += 32 * L::VEC) {
    typename L::Acc v[L::VEC];
    L::load(G, col * ld + r, v);
#pragma unroll
    for (int k = 0; k < L::VEC; k++) {
      double e = (double)v[k];
      if (row_scale) e *= (r + k < nd) ? (double)row_scale[r + k] : 0.0;
      s = fma(e, e, s);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) norms[col] = sqrt(s);
}

}  // namespace

void launch_column_norms(const DevG &G, double *norms, cudaStream_t s) {
  if (G.nm <= 0) return;
  const unsigned blocks = (unsigned)ceil_div(G.nm, GV_THREADS / 32);
  switch (G.kind) {
    case GKind::FP64:
      column_norms_kernel<LoadF64><<<blocks, GV_THREADS, 0, s>>>(G.data, nullptr, G.nd, G.nm, G.ld, norms);
      break;
    case GKind::FP32:
      column_norms_kernel<LoadF32><<<blocks, GV_THREADS, 0, s>>>(G.data, nullptr, G.nd, G.nm, G.ld, norms);
      break;
    case GKind::BF16:
      column_norms_kernel<LoadBF16><<<blocks, GV_THREADS, 0, s>>>(G.data, G.row_scale, G.nd, G.nm,
                                                                   G.ld, norms);
      break;
    case GKind::FP16:
      column_norms_kernel<LoadF16><<<blocks, GV_THREADS, 0, s>>>(G.data, G.row_scale, G.nd, G.nm,
                                                                  G.ld, norms);
      break;
    default:
      throw Error(-4, "column norms need a stored G");
  }
  GRADA_LAUNCH_CHECK();
}

}  // namespace grada
