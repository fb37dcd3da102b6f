// Block products with FP64 G: Y = G X and X = G^T Y for 16 right-hand sides.
//
// Reference: a block of the reference's dense G_vec_mul / GT_vec_mul
// (src/Forward_modelling/Fwd.cpp:145, :111), one per right-hand side.
//
// GB300's FP64 pipe retires 2 FMAs per clock per SM, so a 16-column product
// with FP64 G costs 16 FMAs per 8-byte entry and is bound by the FP64 pipe,
// not by HBM; the kernels are plain shared-memory tiled loops that keep that
// pipe fed.  (FP32 and 16-bit G take the tensor-core kernels of tc_gemm.cu.)
//  * G X: a block owns 64 rows x 16 columns of Y and a range of cells; each
//    thread accumulates one row x 4 columns over 32-cell tiles of G and X
//    staged in shared memory.  Cell ranges give partial rows, summed in range
//    order by a second pass (deterministic).
//  * G^T Y: a block owns 32 cells x 16 columns of X and walks all rows in
//    64-row tiles; each thread accumulates one cell x 2 columns.
#include "cg_kernels.h"
#include "common.cuh"
#include "kernels.h"

namespace grada {

namespace {

constexpr int GX_TR = 64;   // rows per block
constexpr int GX_KC = 32;   // cells per tile
constexpr int GT_TC = 32;   // cells per block
constexpr int GT_KR = 64;   // rows per tile
constexpr int BG_THREADS = 256;

__global__ void __launch_bounds__(BG_THREADS)
    bgx_fp64_kernel(const double *__restrict__ G, int64_t ld, int64_t nm, int64_t cells_per_split,
                    const double *__restrict__ X, double *__restrict__ partial,
                    const int *__restrict__ skip) {
  if (skip && *skip) return;
  __shared__ __align__(16) double gs[GX_KC][GX_TR];
  __shared__ __align__(16) double xs[GX_KC][kBW];
  const int t = threadIdx.x;
  const int row_l = t % GX_TR, q = t / GX_TR;
  const int64_t r0 = (int64_t)blockIdx.x * GX_TR;
  const int64_t c_begin = (int64_t)blockIdx.y * cells_per_split;
  const int64_t c_end = min(nm, c_begin + cells_per_split);
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  for (int64_t c0 = c_begin; c0 < c_end; c0 += GX_KC) {
    const int nc = (int)min((int64_t)GX_KC, c_end - c0);
    __syncthreads();
    // G tile: 32 cells x 64 rows, 16-byte loads along the rows
    for (int v = t; v < GX_KC * GX_TR / 2; v += BG_THREADS) {
      const int k = v / (GX_TR / 2), rr = (v % (GX_TR / 2)) * 2;
      double2 g = make_double2(0.0, 0.0);
      if (k < nc && r0 + rr < ld)
        g = __ldcs(reinterpret_cast<const double2 *>(G + (c0 + k) * ld + r0 + rr));
      gs[k][rr] = g.x;
      gs[k][rr + 1] = g.y;
    }
    for (int v = t; v < GX_KC * kBW; v += BG_THREADS) {
      const int k = v / kBW;
      xs[k][v % kBW] = (k < nc) ? X[(c0 + k) * kBW + v % kBW] : 0.0;
    }
    __syncthreads();
#pragma unroll 8
    for (int k = 0; k < GX_KC; k++) {
      const double g = gs[k][row_l];
      const double2 xa = *reinterpret_cast<const double2 *>(&xs[k][4 * q]);
      const double2 xb = *reinterpret_cast<const double2 *>(&xs[k][4 * q + 2]);
      acc[0] = fma(g, xa.x, acc[0]);
      acc[1] = fma(g, xa.y, acc[1]);
      acc[2] = fma(g, xb.x, acc[2]);
      acc[3] = fma(g, xb.y, acc[3]);
    }
  }
  const int64_t r = r0 + row_l;
  if (r < ld) {
    double *out = partial + ((int64_t)blockIdx.y * ld + r) * kBW + 4 * q;
    *reinterpret_cast<double2 *>(out) = make_double2(acc[0], acc[1]);
    *reinterpret_cast<double2 *>(out + 2) = make_double2(acc[2], acc[3]);
  }
}

// Y(r, c) = post(r) * rs(r) * sum over splits of partial, r < nd.
__global__ void bgx_finish_kernel(const double *__restrict__ partial, int n_split, int64_t ld,
                                  int64_t nd, const float *__restrict__ row_scale,
                                  const double *__restrict__ post, double *__restrict__ Y,
                                  const int *__restrict__ skip) {
  if (skip && *skip) return;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nd * kBW) return;
  const int64_t r = e / kBW;
  double s = 0.0;
  for (int k = 0; k < n_split; k++) s += partial[(int64_t)k * ld * kBW + e];
  if (row_scale) s *= (double)row_scale[r];
  if (post) s *= post[r];
  Y[e] = s;
}

__global__ void __launch_bounds__(BG_THREADS)
    bgty_fp64_kernel(const double *__restrict__ G, int64_t ld, int64_t nd, int64_t nm,
                     const double *__restrict__ Y, const double *__restrict__ pre,
                     double *__restrict__ X, const int *__restrict__ skip) {
  if (skip && *skip) return;
  __shared__ __align__(16) double gs[GT_TC][GT_KR + 1];
  __shared__ __align__(16) double ys[GT_KR][kBW];
  const int t = threadIdx.x;
  const int cl = t / 8, pc = (t % 8) * 2;
  const int64_t j0 = (int64_t)blockIdx.x * GT_TC;
  const int ncell = (int)min((int64_t)GT_TC, nm - j0);
  double a0 = 0.0, a1 = 0.0;
  for (int64_t i0 = 0; i0 < nd; i0 += GT_KR) {
    __syncthreads();
    // G tile: 32 cells x 64 rows (each cell's rows contiguous)
    for (int v = t; v < GT_TC * GT_KR / 2; v += BG_THREADS) {
      const int k = v / (GT_KR / 2), rr = (v % (GT_KR / 2)) * 2;
      double2 g = make_double2(0.0, 0.0);
      if (k < ncell && i0 + rr < ld)
        g = __ldcs(reinterpret_cast<const double2 *>(G + (j0 + k) * ld + i0 + rr));
      gs[k][rr] = g.x;
      gs[k][rr + 1] = g.y;
    }
    for (int v = t; v < GT_KR * kBW; v += BG_THREADS) {
      const int rr = v / kBW;
      const int64_t i = i0 + rr;
      double y = 0.0;
      if (i < nd) {
        y = Y[i * kBW + v % kBW];
        if (pre) y *= pre[i];
      }
      ys[rr][v % kBW] = y;
    }
    __syncthreads();
#pragma unroll 8
    for (int k = 0; k < GT_KR; k++) {
      const double g = gs[cl][k];
      const double2 y = *reinterpret_cast<const double2 *>(&ys[k][pc]);
      a0 = fma(g, y.x, a0);
      a1 = fma(g, y.y, a1);
    }
  }
  if (cl < ncell) {
    double *out = X + (j0 + cl) * kBW + pc;
    *reinterpret_cast<double2 *>(out) = make_double2(a0, a1);
  }
}

int gx_fp64_splits(const DevG &G, int sm_count) {
  const int64_t tiles = ceil_div(G.ld, GX_TR);
  int64_t s = ceil_div((int64_t)sm_count * 8, tiles);
  const int64_t max_s = ceil_div(G.nm, GX_KC * 8);  // at least 8 tiles per range
  if (s > max_s) s = max_s;
  if (s < 1) s = 1;
  if (s > 65535) s = 65535;
  return (int)s;
}

}  // namespace

int64_t block_scratch_bytes(const DevG &G, int sm_count) {
  if (G.kind == GKind::FP64)
    return (int64_t)gx_fp64_splits(G, sm_count) * G.ld * kBW * (int64_t)sizeof(double);
  return tc_scratch_bytes(G, sm_count);
}

void launch_G_mat_mul(const DevG &G, const double *X, double *Y, void *scratch, int sm_count,
                      cudaStream_t s, const GemvOpts &o, int *err) {
  if (G.kind != GKind::FP64) {
    launch_tc_G_mat_mul(G, X, Y, scratch, sm_count, s, o, err);
    return;
  }
  const int splits = gx_fp64_splits(G, sm_count);
  const int64_t per = round_up(ceil_div(G.nm, splits), GX_KC);
  double *partial = static_cast<double *>(scratch);
  dim3 grid((unsigned)ceil_div(G.ld, GX_TR), (unsigned)splits);
  bgx_fp64_kernel<<<grid, BG_THREADS, 0, s>>>(static_cast<const double *>(G.data), G.ld, G.nm, per,
                                              X, partial, o.skip);
  GRADA_LAUNCH_CHECK();
  bgx_finish_kernel<<<(unsigned)ceil_div(G.nd * kBW, 256), 256, 0, s>>>(
      partial, splits, G.ld, G.nd, nullptr, o.scale, Y, o.skip);
  GRADA_LAUNCH_CHECK();
}

void launch_GT_mat_mul(const DevG &G, const double *Y, double *X, void *scratch, int sm_count,
                       cudaStream_t s, const GemvOpts &o, int *err) {
  if (G.kind != GKind::FP64) {
    launch_tc_GT_mat_mul(G, Y, X, scratch, sm_count, s, o, err);
    return;
  }
  bgty_fp64_kernel<<<(unsigned)ceil_div(G.nm, GT_TC), BG_THREADS, 0, s>>>(
      static_cast<const double *>(G.data), G.ld, G.nd, G.nm, Y, o.scale, X, o.skip);
  GRADA_LAUNCH_CHECK();
}

}  // namespace grada
