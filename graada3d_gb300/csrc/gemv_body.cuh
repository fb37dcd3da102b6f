// Per-block bodies of the dense products with the stored G (gemv.cu), shared
// by the one-product kernels and the persistent CG kernel (cg_fused.cu).  A
// body takes the index of its block as an argument instead of blockIdx, so a
// persistent kernel can run the blocks of a product in any grid and gets the
// same sums in the same order: the results are bitwise those of the
// stand-alone kernels.
//
// Vectors that the persistent kernel rewrites between its phases (x, y, the
// partial sums) are read with ld.global.cg (L2, never a stale L1 or the
// read-only path); G itself is streamed with evict-first loads.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>

#include "common.cuh"

namespace grada {
namespace gemv {

constexpr int kThreads = 256;  // threads of every product block
constexpr int kXChunk = 256;   // x entries staged in shared memory at a time (G x)

// ---- element loaders: VEC consecutive entries from a 16-byte load ----------
// (streamed, evict-first: G is read once per product and would only push the
// vectors out of L2)

struct LoadF64 {
  static constexpr int VEC = 2;
  using Acc = double;
  __device__ static void load(const void *base, int64_t idx, double (&v)[2]) {
    const double2 d = __ldcs(reinterpret_cast<const double2 *>(static_cast<const double *>(base) + idx));
    v[0] = d.x;
    v[1] = d.y;
  }
};
struct LoadF32 {
  static constexpr int VEC = 4;
  using Acc = float;
  __device__ static void load(const void *base, int64_t idx, float (&v)[4]) {
    const float4 d = __ldcs(reinterpret_cast<const float4 *>(static_cast<const float *>(base) + idx));
    v[0] = d.x;
    v[1] = d.y;
    v[2] = d.z;
    v[3] = d.w;
  }
};
struct LoadBF16 {
  static constexpr int VEC = 8;
  using Acc = float;
  __device__ static void load(const void *base, int64_t idx, float (&v)[8]) {
    const uint4 d = __ldcs(reinterpret_cast<const uint4 *>(static_cast<const uint16_t *>(base) + idx));
    const uint32_t w[4] = {d.x, d.y, d.z, d.w};
#pragma unroll
    for (int k = 0; k < 4; k++) {
      v[2 * k] = __uint_as_float(w[k] << 16);
      v[2 * k + 1] = __uint_as_float(w[k] & 0xffff0000u);
    }
  }
};
struct LoadF16 {
  static constexpr int VEC = 8;
  using Acc = float;
  __device__ static void load(const void *base, int64_t idx, float (&v)[8]) {
    const uint4 d = __ldcs(reinterpret_cast<const uint4 *>(static_cast<const uint16_t *>(base) + idx));
    const uint32_t w[4] = {d.x, d.y, d.z, d.w};
#pragma unroll
    for (int k = 0; k < 4; k++) {
      __half2 h;
      memcpy(&h, &w[k], 4);
      const float2 f = __half22float2(h);
      v[2 * k] = f.x;
      v[2 * k + 1] = f.y;
    }
  }
};

// ---- G x: block (tile, split) accumulates kThreads * VEC rows over one
// column range; the ranges' partial rows go to partial[split * ld + row].
template <class L>
__device__ __forceinline__ void gx_partial_body(const void *__restrict__ G, int64_t ld, int64_t nm,
                                                int64_t cols_per_split, const double *x,
                                                double *partial, int64_t tile, int64_t split) {
  using Acc = typename L::Acc;
  constexpr int VEC = L::VEC;
  __shared__ Acc xs[kXChunk];
  const int64_t row = (tile * kThreads + threadIdx.x) * VEC;
  const int64_t c_begin = split * cols_per_split;
  const int64_t c_end = min(nm, c_begin + cols_per_split);
  Acc acc[VEC];
#pragma unroll
  for (int v = 0; v < VEC; v++) acc[v] = Acc(0);
  for (int64_t c0 = c_begin; c0 < c_end; c0 += kXChunk) {
    const int nc = (int)min((int64_t)kXChunk, c_end - c0);
    __syncthreads();
    for (int t = threadIdx.x; t < nc; t += kThreads) xs[t] = (Acc)__ldcg(x + c0 + t);
    __syncthreads();
    if (row < ld) {
      const int64_t base = row + c0 * ld;
      int c = 0;
      // eight columns' loads in flight before their FMAs
      for (; c + 8 <= nc; c += 8) {
        Acc g[8][VEC];
#pragma unroll
        for (int q = 0; q < 8; q++) L::load(G, base + (int64_t)(c + q) * ld, g[q]);
#pragma unroll
        for (int q = 0; q < 8; q++) {
          const Acc xq = xs[c + q];
#pragma unroll
          for (int v = 0; v < VEC; v++) acc[v] = fma(g[q][v], xq, acc[v]);
        }
      }
      for (; c < nc; c++) {
        Acc g0[VEC];
        L::load(G, base + (int64_t)c * ld, g0);
#pragma unroll
        for (int v = 0; v < VEC; v++) acc[v] = fma(g0[v], xs[c], acc[v]);
      }
    }
  }
  if (row < ld) {
    double *out = partial + split * ld + row;
#pragma unroll
    for (int v = 0; v < VEC; v++) out[v] = (double)acc[v];
  }
}

// Warps of a fold-body block that share a row tile (the block's 8 warps form
// 8 / kFoldWarps groups that split the unit's columns), and the rows of a
// tile: 1 KB of a column per pair of warp loads for every storage.  Measured
// on 40,832 x 32,000 bf16 G: 417 us with two warps per tile against 495 us
// with one; at 3,392 x 16,384 the same or better.
constexpr int kFoldWarps = 2;
// Two accumulator chains per row (even and odd columns of a batch) for FP64 and
// FP32 G: the FP64 pipe needs the independent FMAs, and FP32's CG loop measured
// a little faster with them (40,832 x 236,226: 10.5-10.8 against 10.9 ms per
// iteration).  16-bit G has eight rows per thread, and there a second chain
// measured slower (40,832 x 32,000 bf16 G x: 542 against 417 us).
template <int VEC>
constexpr bool kFoldTwoChains = VEC < 8;
__host__ __device__ constexpr int fold_tile_rows_for_vec(int vec) { return kFoldWarps * 32 * vec; }
template <class L>
__host__ __device__ constexpr int fold_tile_rows() {
  return fold_tile_rows_for_vec(L::VEC);
}

// G pp's partial row sums for the CG with the direction update folded in:
// the staged entries are pp_j = P_j (-r_j + beta p_old_j); blocks of tile 0
// also store p_new_j = -r_j + beta p_old_j and pp_j (GaussNewtonInversion.cpp:
// 1562-1566), so no separate pass over p is needed before G pp.  Unit (tile,
// split): the tile's fold_tile_rows rows over the split's columns.  Within a
// staged chunk of columns warp group g (kFoldWarps warps on the tile's rows)
// takes the g-th of 8 / kFoldWarps consecutive column sub-ranges (eight
// columns' loads in flight, kFoldTwoChains accumulator chains); the group sums
// of each row are added in group order through shared memory and stored to
// partial[split * ld + row].  Short, wide G thus gets many row tiles and few
// column splits (few partial rows for the finish to add).
template <class L>
__device__ __forceinline__ void gx_partial_fold_body(
    const void *__restrict__ G, int64_t ld, int64_t nm, int64_t cols_per_split, const double *r,
    const double *p_old, const double *__restrict__ P, double beta, double *p_new, double *pp,
    double *partial, int64_t tile, int64_t split) {
  using Acc = typename L::Acc;
  constexpr int VEC = L::VEC;
  constexpr int kGroups = (kThreads / 32) / kFoldWarps;
  constexpr int kRows = fold_tile_rows<L>();
  __shared__ Acc xs[kXChunk];
  __shared__ double wsum[kGroups][kRows];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int grp = warp / kFoldWarps, wig = warp % kFoldWarps;
  const int64_t row = tile * kRows + (wig * 32 + lane) * VEC;
  const int64_t c_begin = split * cols_per_split;
  const int64_t c_end = min(nm, c_begin + cols_per_split);
  Acc acc[VEC], acc2[VEC];
#pragma unroll
  for (int v = 0; v < VEC; v++) acc[v] = acc2[v] = Acc(0);
  for (int64_t c0 = c_begin; c0 < c_end; c0 += kXChunk) {
    const int nc = (int)min((int64_t)kXChunk, c_end - c0);
    __syncthreads();
    for (int t = threadIdx.x; t < nc; t += kThreads) {
      const int64_t j = c0 + t;
      const double v = -__ldcg(r + j) + beta * __ldcg(p_old + j);
      const double q = P[j] * v;
      if (tile == 0) {
        p_new[j] = v;
        pp[j] = q;
      }
      xs[t] = (Acc)q;
    }
    __syncthreads();
    const int lo = (nc * grp) / kGroups, hi = (nc * (grp + 1)) / kGroups;
    if (row < ld) {
      const int64_t base = row + c0 * ld;
      int c = lo;
      for (; c + 8 <= hi; c += 8) {
        Acc g[8][VEC];
#pragma unroll
        for (int q = 0; q < 8; q++) L::load(G, base + (int64_t)(c + q) * ld, g[q]);
        if constexpr (kFoldTwoChains<VEC>) {
#pragma unroll
          for (int q = 0; q < 8; q += 2) {
            const Acc xq = xs[c + q], xr = xs[c + q + 1];
#pragma unroll
            for (int v = 0; v < VEC; v++) {
              acc[v] = fma(g[q][v], xq, acc[v]);
              acc2[v] = fma(g[q + 1][v], xr, acc2[v]);
            }
          }
        } else {
#pragma unroll
          for (int q = 0; q < 8; q++) {
            const Acc xq = xs[c + q];
#pragma unroll
            for (int v = 0; v < VEC; v++) acc[v] = fma(g[q][v], xq, acc[v]);
          }
        }
      }
      for (; c < hi; c++) {
        Acc g0[VEC];
        L::load(G, base + (int64_t)c * ld, g0);
#pragma unroll
        for (int v = 0; v < VEC; v++) acc[v] = fma(g0[v], xs[c], acc[v]);
      }
    }
  }
  __syncthreads();  // wsum may still be read for the caller's previous unit
#pragma unroll
  for (int v = 0; v < VEC; v++)
    wsum[grp][(wig * 32 + lane) * VEC + v] = (double)acc[v] + (double)acc2[v];
  __syncthreads();
  for (int t = threadIdx.x; t < kRows; t += kThreads) {
    const int64_t rr = tile * kRows + t;
    if (rr < ld) {
      double sum = 0.0;
#pragma unroll
      for (int w = 0; w < kGroups; w++) sum += wsum[w][t];
      partial[split * ld + rr] = sum;
    }
  }
}

// y[r] = (sum over splits of the partial rows) * row_scale[r] * post_scale[r]
// for the kFinishRows rows of block b: warp w adds splits w, w + 8, ... of
// its lane's row, then warp 0 adds the 8 warp sums in warp order.  Sharing a
// row's splits among the warps keeps the many column ranges of a tall-thin G
// from turning the sum into one long dependent chain per thread.
constexpr int kFinishRows = 32;

__device__ __forceinline__ void gx_finish_body(const double *partial, int n_split, int64_t ld,
                                               int64_t nd, const float *__restrict__ row_scale,
                                               const double *__restrict__ post_scale, double *y,
                                               int64_t b) {
  __shared__ double part[kThreads / 32][kFinishRows];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t r = b * kFinishRows + lane;
  double s = 0.0;
  if (r < nd)
    for (int k = warp; k < n_split; k += kThreads / 32) s += __ldcg(partial + (int64_t)k * ld + r);
  __syncthreads();  // part is reused by the next block the caller runs
  part[warp][lane] = s;
  __syncthreads();
  if (warp == 0 && r < nd) {
    double v = 0.0;
#pragma unroll
    for (int w = 0; w < kThreads / 32; w++) v += part[w][lane];
    if (row_scale) v *= (double)row_scale[r];
    if (post_scale) v *= post_scale[r];
    y[r] = v;
  }
}

// y (FP64, nd entries) -> padded vector of the accumulation type, times the
// optional pre-scale and the 16-bit row scale, zero in the padding rows;
// 256 rows per block b.
template <typename Acc>
__device__ __forceinline__ void prep_y_body(const double *y, int64_t nd, int64_t ld,
                                            const float *__restrict__ row_scale,
                                            const double *__restrict__ pre_scale, Acc *out,
                                            int64_t b) {
  const int64_t r = b * 256 + threadIdx.x;
  if (r >= ld) return;
  double v = (r < nd) ? __ldcg(y + r) : 0.0;
  if (pre_scale && r < nd) v = pre_scale[r] * v;
  if (row_scale && r < nd) v *= (double)row_scale[r];
  out[r] = (Acc)v;
}

// G^T y for the kGtBlockCols columns of block b: warp w takes columns
// 4w .. 4w + 3 of the block, its lanes striding the rows with 16-byte loads,
// and sums each column with a butterfly.  y goes through shared memory in
// chunks of 32 KB, read once per block with 16-byte loads (not once per warp);
// one chunk, two block barriers, for the heights of most problems.  Lane
// c < 4 of warp w returns column b * kGtBlockCols + 4w + c's sum and sets
// *col to that column; every other thread gets *col = -1.
constexpr int kGtWarpCols = 4;
constexpr int kGtBlockCols = kGtWarpCols * (kThreads / 32);
constexpr int kYChunkBytes = 32768;  // y staged 32 KB at a time: one chunk for ld <= 8,192 (FP32)

// Rows row_begin, row_begin + 32 VEC, ... < row_end of the warp's columns
// c0 .. c0 + ncol - 1 (G rows offset by g_row0), y's VEC values of a row from
// y_at.  Full (ncol = kGtWarpCols, every warp but the last): no per-column
// tests, so every column's loads of a row step issue before its FMAs.  Each
// column adds its rows in the same order either way.
template <class L, int U, bool Full, class YAt>
__device__ __forceinline__ void gty_rows(const void *__restrict__ G, int64_t ld, int64_t c0,
                                         int ncol, int64_t g_row0, int64_t row_begin,
                                         int64_t row_end, YAt y_at,
                                         typename L::Acc (&acc)[kGtWarpCols]) {
  using Acc = typename L::Acc;
  constexpr int VEC = L::VEC;
#pragma unroll U
  for (int64_t row = row_begin; row < row_end; row += 32 * VEC) {
    Acc yv[VEC];
    y_at(row, yv);
    if constexpr (Full) {
      Acc g[kGtWarpCols][VEC];
#pragma unroll
      for (int c = 0; c < kGtWarpCols; c++) L::load(G, g_row0 + row + (c0 + c) * ld, g[c]);
#pragma unroll
      for (int c = 0; c < kGtWarpCols; c++)
#pragma unroll
        for (int v = 0; v < VEC; v++) acc[c] = fma(g[c][v], yv[v], acc[c]);
    } else {
#pragma unroll
      for (int c = 0; c < kGtWarpCols; c++) {
        if (c < ncol) {
          Acc g[VEC];
          L::load(G, g_row0 + row + (c0 + c) * ld, g);
#pragma unroll
          for (int v = 0; v < VEC; v++) acc[c] = fma(g[v], yv[v], acc[c]);
        }
      }
    }
  }
}

// Row steps per trip of G^T y (gty_body's U; the sums do not depend on it):
// two in general, four on tall G (measured on 40,832 x 32,000: FP32 786
// against 875 us, bf16 410 against 447 us), where short G loses with them
// (bf16 at 3,392 x 16,384: 33.9 against 28 us).
constexpr int kGtUnroll = 2, kGtUnrollTall = 4;
constexpr int64_t kGtTallRows = 16384;

template <class L, int U = kGtUnroll>
__device__ __forceinline__ double gty_body(const void *__restrict__ G, int64_t ld, int64_t nm,
                                           const typename L::Acc *y, int64_t b, int64_t *col) {
  using Acc = typename L::Acc;
  constexpr int VEC = L::VEC;
  constexpr int kYChunk = kYChunkBytes / (int)sizeof(Acc);
  __shared__ __align__(16) Acc ys[kYChunk];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t c0 = b * kGtBlockCols + (int64_t)warp * kGtWarpCols;
  const int64_t left = nm - c0;
  const int ncol = left <= 0 ? 0 : (left < kGtWarpCols ? (int)left : kGtWarpCols);
  Acc acc[kGtWarpCols];
#pragma unroll
  for (int c = 0; c < kGtWarpCols; c++) acc[c] = Acc(0);
  // 16 bytes of y per load: 4 floats or 2 doubles
  constexpr int YV = 16 / (int)sizeof(Acc);
  auto y_at = [&](int64_t row, Acc (&yv)[VEC]) {
#pragma unroll
    for (int v = 0; v < VEC; v++) yv[v] = ys[row + v];
  };
  for (int64_t r0 = 0; r0 < ld; r0 += kYChunk) {
    const int n = (int)min((int64_t)kYChunk, ld - r0);  // a multiple of 64 (ld is)
    __syncthreads();
    for (int t = threadIdx.x * YV; t < n; t += kThreads * YV) {
      if constexpr (YV == 4) {
        *reinterpret_cast<float4 *>(&ys[t]) = __ldcg(reinterpret_cast<const float4 *>(y + r0 + t));
      } else {
        *reinterpret_cast<double2 *>(&ys[t]) =
            __ldcg(reinterpret_cast<const double2 *>(y + r0 + t));
      }
    }
    __syncthreads();
    if (ncol == kGtWarpCols)
      gty_rows<L, U, true>(G, ld, c0, ncol, r0, lane * VEC, n, y_at, acc);
    else if (ncol > 0)
      gty_rows<L, U, false>(G, ld, c0, ncol, r0, lane * VEC, n, y_at, acc);
  }
  double mine = 0.0;
#pragma unroll
  for (int c = 0; c < kGtWarpCols; c++) {
    double v = (double)acc[c];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == c) mine = v;
  }
  *col = (lane < ncol) ? c0 + lane : -1;
  return mine;
}

}  // namespace gemv
}  // namespace grada
