// Matrix-free block products: Y = G X and X = G^T Y for 16 right-hand sides
// without storing G, each (point, cell) pair evaluated once for all of them.
//
// Reference: the dense G_vec_mul / GT_vec_mul (src/Forward_modelling/
// Fwd.cpp:145, :111) with G's entries from GravFormula::
// field_caused_by_single_prism (GravFormula.cpp:2-36) recomputed on the fly.
// The prism terms cost several hundred FP64 instructions per pair; the 16
// multiply-adds per component that a block adds are a small fraction of
// that, so a block costs little more than one single product.
//  * G X: one thread per observation point walking the assembly tiles (faces
//    shared in z and y, tile_walk.cuh); accumulators per component and
//    right-hand side stay in registers, RG right-hand sides per pass (RG = 16
//    for up to 2 components, fewer for more components).  Tile ranges
//    (splits) give partial sums added in order by a second pass.
//  * G^T Y: one thread per cell, observation points (coordinates and the 16
//    weighted data values per component) streamed through shared memory;
//    the thread's 16 sums stay in registers.  Point ranges (splits) give
//    partial sums added in order by a second pass.
#include <mutex>

#include "cg_kernels.h"
#include "common.cuh"
#include "kernels.h"
#include "prism.cuh"
#include "tile_walk.cuh"

namespace grada {

namespace {

constexpr int AB_THREADS = 128;
constexpr int AB_CHUNK = 32;

__device__ __forceinline__ void slot_bits(uint32_t mask, int *bits) {
  int s = 0;
  for (int b = 0; b < 10; b++)
    if (mask & (1u << b)) bits[s++] = b;
}

template <int RG>
__global__ void __launch_bounds__(TL_THREADS)
    forward_field_block_kernel(const double *__restrict__ obs, int64_t n_obs,
                               const double *__restrict__ prisms, const int4 *__restrict__ tiles,
                               const int64_t *__restrict__ cells, int64_t n_tiles,
                               int64_t tiles_per_split, const double *__restrict__ X,
                               uint32_t mask, int nf, const double *__restrict__ tables, int r0,
                               double *__restrict__ partial, const int *__restrict__ skip) {
  constexpr int NFMAX = (RG >= 16) ? 2 : (RG >= 8 ? 4 : (RG >= 4 ? 8 : 10));
  if (skip && *skip) return;
  __shared__ double tab[kTabSize];
  __shared__ TileSmem ws;
  __shared__ int bits[10];
  extern __shared__ double zsm[];
  for (int t = threadIdx.x; t < kTabSize; t += TL_THREADS) tab[t] = tables[t];
  if (threadIdx.x == 0) slot_bits(mask, bits);
  const int64_t split = blockIdx.x;
  const int64_t t_begin = split * tiles_per_split;
  const int64_t t_end = min(n_tiles, t_begin + tiles_per_split);
  const int64_t i = (int64_t)blockIdx.y * TL_THREADS + threadIdx.x;
  const bool active = i < n_obs;
  double px = 0, py = 0, pz = 0;
  if (active) {
    px = obs[3 * i];
    py = obs[3 * i + 1];
    pz = obs[3 * i + 2];
  }
  const uint32_t fam = families_for_mask(mask);
  double acc[NFMAX][RG];
#pragma unroll
  for (int s = 0; s < NFMAX; s++)
#pragma unroll
    for (int r = 0; r < RG; r++) acc[s][r] = 0.0;
  for (int64_t tl = t_begin; tl < t_end; tl++) {
    tile_walk<false>(tiles[tl], cells, prisms, ws, zsm, active, px, py, pz, fam, tab,
                     [&](int64_t cell, int, const PrismTerms &t) {
                const double *xc = X + cell * kBW + r0;  // same address in every thread
#pragma unroll
                for (int s = 0; s < NFMAX; s++) {
                  if (s < nf) {
                    const double v = prism_component(t, bits[s]);
#pragma unroll
                    for (int r = 0; r < RG; r++) acc[s][r] = fma(v, __ldg(xc + r), acc[s][r]);
                  }
                }
              });
  }
  if (!active) return;
  // partial[split][i][s][16]
  double *out = partial + ((split * n_obs + i) * nf) * kBW + r0;
#pragma unroll
  for (int s = 0; s < NFMAX; s++)
    if (s < nf) {
#pragma unroll
      for (int r = 0; r < RG; r++) out[s * kBW + r] = acc[s][r];
    }
}

// Y(row, r) = post(row) * sum over splits, row = s * n_obs + i (G's row order).
__global__ void forward_block_sum_kernel(const double *__restrict__ partial, int n_split,
                                         int64_t n_obs, int nf, const double *__restrict__ post,
                                         double *__restrict__ Y, const int *__restrict__ skip) {
  if (skip && *skip) return;
  const int64_t n = n_obs * nf * kBW;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  double v = 0.0;
  for (int k = 0; k < n_split; k++) v += partial[(int64_t)k * n + e];
  const int64_t r = e % kBW, is = e / kBW;
  const int64_t s = is % nf, i = is / nf;
  const int64_t row = s * n_obs + i;
  Y[row * kBW + r] = post ? post[row] * v : v;
}

__global__ void __launch_bounds__(AB_THREADS)
    adjoint_field_block_kernel(const double *__restrict__ obs, int64_t n_obs,
                               const double *__restrict__ prisms, int64_t n_cells, uint32_t mask,
                               int nf, const double *__restrict__ tables,
                               const double *__restrict__ Y, const double *__restrict__ pre,
                               int64_t obs_per_split, double *__restrict__ partial,
                               const int *__restrict__ skip) {
  if (skip && *skip) return;
  extern __shared__ double dyn[];
  double *tab = dyn;                              // kTabSize
  double *pts = tab + kTabSize;                   // AB_CHUNK x 3
  double *ys = pts + AB_CHUNK * 3;                // AB_CHUNK x nf x 16
  __shared__ int bits[10];
  for (int t = threadIdx.x; t < kTabSize; t += AB_THREADS) tab[t] = tables[t];
  if (threadIdx.x == 0) slot_bits(mask, bits);
  const int64_t j = (int64_t)blockIdx.x * AB_THREADS + threadIdx.x;
  const bool active = j < n_cells;
  double x0 = 0, x1 = 1, y0 = 0, y1 = 1, z0 = 0, z1 = 1;
  if (active) {
    const double *p = prisms + 6 * j;
    x0 = p[0]; x1 = p[1]; y0 = p[2]; y1 = p[3]; z0 = p[4]; z1 = p[5];
  }
  const uint32_t fam = families_for_mask(mask);
  double acc[kBW];
#pragma unroll
  for (int r = 0; r < kBW; r++) acc[r] = 0.0;
  const int64_t i_begin = (int64_t)blockIdx.y * obs_per_split;
  const int64_t i_end = min(n_obs, i_begin + obs_per_split);
  for (int64_t i0 = i_begin; i0 < i_end; i0 += AB_CHUNK) {
    const int np = (int)min((int64_t)AB_CHUNK, i_end - i0);
    __syncthreads();
    for (int t = threadIdx.x; t < np * 3; t += AB_THREADS) pts[t] = obs[i0 * 3 + t];
    for (int t = threadIdx.x; t < np * nf * kBW; t += AB_THREADS) {
      const int pi = t / (nf * kBW), s = (t / kBW) % nf, r = t % kBW;
      const int64_t row = (int64_t)s * n_obs + i0 + pi;
      const double y = Y[row * kBW + r];
      ys[t] = pre ? pre[row] * y : y;
    }
    __syncthreads();
    if (!active) continue;
    for (int pi = 0; pi < np; pi++) {
      ZCarry carry;
      PrismTerms t;
      prism_terms(pts[3 * pi], pts[3 * pi + 1], pts[3 * pi + 2], x0, x1, y0, y1, z0, z1, fam, tab,
                  false, carry, t);
      const double *yp = ys + pi * nf * kBW;
      for (int s = 0; s < nf; s++) {
        const double v = prism_component(t, bits[s]);
#pragma unroll
        for (int r = 0; r < kBW; r++) acc[r] = fma(v, yp[s * kBW + r], acc[r]);
      }
    }
  }
  if (!active) return;
  double *out = partial + ((int64_t)blockIdx.y * n_cells + j) * kBW;
#pragma unroll
  for (int r = 0; r < kBW; r++) out[r] = acc[r];
}

__global__ void adjoint_block_sum_kernel(const double *__restrict__ partial, int n_split,
                                         int64_t n_cells, double *__restrict__ X,
                                         const int *__restrict__ skip) {
  if (skip && *skip) return;
  const int64_t n = n_cells * kBW;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  double v = 0.0;
  for (int k = 0; k < n_split; k++) v += partial[(int64_t)k * n + e];
  X[e] = v;
}

int fwd_splits(const DevGeometry &g, int sm_count) {
  const int64_t obs_tiles = ceil_div(g.n_obs, TL_THREADS);
  int64_t s = ceil_div((int64_t)sm_count * 2 * 16, obs_tiles);  // ~16 waves
  const int64_t max_s = g.plan.n_tiles;
  if (s > max_s) s = max_s;
  if (s < 1) s = 1;
  if (s > 65535) s = 65535;
  return (int)s;
}

int adj_splits(const DevGeometry &g, int sm_count) {
  const int64_t cell_blocks = ceil_div(g.n_cells, AB_THREADS);
  int64_t s = ceil_div((int64_t)sm_count * 4, cell_blocks);
  const int64_t max_s = ceil_div(g.n_obs, AB_CHUNK);
  if (s > max_s) s = max_s;
  if (s < 1) s = 1;
  if (s > 65535) s = 65535;
  return (int)s;
}

template <int RG>
void fwd_pass(const DevGeometry &g, const double *X, int splits, int64_t per, int r0,
              double *partial, cudaStream_t s, const int *skip) {
  const int smem = tile_walk_dyn_smem(false);
  {
    static std::mutex mu;
    static bool attr[64] = {};
    int dev = 0;
    GRADA_CUDA_CHECK(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(mu);
    if (dev < 0 || dev >= 64 || !attr[dev]) {
      GRADA_CUDA_CHECK(cudaFuncSetAttribute(forward_field_block_kernel<RG>,
                                            cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
      if (dev >= 0 && dev < 64) attr[dev] = true;
    }
  }
  dim3 grid((unsigned)splits, (unsigned)ceil_div(g.n_obs, TL_THREADS));
  forward_field_block_kernel<RG><<<grid, TL_THREADS, smem, s>>>(
      g.obs, g.n_obs, g.prisms, reinterpret_cast<const int4 *>(g.plan.tiles), g.plan.cells,
      g.plan.n_tiles, per, X, g.mask, g.n_fields, g.tables, r0, partial, skip);
  GRADA_LAUNCH_CHECK();
}

}  // namespace

int64_t mf_block_scratch_doubles(const DevGeometry &g, int sm_count) {
  const int64_t f = (int64_t)fwd_splits(g, sm_count) * g.n_obs * g.n_fields * kBW;
  const int64_t a = (int64_t)adj_splits(g, sm_count) * g.n_cells * kBW;
  return f > a ? f : a;
}

void launch_forward_field_block(const DevGeometry &g, const double *X, double *Y, double *scratch,
                                int sm_count, cudaStream_t s, const GemvOpts &o) {
  if (g.n_obs <= 0) return;
  if (ceil_div(g.n_obs, TL_THREADS) > 65535) throw Error(-1, "too many observation points for one launch");
  const int splits = fwd_splits(g, sm_count);
  const int64_t per = ceil_div(g.plan.n_tiles, splits);
  const int nf = g.n_fields;
  if (nf <= 2) {
    fwd_pass<16>(g, X, splits, per, 0, scratch, s, o.skip);
  } else if (nf <= 4) {
    for (int r0 = 0; r0 < kBW; r0 += 8) fwd_pass<8>(g, X, splits, per, r0, scratch, s, o.skip);
  } else if (nf <= 8) {
    for (int r0 = 0; r0 < kBW; r0 += 4) fwd_pass<4>(g, X, splits, per, r0, scratch, s, o.skip);
  } else {
    for (int r0 = 0; r0 < kBW; r0 += 2) fwd_pass<2>(g, X, splits, per, r0, scratch, s, o.skip);
  }
  const int64_t n = g.n_obs * nf * kBW;
  forward_block_sum_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, s>>>(scratch, splits, g.n_obs, nf,
                                                                      o.scale, Y, o.skip);
  GRADA_LAUNCH_CHECK();
}

void launch_adjoint_field_block(const DevGeometry &g, const double *Y, double *X, double *scratch,
                                int sm_count, cudaStream_t s, const GemvOpts &o) {
  if (g.n_cells <= 0) return;
  const int splits = adj_splits(g, sm_count);
  const int64_t per = round_up(ceil_div(g.n_obs, splits), AB_CHUNK);
  const size_t smem = sizeof(double) * (kTabSize + AB_CHUNK * 3 + (size_t)AB_CHUNK * g.n_fields * kBW);
  {
    static std::mutex mu;
    static bool attr[64] = {};
    int dev = 0;
    GRADA_CUDA_CHECK(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(mu);
    if (dev < 0 || dev >= 64 || !attr[dev]) {
      GRADA_CUDA_CHECK(cudaFuncSetAttribute(adjoint_field_block_kernel,
                                            cudaFuncAttributeMaxDynamicSharedMemorySize, 64 * 1024));
      if (dev >= 0 && dev < 64) attr[dev] = true;
    }
  }
  dim3 grid((unsigned)ceil_div(g.n_cells, AB_THREADS), (unsigned)splits);
  adjoint_field_block_kernel<<<grid, AB_THREADS, smem, s>>>(g.obs, g.n_obs, g.prisms, g.n_cells,
                                                            g.mask, g.n_fields, g.tables, Y,
                                                            o.scale, per, scratch, o.skip);
  GRADA_LAUNCH_CHECK();
  adjoint_block_sum_kernel<<<(unsigned)ceil_div(g.n_cells * kBW, 256), 256, 0, s>>>(
      scratch, splits, g.n_cells, X, o.skip);
  GRADA_LAUNCH_CHECK();
}

}  // namespace grada
