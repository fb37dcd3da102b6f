// K1: sensitivity assembly and the matrix-free field sum.
//
// Reference: Fwd::compute_G (src/Forward_modelling/Fwd.cpp:47-78), which
// loops observations serially and cells in an OpenMP loop, calling
// GravFormula::field_caused_by_single_prism per (observation, cell) pair;
// and the field sum of src/compute.cpp:246-260.
//
// Mapping: a block owns 128 consecutive observation points (one per thread)
// and a chunk of ASM_CHUNK consecutive cells whose geometry is staged in
// shared memory once and read by all 128 threads.  Each thread evaluates the
// closed-form terms of prism.cuh for its point against every cell of the chunk
// and writes the requested components; for a fixed cell and component, a warp
// writes 32 consecutive rows of G's column (256 B for FP64), so every store is
// coalesced.  The kernel is bound by the FP64 pipe (log/atan2/sqrt/division),
// not by memory: the G write is ~1% of the FP64 time.
#include "common.cuh"
#include "kernels.h"
#include <cmath>
#include <cstring>
#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "prism.cuh"
#include "tile_walk.cuh"

namespace grada {

namespace {

constexpr int ASM_THREADS = 128;
constexpr int ASM_CHUNK = 16;

template <typename OutT>
__global__ void __launch_bounds__(ASM_THREADS)
    assemble_kernel(const double *__restrict__ obs, int64_t n_obs,
                    const double *__restrict__ prisms, int64_t n_cells,
                    const int64_t *__restrict__ col_index, int64_t col_offset, uint32_t mask,
                    const double *__restrict__ tables, OutT *__restrict__ G, int64_t ld) {
  __shared__ double sp[ASM_CHUNK * 6];
  __shared__ double tab[kTabSize];
  for (int t = threadIdx.x; t < kTabSize; t += ASM_THREADS) tab[t] = tables[t];
  const int64_t c0 = (int64_t)blockIdx.x * ASM_CHUNK;
  const int64_t left = n_cells - c0;
  const int nc = left < ASM_CHUNK ? (int)left : ASM_CHUNK;
  for (int t = threadIdx.x; t < nc * 6; t += ASM_THREADS) sp[t] = prisms[c0 * 6 + t];
  __syncthreads();
  const int64_t i = (int64_t)blockIdx.y * ASM_THREADS + threadIdx.x;
  if (i >= n_obs) return;
  const double px = obs[3 * i], py = obs[3 * i + 1], pz = obs[3 * i + 2];
  const uint32_t fam = families_for_mask(mask);
  ZCarry carry;
  for (int c = 0; c < nc; c++) {
    const double *p = sp + 6 * c;
    // the same cell for every thread of the block: a uniform branch
    const bool reuse = c > 0 && p[0] == p[-6] && p[1] == p[-5] && p[2] == p[-4] &&
                       p[3] == p[-3] && p[4] == p[-1];
    PrismTerms t;
    prism_terms(px, py, pz, p[0], p[1], p[2], p[3], p[4], p[5], fam, tab, reuse, carry, t);
    const int64_t col = col_index ? col_index[c0 + c] : c0 + c + col_offset;
    OutT *gcol = G + col * ld + i;
    int slot = 0;
#pragma unroll
    for (int b = 0; b < 10; b++) {
      if (mask & (1u << b)) {
        store_entry(gcol + (int64_t)slot * n_obs, prism_component(t, b));
        slot++;
      }
    }
  }
}

template <typename OutT>
void launch_assemble(const DevGeometry &g, const double *prisms, int64_t n_cells,
                     const int64_t *col_index, int64_t col_offset, OutT *G, int64_t ld,
                     cudaStream_t s) {
  if (n_cells <= 0 || g.n_obs <= 0) return;
  dim3 grid((unsigned)ceil_div(n_cells, ASM_CHUNK), (unsigned)ceil_div(g.n_obs, ASM_THREADS));
  if (grid.y > 65535u) throw Error(-1, "too many observation points for one launch");
  assemble_kernel<OutT><<<grid, ASM_THREADS, 0, s>>>(g.obs, g.n_obs, prisms, n_cells, col_index,
                                                     col_offset, g.mask, g.tables, G, ld);
  GRADA_LAUNCH_CHECK();
}

// ---- tiled assembly: cells shared in z, y and x ------------------------------
//
// A tile is up to TL_COLS z-runs (vertical stacks of cells with equal x/y
// extent, each on the one above) with identical levels, arranged as 1 or 2
// runs across x times up to TL_COLS (or TL_COLS/2) y-neighbours: at every
// level, consecutive runs in y have the same x extent and the y0 of one equals
// the y1 of the previous, and the two runs across x have the same y extent and
// the x0 of the second equals the x1 of the first.  The host groups the cell
// list into tiles geometrically (build_tile_plan), whatever its order, so a
// refined mesh in octree leaf order still forms long runs wherever its cells
// are regular.  A thread (one observation point) walks a tile level by level
// and, within a level, y-row by y-row and run by run across x, so the cell
// above, the cell before in y and the cell before in x are always done: their
// bottom, y1 and x1 faces are taken over (prism_terms_tiled).  The z carries
// of the tile's runs and the y carries of its columns live in shared memory,
// the x carry in registers.  Each cell still writes its own column.

template <typename OutT>
__global__ void __launch_bounds__(TL_THREADS)
    assemble_tiled_kernel(const double *__restrict__ obs, int64_t n_obs,
                          const double *__restrict__ prisms, const int4 *__restrict__ tiles,
                          const int64_t *__restrict__ cells, uint32_t mask,
                          const double *__restrict__ tables, OutT *__restrict__ G, int64_t ld) {
  __shared__ double tab[kTabSize];
  __shared__ TileSmem ws;
  extern __shared__ double zsm[];
  for (int t = threadIdx.x; t < kTabSize; t += TL_THREADS) tab[t] = tables[t];
  const int64_t i = (int64_t)blockIdx.y * TL_THREADS + threadIdx.x;
  const bool active = i < n_obs;
  double px = 0, py = 0, pz = 0;
  if (active) {
    px = obs[3 * i];
    py = obs[3 * i + 1];
    pz = obs[3 * i + 2];
  }
  tile_walk<true>(tiles[blockIdx.x], cells, prisms, ws, zsm, active, px, py, pz,
                  families_for_mask(mask), tab, [&](int64_t cell, int, const PrismTerms &t) {
              OutT *gcol = G + cell * ld + i;
              int slot = 0;
#pragma unroll
              for (int b = 0; b < 10; b++) {
                if (mask & (1u << b)) {
                  store_entry(gcol + (int64_t)slot * n_obs, prism_component(t, b));
                  slot++;
                }
              }
            });
}

template <typename OutT>
void launch_assemble_tiled(const DevGeometry &g, const TilePlan &plan, OutT *G, int64_t ld,
                           cudaStream_t s) {
  if (plan.n_tiles <= 0 || g.n_obs <= 0) return;
  static std::mutex mu;
  static bool attr[64] = {};
  const int smem = tile_walk_dyn_smem(true);
  {
    int dev = 0;
    GRADA_CUDA_CHECK(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(mu);
    if (dev < 0 || dev >= 64 || !attr[dev]) {
      GRADA_CUDA_CHECK(cudaFuncSetAttribute(assemble_tiled_kernel<OutT>,
                                            cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
      if (dev >= 0 && dev < 64) attr[dev] = true;
    }
  }
  dim3 grid((unsigned)plan.n_tiles, (unsigned)ceil_div(g.n_obs, TL_THREADS));
  if (grid.y > 65535u || plan.n_tiles > 0x7fffffff)
    throw Error(-1, "too many observation points or tiles for one launch");
  assemble_tiled_kernel<OutT><<<grid, TL_THREADS, smem, s>>>(
      g.obs, g.n_obs, g.prisms, reinterpret_cast<const int4 *>(plan.tiles), plan.cells,
      g.mask, g.tables, G, ld);
  GRADA_LAUNCH_CHECK();
}

// ---- bf16 with a per-row scale ---------------------------------------------

__global__ void row_absmax_kernel(const float *__restrict__ G, int64_t nd, int64_t nm, int64_t ld,
                                  int cols_per_block, unsigned int *__restrict__ row_max_bits) {
  const int64_t row = (int64_t)blockIdx.y * blockDim.x + threadIdx.x;
  if (row >= nd) return;
  const int64_t c0 = (int64_t)blockIdx.x * cols_per_block;
  const int64_t c1 = min(nm, c0 + cols_per_block);
  float m = 0.f;
  for (int64_t c = c0; c < c1; c++) m = fmaxf(m, fabsf(G[row + c * ld]));
  // |x| of a finite float orders like its bit pattern.
  atomicMax(row_max_bits + row, __float_as_uint(m));
}

__global__ void row_scale_kernel(const unsigned int *__restrict__ row_max_bits, int64_t nd,
                                 float *__restrict__ scale) {
  const int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= nd) return;
  const float m = __uint_as_float(row_max_bits[row]);
  scale[row] = (m > 0.f) ? m : 1.f;
}

__global__ void quantize_16_kernel(const float *__restrict__ G, int64_t nd, int64_t nm,
                                   int64_t ld, const float *__restrict__ scale, int half16,
                                   uint16_t *__restrict__ out) {
  const int64_t row = (int64_t)blockIdx.y * blockDim.x + threadIdx.x;
  const int64_t col = blockIdx.x;
  if (row >= ld) return;
  const int64_t idx = row + col * ld;
  const float v = (row < nd) ? G[idx] / scale[row] : 0.f;
  out[idx] = half16 ? __half_as_ushort(__float2half_rn(v))
                    : __bfloat16_as_ushort(__float2bfloat16_rn(v));
}

__global__ void round_to_fp32_kernel(const double *__restrict__ in, float *__restrict__ out,
                                     size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    out[i] = (float)in[i];
}

// ---- matrix-free field sum ------------------------------------------------

// One block: TL_THREADS points x the tiles of one split; each thread sums
// rho_j field_k(point, cell_j) over the split's cells (tile walk, faces shared
// in z and y), the splits are added in order by a second pass.
__global__ void __launch_bounds__(TL_THREADS)
    forward_field_kernel(const double *__restrict__ obs, int64_t n_obs,
                         const double *__restrict__ prisms, const int4 *__restrict__ tiles,
                         const int64_t *__restrict__ cells, int64_t n_tiles,
                         int64_t tiles_per_split, const double *__restrict__ rho, uint32_t mask,
                         int nf, const double *__restrict__ tables, double *__restrict__ partial,
                         const int *__restrict__ skip) {
  if (skip && *skip) return;
  __shared__ double tab[kTabSize];
  __shared__ TileSmem ws;
  extern __shared__ double zsm[];
  for (int t = threadIdx.x; t < kTabSize; t += TL_THREADS) tab[t] = tables[t];
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
  double acc[10];
#pragma unroll
  for (int b = 0; b < 10; b++) acc[b] = 0.0;
  for (int64_t tl = t_begin; tl < t_end; tl++) {
    tile_walk<true>(tiles[tl], cells, prisms, ws, zsm, active, px, py, pz, fam, tab,
                    [&](int64_t cell, int, const PrismTerms &t) {
                const double w = __ldg(rho + cell);
#pragma unroll
                for (int b = 0; b < 10; b++)
                  if (mask & (1u << b)) acc[b] = fma(w, prism_component(t, b), acc[b]);
              });
  }
  if (!active) return;
  double *out = partial + split * n_obs * nf + i * nf;
  int slot = 0;
#pragma unroll
  for (int b = 0; b < 10; b++)
    if (mask & (1u << b)) out[slot++] = acc[b];
}

// Sums the per-split partials in split order.  With g_rows the result is
// written in G's row order (component k of point i at k*n_obs + i) instead of
// point-major order.
__global__ void sum_splits_kernel(const double *__restrict__ partial, int n_split, int64_t n,
                                  int nf, int64_t n_obs, int g_rows,
                                  const double *__restrict__ post_scale, double *__restrict__ out,
                                  const int *__restrict__ skip) {
  if (skip && *skip) return;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  double s = 0.0;
  for (int k = 0; k < n_split; k++) s += partial[(int64_t)k * n + e];
  if (g_rows) {
    const int64_t i = e / nf, c = e - i * nf;
    const int64_t r = c * n_obs + i;
    out[r] = post_scale ? post_scale[r] * s : s;
  } else {
    out[e] = s;
  }
}

// ---- matrix-free adjoint: x_j = sum_i sum_k G(k*n_obs+i, j) y(k*n_obs+i) ---

// Tiled G^T y: a block owns one tile and a range of point blocks.  For every
// cell of the tile each thread forms its point's contribution
// sum_k y(k*n_obs+i) field_k(point, cell); the warp adds its 32 with
// shuffles and lane 0 accumulates the warp sum in shared memory, in point-
// block order.  At the end the four warp sums of each cell are added in
// order and written as the block's partial (no atomics: bit-reproducible).
// Threads past n_obs walk observation 0 with weight 0, so every lane takes
// part in the shuffles.
__global__ void __launch_bounds__(TL_THREADS)
    adjoint_field_tiled_kernel(const double *__restrict__ obs, int64_t n_obs,
                               const double *__restrict__ prisms, const int4 *__restrict__ tiles,
                               const int64_t *__restrict__ cells, int64_t n_cells,
                               uint32_t mask, const double *__restrict__ tables,
                               const double *__restrict__ y, const double *__restrict__ pre_scale,
                               int64_t pblocks_per_split, double *__restrict__ partial,
                               const int *__restrict__ skip) {
  if (skip && *skip) return;
  __shared__ double tab[kTabSize];
  __shared__ TileSmem ws;
  __shared__ double wacc[TL_THREADS / 32][TL_COLS * TL_MAXLEV];
  extern __shared__ double zsm[];
  for (int t = threadIdx.x; t < kTabSize; t += TL_THREADS) tab[t] = tables[t];
  const int4 td = tiles[blockIdx.x];
  const int ncells = td.y * td.z;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int q = lane; q < ncells; q += 32) wacc[warp][q] = 0.0;
  const uint32_t fam = families_for_mask(mask);
  const int64_t n_pb = (n_obs + TL_THREADS - 1) / TL_THREADS;
  const int64_t pb0 = (int64_t)blockIdx.y * pblocks_per_split;
  const int64_t pb1 = min(n_pb, pb0 + pblocks_per_split);
  for (int64_t pb = pb0; pb < pb1; pb++) {
    const int64_t i = pb * TL_THREADS + threadIdx.x;
    const bool real = i < n_obs;
    const int64_t ii = real ? i : 0;
    const double px = obs[3 * ii], py = obs[3 * ii + 1], pz = obs[3 * ii + 2];
    double w[10];
    int slot = 0;
#pragma unroll
    for (int b = 0; b < 10; b++) {
      w[b] = 0.0;
      if (mask & (1u << b)) {
        const int64_t r = (int64_t)slot * n_obs + ii;
        w[b] = real ? (pre_scale ? pre_scale[r] * y[r] : y[r]) : 0.0;
        slot++;
      }
    }
    tile_walk<false>(td, cells, prisms, ws, zsm, true, px, py, pz, fam, tab,
                     [&](int64_t, int q, const PrismTerms &t) {
                double c = 0.0;
#pragma unroll
                for (int b = 0; b < 10; b++)
                  if (mask & (1u << b)) c = fma(w[b], prism_component(t, b), c);
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
                if (lane == 0) wacc[warp][q] += c;
              });
  }
  __syncthreads();
  for (int qq = threadIdx.x; qq < ncells; qq += TL_THREADS) {
    double v = 0.0;
#pragma unroll
    for (int w = 0; w < TL_THREADS / 32; w++) v += wacc[w][qq];
    const int k = qq / td.y, a = qq % td.y;  // q = level * runs + run
    const int64_t cell = cells[td.x + (int64_t)a * td.z + k];
    partial[(int64_t)blockIdx.y * n_cells + cell] = v;
  }
}

__global__ void sum_cell_splits_kernel(const double *__restrict__ partial, int n_split,
                                       int64_t n_cells, double *__restrict__ x,
                                       const int *__restrict__ skip) {
  if (skip && *skip) return;
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n_cells) return;
  double s = 0.0;
  for (int k = 0; k < n_split; k++) s += partial[(int64_t)k * n_cells + j];
  x[j] = s;
}

}  // namespace

void build_math_tables(double *tab) {
  // log bins: c_k ~ 1/(0.75 + k/256), ln(1/c_k) as a hi/lo pair
  for (int k = 0; k < kLogBins; k++) {
    const double c = (k == 64) ? 1.0 : 1.0 / (0.75 + k / 256.0);
    const long double L = -logl((long double)c);
    const double hi = (double)L;
    tab[kTabLog + 3 * k] = c;
    tab[kTabLog + 3 * k + 1] = hi;
    tab[kTabLog + 3 * k + 2] = (double)(L - (long double)hi);
  }
  const long double pi = acosl(-1.0L);
  for (int j = 0; j < kRotSteps; j++) {
    const long double th = pi * (long double)j / 128.0L;
    tab[kTabSinCos + 2 * j] = (double)cosl(th);
    tab[kTabSinCos + 2 * j + 1] = (double)sinl(th);
  }
  // hi parts with trailing significand bits cleared so that e*hi (|e| < 2^11)
  // and j*hi (|j| < 2^9) are exact
  auto clear_low = [](double v, int nbits) {
    uint64_t b;
    memcpy(&b, &v, 8);
    b &= ~((uint64_t(1) << nbits) - 1);
    memcpy(&v, &b, 8);
    return v;
  };
  const long double ln2 = logl(2.0L);
  const double ln2_hi = clear_low((double)ln2, 11);
  tab[kTabConst + 0] = ln2_hi;
  tab[kTabConst + 1] = (double)(ln2 - (long double)ln2_hi);
  const long double step = pi / 128.0L;
  const double step_hi = clear_low((double)step, 9);
  tab[kTabConst + 2] = step_hi;
  tab[kTabConst + 3] = (double)(step - (long double)step_hi);
}

int adjoint_field_splits(const DevGeometry &g, int sm_count) {
  // ~16 waves of the 2 resident blocks per SM over (tiles x point ranges)
  const int64_t n_pb = ceil_div(g.n_obs, TL_THREADS);
  int64_t splits = ceil_div((int64_t)sm_count * 2 * 16, std::max<int64_t>(g.plan.n_tiles, 1));
  if (splits > n_pb) splits = n_pb;
  if (splits < 1) splits = 1;
  if (splits > 65535) splits = 65535;
  return (int)splits;
}

void launch_adjoint_field(const DevGeometry &g, const double *y, const double *pre_scale,
                          int n_split, double *partial, double *x, cudaStream_t s,
                          const int *skip) {
  if (g.n_cells <= 0) return;
  const int64_t n_pb = ceil_div(g.n_obs, TL_THREADS);
  const int64_t per = ceil_div(n_pb, n_split);
  const int smem = tile_walk_dyn_smem(false);
  {
    static std::mutex mu;
    static bool attr[64] = {};
    int dev = 0;
    GRADA_CUDA_CHECK(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(mu);
    if (dev < 0 || dev >= 64 || !attr[dev]) {
      GRADA_CUDA_CHECK(cudaFuncSetAttribute(adjoint_field_tiled_kernel,
                                            cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
      if (dev >= 0 && dev < 64) attr[dev] = true;
    }
  }
  if (g.plan.n_tiles > 0x7fffffff) throw Error(-1, "too many tiles for one launch");
  dim3 grid((unsigned)g.plan.n_tiles, (unsigned)n_split);
  adjoint_field_tiled_kernel<<<grid, TL_THREADS, smem, s>>>(
      g.obs, g.n_obs, g.prisms, reinterpret_cast<const int4 *>(g.plan.tiles), g.plan.cells,
      g.n_cells, g.mask, g.tables, y, pre_scale, per, partial, skip);
  GRADA_LAUNCH_CHECK();
  sum_cell_splits_kernel<<<(unsigned)ceil_div(g.n_cells, 256), 256, 0, s>>>(partial, n_split,
                                                                           g.n_cells, x, skip);
  GRADA_LAUNCH_CHECK();
}

int math_table_size() { return kTabSize; }
void build_math_tables_host(double *tab) { build_math_tables(tab); }

int tile_max_cols() { return TL_COLS; }

void build_tile_plan(const double *p, int64_t n, std::vector<int32_t> &tiles,
                     std::vector<int64_t> &cells) {
  tiles.clear();
  cells.clear();
  // cells ordered by (x0, x1, y0, y1, z0): the stacks of a column become
  // adjacent.  A regular mesh in the reference's leaf order (x outer, y, z
  // inner) is already in this order, which one linear pass detects; otherwise
  // the keys are copied into one contiguous array and sorted.
  auto cell_less = [p](int64_t a, int64_t b) {
    const double *u = p + 6 * a, *v = p + 6 * b;
    for (int q = 0; q < 5; q++)
      if (u[q] != v[q]) return u[q] < v[q];
    return a < b;
  };
  std::vector<int64_t> ord((size_t)n);
  bool sorted = true;
  for (int64_t i = 0; i < n; i++) {
    ord[(size_t)i] = i;
    if (i > 0 && sorted && cell_less(i, i - 1)) sorted = false;
  }
  if (!sorted) {
    struct CellKey {
      double k[5];
      int64_t id;
    };
    std::vector<CellKey> keys((size_t)n);
    for (int64_t i = 0; i < n; i++) {
      for (int q = 0; q < 5; q++) keys[(size_t)i].k[q] = p[6 * i + q];
      keys[(size_t)i].id = i;
    }
    std::sort(keys.begin(), keys.end(), [](const CellKey &a, const CellKey &b) {
      for (int q = 0; q < 5; q++)
        if (a.k[q] != b.k[q]) return a.k[q] < b.k[q];
      return a.id < b.id;
    });
    for (int64_t i = 0; i < n; i++) ord[(size_t)i] = keys[(size_t)i].id;
  }
  // z-runs: equal x/y extents, each z0 the previous z1; sig is a hash of the
  // run's levels (its z0 sequence and last z1) that orders runs cheaply
  struct Run {
    int64_t start, len;
    uint64_t sig;
  };
  std::vector<Run> runs;
  for (int64_t c = 0; c < n;) {
    int64_t e = c;
    while (e + 1 < n) {
      const double *u = p + 6 * ord[e], *v = p + 6 * ord[e + 1];
      if (!(u[0] == v[0] && u[1] == v[1] && u[2] == v[2] && u[3] == v[3] && u[5] == v[4])) break;
      e++;
    }
    uint64_t h = 0x9E3779B97F4A7C15ull;  // multiply-xorshift over the boundaries' bits
    auto mix = [&h](double z) {
      uint64_t b;
      memcpy(&b, &z, 8);
      h = (h ^ b) * 0xBF58476D1CE4E5B9ull;
      h ^= h >> 31;
    };
    for (int64_t k = c; k <= e; k++) mix(p[6 * ord[k] + 4]);
    mix(p[6 * ord[e] + 5]);
    runs.push_back({c, e - c + 1, h});
    c = e + 1;
  }
  // runs ordered by (x0, x1, levels, y0): y-neighbours with identical levels
  // become adjacent (equal levels share count and signature)
  auto cell_of = [&](const Run &r, int64_t k) { return p + 6 * ord[r.start + k]; };
  // equal level sequences: count and signature as a quick reject, then the
  // levels themselves
  auto level_eq = [&](const Run &a, const Run &b) -> bool {
    if (a.len != b.len || a.sig != b.sig) return false;
    for (int64_t k = 0; k < a.len; k++)
      if (cell_of(a, k)[4] != cell_of(b, k)[4]) return false;
    return cell_of(a, a.len - 1)[5] == cell_of(b, b.len - 1)[5];
  };
  // (the sort uses the level count and signature only: runs with equal levels
  // stay adjacent, and a signature collision could at most split a chain,
  // since ynext and the x partners compare the levels themselves)
  std::sort(runs.begin(), runs.end(), [&](const Run &a, const Run &b) {
    const double *u = cell_of(a, 0), *v = cell_of(b, 0);
    if (u[0] != v[0]) return u[0] < v[0];
    if (u[1] != v[1]) return u[1] < v[1];
    if (a.len != b.len) return a.len < b.len;
    if (a.sig != b.sig) return a.sig < b.sig;
    if (u[2] != v[2]) return u[2] < v[2];
    return a.start < b.start;
  });
  auto ynext = [&](const Run &a, const Run &b) {
    const double *u = cell_of(a, 0), *v = cell_of(b, 0);
    return u[0] == v[0] && u[1] == v[1] && u[3] == v[2] && level_eq(a, b);
  };
  // x partner of a run: the run whose x0 is its x1, with the same y extent and
  // levels (candidates looked up by x0, y0, y1, level count and first z0)
  using Key = std::tuple<double, double, double, int64_t, double>;
  std::map<Key, std::vector<size_t>> by_face;
  for (size_t r = 0; r < runs.size(); r++) {
    const double *u = cell_of(runs[r], 0);
    by_face[Key(u[0], u[2], u[3], runs[r].len, u[4])].push_back(r);
  }
  std::vector<char> used(runs.size(), 0);
  auto partner = [&](size_t r) -> int64_t {
    const double *u = cell_of(runs[r], 0);
    auto it = by_face.find(Key(u[1], u[2], u[3], runs[r].len, u[4]));
    if (it == by_face.end()) return -1;
    for (size_t q : it->second)
      if (!used[q] && level_eq(runs[r], runs[q])) return (int64_t)q;
    return -1;
  };
  auto emit = [&](const std::vector<size_t> &order, int nx) {
    const int64_t len = runs[order[0]].len;
    // runs longer than TL_MAXLEV levels go on in further tiles of the same runs
    for (int64_t l0 = 0; l0 < len; l0 += TL_MAXLEV) {
      const int64_t nl = std::min<int64_t>(TL_MAXLEV, len - l0);
      tiles.push_back((int32_t)cells.size());
      tiles.push_back((int32_t)order.size());
      tiles.push_back((int32_t)nl);
      tiles.push_back(nx);
      for (size_t q : order)
        for (int64_t k = 0; k < nl; k++) cells.push_back(ord[runs[q].start + l0 + k]);
    }
  };
  tiles.reserve(4 * (size_t)(n / TL_MAXLEV + runs.size()) + 4);
  cells.reserve((size_t)n);
  // Greedy in (x0, x1, levels, y0) order: a run with an x partner starts a
  // 2 x m tile (m <= TL_COLS/2 y-neighbours, each with its partner, run order
  // y-major, x-minor); one without starts a 1 x m tile (m <= TL_COLS) that
  // stops before a run that could start a 2 x m tile.
  for (size_t r = 0; r < runs.size(); r++) {
    if (used[r]) continue;
    std::vector<size_t> order;
    const int64_t p0 = partner(r);
    if (p0 >= 0) {
      size_t e = r, pe = (size_t)p0;
      used[e] = used[pe] = 1;
      order.push_back(e);
      order.push_back(pe);
      while ((int)order.size() < TL_COLS && e + 1 < runs.size() && !used[e + 1] &&
             ynext(runs[e], runs[e + 1])) {
        const int64_t pn = partner(e + 1);
        if (pn < 0 || !ynext(runs[pe], runs[(size_t)pn])) break;
        e = e + 1;
        pe = (size_t)pn;
        used[e] = used[pe] = 1;
        order.push_back(e);
        order.push_back(pe);
      }
      emit(order, 2);
    } else {
      size_t e = r;
      used[e] = 1;
      order.push_back(e);
      while ((int)order.size() < TL_COLS && e + 1 < runs.size() && !used[e + 1] &&
             ynext(runs[e], runs[e + 1]) && partner(e + 1) < 0) {
        e = e + 1;
        used[e] = 1;
        order.push_back(e);
      }
      emit(order, 1);
    }
  }
}

void launch_round_to_fp32(const double *in, float *out, size_t n, cudaStream_t s) {
  if (n == 0) return;
  const size_t blocks = std::min<size_t>((n + 255) / 256, (size_t)65535 * 16);
  round_to_fp32_kernel<<<(unsigned)blocks, 256, 0, s>>>(in, out, n);
  GRADA_LAUNCH_CHECK();
}

void launch_assemble_tiled_fp64(const DevGeometry &g, const TilePlan &plan, double *G, int64_t ld,
                                cudaStream_t s) {
  launch_assemble_tiled<double>(g, plan, G, ld, s);
}

void launch_assemble_tiled_fp32(const DevGeometry &g, const TilePlan &plan, float *G, int64_t ld,
                                cudaStream_t s) {
  launch_assemble_tiled<float>(g, plan, G, ld, s);
}

void launch_assemble_fp64(const DevGeometry &g, const double *prisms, int64_t n_cells,
                          const int64_t *col_index, int64_t col_offset, double *G, int64_t ld,
                          cudaStream_t s) {
  launch_assemble<double>(g, prisms, n_cells, col_index, col_offset, G, ld, s);
}

void launch_assemble_fp32(const DevGeometry &g, const double *prisms, int64_t n_cells,
                          const int64_t *col_index, int64_t col_offset, float *G, int64_t ld,
                          cudaStream_t s) {
  launch_assemble<float>(g, prisms, n_cells, col_index, col_offset, G, ld, s);
}

void launch_rowscale_16(const float *G32, int64_t nd, int64_t nm, int64_t ld, float *row_scale,
                        uint16_t *G16, bool half16, cudaStream_t s) {
  // row_scale doubles as the atomicMax target (bit patterns) before scaling.
  unsigned int *bits = reinterpret_cast<unsigned int *>(row_scale);
  GRADA_CUDA_CHECK(cudaMemsetAsync(bits, 0, sizeof(unsigned int) * nd, s));
  const int cols_per_block = 256;
  dim3 g1((unsigned)ceil_div(nm, cols_per_block), (unsigned)ceil_div(nd, 256));
  row_absmax_kernel<<<g1, 256, 0, s>>>(G32, nd, nm, ld, cols_per_block, bits);
  GRADA_LAUNCH_CHECK();
  row_scale_kernel<<<(unsigned)ceil_div(nd, 256), 256, 0, s>>>(bits, nd, row_scale);
  GRADA_LAUNCH_CHECK();
  dim3 g3((unsigned)nm, (unsigned)ceil_div(ld, 256));
  quantize_16_kernel<<<g3, 256, 0, s>>>(G32, nd, nm, ld, row_scale, half16 ? 1 : 0, G16);
  GRADA_LAUNCH_CHECK();
}

int forward_field_splits(const DevGeometry &g, int sm_count) {
  // ~16 waves of the 2 resident blocks per SM, so the last wave is a small
  // part of the launch
  const int64_t obs_tiles = ceil_div(g.n_obs, TL_THREADS);
  const int64_t want_blocks = (int64_t)sm_count * 2 * 16;
  int64_t splits = ceil_div(want_blocks, obs_tiles);
  const int64_t max_splits = g.plan.n_tiles;
  if (splits > max_splits) splits = max_splits;
  if (splits < 1) splits = 1;
  if (splits > 65535) splits = 65535;
  return (int)splits;
}

void launch_forward_field(const DevGeometry &g, const double *rho, int n_split, double *partial,
                          double *fields, bool g_rows, cudaStream_t s, const double *post_scale,
                          const int *skip) {
  if (g.n_obs <= 0) return;
  const int64_t per = ceil_div(g.plan.n_tiles, n_split);
  dim3 grid((unsigned)n_split, (unsigned)ceil_div(g.n_obs, TL_THREADS));
  if (grid.y > 65535u) throw Error(-1, "too many observation points for one launch");
  const int smem = tile_walk_dyn_smem(true);
  {
    static std::mutex mu;
    static bool attr[64] = {};
    int dev = 0;
    GRADA_CUDA_CHECK(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(mu);
    if (dev < 0 || dev >= 64 || !attr[dev]) {
      GRADA_CUDA_CHECK(cudaFuncSetAttribute(forward_field_kernel,
                                            cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
      if (dev >= 0 && dev < 64) attr[dev] = true;
    }
  }
  forward_field_kernel<<<grid, TL_THREADS, smem, s>>>(
      g.obs, g.n_obs, g.prisms, reinterpret_cast<const int4 *>(g.plan.tiles), g.plan.cells,
      g.plan.n_tiles, per, rho, g.mask, g.n_fields, g.tables, partial, skip);
  GRADA_LAUNCH_CHECK();
  const int64_t n = g.n_obs * g.n_fields;
  sum_splits_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, s>>>(
      partial, n_split, n, g.n_fields, g.n_obs, g_rows ? 1 : 0, post_scale, fields, skip);
  GRADA_LAUNCH_CHECK();
}

}  // namespace grada
