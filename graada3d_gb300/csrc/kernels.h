// Internal launcher interface between the host context (abi.cu) and the CUDA
// kernels.  Nothing here is part of the C ABI.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

namespace grada {

// Assembly tiles (cells that share faces in z, y and x).  The plan groups the
// cell list, in any order, into tiles of up to tile_max_cols() z-runs (stacks
// of cells with equal x/y extent, each on the one above) that are neighbours
// level by level, nx = 1 or 2 across x times runs / nx along y: int4 {offset,
// runs, levels, nx} per tile; run a sits at x = a % nx, y = a / nx and its
// cell at level k is cells[offset + a * levels + k].
struct TilePlan {
  const int32_t *tiles = nullptr;    // n_tiles x 4
  const int64_t *cells = nullptr;
  int64_t n_tiles = 0;
};

// Device-resident problem geometry (mesh leaf cells and observation points).
struct DevGeometry {
  const double *prisms = nullptr;  // n_cells x 6: x0 x1 y0 y1 z0 z1
  const double *obs = nullptr;     // n_obs x 3
  int64_t n_cells = 0;
  int64_t n_obs = 0;
  uint32_t mask = 0;
  int n_fields = 0;
  const double *tables = nullptr;  // math tables of prism.cuh (kTabSize doubles)
  TilePlan plan;                   // the cell list as assembly tiles
};

// Number of doubles of the math tables and their host-side construction.
int math_table_size();
void build_math_tables_host(double *tab);

// ---- sensitivity assembly (assemble.cu) ---------------------------------
// Writes the columns of G for cells [0, n_cells) of `prisms`; column of cell c
// is col_index[c] when col_index is non-null, else c + col_offset.
void launch_assemble_fp64(const DevGeometry &g, const double *prisms, int64_t n_cells,
                          const int64_t *col_index, int64_t col_offset, double *G, int64_t ld,
                          cudaStream_t s);
void launch_assemble_fp32(const DevGeometry &g, const double *prisms, int64_t n_cells,
                          const int64_t *col_index, int64_t col_offset, float *G, int64_t ld,
                          cudaStream_t s);
int tile_max_cols();
void build_tile_plan(const double *prisms, int64_t n_cells, std::vector<int32_t> &tiles,
                     std::vector<int64_t> &cells);
void launch_assemble_tiled_fp64(const DevGeometry &g, const TilePlan &plan, double *G, int64_t ld,
                                cudaStream_t s);
void launch_assemble_tiled_fp32(const DevGeometry &g, const TilePlan &plan, float *G, int64_t ld,
                                cudaStream_t s);

// Per-row maximum of |G| over the columns, then bf16 entries G/scale with the
// FP32 scale per row (entries of an all-zero row get scale 1).
// half16 = false: bf16; true: IEEE fp16 (entries in [-1, 1] after scaling).
void launch_rowscale_16(const float *G32, int64_t nd, int64_t nm, int64_t ld, float *row_scale,
                        uint16_t *G16, bool half16, cudaStream_t s);

// Matrix-free field sum: fields[i*nf + k] = sum_j rho_j field_k(obs_i, cell_j).
// `partial` must hold n_split * n_obs * nf doubles.
int forward_field_splits(const DevGeometry &g, int sm_count);
// With g_rows the result is in G's row order and may be post-scaled; skip as
// in GemvOpts.
void launch_forward_field(const DevGeometry &g, const double *rho, int n_split, double *partial,
                          double *fields, bool g_rows, cudaStream_t s,
                          const double *post_scale = nullptr, const int *skip = nullptr);
// Matrix-free G^T y (y in G's row order, optionally pre-scaled); `partial`
// holds n_split * n_cells doubles.
int adjoint_field_splits(const DevGeometry &g, int sm_count);
void launch_adjoint_field(const DevGeometry &g, const double *y, const double *pre_scale,
                          int n_split, double *partial, double *x, cudaStream_t s,
                          const int *skip = nullptr);

// ---- dense products (gemv.cu) -------------------------------------------
enum class GKind : int { FP64 = 0, FP32 = 1, BF16 = 2, FP16 = 3 };

struct DevG {
  GKind kind = GKind::FP64;
  const void *data = nullptr;
  const float *row_scale = nullptr;  // bf16 / fp16 only
  int64_t nd = 0, nm = 0, ld = 0;
};

// Optional extras of the products: skip (device flag; when non-zero every
// kernel of the product returns at once, so a captured CG iteration becomes a
// no-op after convergence) and a diagonal row scale (G x: applied to the
// result, y_r *= scale_r; G^T y: applied to the input, y_r -> scale_r y_r).
struct GemvOpts {
  const int *skip = nullptr;
  const double *scale = nullptr;
};

// Partition of G x: column ranges ("splits") per row tile of 256 * vec rows,
// vec = entries per 16-byte load of the storage (vec_of).
int gx_splits(const DevG &G, int sm_count, int vec);
int vec_of(GKind k);
// Scratch (in doubles) the products need for a given G, and the launches.
int64_t gemv_scratch_doubles(const DevG &G, int sm_count);
void launch_G_vec_mul(const DevG &G, const double *x, double *y, double *scratch, int sm_count,
                      cudaStream_t s, const GemvOpts &o = GemvOpts());
void launch_GT_vec_mul(const DevG &G, const double *y, double *x, double *scratch, int sm_count,
                       cudaStream_t s, const GemvOpts &o = GemvOpts());
// norms[j] = ||G(:, j)||_2 of the stored entries (16-bit ones with their row
// scale), FP64 sums; stored storages only.
void launch_column_norms(const DevG &G, double *norms, cudaStream_t s);

// out[i] = (float)in[i] for i < n (round to nearest: the entries the FP32
// assembly writes from the same FP64 values).
void launch_round_to_fp32(const double *in, float *out, size_t n, cudaStream_t s);

// Columns [c0, c0+nc) of G widened to FP64 (scale applied for bf16) into
// out (ld x nc, column-major).
void launch_widen_columns(const DevG &G, int64_t c0, int64_t nc, double *out, cudaStream_t s);
// out[r * nm + j] = G(rows[r], j) in FP64 for n_rows (<= 65535) device row indices.
void launch_gather_rows(const DevG &G, const int64_t *rows, int64_t n_rows, double *out,
                        cudaStream_t s);

// ---- block products (block_gemm.cu, tc_gemm.cu) -------------------------
// Y = G X and X = G^T Y for blocks of kBW = 16 right-hand sides, row-
// interleaved ([row * 16 + col], see cg_kernels.h).  Y has nd rows (rows
// nd..ld-1 are neither read nor written).  GemvOpts as for the products
// above, per row.  FP64 G runs on the FP64 pipe; FP32 and 16-bit G run on the
// tensor cores (tc_gemm.cu).  `err` is a device int that a tensor-core
// launch raises (bit flags) when one of its bounded waits gives up.
int64_t block_scratch_bytes(const DevG &G, int sm_count);
void launch_G_mat_mul(const DevG &G, const double *X, double *Y, void *scratch, int sm_count,
                      cudaStream_t s, const GemvOpts &o, int *err);
void launch_GT_mat_mul(const DevG &G, const double *Y, double *X, void *scratch, int sm_count,
                       cudaStream_t s, const GemvOpts &o, int *err);

// Tensor-core implementation for FP32 (3xTF32 split) and 16-bit G (A exact,
// right-hand sides split into two 16-bit parts).
bool tc_supported(const DevG &G);
int64_t tc_scratch_bytes(const DevG &G, int sm_count);
void launch_tc_G_mat_mul(const DevG &G, const double *X, double *Y, void *scratch, int sm_count,
                         cudaStream_t s, const GemvOpts &o, int *err);
void launch_tc_GT_mat_mul(const DevG &G, const double *Y, double *X, void *scratch, int sm_count,
                          cudaStream_t s, const GemvOpts &o, int *err);

// Matrix-free block products: every (point, cell) pair evaluated once for all
// 16 right-hand sides (FP64).
int64_t mf_block_scratch_doubles(const DevGeometry &g, int sm_count);
void launch_forward_field_block(const DevGeometry &g, const double *X, double *Y, double *scratch,
                                int sm_count, cudaStream_t s, const GemvOpts &o);
void launch_adjoint_field_block(const DevGeometry &g, const double *Y, double *X, double *scratch,
                                int sm_count, cudaStream_t s, const GemvOpts &o);

// ---- diagnostics (diag.cu) ----------------------------------------------
double measure_fp64_fma_rate(int sm_count, cudaStream_t s);

}  // namespace grada
