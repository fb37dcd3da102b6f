// Wavelet-compressed sensitivity matrix (method_id 2 of the reference):
// Fwd::compute_G_wavelet (Fwd.cpp:148-219), Fwd::compress_vec (:298-358) and
// the wavelet branches of Fwd::G_vec_mul / GT_vec_mul (:80-146) with
// wavelet_transform_vec / inverse_wavelet_transform_vec (:257-296, :360-402).
//
// Each row of G, its cells taken in the mesh's reordered sequence
// (Mesh::get_reordered_id, handed in by the host) and zero-padded to n_dy, the
// next power of two, goes through the periodic Daubechies-4 pyramid: the
// four-tap scaling filter h of Daubechies (1988), the wavelet filter
// g_k = (-1)^k h_{3-k}, no offset, levels n = n_dy, ..., 2 with a level's
// approximations in [0, n/2) and its details in [n/2, n) -- the algorithm the
// reference takes from GSL (gsl_wavelet_daubechies, member 4).  A row keeps
// the coefficients with |c| > t or ||c| - t| < 1e-15, t = threshold x the
// row's largest |c|, in coefficient order.
//
// Like the reference, the compression never holds the dense G: the rows are
// assembled (FP64, the tiled assembly) for a batch of observation points at a
// time, transformed and thresholded; a first pass counts each row's kept
// coefficients, a second assembles again and fills them in.
//
//   G x:   x reordered and padded, transformed; one warp per row dots the
//          row's kept coefficients with it, lane l summing entries l, l + 32,
//          ... in order, then a fixed butterfly over the lanes.
//   G^T y: rows in 304 consecutive blocks; a block adds its rows' scaled
//          coefficients into its own partial vector, row after row (a segment
//          of 4096 columns at a time, in shared memory); the partials are
//          added in block order; then the inverse pyramid (levels 2, 4, ...,
//          n_dy) and the cell order.
// These fixed orders differ from the reference's sequential sums at the
// rounding level; the oracle reproduces them.  Every operation is an explicit
// round-to-nearest one.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <vector>

#include <cub/block/block_reduce.cuh>
#include <cub/block/block_scan.cuh>

#include "common.cuh"
#include "context.h"
#include "kernels.h"

namespace grada {
namespace {

constexpr int WV_THREADS = 256;
constexpr int kGtBlocks = 304;       // row blocks of G^T y
constexpr int64_t kGtSegment = 4096;  // columns a block of G^T y accumulates in shared memory

// (1 + sqrt 3, 3 + sqrt 3, 3 - sqrt 3, 1 - sqrt 3) / (4 sqrt 2), correctly rounded
__constant__ double kH[4] = {0.48296291314453416, 0.8365163037378079, 0.2241438680420134,
                             -0.12940952255126037};
__constant__ double kG[4] = {-0.12940952255126037, -0.2241438680420134, 0.8365163037378079,
                             -0.48296291314453416};

unsigned grid_for(int64_t n) { return (unsigned)std::max<int64_t>(1, ceil_div(n, WV_THREADS)); }

// P[r * n_dy + j] = Gb(r, order[j]) for j < nm, zero up to n_dy: a 32 x 32
// tiled transpose (coalesced reads down G's columns, coalesced row writes).
__global__ void load_rows_kernel(const double *__restrict__ Gb, int64_t ldb, int64_t rows,
                                 const int *__restrict__ order, int64_t nm, int64_t n_dy,
                                 double *__restrict__ P) {
  __shared__ double tile[32][33];
  const int64_t j0 = (int64_t)blockIdx.x * 32, r0 = (int64_t)blockIdx.y * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
  for (int q = 0; q < 4; q++) {
    const int64_t j = j0 + ty + 8 * q, r = r0 + tx;
    double v = 0.0;
    if (j < nm && r < rows) v = Gb[(int64_t)order[j] * ldb + r];
    tile[ty + 8 * q][tx] = v;
  }
  __syncthreads();
  for (int q = 0; q < 4; q++) {
    const int64_t r = r0 + ty + 8 * q, j = j0 + tx;
    if (r < rows && j < n_dy) P[r * n_dy + j] = tile[tx][ty + 8 * q];
  }
}

// One forward level of length n on `rows` vectors of stride S: approximations
// to approx[r * S + ii], details to coef[r * S + nh + ii] (at n = 2 approx is
// coef itself: the two writes never meet).
__global__ void forward_level_kernel(const double *__restrict__ src, double *approx, double *coef,
                                     int64_t rows, int64_t S, int64_t n,
                                     const int *__restrict__ skip) {
  if (skip && *skip) return;
  const int64_t nh = n >> 1;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= rows * nh) return;
  const int64_t ii = t % nh, r = t / nh;
  const double *a = src + r * S;
  double h = 0.0, g = 0.0;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const double v = a[(2 * ii + k) & (n - 1)];
    h = __dadd_rn(h, __dmul_rn(kH[k], v));
    g = __dadd_rn(g, __dmul_rn(kG[k], v));
  }
  approx[r * S + ii] = h;
  coef[r * S + nh + ii] = g;
}

__device__ __forceinline__ bool kept(double c, double thr) {
  const double a = fabs(c);
  return a > thr || fabs(__dsub_rn(a, thr)) < 1e-15;
}

// Global row of batch row r: component r / pb of point p0 + r % pb.
__device__ __forceinline__ int64_t global_row(int64_t r, int64_t pb, int64_t p0, int64_t n_obs) {
  return (r / pb) * n_obs + p0 + r % pb;
}

__device__ double block_row_threshold(const double *__restrict__ c, int64_t n_dy, double rel) {
  using Reduce = cub::BlockReduce<double, WV_THREADS>;
  __shared__ typename Reduce::TempStorage tmp;
  __shared__ double thr;
  double mx = 0.0;
  for (int64_t i = threadIdx.x; i < n_dy; i += WV_THREADS) mx = fmax(mx, fabs(c[i]));
  mx = Reduce(tmp).Reduce(mx, [](double a, double b) { return fmax(a, b); });
  if (threadIdx.x == 0) thr = __dmul_rn(rel, mx);
  __syncthreads();
  return thr;
}

// One block per batch row: the number of kept coefficients.
__global__ void __launch_bounds__(WV_THREADS)
    count_rows_kernel(const double *__restrict__ C, int64_t n_dy, double rel, int64_t pb,
                      int64_t p0, int64_t n_obs, int64_t *__restrict__ count) {
  using Reduce = cub::BlockReduce<int64_t, WV_THREADS>;
  __shared__ typename Reduce::TempStorage tmp;
  const int64_t r = blockIdx.x;
  const double *c = C + r * n_dy;
  const double thr = block_row_threshold(c, n_dy, rel);
  int64_t k = 0;
  for (int64_t i = threadIdx.x; i < n_dy; i += WV_THREADS) k += kept(c[i], thr) ? 1 : 0;
  k = Reduce(tmp).Sum(k);
  if (threadIdx.x == 0) count[global_row(r, pb, p0, n_obs)] = k;
}

// One block per batch row: the kept coefficients in index order (as FP32,
// rounded to nearest, when the values are stored in FP32).
template <class V>
__global__ void __launch_bounds__(WV_THREADS)
    fill_rows_kernel(const double *__restrict__ C, int64_t n_dy, double rel, int64_t pb,
                     int64_t p0, int64_t n_obs, const int64_t *__restrict__ rowptr,
                     int *__restrict__ col, V *__restrict__ val) {
  using Scan = cub::BlockScan<int, WV_THREADS>;
  __shared__ typename Scan::TempStorage tmp;
  const int64_t r = blockIdx.x;
  const double *c = C + r * n_dy;
  const double thr = block_row_threshold(c, n_dy, rel);
  int64_t base = rowptr[global_row(r, pb, p0, n_obs)];
  for (int64_t i0 = 0; i0 < n_dy; i0 += WV_THREADS) {
    const int64_t i = i0 + threadIdx.x;
    const double v = i < n_dy ? c[i] : 0.0;
    const int flag = (i < n_dy && kept(v, thr)) ? 1 : 0;
    int pos, total;
    Scan(tmp).ExclusiveSum(flag, pos, total);
    if (flag) {
      col[base + pos] = (int)i;
      val[base + pos] = (V)v;
    }
    base += total;
    __syncthreads();  // tmp is reused by the next chunk
  }
}

// ---- products --------------------------------------------------------------

__global__ void load_vec_kernel(const double *__restrict__ x, const int *__restrict__ order,
                                int64_t nm, int64_t n_dy, double *__restrict__ w,
                                const int *__restrict__ skip) {
  if (skip && *skip) return;
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n_dy) return;
  w[j] = j < nm ? x[order[j]] : 0.0;
}

template <class V>
__global__ void row_dot_kernel(const int64_t *__restrict__ rowptr, const int *__restrict__ col,
                               const V *__restrict__ val, const double *__restrict__ w,
                               int64_t nd, const double *__restrict__ scale,
                               double *__restrict__ y, const int *__restrict__ skip) {
  if (skip && *skip) return;
  const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (r >= nd) return;
  double s = 0.0;
  // unrolled; the additions keep their order
  const int64_t k1 = rowptr[r + 1];
#pragma unroll 4
  for (int64_t k = rowptr[r] + lane; k < k1; k += 32)
    s = __dadd_rn(s, __dmul_rn((double)val[k], w[col[k]]));
#pragma unroll
  for (int off = 16; off >= 1; off >>= 1) s = __dadd_rn(s, __shfl_xor_sync(0xffffffffu, s, off));
  if (lane == 0) y[r] = scale ? __dmul_rn(s, scale[r]) : s;
}

// seg[r * (S + 1) + s] = the first entry of row r with column >= s * SEG
// (columns ascend within a row), s = 0..S.
__global__ void segment_starts_kernel(const int64_t *__restrict__ rowptr,
                                      const int *__restrict__ col, int64_t nd, int64_t S,
                                      int64_t SEG, int64_t *__restrict__ seg) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nd * (S + 1)) return;
  const int64_t r = t / (S + 1), s = t % (S + 1);
  const int64_t c = s * SEG;
  int64_t lo = rowptr[r], hi = rowptr[r + 1];
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (col[mid] < c) lo = mid + 1;
    else hi = mid;
  }
  seg[t] = lo;
}

// Block (b, s) adds the entries of rows [b R, (b + 1) R) with columns in
// segment s into a shared-memory accumulator, row after row, and writes it to
// part[b * n_dy + s * SEG + i]: per column the rows of a block in ascending
// order, as one pass over the whole row would add them.
template <class V>
__global__ void __launch_bounds__(WV_THREADS)
    gt_partial_kernel(const int64_t *__restrict__ seg, const int *__restrict__ col,
                      const V *__restrict__ val, const double *__restrict__ y,
                      const double *__restrict__ scale, int64_t nd, int64_t R, int64_t S,
                      int64_t SEG, int64_t n_dy, double *__restrict__ part,
                      const int *__restrict__ skip) {
  if (skip && *skip) return;
  extern __shared__ double acc[];
  const int64_t b = blockIdx.x, s = blockIdx.y, c0 = s * SEG;
  for (int64_t i = threadIdx.x; i < SEG; i += WV_THREADS) acc[i] = 0.0;
  __syncthreads();
  const int64_t r_last = (b + 1) * R;
  const int64_t r_end = r_last < nd ? r_last : nd;
  for (int64_t r = b * R; r < r_end; r++) {
    const double v = scale ? __dmul_rn(scale[r], y[r]) : y[r];
    const int64_t k1 = seg[r * (S + 1) + s + 1];
#pragma unroll 4
    for (int64_t k = seg[r * (S + 1) + s] + threadIdx.x; k < k1; k += WV_THREADS) {
      const int64_t c = col[k] - c0;
      acc[c] = __dadd_rn(acc[c], __dmul_rn((double)val[k], v));
    }
    __syncthreads();  // the next row may touch the same entries
  }
  double *p = part + b * n_dy + c0;
  for (int64_t i = threadIdx.x; i < SEG; i += WV_THREADS) p[i] = acc[i];
}

__global__ void gt_reduce_kernel(const double *__restrict__ part, int64_t nb, int64_t n_dy,
                                 double *__restrict__ w, const int *__restrict__ skip) {
  if (skip && *skip) return;
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n_dy) return;
  double s = 0.0;
  for (int64_t b = 0; b < nb; b++) s = __dadd_rn(s, part[b * n_dy + c]);
  w[c] = s;
}

// One inverse level of length n: approximations a[0, nh) (the previous
// level's output, or coef[0] at n = 2), details coef[nh, n), result out[0, n).
// Output j takes the contributions of (ii, k) with (2 ii + k) mod n = j in the
// order the pyramid adds them: ascending ii, then ascending k.
__global__ void inverse_level_kernel(const double *__restrict__ a, const double *__restrict__ coef,
                                     double *__restrict__ out, int64_t n,
                                     const int *__restrict__ skip) {
  if (skip && *skip) return;
  const int64_t nh = n >> 1;
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const int k0 = (int)(j & 1);             // k of the contribution from ii = j >> 1
  const int64_t ia = j >> 1;
  const int64_t ib = (ia + nh - 1) % nh;  // the contribution with k0 + 2
  const double ca = __dadd_rn(__dmul_rn(kH[k0], a[ia]), __dmul_rn(kG[k0], coef[nh + ia]));
  const double cb =
      __dadd_rn(__dmul_rn(kH[k0 + 2], a[ib]), __dmul_rn(kG[k0 + 2], coef[nh + ib]));
  // ib < ia except for j = 0, 1 (ib wraps to nh - 1; at nh = 1, ia = ib and k
  // orders them)
  out[j] = ib < ia ? __dadd_rn(__dadd_rn(0.0, cb), ca) : __dadd_rn(__dadd_rn(0.0, ca), cb);
}

__global__ void store_vec_kernel(const double *__restrict__ w, const int *__restrict__ order,
                                 int64_t nm, double *__restrict__ x, const int *__restrict__ skip) {
  if (skip && *skip) return;
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nm) return;
  x[order[j]] = w[j];
}

// Forward pyramid of `rows` vectors of stride n_dy held in P0; details land in
// C, the last approximation in C[r * n_dy]; P0 and P1 take the intermediate
// approximations in turn.
void forward_pyramid(double *P0, double *P1, double *C, int64_t rows, int64_t n_dy,
                     const int *skip, cudaStream_t s) {
  const double *src = P0;
  double *bufs[2] = {P1, P0};
  int flip = 0;
  for (int64_t n = n_dy; n >= 2; n >>= 1) {
    double *dst = n == 2 ? C : bufs[flip];
    forward_level_kernel<<<grid_for(rows * (n >> 1)), WV_THREADS, 0, s>>>(src, dst, C, rows, n_dy,
                                                                          n, skip);
    GRADA_LAUNCH_CHECK();
    src = dst;
    flip ^= 1;
  }
}

}  // namespace

void Context::compute_G_wavelet(const int64_t *h_order, double rel, int value_storage) {
  require_geometry();
  if (value_storage != GRADA_G_FP64 && value_storage != GRADA_G_FP32)
    throw Error(GRADA_ERR_INVALID_ARGUMENT, "wavelet values are stored in FP64 or FP32");
  const bool f32 = value_storage == GRADA_G_FP32;
  if (!h_order) throw Error(GRADA_ERR_INVALID_ARGUMENT, "null cell order");
  if (!std::isfinite(rel) || rel < 0.0)
    throw Error(GRADA_ERR_INVALID_ARGUMENT, "threshold must be finite and >= 0");
  const int64_t nm = n_cells;
  if (nm < 2) throw Error(GRADA_ERR_INVALID_ARGUMENT, "the wavelet G needs two cells or more");
  if (nm >= ((int64_t)1 << 30)) throw Error(GRADA_ERR_INVALID_ARGUMENT, "too many cells");
  std::vector<int> order((size_t)nm);
  {
    std::vector<char> seen((size_t)nm, 0);
    for (int64_t j = 0; j < nm; j++) {
      const int64_t v = h_order[j];
      if (v < 0 || v >= nm || seen[(size_t)v])
        throw Error(GRADA_ERR_INVALID_ARGUMENT, "cell order is not a permutation");
      seen[(size_t)v] = 1;
      order[(size_t)j] = (int)v;
    }
  }
  int64_t n_dy = 1;
  while (n_dy < nm) n_dy <<= 1;
  if (n_dy / std::min<int64_t>(kGtSegment, n_dy) > 65535)
    throw Error(GRADA_ERR_INVALID_ARGUMENT, "too many cells for the wavelet G (2^28 at most)");

  // the old G goes first: the compressed rows replace it
  g_storage = -1;
  g64_valid = false;
  G.release();
  G64.release();
  wv_order.alloc(this, sizeof(int) * (size_t)nm);
  upload(wv_order.ptr, order.data(), sizeof(int) * (size_t)nm);

  // points per batch: the batch's FP64 rows (ldb x nm) and three n_dy-long
  // buffers per row within ~8 GB
  const int64_t budget = (int64_t)8 << 30;
  const int64_t per_row = 8 * (nm + 3 * n_dy);
  int64_t pb = std::max<int64_t>(1, budget / (per_row * n_fields));
  // GRADA_WAVELET_BATCH_POINTS makes batches smaller (tests); it never raises
  // the batch above the ~8 GB budget
  if (const char *e = std::getenv("GRADA_WAVELET_BATCH_POINTS"))
    pb = std::min(pb, std::max<int64_t>(1, std::atoll(e)));
  pb = std::min(pb, n_obs);
  pb = std::min<int64_t>(pb, std::max<int64_t>(1, (int64_t)65535 * 32 / n_fields));  // grid rows
  const int64_t rows_max = pb * n_fields, ldb = round_up(rows_max, 32);
  DevBuf Gb, P0, P1, C, cnt;
  Gb.alloc(this, sizeof(double) * (size_t)(ldb * nm));
  P0.alloc(this, sizeof(double) * (size_t)(rows_max * n_dy));
  P1.alloc(this, sizeof(double) * (size_t)(rows_max * n_dy));
  C.alloc(this, sizeof(double) * (size_t)(rows_max * n_dy));
  cnt.alloc(this, sizeof(int64_t) * (size_t)nd);
  const DevGeometry g_all = geometry();
  const TilePlan plan = tile_plan();
  auto transform_batch = [&](int64_t p0, int64_t np) {
    DevGeometry g = g_all;  // the batch's points only: rows k * np + i
    g.obs = g_all.obs + 3 * p0;
    g.n_obs = np;
    launch_assemble_tiled_fp64(g, plan, Gb.as<double>(), ldb, stream);
    const int64_t rows = np * n_fields;
    dim3 grid((unsigned)ceil_div(n_dy, 32), (unsigned)ceil_div(rows, 32));
    load_rows_kernel<<<grid, dim3(32, 8), 0, stream>>>(Gb.as<double>(), ldb, rows,
                                                      wv_order.as<int>(), nm, n_dy,
                                                      P0.as<double>());
    GRADA_LAUNCH_CHECK();
    forward_pyramid(P0.as<double>(), P1.as<double>(), C.as<double>(), rows, n_dy, nullptr, stream);
    return rows;
  };
  for (int64_t p0 = 0; p0 < n_obs; p0 += pb) {
    const int64_t np = std::min(pb, n_obs - p0);
    const int64_t rows = transform_batch(p0, np);
    count_rows_kernel<<<(unsigned)rows, WV_THREADS, 0, stream>>>(C.as<double>(), n_dy, rel, np, p0,
                                                                n_obs, cnt.as<int64_t>());
    GRADA_LAUNCH_CHECK();
  }
  std::vector<int64_t> counts((size_t)nd), rowptr((size_t)nd + 1, 0);
  download(counts.data(), cnt.ptr, sizeof(int64_t) * (size_t)nd);
  sync();
  for (int64_t r = 0; r < nd; r++) rowptr[(size_t)r + 1] = rowptr[(size_t)r] + counts[(size_t)r];
  const int64_t nnz = rowptr[(size_t)nd];
  wv_rowptr.alloc(this, sizeof(int64_t) * ((size_t)nd + 1));
  wv_col.alloc(this, sizeof(int) * (size_t)std::max<int64_t>(nnz, 1));
  wv_val.alloc(this, (f32 ? sizeof(float) : sizeof(double)) * (size_t)std::max<int64_t>(nnz, 1));
  upload(wv_rowptr.ptr, rowptr.data(), sizeof(int64_t) * ((size_t)nd + 1));
  for (int64_t p0 = 0; p0 < n_obs; p0 += pb) {
    const int64_t np = std::min(pb, n_obs - p0);
    const int64_t rows = transform_batch(p0, np);
    if (f32)
      fill_rows_kernel<float><<<(unsigned)rows, WV_THREADS, 0, stream>>>(
          C.as<double>(), n_dy, rel, np, p0, n_obs, wv_rowptr.as<int64_t>(), wv_col.as<int>(),
          wv_val.as<float>());
    else
      fill_rows_kernel<double><<<(unsigned)rows, WV_THREADS, 0, stream>>>(
          C.as<double>(), n_dy, rel, np, p0, n_obs, wv_rowptr.as<int64_t>(), wv_col.as<int>(),
          wv_val.as<double>());
    GRADA_LAUNCH_CHECK();
  }
  sync();
  Gb.release();
  P0.release();
  P1.release();
  C.release();
  // G^T y's row blocks, their partial vectors and the rows' column segments
  wv_rows_per_block = std::max<int64_t>(1, ceil_div(nd, kGtBlocks));
  wv_blocks = ceil_div(nd, wv_rows_per_block);
  wv_part.alloc(this, sizeof(double) * (size_t)(wv_blocks * n_dy));
  wv_seg_len = std::min<int64_t>(kGtSegment, n_dy);
  wv_nseg = n_dy / wv_seg_len;
  wv_segptr.alloc(this, sizeof(int64_t) * (size_t)(nd * (wv_nseg + 1)));
  segment_starts_kernel<<<grid_for(nd * (wv_nseg + 1)), WV_THREADS, 0, stream>>>(
      wv_rowptr.as<int64_t>(), wv_col.as<int>(), nd, wv_nseg, wv_seg_len,
      wv_segptr.as<int64_t>());
  GRADA_LAUNCH_CHECK();
  sync();
  wv_ndy = n_dy;
  wv_nnz = nnz;
  wv_fp32 = f32;
  g_storage = GRADA_G_WAVELET;
}

void Context::apply_G_wavelet(const double *x, double *y, const GemvOpts &o) {
  double *sc = scratch.as<double>();
  double *P0 = sc, *P1 = sc + wv_ndy, *W = sc + 2 * wv_ndy;
  load_vec_kernel<<<grid_for(wv_ndy), WV_THREADS, 0, stream>>>(x, wv_order.as<int>(), n_cells,
                                                               wv_ndy, P0, o.skip);
  GRADA_LAUNCH_CHECK();
  forward_pyramid(P0, P1, W, 1, wv_ndy, o.skip, stream);
  if (wv_fp32)
    row_dot_kernel<float><<<grid_for(nd * 32), WV_THREADS, 0, stream>>>(
        wv_rowptr.as<int64_t>(), wv_col.as<int>(), wv_val.as<float>(), W, nd, o.scale, y, o.skip);
  else
    row_dot_kernel<double><<<grid_for(nd * 32), WV_THREADS, 0, stream>>>(
        wv_rowptr.as<int64_t>(), wv_col.as<int>(), wv_val.as<double>(), W, nd, o.scale, y, o.skip);
  GRADA_LAUNCH_CHECK();
}

void Context::apply_GT_wavelet(const double *y, double *x, const GemvOpts &o) {
  double *sc = scratch.as<double>();
  double *W = sc + 2 * wv_ndy;
  double *bufs[2] = {sc, sc + wv_ndy};
  const dim3 grid((unsigned)wv_blocks, (unsigned)wv_nseg);
  const size_t smem = sizeof(double) * (size_t)wv_seg_len;
  if (wv_fp32)
    gt_partial_kernel<float><<<grid, WV_THREADS, smem, stream>>>(
        wv_segptr.as<int64_t>(), wv_col.as<int>(), wv_val.as<float>(), y, o.scale, nd,
        wv_rows_per_block, wv_nseg, wv_seg_len, wv_ndy, wv_part.as<double>(), o.skip);
  else
    gt_partial_kernel<double><<<grid, WV_THREADS, smem, stream>>>(
        wv_segptr.as<int64_t>(), wv_col.as<int>(), wv_val.as<double>(), y, o.scale, nd,
        wv_rows_per_block, wv_nseg, wv_seg_len, wv_ndy, wv_part.as<double>(), o.skip);
  GRADA_LAUNCH_CHECK();
  gt_reduce_kernel<<<grid_for(wv_ndy), WV_THREADS, 0, stream>>>(wv_part.as<double>(), wv_blocks,
                                                                wv_ndy, W, o.skip);
  GRADA_LAUNCH_CHECK();
  const double *a = W;  // the level-2 approximation is coef[0]
  int flip = 0;
  for (int64_t n = 2; n <= wv_ndy; n <<= 1) {
    double *out = bufs[flip];
    inverse_level_kernel<<<grid_for(n), WV_THREADS, 0, stream>>>(a, W, out, n, o.skip);
    GRADA_LAUNCH_CHECK();
    a = out;
    flip ^= 1;
  }
  store_vec_kernel<<<grid_for(n_cells), WV_THREADS, 0, stream>>>(a, wv_order.as<int>(), n_cells, x,
                                                                 o.skip);
  GRADA_LAUNCH_CHECK();
}

void Context::get_wavelet_G(int64_t *n_dy, int64_t *nnz, int64_t *rowptr, int *col, double *val) {
  if (g_storage != GRADA_G_WAVELET) throw Error(GRADA_ERR_STATE, "G is not wavelet-compressed");
  if (n_dy) *n_dy = wv_ndy;
  if (nnz) *nnz = wv_nnz;
  if (rowptr) download(rowptr, wv_rowptr.ptr, sizeof(int64_t) * ((size_t)nd + 1));
  if (col) download(col, wv_col.ptr, sizeof(int) * (size_t)wv_nnz);
  if (val && wv_fp32) {
    std::vector<float> tmp((size_t)wv_nnz);
    download(tmp.data(), wv_val.ptr, sizeof(float) * (size_t)wv_nnz);
    sync();
    for (int64_t k = 0; k < wv_nnz; k++) val[k] = (double)tmp[(size_t)k];
  } else if (val) {
    download(val, wv_val.ptr, sizeof(double) * (size_t)wv_nnz);
  }
  sync();
}

}  // namespace grada
