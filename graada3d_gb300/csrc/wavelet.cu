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
//   G x:   x reordered and padded, transformed; each row's kept coefficients
//          dotted with it in stored order.
//   G^T y: the kept coefficients gathered per coefficient index over the rows
//          in ascending order (a stable sort by index gives that layout), the
//          inverse pyramid (levels 2, 4, ..., n_dy), the result put back in
//          cell order.
// Every sum runs in the reference's order from zero, as explicit
// round-to-nearest operations.  The compression assembles the FP64 G first
// (it must fit on the device) and releases it afterwards.
#include <algorithm>
#include <cmath>
#include <vector>

#include <cub/device/device_radix_sort.cuh>

#include "common.cuh"
#include "context.h"
#include "kernels.h"

namespace grada {
namespace {

constexpr int WV_THREADS = 256;

// (1 + sqrt 3, 3 + sqrt 3, 3 - sqrt 3, 1 - sqrt 3) / (4 sqrt 2), correctly rounded
__constant__ double kH[4] = {0.48296291314453416, 0.8365163037378079, 0.2241438680420134,
                             -0.12940952255126037};
__constant__ double kG[4] = {-0.12940952255126037, -0.2241438680420134, 0.8365163037378079,
                             -0.48296291314453416};

unsigned grid_for(int64_t n) { return (unsigned)std::max<int64_t>(1, ceil_div(n, WV_THREADS)); }

// P[j * B + r] = G(rows r0 + r, cell order[j]) for j < nm, zero beyond (and for
// rows past nd).
__global__ void load_rows_kernel(const double *__restrict__ G, int64_t ld, int64_t nd, int64_t r0,
                                 int64_t B, const int *__restrict__ order, int64_t nm,
                                 int64_t n_dy, double *__restrict__ P) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= B * n_dy) return;
  const int64_t r = t % B, j = t / B;
  double v = 0.0;
  if (j < nm && r0 + r < nd) v = G[(int64_t)order[j] * ld + r0 + r];
  P[t] = v;
}

// One forward level of length n on B interleaved vectors: approximations to
// approx[ii * B + r], details to coef[(nh + ii) * B + r] (at n = 2 approx is
// coef itself: the two writes never meet).
__global__ void forward_level_kernel(const double *__restrict__ src, double *approx, double *coef,
                                     int64_t B, int64_t n,
                                     const int *__restrict__ skip) {
  if (skip && *skip) return;
  const int64_t nh = n >> 1;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= B * nh) return;
  const int64_t r = t % B, ii = t / B;
  double h = 0.0, g = 0.0;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const double a = src[((2 * ii + k) & (n - 1)) * B + r];
    h = __dadd_rn(h, __dmul_rn(kH[k], a));
    g = __dadd_rn(g, __dmul_rn(kG[k], a));
  }
  approx[ii * B + r] = h;
  coef[(nh + ii) * B + r] = g;
}

__device__ __forceinline__ bool kept(double c, double thr) {
  const double a = fabs(c);
  return a > thr || fabs(__dsub_rn(a, thr)) < 1e-15;
}

__device__ double row_threshold(const double *__restrict__ coef, int64_t B, int64_t r,
                                int64_t n_dy, double rel) {
  double mx = fabs(coef[r]);
  for (int64_t i = 1; i < n_dy; i++) mx = fmax(mx, fabs(coef[i * B + r]));
  return __dmul_rn(rel, mx);
}

__global__ void count_rows_kernel(const double *__restrict__ coef, int64_t B, int64_t rows,
                                  int64_t n_dy, double rel, int64_t *__restrict__ count) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows) return;
  const double thr = row_threshold(coef, B, r, n_dy, rel);
  int64_t c = 0;
  for (int64_t i = 0; i < n_dy; i++) c += kept(coef[i * B + r], thr) ? 1 : 0;
  count[r] = c;
}

__global__ void fill_rows_kernel(const double *__restrict__ coef, int64_t B, int64_t rows,
                                 int64_t n_dy, double rel, const int64_t *__restrict__ rowptr,
                                 int *__restrict__ col, double *__restrict__ val) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows) return;
  const double thr = row_threshold(coef, B, r, n_dy, rel);
  int64_t p = rowptr[r];
  for (int64_t i = 0; i < n_dy; i++) {
    const double c = coef[i * B + r];
    if (kept(c, thr)) {
      col[p] = (int)i;
      val[p] = c;
      p++;
    }
  }
}

__global__ void row_of_entry_kernel(const int64_t *__restrict__ rowptr, int64_t nd,
                                    int *__restrict__ row_of, int *__restrict__ seq) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nd) return;
  for (int64_t k = rowptr[r]; k < rowptr[r + 1]; k++) {
    row_of[k] = (int)r;
    seq[k] = (int)k;
  }
}

// t_rowptr[c] = first position of a key >= c in the sorted keys (c <= n_dy).
__global__ void column_starts_kernel(const int *__restrict__ keys, int64_t nnz, int64_t n_dy,
                                     int64_t *__restrict__ t_rowptr) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c > n_dy) return;
  int64_t lo = 0, hi = nnz;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (keys[mid] < c) lo = mid + 1;
    else hi = mid;
  }
  t_rowptr[c] = lo;
}

__global__ void gather_transpose_kernel(const int *__restrict__ perm, const int *__restrict__ row_of,
                                        const double *__restrict__ val, int64_t nnz,
                                        int *__restrict__ t_row, double *__restrict__ t_val) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nnz) return;
  const int e = perm[p];
  t_row[p] = row_of[e];
  t_val[p] = val[e];
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

__global__ void row_dot_kernel(const int64_t *__restrict__ rowptr, const int *__restrict__ col,
                               const double *__restrict__ val, const double *__restrict__ w,
                               int64_t nd, const double *__restrict__ scale,
                               double *__restrict__ y, const int *__restrict__ skip) {
  if (skip && *skip) return;
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nd) return;
  double s = 0.0;
  for (int64_t k = rowptr[r]; k < rowptr[r + 1]; k++) s = __dadd_rn(s, __dmul_rn(val[k], w[col[k]]));
  y[r] = scale ? __dmul_rn(s, scale[r]) : s;
}

__global__ void column_gather_kernel(const int64_t *__restrict__ t_rowptr,
                                     const int *__restrict__ t_row, const double *__restrict__ t_val,
                                     const double *__restrict__ y, const double *__restrict__ scale,
                                     int64_t n_dy, double *__restrict__ w,
                                     const int *__restrict__ skip) {
  if (skip && *skip) return;
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n_dy) return;
  double s = 0.0;
  for (int64_t p = t_rowptr[c]; p < t_rowptr[c + 1]; p++) {
    const int r = t_row[p];
    const double v = scale ? __dmul_rn(scale[r], y[r]) : y[r];
    s = __dadd_rn(s, __dmul_rn(t_val[p], v));
  }
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
  const int k0 = (int)(j & 1);                   // k of the contribution from ii = j >> 1
  const int64_t ia = j >> 1;
  const int64_t ib = (ia + nh - 1) % nh;        // k0 + 2
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

}  // namespace

void Context::compute_G_wavelet(const int64_t *h_order, double rel) {
  require_geometry();
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

  compute_G(GRADA_G_FP64);  // the rows to compress; released below
  g_storage = -1;
  wv_order.alloc(this, sizeof(int) * (size_t)nm);
  upload(wv_order.ptr, order.data(), sizeof(int) * (size_t)nm);

  // rows in batches: three n_dy x B buffers of at most ~6 GB together
  const int64_t budget = (int64_t)6 << 30;
  int64_t B = std::max<int64_t>(32, (budget / (3 * 8 * n_dy)) / 32 * 32);
  B = std::min(B, round_up(nd, 32));
  DevBuf P0, P1, C, cnt;
  P0.alloc(this, sizeof(double) * (size_t)(B * n_dy));
  P1.alloc(this, sizeof(double) * (size_t)(B * std::max<int64_t>(n_dy / 2, 1)));
  C.alloc(this, sizeof(double) * (size_t)(B * n_dy));
  cnt.alloc(this, sizeof(int64_t) * (size_t)B);
  const double *Gd = G.as<double>();
  auto transform_batch = [&](int64_t r0) {
    load_rows_kernel<<<grid_for(B * n_dy), WV_THREADS, 0, stream>>>(
        Gd, ld, nd, r0, B, wv_order.as<int>(), nm, n_dy, P0.as<double>());
    GRADA_LAUNCH_CHECK();
    double *src = P0.as<double>();
    double *bufs[2] = {P1.as<double>(), P0.as<double>()};
    int flip = 0;
    for (int64_t n = n_dy; n >= 2; n >>= 1) {
      double *dst = n == 2 ? C.as<double>() : bufs[flip];
      forward_level_kernel<<<grid_for(B * (n >> 1)), WV_THREADS, 0, stream>>>(
          src, dst, C.as<double>(), B, n, nullptr);
      GRADA_LAUNCH_CHECK();
      src = dst;
      flip ^= 1;
    }
  };
  // The level writing into P0 reads P1 and vice versa; P0 holds n_dy, P1 n_dy/2
  // entries per row, enough for every level after the first.
  std::vector<int64_t> rowptr((size_t)nd + 1, 0), part((size_t)B);
  for (int64_t r0 = 0; r0 < nd; r0 += B) {
    const int64_t rows = std::min(B, nd - r0);
    transform_batch(r0);
    count_rows_kernel<<<grid_for(rows), WV_THREADS, 0, stream>>>(C.as<double>(), B, rows, n_dy,
                                                                 rel, cnt.as<int64_t>());
    GRADA_LAUNCH_CHECK();
    download(part.data(), cnt.ptr, sizeof(int64_t) * (size_t)rows);
    sync();
    for (int64_t r = 0; r < rows; r++)
      rowptr[(size_t)(r0 + r + 1)] = rowptr[(size_t)(r0 + r)] + part[(size_t)r];
  }
  const int64_t nnz = rowptr[(size_t)nd];
  if (nnz >= ((int64_t)1 << 31) - 1)
    throw Error(GRADA_ERR_INVALID_ARGUMENT, "too many kept coefficients (raise the threshold)");
  wv_rowptr.alloc(this, sizeof(int64_t) * ((size_t)nd + 1));
  wv_col.alloc(this, sizeof(int) * (size_t)std::max<int64_t>(nnz, 1));
  wv_val.alloc(this, sizeof(double) * (size_t)std::max<int64_t>(nnz, 1));
  upload(wv_rowptr.ptr, rowptr.data(), sizeof(int64_t) * ((size_t)nd + 1));
  for (int64_t r0 = 0; r0 < nd; r0 += B) {
    const int64_t rows = std::min(B, nd - r0);
    transform_batch(r0);
    fill_rows_kernel<<<grid_for(rows), WV_THREADS, 0, stream>>>(
        C.as<double>(), B, rows, n_dy, rel, wv_rowptr.as<int64_t>() + r0, wv_col.as<int>(),
        wv_val.as<double>());
    GRADA_LAUNCH_CHECK();
  }
  sync();
  P0.release();
  P1.release();
  C.release();
  G.release();  // the reference drops the dense G too (Fwd.cpp:159)

  // coefficient-major copy: a stable sort of the entries by coefficient index
  DevBuf row_of, seq, keys_out, perm, sort_tmp;
  const int64_t m = std::max<int64_t>(nnz, 1);
  row_of.alloc(this, sizeof(int) * (size_t)m);
  seq.alloc(this, sizeof(int) * (size_t)m);
  keys_out.alloc(this, sizeof(int) * (size_t)m);
  perm.alloc(this, sizeof(int) * (size_t)m);
  row_of_entry_kernel<<<grid_for(nd), WV_THREADS, 0, stream>>>(wv_rowptr.as<int64_t>(), nd,
                                                               row_of.as<int>(), seq.as<int>());
  GRADA_LAUNCH_CHECK();
  int end_bit = 1;
  while (((int64_t)1 << end_bit) <= n_dy) end_bit++;
  size_t sort_bytes = 0;
  GRADA_CUDA_CHECK(cub::DeviceRadixSort::SortPairs(nullptr, sort_bytes, wv_col.as<int>(),
                                                   keys_out.as<int>(), seq.as<int>(), perm.as<int>(),
                                                   (int)nnz, 0, end_bit, stream));
  sort_tmp.alloc(this, std::max<size_t>(sort_bytes, 16));
  GRADA_CUDA_CHECK(cub::DeviceRadixSort::SortPairs(sort_tmp.ptr, sort_bytes, wv_col.as<int>(),
                                                   keys_out.as<int>(), seq.as<int>(), perm.as<int>(),
                                                   (int)nnz, 0, end_bit, stream));
  wv_trowptr.alloc(this, sizeof(int64_t) * ((size_t)n_dy + 1));
  wv_trow.alloc(this, sizeof(int) * (size_t)m);
  wv_tval.alloc(this, sizeof(double) * (size_t)m);
  column_starts_kernel<<<grid_for(n_dy + 1), WV_THREADS, 0, stream>>>(
      keys_out.as<int>(), nnz, n_dy, wv_trowptr.as<int64_t>());
  GRADA_LAUNCH_CHECK();
  gather_transpose_kernel<<<grid_for(nnz), WV_THREADS, 0, stream>>>(
      perm.as<int>(), row_of.as<int>(), wv_val.as<double>(), nnz, wv_trow.as<int>(),
      wv_tval.as<double>());
  GRADA_LAUNCH_CHECK();
  sync();
  wv_ndy = n_dy;
  wv_nnz = nnz;
  g_storage = GRADA_G_WAVELET;
}

void Context::apply_G_wavelet(const double *x, double *y, const GemvOpts &o) {
  double *sc = scratch.as<double>();
  double *P0 = sc, *P1 = sc + wv_ndy, *W = sc + 2 * wv_ndy;
  load_vec_kernel<<<grid_for(wv_ndy), WV_THREADS, 0, stream>>>(x, wv_order.as<int>(), n_cells,
                                                               wv_ndy, P0, o.skip);
  GRADA_LAUNCH_CHECK();
  double *src = P0;
  double *bufs[2] = {P1, P0};
  int flip = 0;
  for (int64_t n = wv_ndy; n >= 2; n >>= 1) {
    double *dst = n == 2 ? W : bufs[flip];
    forward_level_kernel<<<grid_for(n >> 1), WV_THREADS, 0, stream>>>(src, dst, W, 1, n, o.skip);
    GRADA_LAUNCH_CHECK();
    src = dst;
    flip ^= 1;
  }
  row_dot_kernel<<<grid_for(nd), WV_THREADS, 0, stream>>>(wv_rowptr.as<int64_t>(), wv_col.as<int>(),
                                                          wv_val.as<double>(), W, nd, o.scale, y,
                                                          o.skip);
  GRADA_LAUNCH_CHECK();
}

void Context::apply_GT_wavelet(const double *y, double *x, const GemvOpts &o) {
  double *sc = scratch.as<double>();
  double *W = sc + 2 * wv_ndy;
  double *bufs[2] = {sc, sc + wv_ndy};
  column_gather_kernel<<<grid_for(wv_ndy), WV_THREADS, 0, stream>>>(
      wv_trowptr.as<int64_t>(), wv_trow.as<int>(), wv_tval.as<double>(), y, o.scale, wv_ndy, W,
      o.skip);
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
  if (val) download(val, wv_val.ptr, sizeof(double) * (size_t)wv_nnz);
  sync();
}

}  // namespace grada
