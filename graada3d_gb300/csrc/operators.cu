// Regularisation operators built on the device after a refinement
// (InversionBase::init_matrices, InversionBase.cpp:146-187):
//   V_ii = sqrt(cell volume)                      set_Vmatrix, :452-466
//   Z_ii = 1 / |zp - zc_i|^(beta/2), zp the mean observation height (flag 0),
//          sqrt(||G(:, i)|| / Nd) (flag 1)         set_depth_weighting, :497-529
//   D_x1, D_y1, D_z1 from the face table            set_difference_matrix, :189-434
//   W_* = a_* S_* V D_* Z, S_* = I                  GaussNewtonInversion.cpp:711-714
// and their transposes, straight into the context's operator slots.
//
// The face table gives, per cell and axis, the cells across the face the
// reference differences against: [side, c0, c1, c2, c3], side +1 for the
// +axis face (-w on the diagonal, +w to the neighbour), -1 for the -axis face
// when the +axis face is on the boundary (signs swapped), 0 for no row; one
// neighbour (c1..c3 = -1, same or coarser level) or four finer neighbours,
// each taking a quarter of the off-diagonal weight.  w = 1 / (0.5 (h0 + h1))
// with h the cells' sizes along the axis, h1 that of c0.
//
// Every value is computed with the reference's operations in its order
// (products and sums as explicit round-to-nearest intrinsics, so that nothing
// is contracted into a fused multiply-add); only Z's power may differ from the
// host C library's in the last bits.
#include <cmath>
#include <vector>

#include <cub/device/device_scan.cuh>

#include "common.cuh"
#include "context.h"
#include "kernels.h"

namespace grada {
namespace {

constexpr int OB_THREADS = 256;

// zp = (z_0 + z_1 + ... ) / N_obs, summed in order (InversionBase.cpp:505-510).
__global__ void mean_height_kernel(const double *__restrict__ obs, int64_t n_obs,
                                   double *__restrict__ zp) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  double s = 0.0;
  for (int64_t i = 0; i < n_obs; i++) s = __dadd_rn(s, obs[3 * i + 2]);
  *zp = s / (double)n_obs;
}

__global__ void cell_weights_kernel(const double *__restrict__ prisms, int64_t n,
                                    const double *__restrict__ zp, double half_beta,
                                    const double *__restrict__ norms, double nd, int flag,
                                    double *__restrict__ V, double *__restrict__ Z) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double *c = prisms + 6 * i;
  const double dx = fabs(__dsub_rn(c[1], c[0]));
  const double dy = fabs(__dsub_rn(c[3], c[2]));
  const double dz = fabs(__dsub_rn(c[5], c[4]));
  V[i] = sqrt(__dmul_rn(__dmul_rn(dx, dy), dz));  // RectPrism::get_volumn, RectPrism.h:22-27
  if (flag == 0) {
    const double zc = __dmul_rn(0.5, __dadd_rn(c[4], c[5]));
    Z[i] = 1.0 / pow(fabs(__dsub_rn(*zp, zc)), half_beta);
  } else {
    Z[i] = sqrt(norms[i] / nd);
  }
}

__device__ __forceinline__ double axis_size(const double *__restrict__ prisms, int64_t c, int a) {
  return fabs(__dsub_rn(prisms[6 * c + 2 * a + 1], prisms[6 * c + 2 * a]));
}

// One row of W_axis (axis 0..2) or of W_s (axis < 0), columns ascending.
__global__ void fill_rows_kernel(const int *__restrict__ faces, int axis,
                                 const double *__restrict__ prisms, const double *__restrict__ V,
                                 const double *__restrict__ Z, double a,
                                 const int *__restrict__ rowptr, int *__restrict__ col,
                                 double *__restrict__ val, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double aV = __dmul_rn(a, V[i]);
  const int base = rowptr[i];
  if (axis < 0) {  // D_s = I
    col[base] = (int)i;
    val[base] = __dmul_rn(__dmul_rn(aV, 1.0), Z[i]);
    return;
  }
  const int *f = faces + 15 * i + 5 * axis;
  const int side = f[0];
  if (side == 0) return;
  const double w = 1.0 / __dmul_rn(0.5, __dadd_rn(axis_size(prisms, i, axis),
                                                  axis_size(prisms, f[1], axis)));
  int cols[5];
  double d[5];
  int k = 0;
  cols[k] = (int)i;
  d[k++] = side > 0 ? -w : w;
  const double off = side > 0 ? w : -w;
  if (f[2] < 0) {
    cols[k] = f[1];
    d[k++] = off;
  } else {
    for (int q = 0; q < 4; q++) {
      cols[k] = f[1 + q];
      d[k++] = __dmul_rn(off, 0.25);
    }
  }
  for (int s = 1; s < k; s++) {  // insertion sort by column
    const int cc = cols[s];
    const double dd = d[s];
    int t = s - 1;
    while (t >= 0 && cols[t] > cc) {
      cols[t + 1] = cols[t];
      d[t + 1] = d[t];
      t--;
    }
    cols[t + 1] = cc;
    d[t + 1] = dd;
  }
  for (int s = 0; s < k; s++) {
    col[base + s] = cols[s];
    val[base + s] = __dmul_rn(__dmul_rn(aV, d[s]), Z[cols[s]]);
  }
}

__global__ void column_count_kernel(const int *__restrict__ rowptr, const int *__restrict__ col,
                                    int64_t n, int *__restrict__ count) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  for (int k = rowptr[r]; k < rowptr[r + 1]; k++) atomicAdd(count + col[k], 1);
}

__global__ void scatter_kernel(const int *__restrict__ rowptr, const int *__restrict__ col,
                               const double *__restrict__ val, int64_t n,
                               const int *__restrict__ t_rowptr, int *__restrict__ cursor,
                               int *__restrict__ t_col, double *__restrict__ t_val) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  for (int k = rowptr[r]; k < rowptr[r + 1]; k++) {
    const int c = col[k];
    const int p = t_rowptr[c] + atomicAdd(cursor + c, 1);
    t_col[p] = (int)r;
    t_val[p] = val[k];
  }
}

// The scatter's order within a row depends on the atomics; sorting each row
// by column gives the host transpose's layout (rows ascending).
__global__ void sort_rows_kernel(const int *__restrict__ rowptr, int *__restrict__ col,
                                 double *__restrict__ val, int64_t n) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const int b = rowptr[r], e = rowptr[r + 1];
  for (int s = b + 1; s < e; s++) {
    const int cc = col[s];
    const double vv = val[s];
    int t = s - 1;
    while (t >= b && col[t] > cc) {
      col[t + 1] = col[t];
      val[t + 1] = val[t];
      t--;
    }
    col[t + 1] = cc;
    val[t + 1] = vv;
  }
}

unsigned grid_for(int64_t n) { return (unsigned)std::max<int64_t>(1, ceil_div(n, OB_THREADS)); }

}  // namespace

void Context::build_operators(const int *h_faces, double beta, int depth_flag,
                              const double *alphas) {
  require_geometry();
  if (!h_faces || !alphas) throw Error(GRADA_ERR_INVALID_ARGUMENT, "null face table or weights");
  if (depth_flag != 0 && depth_flag != 1)
    throw Error(GRADA_ERR_INVALID_ARGUMENT, "depth weighting flag must be 0 or 1");
  if (depth_flag == 1) {
    require_G();
    if (g_storage == GRADA_G_MATRIX_FREE)
      throw Error(GRADA_ERR_STATE, "depth weighting from G needs a stored G (not matrix-free)");
  }
  for (int k = 0; k < 4; k++)
    if (!std::isfinite(alphas[k])) throw Error(GRADA_ERR_NONFINITE, "non-finite weight");
  if (!std::isfinite(beta)) throw Error(GRADA_ERR_NONFINITE, "non-finite beta");
  const int64_t n = n_cells;
  if (n >= (int64_t)1 << 31) throw Error(GRADA_ERR_INVALID_ARGUMENT, "too many cells for int32 indices");
  // Check the table and lay out the rows on the host: every index the kernels
  // follow is in range before anything is launched.
  std::vector<int> rp[3];
  for (int a = 0; a < 3; a++) {
    rp[a].resize((size_t)n + 1);
    rp[a][0] = 0;
  }
  for (int64_t i = 0; i < n; i++) {
    for (int a = 0; a < 3; a++) {
      const int *f = h_faces + 15 * i + 5 * a;
      int cnt = 0;
      if (f[0] != 0) {
        if (f[0] != 1 && f[0] != -1)
          throw Error(GRADA_ERR_INVALID_ARGUMENT, "face side must be -1, 0 or 1");
        if (f[1] < 0 || f[1] >= n || f[1] == i)
          throw Error(GRADA_ERR_INVALID_ARGUMENT,
                      "face neighbour out of range at cell " + std::to_string(i));
        if (f[2] < 0) {
          if (f[3] >= 0 || f[4] >= 0)
            throw Error(GRADA_ERR_INVALID_ARGUMENT, "one face neighbour or four expected");
          cnt = 2;
        } else {
          for (int q = 1; q < 4; q++)
            if (f[1 + q] < 0 || f[1 + q] >= n || f[1 + q] == i)
              throw Error(GRADA_ERR_INVALID_ARGUMENT,
                          "face neighbour out of range at cell " + std::to_string(i));
          for (int p = 0; p < 4; p++)
            for (int q = p + 1; q < 4; q++)
              if (f[1 + p] == f[1 + q])
                throw Error(GRADA_ERR_INVALID_ARGUMENT, "repeated face neighbour");
          cnt = 5;
        }
      }
      rp[a][(size_t)i + 1] = rp[a][(size_t)i] + cnt;
    }
  }

  DevBuf faces, cellV, cellZ, scal, norms, count, cursor, scan_tmp;
  faces.alloc(this, sizeof(int) * 15 * (size_t)n);
  cellV.alloc(this, sizeof(double) * (size_t)n);
  cellZ.alloc(this, sizeof(double) * (size_t)n);
  scal.alloc(this, sizeof(double));
  upload(faces.ptr, h_faces, sizeof(int) * 15 * (size_t)n);
  if (depth_flag == 0) {
    mean_height_kernel<<<1, 32, 0, stream>>>(obs.as<double>(), n_obs, scal.as<double>());
    GRADA_LAUNCH_CHECK();
  } else {
    norms.alloc(this, sizeof(double) * (size_t)n);
    launch_column_norms(devG(), norms.as<double>(), stream);
  }
  cell_weights_kernel<<<grid_for(n), OB_THREADS, 0, stream>>>(
      prisms.as<double>(), n, scal.as<double>(), 0.5 * beta,
      depth_flag == 1 ? norms.as<double>() : nullptr, (double)nd, depth_flag, cellV.as<double>(),
      cellZ.as<double>());
  GRADA_LAUNCH_CHECK();

  count.alloc(this, sizeof(int) * ((size_t)n + 1));
  cursor.alloc(this, sizeof(int) * (size_t)n);
  size_t scan_bytes = 0;
  GRADA_CUDA_CHECK(cub::DeviceScan::ExclusiveSum(nullptr, scan_bytes, count.as<int>(),
                                                 count.as<int>(), (int)(n + 1), stream));
  scan_tmp.alloc(this, std::max<size_t>(scan_bytes, 16));

  const int slots[4] = {GRADA_OP_WS, GRADA_OP_WX, GRADA_OP_WY, GRADA_OP_WZ};
  // alphas = (a_s, a_z, a_x, a_y), the order of set_weights_of_objectives
  const double a_of[4] = {alphas[0], alphas[2], alphas[3], alphas[1]};
  for (int s = 0; s < 4; s++) {
    DevOperator &op = ops[slots[s]];
    op.set = false;
    const int axis = s - 1;  // -1: Ws, 0: Wx, 1: Wy, 2: Wz
    std::vector<int> ident;
    const std::vector<int> *rows = nullptr;
    if (axis < 0) {
      ident.resize((size_t)n + 1);
      for (int64_t i = 0; i <= n; i++) ident[(size_t)i] = (int)i;
      rows = &ident;
    } else {
      rows = &rp[axis];
    }
    const int64_t nnz = (*rows)[(size_t)n];
    op.rowptr.alloc(this, sizeof(int) * ((size_t)n + 1));
    op.col.alloc(this, sizeof(int) * (size_t)std::max<int64_t>(nnz, 1));
    op.val.alloc(this, sizeof(double) * (size_t)std::max<int64_t>(nnz, 1));
    op.t_rowptr.alloc(this, sizeof(int) * ((size_t)n + 1));
    op.t_col.alloc(this, sizeof(int) * (size_t)std::max<int64_t>(nnz, 1));
    op.t_val.alloc(this, sizeof(double) * (size_t)std::max<int64_t>(nnz, 1));
    upload(op.rowptr.ptr, rows->data(), sizeof(int) * ((size_t)n + 1));
    fill_rows_kernel<<<grid_for(n), OB_THREADS, 0, stream>>>(
        faces.as<int>(), axis, prisms.as<double>(), cellV.as<double>(), cellZ.as<double>(),
        a_of[s], op.rowptr.as<int>(), op.col.as<int>(), op.val.as<double>(), n);
    GRADA_LAUNCH_CHECK();
    // transpose: column counts, their exclusive sum, scatter, rows sorted
    GRADA_CUDA_CHECK(cudaMemsetAsync(count.ptr, 0, sizeof(int) * ((size_t)n + 1), stream));
    GRADA_CUDA_CHECK(cudaMemsetAsync(cursor.ptr, 0, sizeof(int) * (size_t)n, stream));
    column_count_kernel<<<grid_for(n), OB_THREADS, 0, stream>>>(op.rowptr.as<int>(),
                                                               op.col.as<int>(), n, count.as<int>());
    GRADA_LAUNCH_CHECK();
    size_t bytes = scan_tmp.bytes;
    GRADA_CUDA_CHECK(cub::DeviceScan::ExclusiveSum(scan_tmp.ptr, bytes, count.as<int>(),
                                                   op.t_rowptr.as<int>(), (int)(n + 1), stream));
    scatter_kernel<<<grid_for(n), OB_THREADS, 0, stream>>>(
        op.rowptr.as<int>(), op.col.as<int>(), op.val.as<double>(), n, op.t_rowptr.as<int>(),
        cursor.as<int>(), op.t_col.as<int>(), op.t_val.as<double>());
    GRADA_LAUNCH_CHECK();
    sort_rows_kernel<<<grid_for(n), OB_THREADS, 0, stream>>>(op.t_rowptr.as<int>(),
                                                            op.t_col.as<int>(),
                                                            op.t_val.as<double>(), n);
    GRADA_LAUNCH_CHECK();
    op.n = n;
    op.nnz = nnz;
  }
  sync();  // the host row layouts and scratch buffers go out of scope
  for (int s = 0; s < 4; s++) ops[slots[s]].set = true;
}

void Context::get_operator(int which, int64_t *nnz, int *rowptr, int *col, double *val) {
  if (which < GRADA_OP_WS || which > GRADA_OP_TZ)
    throw Error(GRADA_ERR_INVALID_ARGUMENT, "unknown operator slot");
  const DevOperator &op = ops[which];
  if (!op.set) throw Error(GRADA_ERR_STATE, "operator not set");
  if (nnz) *nnz = op.nnz;
  if (rowptr) download(rowptr, op.rowptr.ptr, sizeof(int) * ((size_t)op.n + 1));
  if (col) download(col, op.col.ptr, sizeof(int) * (size_t)op.nnz);
  if (val) download(val, op.val.ptr, sizeof(double) * (size_t)op.nnz);
  sync();
}

}  // namespace grada
