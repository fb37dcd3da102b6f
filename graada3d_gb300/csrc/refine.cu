// Refinement indicator of the adaptive inversion on the device.
//
// Reference: AdaptiveInversion::indicator_calculator (src/Inversion/
// AdaptiveInversion.cpp:108-204): for every leaf cell, the sum over the cells
// across its faces of (m_neighbour - m_cell)^2 times a face area.  The
// neighbour structure lives in the host mesh (its faces and their children),
// so the host hands the device each cell's (neighbour, area) pairs in the
// order the reference adds them; one thread per cell then forms the sum with
// the same operations in the same order, rounded separately (no fused
// multiply-add), so the result is bitwise the reference's.
#include "../../include/grada_gpu.h"
#include "common.cuh"
#include "context.h"

namespace grada {

namespace {

__global__ void indicator_kernel(const double *__restrict__ m, const int64_t *__restrict__ rowptr,
                                 const int64_t *__restrict__ nb, const double *__restrict__ area,
                                 int64_t n, double *__restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double mc = m[i];
  double acc = 0.0;
  for (int64_t k = rowptr[i]; k < rowptr[i + 1]; k++) {
    const double d = __dsub_rn(m[nb[k]], mc);
    acc = __dadd_rn(acc, __dmul_rn(__dmul_rn(d, d), area[k]));
  }
  out[i] = acc;
}

}  // namespace

void Context::refinement_indicator(const double *h_m, const int64_t *h_rowptr,
                                   const int64_t *h_nb, const double *h_area, double *h_out) {
  require_geometry();
  if (!h_m || !h_rowptr || !h_out) throw Error(GRADA_ERR_INVALID_ARGUMENT, "null argument");
  const int64_t n = n_cells;
  if (h_rowptr[0] != 0) throw Error(GRADA_ERR_INVALID_ARGUMENT, "rowptr[0] must be 0");
  for (int64_t i = 0; i < n; i++)
    if (h_rowptr[i + 1] < h_rowptr[i]) throw Error(GRADA_ERR_INVALID_ARGUMENT, "rowptr not monotone");
  const int64_t nnz = h_rowptr[n];
  if (nnz > 0 && (!h_nb || !h_area)) throw Error(GRADA_ERR_INVALID_ARGUMENT, "null neighbour list");
  for (int64_t k = 0; k < nnz; k++)
    if (h_nb[k] < 0 || h_nb[k] >= n) throw Error(GRADA_ERR_INVALID_ARGUMENT, "neighbour out of range");
  DevBuf dm, drp, dnb, dar, dout;
  dm.alloc(this, sizeof(double) * n);
  drp.alloc(this, sizeof(int64_t) * (n + 1));
  dnb.alloc(this, sizeof(int64_t) * std::max<int64_t>(nnz, 1));
  dar.alloc(this, sizeof(double) * std::max<int64_t>(nnz, 1));
  dout.alloc(this, sizeof(double) * n);
  upload(dm.ptr, h_m, sizeof(double) * n);
  upload(drp.ptr, h_rowptr, sizeof(int64_t) * (n + 1));
  upload(dnb.ptr, h_nb, sizeof(int64_t) * nnz);
  upload(dar.ptr, h_area, sizeof(double) * nnz);
  indicator_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, stream>>>(
      dm.as<double>(), drp.as<int64_t>(), dnb.as<int64_t>(), dar.as<double>(), n,
      dout.as<double>());
  GRADA_LAUNCH_CHECK();
  download(h_out, dout.ptr, sizeof(double) * n);
  sync();
}

}  // namespace grada
