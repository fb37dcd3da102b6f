// AdaptiveInversion::expand_G on the device.
//
// Reference: src/Inversion/AdaptiveInversion.cpp:23-106.  After the host's
// Mesh::refinement has split some leaf cells into 8 children (created in
// x-outer, y, z-inner order at the cell centre, Mesh.cpp:1579-1600, and put in
// the parent's place in the leaf list, :1934-1941), G gains 7 columns per
// split: the parent's column is replaced, in place, by the 8 children's
// columns, and every other column keeps its relative order.
//
// Here the old columns move as contiguous runs (one device-to-device copy per
// run between two parents) and the children's columns are evaluated by the
// assembly kernel writing straight into their new positions.  The cell list of
// the context is updated the same way, so later products and assemblies see
// the refined mesh.
#include <algorithm>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "context.h"

namespace grada {

void Context::expand_G(int64_t n_split, const int64_t *parent, const double *children) {
  require_G();
  const bool matrix_free = g_storage == GRADA_G_MATRIX_FREE;
  if (!matrix_free && g_storage != GRADA_G_FP64 && g_storage != GRADA_G_FP32)
    throw Error(GRADA_ERR_INVALID_ARGUMENT,
                "expand_G needs G stored in FP64 or FP32 (re-assemble 16-bit storage instead)");
  if (n_split < 0) throw Error(GRADA_ERR_INVALID_ARGUMENT, "negative split count");
  if (n_split == 0) return;
  if (!parent) throw Error(GRADA_ERR_INVALID_ARGUMENT, "null parent index array");
  for (int64_t k = 0; k < n_split; k++) {
    if (parent[k] < 0 || parent[k] >= n_cells)
      throw Error(GRADA_ERR_INVALID_ARGUMENT, "parent index out of range");
    if (k > 0 && parent[k] <= parent[k - 1])
      throw Error(GRADA_ERR_INVALID_ARGUMENT, "parent indices must be strictly ascending");
  }
  const int64_t nm_old = n_cells, nm_new = n_cells + 7 * n_split;
  // children: given, or split at the centre like Mesh::refinement
  std::vector<double> kids((size_t)n_split * 48);
  for (int64_t k = 0; k < n_split; k++) {
    double *out = kids.data() + 48 * k;
    if (children) {
      std::memcpy(out, children + 48 * k, sizeof(double) * 48);
    } else {
      const double *p = host_prisms.data() + 6 * parent[k];
      const double xs[3] = {p[0], 0.5 * (p[1] + p[0]), p[1]};
      const double ys[3] = {p[2], 0.5 * (p[3] + p[2]), p[3]};
      const double zs[3] = {p[4], 0.5 * (p[5] + p[4]), p[5]};
      int id = 0;
      for (int i = 0; i < 2; i++)
        for (int j = 0; j < 2; j++)
          for (int l = 0; l < 2; l++, id++) {
            double *c = out + 6 * id;
            c[0] = xs[i]; c[1] = xs[i + 1];
            c[2] = ys[j]; c[3] = ys[j + 1];
            c[4] = zs[l]; c[5] = zs[l + 1];
          }
    }
    for (int c = 0; c < 8; c++) {
      const double *q = out + 6 * c;
      for (int t = 0; t < 6; t++)
        if (!std::isfinite(q[t])) throw Error(GRADA_ERR_NONFINITE, "non-finite child coordinate");
      if (!(q[0] < q[1] && q[2] < q[3] && q[4] < q[5]))
        throw Error(GRADA_ERR_INVALID_ARGUMENT, "child prism is not (x0<x1, y0<y1, z0<z1)");
    }
  }
  // new cell list and the new column of every child
  std::vector<double> new_prisms((size_t)nm_new * 6);
  std::vector<int64_t> child_col((size_t)n_split * 8);
  struct Run {
    int64_t src, dst, n;
  };
  std::vector<Run> runs;
  int64_t src = 0, dst = 0;
  for (int64_t k = 0; k <= n_split; k++) {
    const int64_t end = (k < n_split) ? parent[k] : nm_old;
    if (end > src) {
      runs.push_back({src, dst, end - src});
      std::memcpy(new_prisms.data() + 6 * dst, host_prisms.data() + 6 * src,
                  sizeof(double) * 6 * (end - src));
      dst += end - src;
    }
    if (k < n_split) {
      std::memcpy(new_prisms.data() + 6 * dst, kids.data() + 48 * k, sizeof(double) * 48);
      for (int c = 0; c < 8; c++) child_col[8 * k + c] = dst + c;
      dst += 8;
      src = parent[k] + 1;
    }
  }
  if (matrix_free) {  // no matrix to splice: only the cell list changes
    n_cells = nm_new;
    host_prisms.swap(new_prisms);
    plan_valid = false;
    tile_plan();
    prisms.alloc(this, sizeof(double) * 6 * nm_new);
    upload(prisms.ptr, host_prisms.data(), sizeof(double) * 6 * nm_new);
    sync();
    for (auto &o : ops) o.set = false;
    for (auto &o : crg) o.set = false;
    return;
  }
  const size_t esz = (g_storage == GRADA_G_FP64) ? sizeof(double) : sizeof(float);
  DevBuf newG;
  newG.alloc(this, esz * (size_t)ld * (size_t)nm_new);
  for (const Run &r : runs)
    GRADA_CUDA_CHECK(cudaMemcpyAsync(static_cast<char *>(newG.ptr) + esz * ld * r.dst,
                                     static_cast<char *>(G.ptr) + esz * ld * r.src,
                                     esz * ld * r.n, cudaMemcpyDeviceToDevice, stream));
  DevBuf d_kids, d_cols;
  d_kids.alloc(this, sizeof(double) * kids.size());
  d_cols.alloc(this, sizeof(int64_t) * child_col.size());
  upload(d_kids.ptr, kids.data(), sizeof(double) * kids.size());
  upload(d_cols.ptr, child_col.data(), sizeof(int64_t) * child_col.size());
  if (ld > nd) {  // zero the padding rows of the children's columns
    for (int64_t k = 0; k < n_split; k++)
      GRADA_CUDA_CHECK(cudaMemsetAsync(static_cast<char *>(newG.ptr) + esz * ld * child_col[8 * k],
                                       0, esz * ld * 8, stream));
  }
  const DevGeometry g = geometry();
  if (g_storage == GRADA_G_FP64)
    launch_assemble_fp64(g, d_kids.as<double>(), 8 * n_split, d_cols.as<int64_t>(), 0,
                         newG.as<double>(), ld, stream);
  else
    launch_assemble_fp32(g, d_kids.as<double>(), 8 * n_split, d_cols.as<int64_t>(), 0,
                         newG.as<float>(), ld, stream);
  sync();
  // swap in the new matrix and cell list; a kept FP64 G no longer matches
  g64_valid = false;
  G64.release();
  std::swap(G.ptr, newG.ptr);
  std::swap(G.bytes, newG.bytes);
  n_cells = nm_new;
  host_prisms.swap(new_prisms);
  plan_valid = false;
  prisms.alloc(this, sizeof(double) * 6 * nm_new);
  upload(prisms.ptr, host_prisms.data(), sizeof(double) * 6 * nm_new);
  sync();
  tile_plan();
  // the regularisation operators are Nm x Nm: the host rebuilds them after a refinement
  for (auto &o : ops) o.set = false;
  for (auto &o : crg) o.set = false;
}

}  // namespace grada
