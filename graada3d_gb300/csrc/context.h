// Host-side state of one library context: the device copies of the reference
// Fwd object's data (mesh leaf cells, observation points, field flag, dense G)
// plus the inversion operators and work vectors.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "kernels.h"

namespace grada {

struct Context;

// Owning device allocation, accounted against its context.
struct DevBuf {
  void *ptr = nullptr;
  size_t bytes = 0;
  Context *owner = nullptr;
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  ~DevBuf();
  void alloc(Context *ctx, size_t nbytes);  // keeps the buffer if already large enough
  void release();
  template <typename T>
  T *as() const {
    return static_cast<T *>(ptr);
  }
};

struct Context {
  int device = 0;
  int sm_count = 0;
  cudaStream_t stream = nullptr;
  std::string last_error;
  int64_t bytes_held = 0;

  // Geometry (Fwd::mesh leaf cells, Fwd::ob, Fwd::field_flag).
  DevBuf prisms, obs;
  int64_t n_cells = 0, n_obs = 0, nd = 0, ld = 0;
  uint32_t mask = 0;
  int n_fields = 0;

  // Dense sensitivity matrix (Fwd::G), column-major, leading dimension ld.
  int g_storage = -1;
  DevBuf G, row_scale;

  // Work space.
  DevBuf scratch, vx, vy;

  void release_all() {
    prisms.release();
    obs.release();
    G.release();
    row_scale.release();
    scratch.release();
    vx.release();
    vy.release();
  }

  void upload(void *dst, const void *src, size_t nbytes);
  void download(void *dst, const void *src, size_t nbytes);
  void sync();
  DevGeometry geometry() const;
  DevG devG() const;
  double *scratch_doubles(int64_t n);
  void require_G() const;
  void require_geometry() const;

  void set_geometry(const double *h_prisms, int64_t nc, const double *h_obs, int64_t no,
                    uint32_t fmask);
  void compute_G(int storage);
  void G_vec_mul_dev(const double *d_x, double *d_y);
  void GT_vec_mul_dev(const double *d_y, double *d_x);
  void forward_field_dev(const double *d_rho, double *d_fields);
};

}  // namespace grada
