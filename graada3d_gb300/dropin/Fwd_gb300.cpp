// Drop-in bodies for the reference's Fwd class (src/Forward_modelling/Fwd.cpp:
// 47-219), against the unchanged Fwd.h.  A maintainer removes Fwd::compute_G,
// Fwd::GT_vec_mul, Fwd::G_vec_mul and Fwd::compute_G_wavelet from Fwd.cpp
// (keeping the constructors and the wavelet helpers there) and links this file,
// gb300_bridge.cpp and libgrada_gpu.so instead.  With the wavelet-compressed G
// the library keeps the compressed rows and both products use them, as the
// reference's G_vec_mul / GT_vec_mul do when use_wavelet is set.
//
// G is assembled and kept on the GPU.  Because the reference also reads the
// member G directly (InversionBase::get_predicted_field, set_depth_weighting
// with flag 1, AdaptiveInversion::expand_G), compute_G copies it back into the
// member unless GRADA_KEEP_G_ON_DEVICE is set, in which case those readers must
// go through G_vec_mul instead.
#include <cstdlib>
#include <vector>

#include "Fwd.h"
#include "gb300_bridge.h"

namespace {

// Fwd::compute_G's inputs in the library layout: cells (x0,x1,y0,y1,z0,z1) in
// leaf order, points (x,y,z), the field bitset as a mask.
void bind_geometry(grada_ctx *ctx, Mesh &mesh, const Observation &ob,
                   const std::bitset<10> &flag, int Nm, int N_obs) {
  std::vector<double> prisms(6 * (size_t)Nm), obs(3 * (size_t)N_obs);
  for (int j = 0; j < Nm; j++) {
    const RectPrism &r = mesh.get_elem(j);
    double *p = &prisms[6 * (size_t)j];
    p[0] = r._x[0]; p[1] = r._x[1];
    p[2] = r._y[0]; p[3] = r._y[1];
    p[4] = r._z[0]; p[5] = r._z[1];
  }
  for (int i = 0; i < N_obs; i++) {
    const Point &q = ob(i);
    obs[3 * (size_t)i] = q.x();
    obs[3 * (size_t)i + 1] = q.y();
    obs[3 * (size_t)i + 2] = q.z();
  }
  gb300::check(ctx, grada_set_geometry(ctx, prisms.data(), Nm, obs.data(), N_obs,
                                       (uint32_t)flag.to_ulong()),
               "grada_set_geometry");
}

}  // namespace

void Fwd::compute_G()
{
  assert(Nm > 0);
  assert(N_obs > 0);
  grada_ctx *ctx = gb300::context_for(this);
  bind_geometry(ctx, mesh, ob, field_flag, Nm, N_obs);
  gb300::check(ctx, grada_compute_G(ctx, GRADA_G_FP64), "grada_compute_G");
  if (!std::getenv("GRADA_KEEP_G_ON_DEVICE")) {
    const int n_fields = field_flag.count();
    G.resize(n_fields * N_obs, Nm);
    gb300::check(ctx, grada_get_G(ctx, G.data(), G.rows()), "grada_get_G");
  }
}

void Fwd::GT_vec_mul(const VectorXd &vec, VectorXd &product) const
{
  grada_ctx *ctx = gb300::context_for(this);
  product.resize(Nm);
  gb300::check(ctx, grada_GT_vec_mul(ctx, vec.data(), product.data()), "grada_GT_vec_mul");
}

void Fwd::G_vec_mul(const VectorXd &vec, VectorXd &product) const
{
  grada_ctx *ctx = gb300::context_for(this);
  product.resize(Nd);
  gb300::check(ctx, grada_G_vec_mul(ctx, vec.data(), product.data()), "grada_G_vec_mul");
}

// Fwd::compute_G_wavelet (Fwd.cpp:148-219): the rows along the mesh's
// reordered sequence, compressed on the device at compression_threshold; the
// member G is emptied as in the reference.
void Fwd::compute_G_wavelet()
{
  assert(Nm > 0);
  assert(N_obs > 0);
  grada_ctx *ctx = gb300::context_for(this);
  bind_geometry(ctx, mesh, ob, field_flag, Nm, N_obs);
  std::vector<int64_t> order((size_t)Nm);
  for (int j = 0; j < Nm; j++) order[(size_t)j] = mesh.get_reordered_id((unsigned)j);
  gb300::check(ctx, grada_compute_G_wavelet(ctx, order.data(), compression_threshold),
               "grada_compute_G_wavelet");
  int64_t n_dy = 0, nnz = 0;
  gb300::check(ctx, grada_get_wavelet_G(ctx, &n_dy, &nnz, nullptr, nullptr, nullptr),
               "grada_get_wavelet_G");
  n_dy_for_wavelet = (int)n_dy;
  comp_col_ids.clear();
  comp_G_coeffs.clear();
  G.resize(0, 0);
}
