// Drop-in bodies for the dense path of the reference's Fwd class
// (src/Forward_modelling/Fwd.cpp:47-146), against the unchanged Fwd.h.
// A maintainer removes Fwd::compute_G, Fwd::GT_vec_mul and Fwd::G_vec_mul from
// Fwd.cpp (keeping the constructors and the wavelet members there) and links
// this file, gb300_bridge.cpp and libgrada_gpu.so instead.
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
