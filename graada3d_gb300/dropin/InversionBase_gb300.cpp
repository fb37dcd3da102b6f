// Drop-in bodies for the members of InversionBase that read the member G
// (src/Inversion/InversionBase.cpp), against the unchanged InversionBase.h:
// set_depth_weighting (:497-528) and get_predicted_field (:696-708).  A
// maintainer removes both from InversionBase.cpp and links this file with the
// other drop-in units.
//
// set_depth_weighting: flag 0 (distance of each cell centre from the mean
// observation height, raised to -beta/2) is host arithmetic on the mesh and
// the points, in the reference's order.  flag 1 (sensitivity weighting,
// sqrt(||G(:, j)|| / Nd)) reads every column of G; here the norms come from the
// GPU copy of G (grada_G_column_norms), so it also works when the member G is
// left empty (GRADA_KEEP_G_ON_DEVICE) and never moves G to the host.
#include <cassert>
#include <cmath>
#include <vector>

#include "InversionBase.h"
#include "gb300_bridge.h"

void InversionBase::set_depth_weighting(double beta, int flag)
{
  depth_weighting_factor = beta;
  Z.setZero();
  assert(N_obs != 0);
  assert(Nm != 0);
  if (flag == 0) {
    double mean_height = 0.0;
    for (int i = 0; i < N_obs; i++) mean_height += ob(i).z();
    mean_height /= N_obs;
    for (int j = 0; j < Nm; j++) {
      const RectPrism &cell = mesh.get_elem(j);
      const double centre = 0.5 * (cell._z[0] + cell._z[1]);
      Z.coeffRef(j, j) += 1.0 / std::pow(std::abs(mean_height - centre), beta * 0.5);
    }
  }
  if (flag == 1) {
    std::vector<double> norms((size_t)Nm);
    grada_ctx *ctx = gb300::context_for(static_cast<const Fwd *>(this));
    gb300::check(ctx, grada_G_column_norms(ctx, norms.data()), "grada_G_column_norms");
    for (int j = 0; j < Nm; j++) Z.coeffRef(j, j) += std::sqrt(norms[(size_t)j] / Nd);
  }
}

// InversionBase::get_predicted_field (InversionBase.cpp:696-708): G m, here
// always through G_vec_mul (the drop-in Fwd::G_vec_mul multiplies by the GPU
// copy), since the member G may be left empty.
VectorXd InversionBase::get_predicted_field()
{
  VectorXd d_pre;
  this->G_vec_mul(this->m, d_pre);
  return d_pre;
}
