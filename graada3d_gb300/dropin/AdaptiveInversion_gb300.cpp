// Drop-in body for AdaptiveInversion::expand_G
// (src/Inversion/AdaptiveInversion.cpp:23-106) against the unchanged
// AdaptiveInversion.h.  A maintainer removes expand_G from
// AdaptiveInversion.cpp and links this file with the other drop-in units;
// refine_mesh keeps calling it after Mesh::refinement and rearrange_id.
//
// The split parents (the map's keys, ascending: their column indices before
// the refinement) and each parent's eight children in Cell::child_cells order
// go to grada_expand_G, which splices the children's columns into the GPU
// copy of G exactly as the reference splices them into the member G.  The
// member G is refreshed from the GPU unless GRADA_KEEP_G_ON_DEVICE is set.
#include <cstdlib>
#include <map>
#include <vector>

#include "AdaptiveInversion.h"
#include "gb300_bridge.h"

void AdaptiveInversion::expand_G(const map<unsigned int, Cell *> &split_cells)
{
  grada_ctx *ctx = gb300::context_for(static_cast<const Fwd *>(this));
  std::vector<int64_t> parents;
  std::vector<double> children;
  parents.reserve(split_cells.size());
  children.reserve(48 * split_cells.size());
  for (const auto &kv : split_cells) {
    parents.push_back((int64_t)kv.first);
    for (int j = 0; j < 8; j++) {
      const Cell *c = kv.second->child_cells[j];
      const double box[6] = {c->_x[0], c->_x[1], c->_y[0], c->_y[1], c->_z[0], c->_z[1]};
      children.insert(children.end(), box, box + 6);
    }
  }
  gb300::check(ctx,
               grada_expand_G(ctx, (int64_t)parents.size(), parents.data(), children.data()),
               "grada_expand_G");
  if (!std::getenv("GRADA_KEEP_G_ON_DEVICE")) {
    int64_t n_cells = 0, n_obs = 0;
    int n_fields = 0;
    gb300::check(ctx, grada_get_dims(ctx, &n_cells, &n_obs, &n_fields, nullptr, nullptr),
                 "grada_get_dims");
    G.resize((Eigen::Index)(n_fields * n_obs), (Eigen::Index)n_cells);
    gb300::check(ctx, grada_get_G(ctx, G.data(), G.rows()), "grada_get_G");
  }
}
