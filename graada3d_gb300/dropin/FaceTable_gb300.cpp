// The face table grada_build_operators takes, read from the reference's own
// mesh faces: per leaf cell and axis the face InversionBase::
// set_difference_matrix (InversionBase.cpp:189-434) differences against, as
// [side, c0, c1, c2, c3] int32 (15 per cell, axes x, y, z):
//   +axis face split (the neighbour was refined): side +1, its four child
//     faces' cells on the + side                                   (:251-263)
//   +axis face a leaf with cells on both sides: side +1, the cell across (:208-220)
//   +axis face on the boundary: the -axis face instead, side -1 -- split: its
//     four child faces' cells on the - side (:236-248), a leaf: the cell
//     across (:223-235), no cell (a one-cell axis): side 0, no row (:389)
// A host that keeps the reference's Mesh calls this after a refinement and
// hands the table to grada_build_operators in place of uploading host-built
// Ws/Wx/Wy/Wz.
#include <cstdint>
#include <vector>

#include "Mesh.h"
#include "gb300_bridge.h"

namespace gb300 {
namespace {

void entry(Face *plus, Face *minus, int32_t *f) {
  f[0] = 0;
  f[1] = f[2] = f[3] = f[4] = -1;
  if (!plus->isleaf) {
    f[0] = 1;
    for (int k = 0; k < 4; k++) f[1 + k] = plus->child_faces[k]->neigh_cells[1]->get_id();
    return;
  }
  if (plus->neigh_cells[0] != nullptr && plus->neigh_cells[1] != nullptr) {
    f[0] = 1;
    f[1] = plus->neigh_cells[1]->get_id();
    return;
  }
  if (!minus->isleaf) {
    f[0] = -1;
    for (int k = 0; k < 4; k++) f[1 + k] = minus->child_faces[k]->neigh_cells[0]->get_id();
    return;
  }
  if (minus->neigh_cells[0] != nullptr) {
    f[0] = -1;
    f[1] = minus->neigh_cells[0]->get_id();
  }
}

}  // namespace

void face_table(Mesh &mesh, std::vector<int32_t> &table) {
  const size_t n = mesh.leaf_cells.size();
  table.assign(15 * n, -1);
  for (size_t i = 0; i < n; i++) {
    Cell *c = mesh.leaf_cells[i];
    entry(c->external_faces_x[1], c->external_faces_x[0], &table[15 * i]);
    entry(c->external_faces_y[1], c->external_faces_y[0], &table[15 * i + 5]);
    entry(c->external_faces_z[1], c->external_faces_z[0], &table[15 * i + 10]);
  }
}

}  // namespace gb300
