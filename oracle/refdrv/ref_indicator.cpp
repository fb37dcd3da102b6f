// Fixture driver (test infrastructure, built only in the oracle's _ref/ tree
// from the reference sources).  On a regular mesh refined at a few cells
// (Mesh::refinement, Mesh::rearrange_id), with a seeded model m, dumps the
// reference's refinement indicator (AdaptiveInversion::indicator_calculator,
// src/Inversion/AdaptiveInversion.cpp:108-204) and, for every leaf cell, the
// (neighbour id, face area) pairs its sum runs over, in the order it adds them:
// for j = 0, 1 the x, y and z faces on side j; a leaf face with cells on both
// sides contributes the cell across it with the cell's own face area, a split
// face its four child faces' cells with those cells' face areas.  This list is
// what a host hands to the device indicator.
//
// Usage: ref_indicator <in.bin> <out.bin>
#include <cstdint>
#include <cstdio>
#include <map>
#include <stdexcept>
#include <vector>

#include "GaussNewtonInversion.h"

namespace {

struct Reader {
  FILE *f;
  template <typename T>
  T get() {
    T v{};
    if (std::fread(&v, sizeof(T), 1, f) != 1) throw std::runtime_error("short input");
    return v;
  }
};

class Drv : public GaussNewtonInversion {
 public:
  Drv(const Mesh &mesh, const Observation &ob, unsigned long long flag)
      : GaussNewtonInversion(mesh, ob, flag) {}
  Mesh &mesh_() { return mesh; }
  void put_m(const Eigen::VectorXd &v) { m = v; Nm = (int)v.size(); }
};

// Neighbour pairs of one face direction, in indicator_calculator's order.
void face_pairs(Face *f, int j, Cell *c, int axis, std::vector<int64_t> &nb,
                std::vector<double> &area) {
  auto face_area = [axis](const Cell *x) {
    if (axis == 0) return (x->_z[1] - x->_z[0]) * (x->_y[1] - x->_y[0]);
    if (axis == 1) return (x->_z[1] - x->_z[0]) * (x->_x[1] - x->_x[0]);
    return (x->_x[1] - x->_x[0]) * (x->_y[1] - x->_y[0]);
  };
  if (f->isleaf) {
    if (f->neigh_cells[0] != nullptr && f->neigh_cells[1] != nullptr) {
      nb.push_back(f->neigh_cells[j]->get_id());
      area.push_back(face_area(c));
    }
  } else {
    for (int k = 0; k < 4; k++) {
      Cell *n = f->child_faces[k]->neigh_cells[j];
      nb.push_back(n->get_id());
      area.push_back(face_area(n));
    }
  }
}

}  // namespace

int main(int argc, char **argv) {
  if (argc != 3) {
    std::fprintf(stderr, "usage: %s in.bin out.bin\n", argv[0]);
    return 2;
  }
  FILE *fi = std::fopen(argv[1], "rb");
  if (!fi) return 3;
  Reader in{fi};
  const int64_t nx = in.get<int64_t>(), ny = in.get<int64_t>(), nz = in.get<int64_t>();
  double xl[2], yl[2], zl[2];
  xl[0] = in.get<double>(); xl[1] = in.get<double>();
  yl[0] = in.get<double>(); yl[1] = in.get<double>();
  zl[0] = in.get<double>(); zl[1] = in.get<double>();
  const int64_t n_par = in.get<int64_t>();
  std::vector<int64_t> parents(n_par);
  for (auto &p : parents) p = in.get<int64_t>();
  const uint64_t seed = in.get<uint64_t>();
  std::fclose(fi);

  Mesh mesh;
  mesh.generate_regular_mesh(xl, (int)nx, yl, (int)ny, zl, (int)nz);
  Observation ob;
  ob.add_point(0.5 * (xl[0] + xl[1]), 0.5 * (yl[0] + yl[1]), -1.0);
  Drv inv(mesh, ob, 0x002);
  Mesh &m = inv.mesh_();
  std::vector<Cell *> marked;
  for (int64_t p : parents) marked.push_back(m.leaf_cells[p]);
  for (Cell *c : marked)
    if (c->isleaf) m.refinement(c);
  m.rearrange_id();
  const int64_t n = m.n_elems();

  // a seeded model with jumps (linear congruential, reproducible anywhere)
  Eigen::VectorXd mv(n);
  uint64_t s = seed;
  for (int64_t i = 0; i < n; i++) {
    s = s * 6364136223846793005ull + 1442695040888963407ull;
    mv(i) = (double)((s >> 11) % 2001) - 1000.0;
  }
  inv.put_m(mv);
  Eigen::VectorXd ind;
  inv.indicator_calculator(ind);

  std::vector<int64_t> rowptr(1, 0), nb;
  std::vector<double> area;
  for (int64_t i = 0; i < n; i++) {
    Cell *c = m.leaf_cells[i];
    for (int j = 0; j < 2; j++) {
      face_pairs(c->external_faces_x[j], j, c, 0, nb, area);
      face_pairs(c->external_faces_y[j], j, c, 1, nb, area);
      face_pairs(c->external_faces_z[j], j, c, 2, nb, area);
    }
    rowptr.push_back((int64_t)nb.size());
  }

  FILE *fo = std::fopen(argv[2], "wb");
  if (!fo) return 6;
  std::fwrite(&n, 8, 1, fo);
  for (int64_t i = 0; i < n; i++) {
    const Cell *c = m.leaf_cells[i];
    const double v[6] = {c->_x[0], c->_x[1], c->_y[0], c->_y[1], c->_z[0], c->_z[1]};
    std::fwrite(v, 8, 6, fo);
  }
  std::fwrite(mv.data(), 8, (size_t)n, fo);
  std::fwrite(ind.data(), 8, (size_t)n, fo);
  const int64_t nnz = (int64_t)nb.size();
  std::fwrite(&nnz, 8, 1, fo);
  std::fwrite(rowptr.data(), 8, rowptr.size(), fo);
  std::fwrite(nb.data(), 8, nb.size(), fo);
  std::fwrite(area.data(), 8, area.size(), fo);
  std::fclose(fo);
  return 0;
}
