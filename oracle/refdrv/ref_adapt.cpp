// Fixture driver (test infrastructure, built only in the oracle's _ref/ tree
// from the reference sources).  One refinement of the adaptive inversion with
// the reference's own AdaptiveInversion::refine_mesh(a)
// (src/Inversion/AdaptiveInversion.cpp:637-735): a regular mesh refined first
// at the leaves containing given points (so that levels are mixed), a seeded
// model, then refine_mesh with a refinement fraction and minimum cell sizes.
// Dumps the leaves and the model before, the indicator the refinement is
// driven by, and the leaves and the inherited model after.
//
// Usage: ref_adapt <in.bin> <out.bin>
#include <cstdint>
#include <cstdio>
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
  void rebuild() {
    mesh.rearrange_id();
    Nm = mesh.n_elems();
    init_matrices();
  }
  void put_m(const Eigen::VectorXd &v) {
    m = v;
    m0 = Eigen::VectorXd::Zero(v.size());
    m0_s = Eigen::VectorXd::Zero(v.size());
    m_min = Eigen::VectorXd::Constant(v.size(), -1e6);
    m_max = Eigen::VectorXd::Constant(v.size(), 1e6);
  }
  const Eigen::VectorXd &m_() const { return m; }
};

void dump_leaves(FILE *fo, Mesh &m) {
  const int64_t n = m.n_elems();
  std::fwrite(&n, 8, 1, fo);
  for (int64_t i = 0; i < n; i++) {
    const Cell *c = m.leaf_cells[i];
    const double v[6] = {c->_x[0], c->_x[1], c->_y[0], c->_y[1], c->_z[0], c->_z[1]};
    std::fwrite(v, 8, 6, fo);
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
  const int64_t np = in.get<int64_t>();
  std::vector<double> pts(3 * np);
  for (auto &v : pts) v = in.get<double>();
  const double fraction = in.get<double>();
  const double mdx = in.get<double>(), mdy = in.get<double>(), mdz = in.get<double>();
  const uint64_t seed = in.get<uint64_t>();
  std::fclose(fi);

  Mesh mesh;
  mesh.generate_regular_mesh(xl, (int)nx, yl, (int)ny, zl, (int)nz);
  Observation ob;
  ob.add_point(0.5 * (xl[0] + xl[1]), 0.5 * (yl[0] + yl[1]), -10.0);
  Drv inv(mesh, ob, 0x002);
  Mesh &m = inv.mesh_();
  std::vector<Cell *> marked;
  for (size_t i = 0; i < m.leaf_cells.size(); i++) {
    Cell *c = m.leaf_cells[i];
    for (int64_t p = 0; p < np; p++)
      if (pts[3 * p] > c->_x[0] && pts[3 * p] < c->_x[1] && pts[3 * p + 1] > c->_y[0] &&
          pts[3 * p + 1] < c->_y[1] && pts[3 * p + 2] > c->_z[0] && pts[3 * p + 2] < c->_z[1]) {
        marked.push_back(c);
        break;
      }
  }
  for (Cell *c : marked)
    if (c->isleaf) m.refinement(c);
  inv.rebuild();
  const int64_t n = m.n_elems();
  // a seeded model with jumps and decimals (linear congruential)
  Eigen::VectorXd mv(n);
  uint64_t s = seed;
  for (int64_t i = 0; i < n; i++) {
    s = s * 6364136223846793005ull + 1442695040888963407ull;
    mv(i) = ((double)((s >> 11) % 200001) - 100000.0) / 137.0;
  }
  inv.put_m(mv);
  inv.compute_G();
  Eigen::VectorXd ind;
  inv.indicator_calculator(ind);
  inv.set_min_cell_size_in_adaptive_mesh(mdx, mdy, mdz);

  FILE *fo = std::fopen(argv[2], "wb");
  if (!fo) return 6;
  dump_leaves(fo, m);
  std::fwrite(mv.data(), 8, (size_t)n, fo);
  std::fwrite(ind.data(), 8, (size_t)n, fo);
  inv.refine_mesh(fraction);
  dump_leaves(fo, m);
  const Eigen::VectorXd &m2 = inv.m_();
  std::fwrite(m2.data(), 8, (size_t)m2.size(), fo);
  std::fclose(fo);
  return 0;
}
