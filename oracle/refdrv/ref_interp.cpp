// Fixture driver (test infrastructure, built only in the oracle's _ref/ tree
// from the reference sources).  The structure-model interpolation of the
// cross-gradient inversion and its use in a refinement:
//   InversionBase::create_crg_model_from_data (InversionBase.cpp:913-1340) on a
//   seeded gridded model written as an "xyz" file, the cell-centre values it
//   gives the leaves (GaussNewtonInversion.cpp:677-692), the interpolator at
//   probe points (inside, on grid points, outside the grid), and one
//   AdaptiveInversion::refine_mesh(a, interpolator, "crg")
//   (AdaptiveInversion.cpp:206-386) whose children take interpolated values.
//
// Usage: ref_interp <in.bin> <out.bin>   (writes crg_model.xyz and
// crg_model.vtk into the working directory)
#include <array>
#include <cstdint>
#include <cstdio>
#include <fstream>
#include <iomanip>
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
  // the cell-centre values invert_with_own_CG gives the leaves (:677-692)
  void centre_values() {
    for (int i = 0; i < Nm; i++) {
      Cell *c = mesh.leaf_cells[i];
      double xc, yc, zc;
      c->get_center(xc, yc, zc);
      std::array<double, 3> args = {xc, yc, zc};
      c->set_parameter(interpolator_m0s->interp(args.begin()), 2);
    }
    m0_s.resize(Nm);
    mesh.get_model_parameter_from_mesh(m0_s, 2);
  }
  double probe(double x, double y, double z) const {
    std::array<double, 3> args = {x, y, z};
    return interpolator_m0s->interp(args.begin());
  }
  void put_m(const Eigen::VectorXd &v) {
    m = v;
    m0 = Eigen::VectorXd::Zero(v.size());
    m_min = Eigen::VectorXd::Constant(v.size(), -1e6);
    m_max = Eigen::VectorXd::Constant(v.size(), 1e6);
  }
  void refine_crg(double a) { refine_mesh(a, *interpolator_m0s, "crg"); }
  const Eigen::VectorXd &m0s_() const { return m0_s; }
};

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
  int64_t gn[3];
  std::vector<double> grid[3];
  for (int d = 0; d < 3; d++) {
    gn[d] = in.get<int64_t>();
    grid[d].resize(gn[d]);
    for (auto &v : grid[d]) v = in.get<double>();
  }
  std::vector<double> vals(gn[0] * gn[1] * gn[2]);  // x outer, z inner
  for (auto &v : vals) v = in.get<double>();
  const int64_t nprobe = in.get<int64_t>();
  std::vector<double> probes(3 * nprobe);
  for (auto &v : probes) v = in.get<double>();
  const double fraction = in.get<double>();
  const uint64_t seed = in.get<uint64_t>();
  std::fclose(fi);

  {  // the gridded model as the reference reads it: x fastest, then y, then z
    std::ofstream o("crg_model.xyz");
    o << std::setprecision(17);
    for (int64_t k = 0; k < gn[2]; k++)
      for (int64_t j = 0; j < gn[1]; j++)
        for (int64_t i = 0; i < gn[0]; i++)
          o << grid[0][i] << " " << grid[1][j] << " " << grid[2][k] << " "
            << vals[(i * gn[1] + j) * gn[2] + k] << "\n";
  }

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
  inv.create_crg_model_from_data("crg_model.xyz", (int)gn[0], (int)gn[1], (int)gn[2], "xyz",
                                 "xyz");
  inv.centre_values();
  const int64_t n0 = m.n_elems();
  Eigen::VectorXd mv(n0);
  uint64_t s = seed;
  for (int64_t i = 0; i < n0; i++) {
    s = s * 6364136223846793005ull + 1442695040888963407ull;
    mv(i) = ((double)((s >> 11) % 200001) - 100000.0) / 137.0;
  }
  inv.put_m(mv);
  inv.compute_G();

  FILE *fo = std::fopen(argv[2], "wb");
  if (!fo) return 6;
  std::fwrite(&n0, 8, 1, fo);
  std::fwrite(inv.m0s_().data(), 8, (size_t)n0, fo);
  std::vector<double> pv(nprobe);
  for (int64_t p = 0; p < nprobe; p++)
    pv[p] = inv.probe(probes[3 * p], probes[3 * p + 1], probes[3 * p + 2]);
  std::fwrite(pv.data(), 8, (size_t)nprobe, fo);
  inv.set_min_cell_size_in_adaptive_mesh(1.0, 1.0, 1.0);
  inv.refine_crg(fraction);
  const int64_t n1 = m.n_elems();
  std::fwrite(&n1, 8, 1, fo);
  for (int64_t i = 0; i < n1; i++) {
    const Cell *c = m.leaf_cells[i];
    const double v[6] = {c->_x[0], c->_x[1], c->_y[0], c->_y[1], c->_z[0], c->_z[1]};
    std::fwrite(v, 8, 6, fo);
  }
  std::fwrite(inv.m0s_().data(), 8, (size_t)n1, fo);
  std::fclose(fo);
  return 0;
}
