// Fixture driver (test infrastructure, built only in the oracle's _ref/ tree
// from the reference sources).  Runs the reference's own result writers on a
// refined mesh with seeded models and data, in the working directory:
//   InversionBase::result2text   -> model.txt        (Mesh::out_model_txt, Mesh.cpp:1416-1460)
//   InversionBase::result2vtk    -> model.vtk, model_points.vtk
//                                   (Mesh::out_model_vtk / out_model_vtk_points, Mesh.cpp:1160-1415)
//   InversionBase::output_obs_data      -> dobs_<component>  (InversionBase::out_data, :743-784)
//   InversionBase::output_obs_data_vtk  -> dobs.vtk          (InversionBase::out_data_vtk, :798-880)
// and dumps the inputs (leaf cells, observation points, m, m0, m0s, dobs) to
// out.bin.  The mesh is refined as the operator driver does it: passes of
// points whose containing leaves are split with Mesh::refinement.
//
// Usage: ref_output <in.bin> <out.bin>
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
  void put(const Eigen::VectorXd &m_, const Eigen::VectorXd &m0_, const Eigen::VectorXd &m0s_) {
    m = m_;
    m0 = m0_;
    m0_s = m0s_;
  }
};

// values with many significant digits, both signs, a few exact zeros and a
// spread of magnitudes (linear congruential, reproducible anywhere)
double seeded(uint64_t &s) {
  s = s * 6364136223846793005ull + 1442695040888963407ull;
  const int64_t k = (int64_t)((s >> 11) % 2000001) - 1000000;
  const int e = (int)((s >> 40) % 13) - 6;
  if ((s >> 56) % 17 == 0) return 0.0;
  double v = (double)k / 997.0;
  for (int i = 0; i < e; i++) v *= 10.0;
  for (int i = 0; i > e; i--) v /= 10.0;
  return v;
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
  const int64_t n_passes = in.get<int64_t>();
  std::vector<std::vector<double>> passes(n_passes);
  for (auto &r : passes) {
    const int64_t np = in.get<int64_t>();
    r.resize(3 * np);
    for (auto &v : r) v = in.get<double>();
  }
  const int64_t n_obs = in.get<int64_t>();
  std::vector<double> obs(3 * n_obs);
  for (auto &v : obs) v = in.get<double>();
  const uint32_t mask = in.get<uint32_t>();
  const uint64_t seed = in.get<uint64_t>();
  std::fclose(fi);

  Mesh mesh;
  mesh.generate_regular_mesh(xl, (int)nx, yl, (int)ny, zl, (int)nz);
  Observation ob;
  for (int64_t i = 0; i < n_obs; i++) ob.add_point(obs[3 * i], obs[3 * i + 1], obs[3 * i + 2]);
  Drv inv(mesh, ob, mask);
  Mesh &m = inv.mesh_();
  for (const auto &r : passes) {
    std::vector<Cell *> marked;
    for (size_t i = 0; i < m.leaf_cells.size(); i++) {
      Cell *c = m.leaf_cells[i];
      for (size_t p = 0; p < r.size(); p += 3) {
        if (r[p] > c->_x[0] && r[p] < c->_x[1] && r[p + 1] > c->_y[0] && r[p + 1] < c->_y[1] &&
            r[p + 2] > c->_z[0] && r[p + 2] < c->_z[1]) {
          marked.push_back(c);
          break;
        }
      }
    }
    for (Cell *c : marked)
      if (c->isleaf) m.refinement(c);
    inv.rebuild();
  }
  const int64_t n = m.n_elems();
  int nf = 0;
  for (int b = 0; b < 10; b++) nf += (mask >> b) & 1;
  const int64_t nd = nf * n_obs;

  uint64_t s = seed;
  Eigen::VectorXd mv(n), m0(n), m0s(n), dobs(nd);
  for (int64_t i = 0; i < n; i++) mv(i) = seeded(s);
  for (int64_t i = 0; i < n; i++) m0(i) = seeded(s);
  for (int64_t i = 0; i < n; i++) m0s(i) = seeded(s);
  for (int64_t i = 0; i < nd; i++) dobs(i) = seeded(s);
  inv.put(mv, m0, m0s);
  inv.set_dobs(dobs, 0.02, 1e-3);

  inv.result2text("model");
  inv.result2vtk("model");
  inv.output_obs_data("dobs");
  inv.output_obs_data_vtk("dobs.vtk");

  FILE *fo = std::fopen(argv[2], "wb");
  if (!fo) return 6;
  std::fwrite(&n, 8, 1, fo);
  for (int64_t i = 0; i < n; i++) {
    const Cell *c = m.leaf_cells[i];
    const double v[6] = {c->_x[0], c->_x[1], c->_y[0], c->_y[1], c->_z[0], c->_z[1]};
    std::fwrite(v, 8, 6, fo);
  }
  std::fwrite(mv.data(), 8, (size_t)n, fo);
  std::fwrite(m0.data(), 8, (size_t)n, fo);
  std::fwrite(m0s.data(), 8, (size_t)n, fo);
  std::fwrite(&nd, 8, 1, fo);
  std::fwrite(dobs.data(), 8, (size_t)nd, fo);
  std::fclose(fo);
  return 0;
}
