// Fixture driver (test infrastructure, built only in the oracle's _ref/ tree
// from the reference sources).  Builds the reference's padded regular mesh
// (Mesh::generate_regular_mesh_with_padding, src/Forward_modelling/
// Mesh.cpp:516-795: the area of interest plus stretched padding cells on the
// x, y sides and below) and dumps its leaf cells and Fwd::compute_G.
//
// Usage: ref_padded <in.bin> <out.bin>
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
  const Eigen::MatrixXd &G_() const { return G; }
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
  const int64_t px = in.get<int64_t>(), py = in.get<int64_t>(), pz = in.get<int64_t>();
  const double sx = in.get<double>(), sy = in.get<double>(), sz = in.get<double>();
  const int64_t n_obs = in.get<int64_t>();
  std::vector<double> obs(3 * n_obs);
  for (auto &v : obs) v = in.get<double>();
  const uint32_t mask = in.get<uint32_t>();
  std::fclose(fi);

  Mesh mesh;
  mesh.generate_regular_mesh_with_padding(xl, (int)nx, yl, (int)ny, zl, (int)nz, (int)px, sx,
                                          (int)py, sy, (int)pz, sz);
  Observation ob;
  for (int64_t i = 0; i < n_obs; i++) ob.add_point(obs[3 * i], obs[3 * i + 1], obs[3 * i + 2]);
  Drv inv(mesh, ob, mask);
  inv.compute_G();

  FILE *fo = std::fopen(argv[2], "wb");
  if (!fo) return 6;
  Mesh &m = inv.mesh_();
  const int64_t n_leaf = m.n_elems();
  std::fwrite(&n_leaf, 8, 1, fo);
  for (int64_t i = 0; i < n_leaf; i++) {
    const Cell *c = m.leaf_cells[i];
    const double v[6] = {c->_x[0], c->_x[1], c->_y[0], c->_y[1], c->_z[0], c->_z[1]};
    std::fwrite(v, 8, 6, fo);
  }
  const Eigen::MatrixXd &G = inv.G_();
  const int64_t rows = G.rows(), cols = G.cols();
  std::fwrite(&rows, 8, 1, fo);
  std::fwrite(&cols, 8, 1, fo);
  std::fwrite(G.data(), 8, (size_t)(rows * cols), fo);
  std::fclose(fo);
  return 0;
}
