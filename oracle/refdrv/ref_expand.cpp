// Fixture driver (test infrastructure, built only in the oracle's _ref/ tree
// from the reference sources).  Runs the reference's own refinement path on a
// regular mesh: Fwd::compute_G, Mesh::refinement of the listed cells, then
// Mesh::rearrange_id and AdaptiveInversion::expand_G (the steps and order of
// AdaptiveInversion::refine_mesh, src/Inversion/AdaptiveInversion.cpp:
// 264-334), and dumps the expanded G, the refined leaf list and each parent's
// children in Cell::child_cells order.
//
// Usage: ref_expand <in.bin> <out.bin>
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
  std::vector<double> vec(size_t n) {
    std::vector<double> v(n);
    if (n && std::fread(v.data(), 8, n, f) != n) throw std::runtime_error("short input");
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

void put_cell(FILE *fo, const Cell *c) {
  const double v[6] = {c->_x[0], c->_x[1], c->_y[0], c->_y[1], c->_z[0], c->_z[1]};
  std::fwrite(v, 8, 6, fo);
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
  const int64_t n_obs = in.get<int64_t>();
  const std::vector<double> obs = in.vec(3 * n_obs);
  const uint32_t mask = in.get<uint32_t>();
  const int64_t n_par = in.get<int64_t>();
  std::vector<int64_t> parents(n_par);
  for (auto &p : parents) p = in.get<int64_t>();
  std::fclose(fi);

  Mesh mesh;
  mesh.generate_regular_mesh(xl, (int)nx, yl, (int)ny, zl, (int)nz);
  Observation ob;
  for (int64_t i = 0; i < n_obs; i++) ob.add_point(obs[3 * i], obs[3 * i + 1], obs[3 * i + 2]);
  Drv inv(mesh, ob, mask);
  inv.compute_G();

  // the cells to split, taken before any refinement (refine_mesh marks first)
  Mesh &m = inv.mesh_();
  std::vector<Cell *> marked;
  for (int64_t p : parents) marked.push_back(m.leaf_cells[p]);
  std::map<unsigned int, Cell *> split;
  for (Cell *c : marked) {
    if (!c->isleaf) continue;
    std::map<unsigned int, Cell *> s0 = m.refinement(c);
    split.insert(s0.begin(), s0.end());
  }
  m.rearrange_id();
  inv.expand_G(split);

  FILE *fo = std::fopen(argv[2], "wb");
  if (!fo) return 6;
  const Eigen::MatrixXd &G = inv.G_();
  const int64_t rows = G.rows(), cols = G.cols(), n_leaf = m.n_elems(), n_split = split.size();
  std::fwrite(&rows, 8, 1, fo);
  std::fwrite(&cols, 8, 1, fo);
  std::fwrite(G.data(), 8, (size_t)(rows * cols), fo);
  std::fwrite(&n_leaf, 8, 1, fo);
  for (int64_t i = 0; i < n_leaf; i++) put_cell(fo, m.leaf_cells[i]);
  std::fwrite(&n_split, 8, 1, fo);
  for (const auto &kv : split) {
    const int64_t idx = kv.first;
    std::fwrite(&idx, 8, 1, fo);
    for (int j = 0; j < 8; j++) put_cell(fo, kv.second->child_cells[j]);
  }
  std::fclose(fo);
  return 0;
}
