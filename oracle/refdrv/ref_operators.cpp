// Fixture driver (test infrastructure, built only in the oracle's _ref/ tree
// from the reference sources).  Builds a regular mesh, refines it in passes
// with the reference's own Mesh::refinement (face-balance cascade included,
// Mesh.cpp:1462-1942) and Mesh::rearrange_id, rebuilds the inversion matrices
// the way AdaptiveInversion does after a refinement (init_matrices,
// AdaptiveInversion.cpp:278-283) and dumps the leaf cells with the
// regularisation operators: D_x1, D_y1, D_z1 (InversionBase::set_difference_matrix,
// InversionBase.cpp:189-434), V, Z, Ws/Wx/Wy/Wz (GaussNewtonInversion.cpp:711-714)
// and, for a seeded structure model, T_x, T_y, T_z (InversionBase::set_Tmatrix,
// InversionBase.cpp:468-495).
//
// Also dumps Mesh::get_reordered_id of every position (the order the
// wavelet compression runs along) and the face table of the drop-in's face_table
// (graada3d_gb300/dropin/FaceTable_gb300.cpp, compiled in here) read from the
// reference's own Face objects, the input a C++ host hands to
// grada_build_operators.
//
// A pass names points; the leaves that contain a point (strictly inside)
// are refined in leaf order, skipping cells a cascade already split, as
// AdaptiveInversion::refine_mesh does with its marked cells.
//
// Usage: ref_operators <in.bin> <out.bin>
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <vector>

#include "GaussNewtonInversion.h"
#include "../../graada3d_gb300/dropin/FaceTable_gb300.cpp"

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

struct Writer {
  FILE *f;
  void i64(int64_t v) { std::fwrite(&v, 8, 1, f); }
  void vec(const Eigen::VectorXd &v) { std::fwrite(v.data(), 8, (size_t)v.size(), f); }
  void csr(const SMatrix &m0) {
    SMatrix m = m0;
    m.makeCompressed();
    const int64_t n = m.rows();
    i64(n);
    i64((int64_t)m.nonZeros());
    for (int64_t r = 0; r <= n; r++) i64((int64_t)m.outerIndexPtr()[r]);
    for (int64_t k = 0; k < m.nonZeros(); k++) i64((int64_t)m.innerIndexPtr()[k]);
    std::fwrite(m.valuePtr(), 8, (size_t)m.nonZeros(), f);
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
  SMatrix Ws() { return a_s * S_s * V * D_s * Z; }  // GaussNewtonInversion.cpp:711
  SMatrix Wx() { return a_x * S_x * V * D_x1 * Z; } // :712
  SMatrix Wy() { return a_y * S_y * V * D_y1 * Z; } // :713
  SMatrix Wz() { return a_z * S_z * V * D_z1 * Z; } // :714
  const SMatrix &Dx() const { return D_x1; }
  const SMatrix &Dy() const { return D_y1; }
  const SMatrix &Dz() const { return D_z1; }
  const SMatrix &V_() const { return V; }
  const SMatrix &Z_() const { return Z; }
  void structure(const Eigen::VectorXd &m0s) {
    m0_s = m0s;
    set_Tmatrix();
  }
  const SMatrix &Tx() const { return T_x; }
  const SMatrix &Ty() const { return T_y; }
  const SMatrix &Tz() const { return T_z; }
};

Eigen::VectorXd diag_of(const SMatrix &m) {
  Eigen::VectorXd d(m.rows());
  for (int i = 0; i < m.rows(); i++) d(i) = m.coeff(i, i);
  return d;
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
  const double beta = in.get<double>();
  const double a_s = in.get<double>(), a_z = in.get<double>(), a_x = in.get<double>(),
               a_y = in.get<double>();
  const uint64_t seed = in.get<uint64_t>();
  std::fclose(fi);

  Mesh mesh;
  mesh.generate_regular_mesh(xl, (int)nx, yl, (int)ny, zl, (int)nz);
  Observation ob;
  for (int64_t i = 0; i < n_obs; i++) ob.add_point(obs[3 * i], obs[3 * i + 1], obs[3 * i + 2]);
  Drv inv(mesh, ob, 0x002);
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
  inv.set_depth_weighting(beta);
  inv.set_weights_of_objectives(a_s, a_z, a_x, a_y, 1.0);
  const int64_t n = m.n_elems();

  // a seeded structure model (linear congruential, reproducible anywhere)
  Eigen::VectorXd m0s(n);
  uint64_t s = seed;
  for (int64_t i = 0; i < n; i++) {
    s = s * 6364136223846793005ull + 1442695040888963407ull;
    m0s(i) = (double)((s >> 11) % 2001) - 1000.0;
  }
  inv.structure(m0s);

  FILE *fo = std::fopen(argv[2], "wb");
  if (!fo) return 6;
  Writer out{fo};
  out.i64(n);
  for (int64_t i = 0; i < n; i++) {
    const Cell *c = m.leaf_cells[i];
    const double v[6] = {c->_x[0], c->_x[1], c->_y[0], c->_y[1], c->_z[0], c->_z[1]};
    std::fwrite(v, 8, 6, fo);
  }
  for (int64_t i = 0; i < n; i++) out.i64(m.leaf_cells[i]->get_level());
  out.csr(inv.Dx());
  out.csr(inv.Dy());
  out.csr(inv.Dz());
  out.vec(diag_of(inv.V_()));
  out.vec(diag_of(inv.Z_()));
  out.csr(inv.Ws());
  out.csr(inv.Wx());
  out.csr(inv.Wy());
  out.csr(inv.Wz());
  out.vec(m0s);
  out.csr(inv.Tx());
  out.csr(inv.Ty());
  out.csr(inv.Tz());
  std::vector<int32_t> table;
  gb300::face_table(m, table);
  std::fwrite(table.data(), 4, table.size(), fo);
  for (int64_t i = 0; i < n; i++) out.i64(m.get_reordered_id((unsigned)i));
  std::fclose(fo);
  return 0;
}
