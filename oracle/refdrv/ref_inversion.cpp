// Fixture driver (test infrastructure, built only in the oracle's _ref/ tree
// from the reference sources).  Sets up the reference GaussNewtonInversion on
// a regular mesh the way GraAdaInv::start_inversion does
// (src/GraAda3D.cpp:684-787) and dumps what the GPU path must reproduce:
// the sensitivity matrix, the host-built regularisation operators, one
// solve_cg call (GaussNewtonInversion.cpp:1417-1698) and, optionally, a full
// invert_with_own_CG run (GaussNewtonInversion.cpp:657-1308).
//
// Mode 3 runs the adaptive inversion instead: invert_with_own_CG with its
// refinement branch (GaussNewtonInversion.cpp:1098-1294, refine_mesh
// AdaptiveInversion.cpp:637-735), reading the refinement settings after the
// mode, and dumps the final model, misfit, lambda and the final leaves.
//
// Usage: ref_inversion <in.bin> <out.bin>   (run in a scratch directory: the
// reference writes lambda_misfit_GN and Iteration_misfit_GN into the cwd)
#include <cstdint>
#include <cstdio>
#include <fstream>
#include <iomanip>
#include <string>
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

struct Writer {
  FILE *f;
  void i64(int64_t v) { std::fwrite(&v, 8, 1, f); }
  void f64(double v) { std::fwrite(&v, 8, 1, f); }
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

// Gives the driver access to the protected state it needs to dump.
class Drv : public GaussNewtonInversion {
 public:
  Drv(const Mesh &mesh, const Observation &ob, unsigned long long flag)
      : GaussNewtonInversion(mesh, ob, flag) {}
  SMatrix Ws() { return a_s * S_s * V * D_s * Z; }  // GaussNewtonInversion.cpp:711
  SMatrix Wx() { return a_x * S_x * V * D_x1 * Z; } // :712
  SMatrix Wy() { return a_y * S_y * V * D_y1 * Z; } // :713
  SMatrix Wz() { return a_z * S_z * V * D_z1 * Z; } // :714
  void set_structure_model(const Eigen::VectorXd &m0s) {
    m0_s = m0s;
    use_cross_gradient_constraint = true;
    set_Tmatrix();
  }
  void set_reference(const Eigen::VectorXd &r) { m0 = r; }
  const SMatrix &Tx() const { return T_x; }
  const SMatrix &Ty() const { return T_y; }
  const SMatrix &Tz() const { return T_z; }
  const SMatrix &Wd_() const { return Wd; }
  const SMatrix &Scrg() const { return S_crg; }
  const Eigen::MatrixXd &G_() const { return G; }
  Eigen::VectorXd m_() const { return m; }
  void use_crg(bool b) { use_cross_gradient_constraint = b; }
  Mesh &mesh_() { return mesh; }
};

SMatrix diag(const Eigen::VectorXd &d) {
  SMatrix m(d.size(), d.size());
  m.reserve(d.size());
  for (int i = 0; i < d.size(); i++) m.insert(i, i) = d(i);
  m.makeCompressed();
  return m;
}

Eigen::VectorXd diag_of(const SMatrix &m) {
  Eigen::VectorXd d(m.rows());
  for (int i = 0; i < m.rows(); i++) d(i) = m.coeff(i, i);
  return d;
}

// Gridded xyz file of values at cell centres, x fastest then y then z, the
// layout create_*_model_from_data reads with fast_dimension "xyz".
void write_center_grid(const std::string &path, const Mesh &mesh, int nx, int ny, int nz,
                       const Eigen::VectorXd &leaf_values) {
  std::ofstream o(path);
  o << std::setprecision(17);
  Mesh &m = const_cast<Mesh &>(mesh);
  for (int k = 0; k < nz; k++)
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nx; i++) {
        const int id = i * ny * nz + j * nz + k;  // leaf order, Mesh.cpp:830-847
        double xc, yc, zc;
        m.get_elem(id).get_center(xc, yc, zc);
        o << xc << " " << yc << " " << zc << " " << leaf_values(id) << "\n";
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
  const int64_t n_obs = in.get<int64_t>();
  const std::vector<double> obs = in.vec(3 * n_obs);
  const uint32_t mask = in.get<uint32_t>();
  int nf = 0;
  for (int b = 0; b < 10; b++) nf += (mask >> b) & 1;
  const int64_t nd = nf * n_obs;
  const int64_t nm = nx * ny * nz;
  Eigen::VectorXd dobs = Eigen::Map<const Eigen::VectorXd>(in.vec(nd).data(), nd);
  std::vector<double> rel = in.vec(nf), absf = in.vec(nf);
  const double beta = in.get<double>();
  const double a_s = in.get<double>(), a_z = in.get<double>(), a_x = in.get<double>(),
               a_y = in.get<double>(), a_crg = in.get<double>();
  const double max_lambda = in.get<double>();
  const int64_t n_lambda = in.get<int64_t>();
  const double rate = in.get<double>();
  const double target = in.get<double>(), stag = in.get<double>(), cg_tol = in.get<double>(),
               cg_factor = in.get<double>();
  const int64_t gn_iter = in.get<int64_t>();
  const int64_t lps = in.get<int64_t>(), lpx = in.get<int64_t>(), lpy = in.get<int64_t>(),
                lpz = in.get<int64_t>(), lpt = in.get<int64_t>();
  const double eps2 = in.get<double>();
  const double m_min = in.get<double>(), m_max = in.get<double>(), m_ini = in.get<double>();
  const int64_t use_crg = in.get<int64_t>();
  std::vector<double> m0s_v = use_crg ? in.vec(nm) : std::vector<double>();
  const int64_t use_ref = in.get<int64_t>();
  std::vector<double> m0_v = use_ref ? in.vec(nm) : std::vector<double>();
  const int64_t mode = in.get<int64_t>();
  int64_t max_ref = 0, interval = 1;
  double fraction = 0.1, min_dx = 0, min_dy = 0, min_dz = 0;
  if (mode == 3) {
    max_ref = in.get<int64_t>();
    interval = in.get<int64_t>();
    fraction = in.get<double>();
    min_dx = in.get<double>();
    min_dy = in.get<double>();
    min_dz = in.get<double>();
  }

  Mesh mesh;
  mesh.generate_regular_mesh(xl, (int)nx, yl, (int)ny, zl, (int)nz);
  Observation ob;
  for (int64_t i = 0; i < n_obs; i++) ob.add_point(obs[3 * i], obs[3 * i + 1], obs[3 * i + 2]);

  Drv inv(mesh, ob, mask);
  inv.set_dobs(dobs, rel, absf);
  inv.set_depth_weighting(beta);
  inv.set_weights_of_objectives(a_s, a_z, a_x, a_y, a_crg);
  inv.set_max_lambda(max_lambda);
  inv.set_max_GN_iterations((int)gn_iter);
  inv.set_lambda_decreasing_rate(rate);
  inv.set_n_lambda((int)n_lambda);
  inv.set_CG_parameter(cg_tol, cg_factor);
  inv.set_max_refinement_number((int)max_ref);
  if (mode == 3) {
    inv.set_interval_between_refinements((int)interval);
    inv.set_refinement_percentage(fraction);
    inv.set_min_cell_size_in_adaptive_mesh(min_dx, min_dy, min_dz);
  }
  inv.set_stagnation_tolerance(stag);
  inv.set_target_misfit(target);
  inv.set_Lp_inversion_parameter((int)lps, (int)lpx, (int)lpy, (int)lpz, (int)lpt, eps2);
  if (use_crg) {
    write_center_grid("crg_model.xyz", mesh, (int)nx, (int)ny, (int)nz,
                      Eigen::Map<const Eigen::VectorXd>(m0s_v.data(), nm));
    inv.create_crg_model_from_data("crg_model.xyz", (int)nx, (int)ny, (int)nz, "xyz", "xyz");
  }
  if (use_ref) {
    write_center_grid("ref_model.xyz", mesh, (int)nx, (int)ny, (int)nz,
                      Eigen::Map<const Eigen::VectorXd>(m0_v.data(), nm));
    inv.create_ref_model_from_data("ref_model.xyz", (int)nx, (int)ny, (int)nz, "xyz", "xyz");
  }
  inv.set_method_id(1);
  Eigen::VectorXd vmin = Eigen::VectorXd::Constant(nm, m_min);
  Eigen::VectorXd vmax = Eigen::VectorXd::Constant(nm, m_max);
  Eigen::VectorXd vini = Eigen::VectorXd::Constant(nm, m_ini);
  inv.set_min_max(vmin, vmax);
  inv.set_m_ini(vini);
  inv.compute_G();
  if (use_crg) inv.set_structure_model(Eigen::Map<const Eigen::VectorXd>(m0s_v.data(), nm));

  FILE *fo = std::fopen(argv[2], "wb");
  if (!fo) return 6;
  Writer out{fo};
  const Eigen::MatrixXd &G = inv.G_();
  out.i64(G.rows());
  out.i64(G.cols());
  std::fwrite(G.data(), 8, (size_t)(G.rows() * G.cols()), fo);
  out.csr(inv.Ws());
  out.csr(inv.Wx());
  out.csr(inv.Wy());
  out.csr(inv.Wz());
  out.i64(use_crg);
  if (use_crg) {
    out.csr(inv.Tx());
    out.csr(inv.Ty());
    out.csr(inv.Tz());
    out.vec(diag_of(inv.Scrg()));
  }
  out.vec(diag_of(inv.Wd_()));

  if (mode == 1) {
    const double lambda = in.get<double>();
    const double tol = in.get<double>();
    const int64_t maxit = in.get<int64_t>();
    Eigen::VectorXd mk = Eigen::Map<const Eigen::VectorXd>(in.vec(nm).data(), nm);
    Eigen::VectorXd mref = Eigen::Map<const Eigen::VectorXd>(in.vec(nm).data(), nm);
    Eigen::VectorXd P = Eigen::Map<const Eigen::VectorXd>(in.vec(nm).data(), nm);
    std::vector<SMatrix> WL;
    for (int t = 0; t < 7; t++) WL.push_back(diag(Eigen::Map<const Eigen::VectorXd>(in.vec(nm).data(), nm)));
    SMatrix Tx0(nm, nm), Ty0(nm, nm), Tz0(nm, nm);
    if (use_crg) {
      Tx0 = inv.Tx();
      Ty0 = inv.Ty();
      Tz0 = inv.Tz();
    }
    double err = 0.0;
    int iters = 0;
    const int imaxit = (int)maxit;
    Eigen::VectorXd dx = inv.solve_cg(tol, imaxit, err, iters, lambda, mk, mref, inv.Wd_(), dobs,
                                      diag(P), inv.Ws(), inv.Wx(), inv.Wy(), inv.Wz(), Tx0, Ty0,
                                      Tz0, WL[0], WL[1], WL[2], WL[3], WL[4], WL[5], WL[6]);
    out.vec(dx);
    out.f64(err);
    out.i64(iters);
  } else if (mode == 2) {
    inv.invert();
    out.vec(inv.m_());
    out.f64(inv.get_final_misfit());
    out.f64(inv.get_final_lambda());
  } else if (mode == 3) {
    inv.invert();
    Mesh &msh = inv.mesh_();
    const int64_t n = msh.n_elems();
    out.i64(n);
    for (int64_t i = 0; i < n; i++) {
      const Cell *c = msh.leaf_cells[i];
      const double v[6] = {c->_x[0], c->_x[1], c->_y[0], c->_y[1], c->_z[0], c->_z[1]};
      std::fwrite(v, 8, 6, fo);
    }
    out.vec(inv.m_());
    out.f64(inv.get_final_misfit());
    out.f64(inv.get_final_lambda());
  }
  std::fclose(fo);
  std::fclose(fi);
  return 0;
}
