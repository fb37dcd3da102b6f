/*
 * TEST INFRASTRUCTURE ONLY -- the CPU oracle for the prism forward model.
 *
 * This file restates, in plain C, the reference GraAda3D algorithm for the
 * gravity field of a right-rectangular prism: every component is evaluated
 * separately as the difference of two opposite-face surface integrals
 * (Gauss divergence theorem), each face integral being built from per-edge
 * log/atan terms with the reference's 1e-12 singular branches.  It exists to
 * check the CUDA kernels (which use a different, corner-based formulation) and
 * to time the reference's CPU path on the host cores.  Only tests/, the
 * smoke() check and bench.py's CPU-baseline leg may call it; the product path
 * never does.
 *
 * Reference citations are paths inside the GraAda3D project:
 *   src/Forward_modelling/Integral.cpp   (line/surface integrals)
 *   src/Forward_modelling/GravFormula.cpp (component formulae, face lists)
 *   src/Forward_modelling/Point.cpp      (vector helpers)
 *   src/Forward_modelling/gs.h           (constants, field bit layout)
 *   src/Forward_modelling/Fwd.cpp        (sensitivity assembly)
 *   src/compute.cpp                      (forward field sum)
 *
 * Compiled with -ffp-contract=off so that x86 and Arm hosts round alike.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>

/* gs.h:17-25 */
#define OR_TOL 1.000e-12
#define OR_G0 6.673e-11
#define OR_SI2EOTVOS 1000000000.0
#define OR_SI2MGAL 100000.0

typedef struct { double x, y, z; } v3;

static inline v3 v3_make(double x, double y, double z) { v3 r = {x, y, z}; return r; }
static inline v3 v3_sub(v3 a, v3 b) { return v3_make(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 v3_add(v3 a, v3 b) { return v3_make(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 v3_scale(v3 a, double s) { return v3_make(a.x * s, a.y * s, a.z * s); }
/* Point::operator*(const Point&), Point.cpp:78-81 */
static inline double v3_dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
/* Point::size, Point.cpp:208-213 */
static inline double v3_norm(v3 a) { return sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
/* Point::getUnit, Point.cpp:190-195 (Point::unit is the same arithmetic) */
static inline v3 v3_unit(v3 a)
{
  double n = sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
  return v3_make(a.x / n, a.y / n, a.z / n);
}
/* cross, Point.cpp:158-168 */
static inline v3 v3_cross(v3 a, v3 b)
{
  return v3_make(a.y * b.z - b.y * a.z, b.x * a.z - a.x * b.z, a.x * b.y - b.x * a.y);
}
/* unitCross, Point.cpp:171-182 */
static inline v3 v3_unit_cross(v3 a, v3 b) { return v3_unit(v3_cross(a, b)); }
/* Point::distance, Point.cpp:229-234: sqrt of (other - this) squared */
static inline double v3_dist(v3 self, v3 other)
{
  double dx = other.x - self.x, dy = other.y - self.y, dz = other.z - self.z;
  return sqrt(dx * dx + dy * dy + dz * dz);
}
/* Point::projection_line, Point.cpp:222-227 */
static inline v3 v3_project_line(v3 self, v3 p1, v3 p2)
{
  v3 t = v3_unit(v3_sub(p2, p1));
  return v3_add(p1, v3_scale(t, v3_dot(v3_sub(self, p1), t)));
}

/* Integral::getBeta, Integral.cpp:540-572: signed angle sum of a face. */
static double face_beta(v3 ob, const v3 *f)
{
  v3 n = v3_unit_cross(v3_sub(f[1], f[0]), v3_sub(f[2], f[1]));
  double beta = 0.0;
  for (int i = 0; i < 4; i++) {
    int k = (i + 1) % 4;
    v3 t = v3_unit(v3_sub(f[k], f[i]));
    double s0 = v3_dot(v3_sub(f[i], ob), t);
    double s1 = v3_dot(v3_sub(f[k], ob), t);
    v3 m = v3_cross(t, n);
    double mval = v3_dot(m, v3_sub(f[i], ob));
    double mp = v3_dot(m, v3_sub(f[k], ob));
    double tt = (fabs(mp) < OR_TOL) ? 0.0 : (mp > 0 ? 1.0 : -1.0);
    if (fabs(mval) < OR_TOL) {
      beta += 0.0;
    } else {
      beta = beta + tt * (atan(s1 / fabs(mval)) - atan(s0 / fabs(mval)));
    }
  }
  return beta;
}

/* Integral::Surface_R_1, Integral.cpp:593-633: integral of 1/R over a face. */
static double face_inv_r(v3 ob, const v3 *f)
{
  double beta = face_beta(ob, f);
  v3 n = v3_unit_cross(v3_sub(f[1], f[0]), v3_sub(f[3], f[0]));
  double h = v3_dot(v3_sub(ob, f[0]), n);
  double acc = 0.0;
  for (int j = 0; j < 4; j++) {
    int k = (j + 1) % 4;
    v3 t = v3_unit(v3_sub(f[k], f[j]));
    v3 m = v3_unit_cross(t, n);
    double mval = v3_dot(v3_sub(f[j], ob), m);
    double bj = 0.0;
    if (!(fabs(mval) < OR_TOL)) {
      double s0 = v3_dot(t, v3_sub(f[j], ob));
      double s1 = v3_dot(t, v3_sub(f[k], ob));
      double r0 = v3_dist(ob, f[j]);
      double r1 = v3_dist(ob, f[k]);
      bj = fabs(h) * (atan((fabs(h) * s1) / (mval * r1)) - atan((fabs(h) * s0) / (mval * r0))) +
           mval * log((s1 + r1) / (s0 + r0));
    }
    acc += bj;
  }
  return acc - beta * fabs(h);
}

/* Integral::Line_R_1, Integral.cpp:59-85: integral of 1/R along an edge.
 * The reference asserts s0*s1 > 0 in the singular branch; the oracle returns
 * NaN there instead of aborting so a test can report the offending point. */
static double edge_inv_r(v3 ob, v3 v0, v3 v1)
{
  v3 t = v3_unit(v3_sub(v1, v0));
  double s0 = v3_dot(v3_sub(v0, ob), t);
  double s1 = v3_dot(v3_sub(v1, ob), t);
  double r0 = v3_dist(v0, ob);
  double r1 = v3_dist(v1, ob);
  if (fabs(s0 + r0) < OR_TOL) {
    if (!(s0 * s1 > 0)) return NAN;
    return fabs(log(s1 / s0));
  }
  return log((r1 + s1) / (r0 + s0));
}

/* Integral::Surface_R_3, Integral.cpp:764-793: integral of 1/R^3 over a face
 * (valid off the face plane). */
static double face_inv_r3(v3 ob, const v3 *f)
{
  v3 n = v3_unit_cross(v3_sub(f[1], f[0]), v3_sub(f[2], f[1]));
  double h = v3_dot(v3_sub(ob, f[0]), n);
  double acc = 0.0;
  for (int i = 0; i < 4; i++) {
    int k = (i + 1) % 4;
    v3 e = v3_unit(v3_sub(f[k], f[i]));
    v3 m = v3_unit_cross(v3_sub(f[k], f[i]), n);
    v3 prj = v3_project_line(ob, f[k], f[i]);
    double l0 = v3_norm(v3_sub(prj, ob));
    double s1 = v3_dot(v3_sub(f[k], ob), e);
    double s0 = v3_dot(v3_sub(f[i], ob), e);
    double r1 = v3_dist(ob, f[k]);
    double r0 = v3_dist(ob, f[i]);
    double m0 = v3_dot(v3_sub(f[i], ob), m);
    acc += atan((m0 * s1) / (l0 * l0 + fabs(h) * r1)) - atan((m0 * s0) / (l0 * l0 + fabs(h) * r0));
  }
  return acc / fabs(h);
}

/* Integral::Surface_rR_3, Integral.cpp:795-823: integral of (r'-r)/R^3 over a
 * face; the normal part is skipped when the point lies in the face plane. */
static v3 face_r_over_r3(v3 ob, const v3 *f)
{
  v3 n = v3_unit_cross(v3_sub(f[1], f[0]), v3_sub(f[2], f[1]));
  double h = v3_dot(v3_sub(ob, f[0]), n);
  v3 acc = v3_make(0, 0, 0);
  for (int i = 0; i < 4; i++) {
    int k = (i + 1) % 4;
    v3 m = v3_unit_cross(v3_sub(f[k], f[i]), n);
    acc = v3_sub(acc, v3_scale(m, edge_inv_r(ob, f[i], f[k])));
  }
  if (!(fabs(h) < OR_TOL)) {
    double s = face_inv_r3(ob, f);
    acc = v3_sub(acc, v3_scale(v3_scale(n, h), s));
  }
  return acc;
}

/* The eight prism vertices in the reference's numbering, GravFormula.cpp:44-51. */
static void prism_vertices(const double *pr, v3 *p)
{
  double x0 = pr[0], x1 = pr[1], y0 = pr[2], y1 = pr[3], z0 = pr[4], z1 = pr[5];
  p[0] = v3_make(x0, y0, z0);
  p[1] = v3_make(x1, y0, z0);
  p[2] = v3_make(x1, y1, z0);
  p[3] = v3_make(x0, y1, z0);
  p[4] = v3_make(x0, y0, z1);
  p[5] = v3_make(x1, y0, z1);
  p[6] = v3_make(x1, y1, z1);
  p[7] = v3_make(x0, y1, z1);
}

/* Face vertex orders, GravFormula.cpp:53-60 (V) and per component. */
static void make_face(const v3 *p, int a, int b, int c, int d, v3 *f)
{
  f[0] = p[a]; f[1] = p[b]; f[2] = p[c]; f[3] = p[d];
}

/*
 * GravFormula::field_caused_by_single_prism, GravFormula.cpp:2-36, with the
 * component functions of GravFormula.cpp:38-272.  out[10] follows the bit
 * layout of gs.h:46-57: 0 V, 1 gz, 2 gx, 3 gy, 4 Tzz, 5 Txz, 6 Tyz, 7 Txx,
 * 8 Txy, 9 Tyy; components not in mask are 0.
 */
void oracle_prism_field(const double *obs, const double *prism, double rho, uint32_t mask,
                        double *out)
{
  v3 ob = v3_make(obs[0], obs[1], obs[2]);
  v3 p[8];
  prism_vertices(prism, p);
  v3 fx0[4], fx1[4], fy0[4], fy1[4], fz0[4], fz1[4];
  make_face(p, 0, 4, 7, 3, fx0); /* GravFormula.cpp:87 */
  make_face(p, 1, 2, 6, 5, fx1); /* GravFormula.cpp:88 */
  make_face(p, 0, 1, 5, 4, fy0); /* GravFormula.cpp:110 */
  make_face(p, 2, 3, 7, 6, fy1); /* GravFormula.cpp:111 */
  make_face(p, 3, 2, 1, 0, fz0); /* GravFormula.cpp:133 */
  make_face(p, 4, 5, 6, 7, fz1); /* GravFormula.cpp:134 */
  for (int i = 0; i < 10; i++) out[i] = 0.0;

  if (mask & 0x001u) { /* V, GravFormula.cpp:38-73 */
    double h1 = -(p[0].x - ob.x), h2 = p[1].x - ob.x;
    double h3 = -(p[0].y - ob.y), h4 = p[2].y - ob.y;
    double h5 = -(p[0].z - ob.z), h6 = p[6].z - ob.z;
    out[0] += 0.5 * OR_G0 * rho *
              (h1 * face_inv_r(ob, fx0) + h2 * face_inv_r(ob, fx1) + h3 * face_inv_r(ob, fy0) +
               h4 * face_inv_r(ob, fy1) + h5 * face_inv_r(ob, fz0) + h6 * face_inv_r(ob, fz1));
  }
  if (mask & 0x002u) { /* gz, GravFormula.cpp:120-141 */
    double i1 = face_inv_r(ob, fz0), i2 = face_inv_r(ob, fz1);
    out[1] += -OR_SI2MGAL * OR_G0 * rho * (-i1 + i2);
  }
  if (mask & 0x004u) { /* gx, GravFormula.cpp:75-96 */
    double i1 = face_inv_r(ob, fx0), i2 = face_inv_r(ob, fx1);
    out[2] += -OR_SI2MGAL * OR_G0 * rho * (-i1 + i2);
  }
  if (mask & 0x008u) { /* gy, GravFormula.cpp:98-118 */
    double i1 = face_inv_r(ob, fy0), i2 = face_inv_r(ob, fy1);
    out[3] += -OR_SI2MGAL * OR_G0 * rho * (-i1 + i2);
  }
  v3 tx0, tx1, ty0, ty1, tz0, tz1;
  int need_x = (mask & (0x020u | 0x080u | 0x100u)) != 0;
  int need_y = (mask & (0x040u | 0x200u)) != 0;
  int need_z = (mask & 0x010u) != 0;
  if (need_x) { tx0 = face_r_over_r3(ob, fx0); tx1 = face_r_over_r3(ob, fx1); }
  if (need_y) { ty0 = face_r_over_r3(ob, fy0); ty1 = face_r_over_r3(ob, fy1); }
  if (need_z) { tz0 = face_r_over_r3(ob, fz0); tz1 = face_r_over_r3(ob, fz1); }
  if (mask & 0x010u) out[4] += -OR_SI2EOTVOS * OR_G0 * rho * (-tz0.z + tz1.z); /* Tzz :251-272 */
  if (mask & 0x020u) out[5] += -OR_SI2EOTVOS * OR_G0 * rho * (-tx0.z + tx1.z); /* Txz :183-203 */
  if (mask & 0x040u) out[6] += -OR_SI2EOTVOS * OR_G0 * rho * (-ty0.z + ty1.z); /* Tyz :228-249 */
  if (mask & 0x080u) out[7] += -OR_SI2EOTVOS * OR_G0 * rho * (-tx0.x + tx1.x); /* Txx :143-163 */
  if (mask & 0x100u) out[8] += -OR_SI2EOTVOS * OR_G0 * rho * (-tx0.y + tx1.y); /* Txy :164-182 */
  if (mask & 0x200u) out[9] += -OR_SI2EOTVOS * OR_G0 * rho * (-ty0.y + ty1.y); /* Tyy :205-226 */
}

static int mask_components(uint32_t mask, int *idx)
{
  int n = 0;
  for (int b = 0; b < 10; b++)
    if (mask & (1u << b)) idx[n++] = b;
  return n;
}

/*
 * Fwd::compute_G, Fwd.cpp:47-78.  G is column-major with leading dimension
 * ld >= n_fields*n_obs; row i + k*n_obs holds component k (ascending bit
 * order) at observation i, column j is cell j.  Like the reference, the
 * observation loop is serial and the cell loop is OpenMP-parallel.
 */
void oracle_compute_G(const double *prisms, int64_t n_cells, const double *obs, int64_t n_obs,
                      uint32_t mask, double *G, int64_t ld)
{
  int idx[10];
  int nf = mask_components(mask, idx);
  for (int64_t i = 0; i < n_obs; i++) {
#pragma omp parallel for schedule(static)
    for (int64_t j = 0; j < n_cells; j++) {
      double f[10];
      oracle_prism_field(obs + 3 * i, prisms + 6 * j, 1.0, mask, f);
      for (int k = 0; k < nf; k++) G[(i + k * n_obs) + j * ld] = f[idx[k]];
    }
  }
}

/*
 * The forward field sum of compute.cpp:246-260: out[i*n_fields + k] is the
 * sum over cells of rho_j * field_k(obs_i, cell_j), accumulated in cell order.
 * OpenMP-parallel over observations as in the reference.
 */
void oracle_forward_field(const double *prisms, const double *rho, int64_t n_cells,
                          const double *obs, int64_t n_obs, uint32_t mask, double *out)
{
  int idx[10];
  int nf = mask_components(mask, idx);
#pragma omp parallel for schedule(dynamic, 4)
  for (int64_t i = 0; i < n_obs; i++) {
    double acc[10] = {0};
    for (int64_t j = 0; j < n_cells; j++) {
      double f[10];
      oracle_prism_field(obs + 3 * i, prisms + 6 * j, rho[j], mask, f);
      for (int k = 0; k < nf; k++) acc[k] += f[idx[k]];
    }
    for (int k = 0; k < nf; k++) out[i * nf + k] = acc[k];
  }
}

/* Number of OpenMP threads the oracle would use (for reporting). */
int oracle_num_threads(void)
{
#ifdef _OPENMP
  extern int omp_get_max_threads(void);
  return omp_get_max_threads();
#else
  return 1;
#endif
}
