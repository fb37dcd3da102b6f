// Closed-form gravity field of a right-rectangular prism, evaluated jointly for
// all requested components from the prism's eight corners.
//
// Reference: GravFormula::field_caused_by_single_prism and the component
// functions (src/Forward_modelling/GravFormula.cpp:2-272).  The reference
// evaluates each component on its own as the difference of two opposite-face
// surface integrals (Integral.cpp:540-823), about 32 atan + 8 log per
// component.  Here the same fields come from the triple antiderivatives of
// 1/r at the corners (X, Y, Z) = corner - observation, z positive down,
// r = |(X, Y, Z)|, sigma = -1/+1 for the lower/upper limit of each axis and
// S = sigma_i sigma_j sigma_k:
//
//   V   =  G0 sum S [XY ln(Z+r) + YZ ln(X+r) + ZX ln(Y+r)
//                    - X^2/2 atan(YZ/(Xr)) - Y^2/2 atan(ZX/(Yr)) - Z^2/2 atan(XY/(Zr))]
//   gz  = -G0 sum S [X ln(Y+r) + Y ln(X+r) - Z atan(XY/(Zr))]      (and cyclic gx, gy)
//   Tzz = -G0 sum S atan(XY/(Zr)),  Txx, Tyy cyclic
//   Txz =  G0 sum S ln(Y+r),  Tyz = G0 sum S ln(X+r),  Txy = G0 sum S ln(Z+r)
//
// (times 1e5 for mGal and 1e9 for Eotvos, as GravFormula.h:6-14).
//
// Work sharing between components:
//  * the eight-term sums of ln(A+r) are regrouped per prism edge: for the edge
//    along axis A at fixed other two corner indices, ln(A1+r1) - ln(A0+r0) is
//    ONE log of a ratio (12 logs per prism serve all ten components instead of
//    24 corner logs), and the ratio is formed without cancellation (for A<0,
//    A+r = rho^2/(r-A), rho^2 the squared distance to the edge line);
//  * the four-term sums of atan per face are the argument of a product of four
//    complex numbers (Z r + i X Y or its conjugate), so each face costs one
//    atan2; the 2*pi branch of that argument is picked with a cheap FP32
//    estimate of the same sum (6 FP64 atan2 per prism instead of 24 atan).
// Every quantity that reaches a result is computed in FP64.
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

namespace grada {

constexpr double kG0 = 6.673e-11;           // gs.h:20
constexpr double kSI2mGal = 100000.0;       // gs.h:25
constexpr double kSI2Eotvos = 1000000000.0; // gs.h:24
constexpr double kTwoPi = 6.283185307179586476925286766559;

// Field bits (gs.h:46-57).
enum : uint32_t {
  F_V = 0x001u, F_GZ = 0x002u, F_GX = 0x004u, F_GY = 0x008u, F_TZZ = 0x010u,
  F_TXZ = 0x020u, F_TYZ = 0x040u, F_TXX = 0x080u, F_TXY = 0x100u, F_TYY = 0x200u,
  F_ALL = 0x3FFu
};

// Families of transcendental terms a component needs.
enum : uint32_t {
  FAM_LX = 1u,  // ln(X+r): gy, gz, Tyz, V
  FAM_LY = 2u,  // ln(Y+r): gx, gz, Txz, V
  FAM_LZ = 4u,  // ln(Z+r): gx, gy, Txy, V
  FAM_AX = 8u,  // atan(YZ/(Xr)): gx, Txx, V
  FAM_AY = 16u, // atan(ZX/(Yr)): gy, Tyy, V
  FAM_AZ = 32u  // atan(XY/(Zr)): gz, Tzz, V
};

__host__ __device__ inline uint32_t families_for_mask(uint32_t m) {
  uint32_t f = 0;
  if (m & (F_V | F_GY | F_GZ | F_TYZ)) f |= FAM_LX;
  if (m & (F_V | F_GX | F_GZ | F_TXZ)) f |= FAM_LY;
  if (m & (F_V | F_GX | F_GY | F_TXY)) f |= FAM_LZ;
  if (m & (F_V | F_GX | F_TXX)) f |= FAM_AX;
  if (m & (F_V | F_GY | F_TYY)) f |= FAM_AY;
  if (m & (F_V | F_GZ | F_TZZ)) f |= FAM_AZ;
  return f;
}

// ln((a1 + r1) / (a0 + r0)) along one edge, a0 <= a1 the edge's end
// coordinates relative to the point, r0/r1 the corner distances, perp2 the
// squared distance from the point to the edge line.  Each factor a + r with
// a < 0 is rewritten as perp2 / (r - a), so no subtraction of near-equal
// numbers happens in any branch.
__device__ __forceinline__ double edge_log_ratio(double a0, double a1, double r0, double r1,
                                                 double perp2) {
  double num, den;
  if (a0 >= 0.0) {
    num = a1 + r1;
    den = a0 + r0;
  } else if (a1 < 0.0) {
    num = r0 - a0;
    den = r1 - a1;
  } else {
    num = (a1 + r1) * (r0 - a0);
    den = perp2;
  }
  return log(num / den);
}

// Normalises (a, b) so that arg(a + i b) equals atan(b / a) as the corner
// formula uses it (a < 0 flips both parts; 0/0 at a corner on an edge line of
// the face's axis is taken as 0, which cancels between the two faces it
// touches).
__device__ __forceinline__ void atan_factor(double &a, double &b) {
  if (a < 0.0) {
    a = -a;
    b = -b;
  }
  if (a == 0.0 && b == 0.0) a = 1.0;
}

// sum_c s_c atan(b_c / a_c) over the four corners of a face, signs (+,-,-,+)
// for corners (00, 01, 10, 11).  FP64 argument of the complex product; the
// multiple of 2*pi comes from an FP32 sum of the four atan2f.
__device__ __forceinline__ double face_atan_sum(double a00, double b00, double a01, double b01,
                                                double a10, double b10, double a11, double b11) {
  atan_factor(a00, b00);
  atan_factor(a01, b01);
  atan_factor(a10, b10);
  atan_factor(a11, b11);
  b01 = -b01;  // conjugate the negative-sign corners
  b10 = -b10;
  double re = fma(a00, a01, -b00 * b01);
  double im = fma(a00, b01, b00 * a01);
  double re2 = fma(re, a10, -im * b10);
  double im2 = fma(re, b10, im * a10);
  double re3 = fma(re2, a11, -im2 * b11);
  double im3 = fma(re2, b11, im2 * a11);
  double theta = atan2(im3, re3);
  float est = atan2f((float)b00, (float)a00) + atan2f((float)b01, (float)a01) +
              atan2f((float)b10, (float)a10) + atan2f((float)b11, (float)a11);
  float turns = rintf((est - (float)theta) * 0.15915494309189535f);
  return fma((double)turns, kTwoPi, theta);
}

// Unscaled per-prism sums shared by the components (see the header comment).
struct PrismTerms {
  double qx[2][2];  // [j][k] sum_i sigma_i ln(X_i + r)
  double qy[2][2];  // [i][k] sum_j sigma_j ln(Y_j + r)
  double qz[2][2];  // [i][j] sum_k sigma_k ln(Z_k + r)
  double tx[2];     // [i] sum_jk sigma_j sigma_k atan(Y_j Z_k / (X_i r))
  double ty[2];     // [j] sum_ik sigma_i sigma_k atan(X_i Z_k / (Y_j r))
  double tz[2];     // [k] sum_ij sigma_i sigma_j atan(X_i Y_j / (Z_k r))
  double X[2], Y[2], Z[2];
};

__device__ __forceinline__ void prism_terms(double px, double py, double pz, double x0, double x1,
                                            double y0, double y1, double z0, double z1,
                                            uint32_t fam, PrismTerms &t) {
  t.X[0] = x0 - px; t.X[1] = x1 - px;
  t.Y[0] = y0 - py; t.Y[1] = y1 - py;
  t.Z[0] = z0 - pz; t.Z[1] = z1 - pz;
  const double X2[2] = {t.X[0] * t.X[0], t.X[1] * t.X[1]};
  const double Y2[2] = {t.Y[0] * t.Y[0], t.Y[1] * t.Y[1]};
  const double Z2[2] = {t.Z[0] * t.Z[0], t.Z[1] * t.Z[1]};
  double r[2][2][2];
#pragma unroll
  for (int i = 0; i < 2; i++)
#pragma unroll
    for (int j = 0; j < 2; j++) {
      const double xy = X2[i] + Y2[j];
#pragma unroll
      for (int k = 0; k < 2; k++) r[i][j][k] = sqrt(xy + Z2[k]);
    }
  if (fam & FAM_LX) {
#pragma unroll
    for (int j = 0; j < 2; j++)
#pragma unroll
      for (int k = 0; k < 2; k++)
        t.qx[j][k] = edge_log_ratio(t.X[0], t.X[1], r[0][j][k], r[1][j][k], Y2[j] + Z2[k]);
  }
  if (fam & FAM_LY) {
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
      for (int k = 0; k < 2; k++)
        t.qy[i][k] = edge_log_ratio(t.Y[0], t.Y[1], r[i][0][k], r[i][1][k], X2[i] + Z2[k]);
  }
  if (fam & FAM_LZ) {
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
      for (int j = 0; j < 2; j++)
        t.qz[i][j] = edge_log_ratio(t.Z[0], t.Z[1], r[i][j][0], r[i][j][1], X2[i] + Y2[j]);
  }
  if (fam & FAM_AX) {
    const double yz00 = t.Y[0] * t.Z[0], yz01 = t.Y[0] * t.Z[1];
    const double yz10 = t.Y[1] * t.Z[0], yz11 = t.Y[1] * t.Z[1];
#pragma unroll
    for (int i = 0; i < 2; i++)
      t.tx[i] = face_atan_sum(t.X[i] * r[i][0][0], yz00, t.X[i] * r[i][0][1], yz01,
                              t.X[i] * r[i][1][0], yz10, t.X[i] * r[i][1][1], yz11);
  }
  if (fam & FAM_AY) {
    const double xz00 = t.X[0] * t.Z[0], xz01 = t.X[0] * t.Z[1];
    const double xz10 = t.X[1] * t.Z[0], xz11 = t.X[1] * t.Z[1];
#pragma unroll
    for (int j = 0; j < 2; j++)
      t.ty[j] = face_atan_sum(t.Y[j] * r[0][j][0], xz00, t.Y[j] * r[0][j][1], xz01,
                              t.Y[j] * r[1][j][0], xz10, t.Y[j] * r[1][j][1], xz11);
  }
  if (fam & FAM_AZ) {
    const double xy00 = t.X[0] * t.Y[0], xy01 = t.X[0] * t.Y[1];
    const double xy10 = t.X[1] * t.Y[0], xy11 = t.X[1] * t.Y[1];
#pragma unroll
    for (int k = 0; k < 2; k++)
      t.tz[k] = face_atan_sum(t.Z[k] * r[0][0][k], xy00, t.Z[k] * r[0][1][k], xy01,
                              t.Z[k] * r[1][0][k], xy10, t.Z[k] * r[1][1][k], xy11);
  }
}

// sum over two indices with signs sigma_a sigma_b of c_ab q_ab where
// c_ab = u_a (or v_b); helpers keep the sign pattern (+,-,-,+) in one place.
__device__ __forceinline__ double signed4(const double q[2][2]) {
  return (q[1][1] - q[1][0]) - (q[0][1] - q[0][0]);
}
__device__ __forceinline__ double signed4_first(const double q[2][2], const double u[2]) {
  return u[1] * (q[1][1] - q[1][0]) - u[0] * (q[0][1] - q[0][0]);
}
__device__ __forceinline__ double signed4_second(const double q[2][2], const double v[2]) {
  return v[1] * (q[1][1] - q[0][1]) - v[0] * (q[1][0] - q[0][0]);
}
__device__ __forceinline__ double signed2(const double t[2], const double u[2]) {
  return u[1] * t[1] - u[0] * t[0];
}
__device__ __forceinline__ double signed2(const double t[2]) { return t[1] - t[0]; }

// Writes component value `b` (field bit index) for unit density.
__device__ __forceinline__ double prism_component(const PrismTerms &t, int b) {
  const double cg = -kSI2mGal * kG0;    // GravFormula.cpp:94/116/139 with rho = 1
  const double cT = -kSI2Eotvos * kG0;  // GravFormula.cpp:161-270 with rho = 1
  switch (b) {
    case 0: {  // V
      const double XY[2][2] = {{t.X[0] * t.Y[0], t.X[0] * t.Y[1]}, {t.X[1] * t.Y[0], t.X[1] * t.Y[1]}};
      const double YZ[2][2] = {{t.Y[0] * t.Z[0], t.Y[0] * t.Z[1]}, {t.Y[1] * t.Z[0], t.Y[1] * t.Z[1]}};
      const double ZX[2][2] = {{t.X[0] * t.Z[0], t.X[0] * t.Z[1]}, {t.X[1] * t.Z[0], t.X[1] * t.Z[1]}};
      double s = 0.0;
#pragma unroll
      for (int a = 0; a < 2; a++)
#pragma unroll
        for (int c = 0; c < 2; c++) {
          const double sg = (a == c) ? 1.0 : -1.0;
          s += sg * (XY[a][c] * t.qz[a][c] + YZ[a][c] * t.qx[a][c] + ZX[a][c] * t.qy[a][c]);
        }
      const double X2[2] = {t.X[0] * t.X[0], t.X[1] * t.X[1]};
      const double Y2[2] = {t.Y[0] * t.Y[0], t.Y[1] * t.Y[1]};
      const double Z2[2] = {t.Z[0] * t.Z[0], t.Z[1] * t.Z[1]};
      s -= 0.5 * (signed2(t.tx, X2) + signed2(t.ty, Y2) + signed2(t.tz, Z2));
      return kG0 * s;
    }
    case 1:  // gz = -G0 sum S [X ln(Y+r) + Y ln(X+r) - Z atan(XY/(Zr))]
      return cg * (signed4_first(t.qy, t.X) + signed4_first(t.qx, t.Y) - signed2(t.tz, t.Z));
    case 2:  // gx
      return cg * (signed4_second(t.qz, t.Y) + signed4_second(t.qy, t.Z) - signed2(t.tx, t.X));
    case 3:  // gy
      return cg * (signed4_second(t.qx, t.Z) + signed4_first(t.qz, t.X) - signed2(t.ty, t.Y));
    case 4:  // Tzz
      return cT * signed2(t.tz);
    case 5:  // Txz
      return -cT * signed4(t.qy);
    case 6:  // Tyz
      return -cT * signed4(t.qx);
    case 7:  // Txx
      return cT * signed2(t.tx);
    case 8:  // Txy
      return -cT * signed4(t.qz);
    default:  // 9 Tyy
      return cT * signed2(t.ty);
  }
}

}  // namespace grada
