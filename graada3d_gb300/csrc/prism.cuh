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
//    argument evaluation (6 per prism instead of 24 atan), done by the
//    table rotation below; the 2*pi branch is picked with a cheap FP32
//    estimate of the same sum;
//  * faces shared by neighbouring cells (a column in z, and with
//    prism_terms_tiled also the previous cells in y and x) are taken over
//    from the neighbour instead of being evaluated again.
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

// ---------------------------------------------------------------------------
// FP64 logarithm and face-angle sums with few FP64 instructions.
//
// On GB300 the FP64 pipe is the bottleneck of this kernel while the FP32 and
// integer pipes are idle, so the two transcendental kernels below are written
// to spend FP64 instructions only where FP64 accuracy is needed:
//  * log: table-driven reduction (P. T. P. Tang, "Table-driven implementation
//    of the logarithm function in IEEE floating-point arithmetic", ACM TOMS
//    16(4), 1990): q = 2^e m, m in [0.75, 1.5]; the table entry c_k is near
//    1/m (193 bins of width 1/256 centred on 0.75 + k/256; the bin of 1.0 has
//    c = 1 exactly), so t = m c_k - 1 is one FMA, |t| < 0.0027, and
//    ln q = e ln2 + ln(1/c_k) + ln(1+t) with the Taylor series of ln(1+t) to
//    t^6 (truncation below 4.5e-17 relative).  ln2 and ln(1/c_k) carry a low
//    part, so q near 1 keeps full relative accuracy.  The exponent and bin
//    come from integer operations on the bits.
//  * face angle sums: the FP32 estimate of the sum (which is needed anyway
//    for the 2*pi branch) picks theta_j = j*pi/128 nearest to it; the FP64
//    complex product is rotated by -theta_j (cos/sin table), leaving an
//    argument below pi/256 + 1e-6 whose arctangent is a short odd series
//    (to delta^7; the first term left out, delta^9/9, is below 5.4e-17 of
//    delta).  Sum = theta_j + atan(delta).
// The tables are built once per context on the host in extended precision
// (build_math_tables) and staged into shared memory by each block.
// ---------------------------------------------------------------------------

constexpr int kLogBins = 193;                   // k = 0..192, centres 0.75 + k/256
constexpr int kTabLog = 0;                      // [c, ln(1/c) hi, ln(1/c) lo] x 97
constexpr int kRotSteps = 256;                  // table angles j*pi/128, j = 0..255
constexpr int kTabSinCos = kTabLog + 3 * kLogBins;  // [cos, sin] of j*pi/128
constexpr int kTabConst = kTabSinCos + 2 * kRotSteps;  // ln2 hi/lo, pi/128 hi/lo
constexpr int kTabSize = kTabConst + 4;

// Fills `tab` (kTabSize doubles).  Host only.
void build_math_tables(double *tab);

// Sign tests on the bit pattern: integer instructions instead of FP64
// compares, which would take FP64-pipe slots.  Exact for every non-NaN double
// (-0.0 is not negative).
__device__ __forceinline__ bool neg_strict(double v) {
  return (unsigned long long)__double_as_longlong(v) > 0x8000000000000000ull;
}
__device__ __forceinline__ bool both_zero(double a, double b) {
  return (((unsigned long long)__double_as_longlong(a) |
           (unsigned long long)__double_as_longlong(b)) << 1) == 0ull;
}

// Exact int -> double for |v| < 2^21 from integer instructions (the
// conversion instruction would take an FP64-pipe slot): exponent from the
// leading-zero count, the bits below the leading one as the fraction.
__device__ __forceinline__ double small_int_to_double(int v) {
  if (v == 0) return 0.0;
  const unsigned s = v < 0 ? 0x80000000u : 0u;
  const unsigned u = v < 0 ? 0u - (unsigned)v : (unsigned)v;
  const int lz = __clz(u);  // 11..31
  const unsigned hi = s | ((unsigned)(1054 - lz) << 20) | ((u ^ (0x80000000u >> lz)) << (lz - 11));
  return __hiloint2double((int)hi, 0);
}

// double -> float rounded to nearest even, as the conversion instruction does,
// from integer instructions where the result is a normal float; zero, and
// anything that rounds to a subnormal, infinity or NaN, takes the instruction.
__device__ __forceinline__ float double_to_float_rn(double v) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  const unsigned hi = (unsigned)(b >> 32);
  const unsigned ex = (hi >> 20) & 0x7FFu;
  if (ex - 897u > 253u) {  // float exponent ex - 896 outside [1, 254]
    if ((b << 1) == 0ull) return __uint_as_float(hi & 0x80000000u);
    return (float)v;
  }
  const unsigned long long mant = b & 0x000FFFFFFFFFFFFFull;
  unsigned f = ((ex - 896u) << 23) | (unsigned)(mant >> 29);
  const unsigned rem = (unsigned)mant & 0x1FFFFFFFu;
  f += (rem > 0x10000000u || (rem == 0x10000000u && (f & 1u))) ? 1u : 0u;  // carries into
  return __uint_as_float((hi & 0x80000000u) | f);                          // the exponent
}

__device__ __forceinline__ double fast_log(double q, const double *__restrict__ tab) {
  // q outside [DBL_MIN, DBL_MAX] (zero, subnormal, negative, inf, NaN), tested
  // on the high word: the library log handles those
  if ((unsigned)__double2hiint(q) - 0x00100000u >= 0x7FE00000u) return log(q);
  const long long bits = __double_as_longlong(q);
  const long long f = bits & 0x000FFFFFFFFFFFFFll;
  int e = (int)(bits >> 52) - 1023;
  long long mbits;
  int k;
  if (f >= (1ll << 51)) {  // m_raw >= 1.5: halve into [0.75, 1)
    mbits = (1022ll << 52) | f;
    e += 1;
    k = (int)((f + (1ll << 44)) >> 45) - 64;
  } else {
    mbits = (1023ll << 52) | f;
    k = 64 + (int)((f + (1ll << 43)) >> 44);
  }
  const double m = __longlong_as_double(mbits);
  const double *L = tab + kTabLog + 3 * k;
  const double t = fma(m, L[0], -1.0);
  const double t2 = t * t;
  double p = -1.0 / 6.0;
  p = fma(p, t, 1.0 / 5.0);
  p = fma(p, t, -1.0 / 4.0);
  p = fma(p, t, 1.0 / 3.0);
  p = fma(p, t, -0.5);
  const double l1p = fma(t2, p, t);
  const double ed = small_int_to_double(e);
  const double hi = fma(ed, tab[kTabConst + 0], L[1]);
  const double lo = fma(ed, tab[kTabConst + 1], L[2]);
  return hi + (l1p + lo);
}

// 1/x without the correctly rounded division sequence: the hardware seed
// y0 = rcp.approx.ftz.f64(x) (relative error e = 1 - x y0 below 2^-19.9,
// measured on GB300 over 4M inputs spread across 2^-60..2^60) refined by the
// series 1/x = y0 / (1 - e) = y0 (1 + e + e^2 + ...) cut after e^2
// (M. J. Flynn, "On division by functional iteration", IEEE Trans. Computers
// C-19(8), 1970): truncation e^3 < 2^-59, so within ~0.5 ulp.  Three FP64
// instructions; x outside 2^-1000..2^1000 (zero, subnormal, inf, NaN) takes
// the correctly rounded reciprocal.
__device__ __forceinline__ double fast_rcp(double x) {
  const unsigned hx = (unsigned)__double2hiint(x) & 0x7FFFFFFFu;
  if (hx - 0x01700000u >= 0x7D100000u) return __drcp_rn(x);
  double y0;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y0) : "d"(x));
  const double e = fma(-x, y0, 1.0);
  return fma(y0, fma(e, e, e), y0);
}

// sqrt(x) the same way: seed y0 = rsqrt.approx.ftz.f64(x) (relative error
// below 2^-20, measured as for the reciprocal), t = x y0 ~ sqrt(x) and
// e = 1 - t y0 = 1 - x y0^2, then sqrt(x) = t (1 - e)^(-1/2) with the binomial
// series t (1 + e/2 + 3e^2/8 + ...) cut after e^2 (|e| < 2^-19, truncation
// below 2^-58; the rounding of t adds half of its own 2^-53).  Five FP64
// instructions; x outside 2^-1000..2^1000 or negative takes sqrt().
__device__ __forceinline__ double fast_sqrt(double x) {
  const unsigned hx = (unsigned)__double2hiint(x);
  if (hx - 0x01700000u >= 0x7D100000u) return sqrt(x);
  double y0;
  asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y0) : "d"(x));
  const double t = x * y0;
  const double e = fma(-t, y0, 1.0);
  const double p = fma(e, 0.375, 0.5) * e;
  return fma(t, p, t);
}

// ln((a1 + r1) / (a0 + r0)) along one edge, a0 <= a1 the edge's end
// coordinates relative to the point, r0/r1 the corner distances, perp2 the
// squared distance from the point to the edge line.  Each factor a + r with
// a < 0 is rewritten as perp2 / (r - a), so no subtraction of near-equal
// numbers happens in any branch.
__device__ __forceinline__ double edge_log_ratio(double a0, double a1, double r0, double r1,
                                                 double perp2, const double *__restrict__ tab) {
  double num, den;
  if (!neg_strict(a0)) {
    num = a1 + r1;
    den = a0 + r0;
  } else if (neg_strict(a1)) {
    num = r0 - a0;
    den = r1 - a1;
  } else {
    num = (a1 + r1) * (r0 - a0);
    den = perp2;
  }
  return fast_log(num * fast_rcp(den), tab);
}

// Normalises (a, b) so that arg(a + i b) equals atan(b / a) as the corner
// formula uses it (a < 0 flips both parts; 0/0 at a corner on an edge line of
// the face's axis is taken as 0, which cancels between the two faces it
// touches).  Applied to the FP32 estimate of a face sum.
template <typename T>
__device__ __forceinline__ void atan_factor(T &a, T &b) {
  if (a < T(0)) {
    a = -a;
    b = -b;
  }
  if (a == T(0) && b == T(0)) a = T(1);
}

// sum_c s_c atan(b_c / a_c) over the four corners of a face, signs (+,-,-,+)
// for corners (00, 01, 10, 11).  (a, b) in FP64, (af, bf) the same in FP32.
// The FP64 factors skip the sign normalisation of atan_factor (a < 0 flips
// both parts): a flipped factor negates the product and so both rotated parts
// xr, yr exactly (round-to-nearest is symmetric), leaving d = yr / xr
// bitwise unchanged.  Only the FP32 estimate, which picks the table angle
// and the 2*pi branch, needs the principal values.  The 0/0 rule stays.
__device__ __forceinline__ double face_atan_sum(const double (&a)[4], const double (&b)[4],
                                                const float (&af)[4], const float (&bf)[4],
                                                const double *__restrict__ tab) {
  double A[4], B[4];
  float est = 0.f;
#pragma unroll
  for (int c = 0; c < 4; c++) {
    A[c] = both_zero(a[c], b[c]) ? 1.0 : a[c];
    B[c] = b[c];
    float x = af[c], y = bf[c];
    atan_factor(x, y);
    const bool neg = (c == 1 || c == 2);  // conjugate the negative-sign corners
    if (neg) {
      B[c] = -B[c];
      y = -y;
    }
    est += atan2f(y, x);
  }
  double re = fma(A[0], A[1], -B[0] * B[1]);
  double im = fma(A[0], B[1], B[0] * A[1]);
  double re2 = fma(re, A[2], -im * B[2]);
  double im2 = fma(re, B[2], im * A[2]);
  const double re3 = fma(re2, A[3], -im2 * B[3]);
  const double im3 = fma(re2, B[3], im2 * A[3]);
  // rotate by -j*pi/64, j nearest to the FP32 estimate of the sum
  const int j = __float2int_rn(est * 40.743665431525208f);  // 128/pi
  const double *cs = tab + kTabSinCos + 2 * (j & (kRotSteps - 1));
  const double c = cs[0], s = cs[1];
  const double xr = fma(re3, c, im3 * s);
  const double yr = fma(im3, c, -re3 * s);
  const double d = yr * fast_rcp(xr);
  const double d2 = d * d;
  double p = -1.0 / 7.0;
  p = fma(p, d2, 1.0 / 5.0);
  p = fma(p, d2, -1.0 / 3.0);
  const double at = fma(d * d2, p, d);
  const double jd = small_int_to_double(j);
  return fma(jd, tab[kTabConst + 2], fma(jd, tab[kTabConst + 3], at));
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

// Quantities of a cell's bottom face (z1) that the next cell of the same
// vertical column (same x/y extent, its z0 equal to this z1) needs for its top
// face: corner distances, the x/y-edge log ratios and the z-face angle sum.
// Reusing them is exact (the same FP64 operands give the same values) and
// saves 4 sqrt, 4 logs and 1 angle sum per cell of a column.
struct ZCarry {
  double r[2][2];
  double qx[2];
  double qy[2];
  double tz;
};

__device__ __forceinline__ void prism_terms(double px, double py, double pz, double x0, double x1,
                                            double y0, double y1, double z0, double z1,
                                            uint32_t fam, const double *__restrict__ tab,
                                            bool reuse_top, ZCarry &carry, PrismTerms &t) {
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
      r[i][j][0] = reuse_top ? carry.r[i][j] : fast_sqrt(xy + Z2[0]);
      r[i][j][1] = fast_sqrt(xy + Z2[1]);
    }
  if (fam & FAM_LX) {
#pragma unroll
    for (int j = 0; j < 2; j++) {
      t.qx[j][0] = reuse_top ? carry.qx[j]
                             : edge_log_ratio(t.X[0], t.X[1], r[0][j][0], r[1][j][0],
                                              Y2[j] + Z2[0], tab);
      t.qx[j][1] = edge_log_ratio(t.X[0], t.X[1], r[0][j][1], r[1][j][1], Y2[j] + Z2[1], tab);
    }
  }
  if (fam & FAM_LY) {
#pragma unroll
    for (int i = 0; i < 2; i++) {
      t.qy[i][0] = reuse_top ? carry.qy[i]
                             : edge_log_ratio(t.Y[0], t.Y[1], r[i][0][0], r[i][1][0],
                                              X2[i] + Z2[0], tab);
      t.qy[i][1] = edge_log_ratio(t.Y[0], t.Y[1], r[i][0][1], r[i][1][1], X2[i] + Z2[1], tab);
    }
  }
  if (fam & FAM_LZ) {
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
      for (int j = 0; j < 2; j++)
        t.qz[i][j] = edge_log_ratio(t.Z[0], t.Z[1], r[i][j][0], r[i][j][1], X2[i] + Y2[j], tab);
  }
  if (!(fam & (FAM_AX | FAM_AY | FAM_AZ))) {
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
      for (int j = 0; j < 2; j++) carry.r[i][j] = r[i][j][1];
    if (fam & FAM_LX) {
      carry.qx[0] = t.qx[0][1];
      carry.qx[1] = t.qx[1][1];
    }
    if (fam & FAM_LY) {
      carry.qy[0] = t.qy[0][1];
      carry.qy[1] = t.qy[1][1];
    }
    return;
  }
  // FP32 copies for the branch/rotation estimates of the face angle sums
  // (6 conversions, by integer instructions; the rest of the estimate runs on the FP32 pipe).
  const float Xf[2] = {double_to_float_rn(t.X[0]), double_to_float_rn(t.X[1])};
  const float Yf[2] = {double_to_float_rn(t.Y[0]), double_to_float_rn(t.Y[1])};
  const float Zf[2] = {double_to_float_rn(t.Z[0]), double_to_float_rn(t.Z[1])};
  float rf[2][2][2];
#pragma unroll
  for (int i = 0; i < 2; i++)
#pragma unroll
    for (int j = 0; j < 2; j++)
#pragma unroll
      for (int k = 0; k < 2; k++)
        rf[i][j][k] = sqrtf(fmaf(Xf[i], Xf[i], fmaf(Yf[j], Yf[j], Zf[k] * Zf[k])));
  if (fam & FAM_AX) {
    const double b[4] = {t.Y[0] * t.Z[0], t.Y[0] * t.Z[1], t.Y[1] * t.Z[0], t.Y[1] * t.Z[1]};
    const float bf[4] = {Yf[0] * Zf[0], Yf[0] * Zf[1], Yf[1] * Zf[0], Yf[1] * Zf[1]};
#pragma unroll
    for (int i = 0; i < 2; i++) {
      const double a[4] = {t.X[i] * r[i][0][0], t.X[i] * r[i][0][1], t.X[i] * r[i][1][0],
                           t.X[i] * r[i][1][1]};
      const float af[4] = {Xf[i] * rf[i][0][0], Xf[i] * rf[i][0][1], Xf[i] * rf[i][1][0],
                           Xf[i] * rf[i][1][1]};
      t.tx[i] = face_atan_sum(a, b, af, bf, tab);
    }
  }
  if (fam & FAM_AY) {
    const double b[4] = {t.X[0] * t.Z[0], t.X[0] * t.Z[1], t.X[1] * t.Z[0], t.X[1] * t.Z[1]};
    const float bf[4] = {Xf[0] * Zf[0], Xf[0] * Zf[1], Xf[1] * Zf[0], Xf[1] * Zf[1]};
#pragma unroll
    for (int j = 0; j < 2; j++) {
      const double a[4] = {t.Y[j] * r[0][j][0], t.Y[j] * r[0][j][1], t.Y[j] * r[1][j][0],
                           t.Y[j] * r[1][j][1]};
      const float af[4] = {Yf[j] * rf[0][j][0], Yf[j] * rf[0][j][1], Yf[j] * rf[1][j][0],
                           Yf[j] * rf[1][j][1]};
      t.ty[j] = face_atan_sum(a, b, af, bf, tab);
    }
  }
  if (fam & FAM_AZ) {
    const double b[4] = {t.X[0] * t.Y[0], t.X[0] * t.Y[1], t.X[1] * t.Y[0], t.X[1] * t.Y[1]};
    const float bf[4] = {Xf[0] * Yf[0], Xf[0] * Yf[1], Xf[1] * Yf[0], Xf[1] * Yf[1]};
#pragma unroll
    for (int k = 0; k < 2; k++) {
      if (k == 0 && reuse_top) {
        t.tz[0] = carry.tz;
        continue;
      }
      const double a[4] = {t.Z[k] * r[0][0][k], t.Z[k] * r[0][1][k], t.Z[k] * r[1][0][k],
                           t.Z[k] * r[1][1][k]};
      const float af[4] = {Zf[k] * rf[0][0][k], Zf[k] * rf[0][1][k], Zf[k] * rf[1][0][k],
                           Zf[k] * rf[1][1][k]};
      t.tz[k] = face_atan_sum(a, b, af, bf, tab);
    }
  }
  // hand the bottom face to the next cell of the column
#pragma unroll
  for (int i = 0; i < 2; i++)
#pragma unroll
    for (int j = 0; j < 2; j++) carry.r[i][j] = r[i][j][1];
  if (fam & FAM_LX) {
    carry.qx[0] = t.qx[0][1];
    carry.qx[1] = t.qx[1][1];
  }
  if (fam & FAM_LY) {
    carry.qy[0] = t.qy[0][1];
    carry.qy[1] = t.qy[1][1];
  }
  if (fam & FAM_AZ) carry.tz = t.tz[1];
}

// Quantities of a cell's y1 face that the next column of a tile (the cell at
// the same level, same x extent and z levels, its y0 equal to this y1) needs
// for its y0 face: corner distances, the x-edge log ratios on that face, the
// z-edge log ratios along it and its angle sum.
struct YCarry {
  double r[2][2];  // [i][k]
  double qx[2];    // [k]
  double qz[2];    // [i]
  double ty;
};

// The same for a cell's x1 face and the cell after it in x (same y extent and
// z levels, its x0 equal to this x1).
struct XCarry {
  double r[2][2];  // [j][k]
  double qy[2];    // [k]
  double qz[2];    // [j]
  double tx;
};

// prism_terms with the neighbours' faces available: `top` (the cell above in
// the same column, ZCarry), `yprev` (the cell before it in y at the same
// level, YCarry) and `xprev` (the cell before it in x, XCarry).  A quantity
// on several shared faces is taken from the first of z, y, x; shared
// quantities are taken over instead of being recomputed, and every computed
// quantity uses the same FP64 operands in the same order as prism_terms, so
// the result is bitwise that of prism_terms.  The faces this cell hands on
// (bottom, y1, x1) are written to zout, yout, xout.
__device__ __forceinline__ void prism_terms_tiled(double px, double py, double pz, double x0,
                                                  double x1, double y0, double y1, double z0,
                                                  double z1, uint32_t fam,
                                                  const double *__restrict__ tab, bool top,
                                                  const ZCarry &zin, bool yprev,
                                                  const YCarry &yin, bool xprev,
                                                  const XCarry &xin, ZCarry &zout, YCarry &yout,
                                                  XCarry &xout, PrismTerms &t) {
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
      for (int k = 0; k < 2; k++) {
        if (top && k == 0) r[i][j][k] = zin.r[i][j];
        else if (yprev && j == 0) r[i][j][k] = yin.r[i][k];
        else if (xprev && i == 0) r[i][j][k] = xin.r[j][k];
        else r[i][j][k] = fast_sqrt(xy + Z2[k]);
      }
    }
  if (fam & FAM_LX) {  // x-edges lie on z and y faces
#pragma unroll
    for (int j = 0; j < 2; j++)
#pragma unroll
      for (int k = 0; k < 2; k++) {
        if (top && k == 0) t.qx[j][k] = zin.qx[j];
        else if (yprev && j == 0) t.qx[j][k] = yin.qx[k];
        else
          t.qx[j][k] = edge_log_ratio(t.X[0], t.X[1], r[0][j][k], r[1][j][k], Y2[j] + Z2[k], tab);
      }
  }
  if (fam & FAM_LY) {  // y-edges lie on z and x faces
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
      for (int k = 0; k < 2; k++) {
        if (top && k == 0) t.qy[i][k] = zin.qy[i];
        else if (xprev && i == 0) t.qy[i][k] = xin.qy[k];
        else
          t.qy[i][k] = edge_log_ratio(t.Y[0], t.Y[1], r[i][0][k], r[i][1][k], X2[i] + Z2[k], tab);
      }
  }
  if (fam & FAM_LZ) {  // z-edges lie on y and x faces
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
      for (int j = 0; j < 2; j++) {
        if (yprev && j == 0) t.qz[i][j] = yin.qz[i];
        else if (xprev && i == 0) t.qz[i][j] = xin.qz[j];
        else
          t.qz[i][j] = edge_log_ratio(t.Z[0], t.Z[1], r[i][j][0], r[i][j][1], X2[i] + Y2[j], tab);
      }
  }
  if (fam & (FAM_AX | FAM_AY | FAM_AZ)) {
    const float Xf[2] = {double_to_float_rn(t.X[0]), double_to_float_rn(t.X[1])};
    const float Yf[2] = {double_to_float_rn(t.Y[0]), double_to_float_rn(t.Y[1])};
    const float Zf[2] = {double_to_float_rn(t.Z[0]), double_to_float_rn(t.Z[1])};
    float rf[2][2][2];
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
      for (int j = 0; j < 2; j++)
#pragma unroll
        for (int k = 0; k < 2; k++)
          rf[i][j][k] = sqrtf(fmaf(Xf[i], Xf[i], fmaf(Yf[j], Yf[j], Zf[k] * Zf[k])));
    if (fam & FAM_AX) {
      const double b[4] = {t.Y[0] * t.Z[0], t.Y[0] * t.Z[1], t.Y[1] * t.Z[0], t.Y[1] * t.Z[1]};
      const float bf[4] = {Yf[0] * Zf[0], Yf[0] * Zf[1], Yf[1] * Zf[0], Yf[1] * Zf[1]};
#pragma unroll
      for (int i = 0; i < 2; i++) {
        if (xprev && i == 0) {
          t.tx[0] = xin.tx;
          continue;
        }
        const double a[4] = {t.X[i] * r[i][0][0], t.X[i] * r[i][0][1], t.X[i] * r[i][1][0],
                             t.X[i] * r[i][1][1]};
        const float af[4] = {Xf[i] * rf[i][0][0], Xf[i] * rf[i][0][1], Xf[i] * rf[i][1][0],
                             Xf[i] * rf[i][1][1]};
        t.tx[i] = face_atan_sum(a, b, af, bf, tab);
      }
    }
    if (fam & FAM_AY) {
      const double b[4] = {t.X[0] * t.Z[0], t.X[0] * t.Z[1], t.X[1] * t.Z[0], t.X[1] * t.Z[1]};
      const float bf[4] = {Xf[0] * Zf[0], Xf[0] * Zf[1], Xf[1] * Zf[0], Xf[1] * Zf[1]};
#pragma unroll
      for (int j = 0; j < 2; j++) {
        if (yprev && j == 0) {
          t.ty[0] = yin.ty;
          continue;
        }
        const double a[4] = {t.Y[j] * r[0][j][0], t.Y[j] * r[0][j][1], t.Y[j] * r[1][j][0],
                             t.Y[j] * r[1][j][1]};
        const float af[4] = {Yf[j] * rf[0][j][0], Yf[j] * rf[0][j][1], Yf[j] * rf[1][j][0],
                             Yf[j] * rf[1][j][1]};
        t.ty[j] = face_atan_sum(a, b, af, bf, tab);
      }
    }
    if (fam & FAM_AZ) {
      const double b[4] = {t.X[0] * t.Y[0], t.X[0] * t.Y[1], t.X[1] * t.Y[0], t.X[1] * t.Y[1]};
      const float bf[4] = {Xf[0] * Yf[0], Xf[0] * Yf[1], Xf[1] * Yf[0], Xf[1] * Yf[1]};
#pragma unroll
      for (int k = 0; k < 2; k++) {
        if (top && k == 0) {
          t.tz[0] = zin.tz;
          continue;
        }
        const double a[4] = {t.Z[k] * r[0][0][k], t.Z[k] * r[0][1][k], t.Z[k] * r[1][0][k],
                             t.Z[k] * r[1][1][k]};
        const float af[4] = {Zf[k] * rf[0][0][k], Zf[k] * rf[0][1][k], Zf[k] * rf[1][0][k],
                             Zf[k] * rf[1][1][k]};
        t.tz[k] = face_atan_sum(a, b, af, bf, tab);
      }
    }
  }
  // faces handed on: bottom (z1) down the column, y1 and x1 to the next runs
#pragma unroll
  for (int i = 0; i < 2; i++)
#pragma unroll
    for (int j = 0; j < 2; j++) zout.r[i][j] = r[i][j][1];
#pragma unroll
  for (int a = 0; a < 2; a++)
#pragma unroll
    for (int k = 0; k < 2; k++) {
      yout.r[a][k] = r[a][1][k];
      xout.r[a][k] = r[1][a][k];
    }
  if (fam & FAM_LX) {
    zout.qx[0] = t.qx[0][1];
    zout.qx[1] = t.qx[1][1];
    yout.qx[0] = t.qx[1][0];
    yout.qx[1] = t.qx[1][1];
  }
  if (fam & FAM_LY) {
    zout.qy[0] = t.qy[0][1];
    zout.qy[1] = t.qy[1][1];
    xout.qy[0] = t.qy[1][0];
    xout.qy[1] = t.qy[1][1];
  }
  if (fam & FAM_LZ) {
    yout.qz[0] = t.qz[0][1];
    yout.qz[1] = t.qz[1][1];
    xout.qz[0] = t.qz[1][0];
    xout.qz[1] = t.qz[1][1];
  }
  if (fam & FAM_AX) xout.tx = t.tx[1];
  if (fam & FAM_AY) yout.ty = t.ty[1];
  if (fam & FAM_AZ) zout.tz = t.tz[1];
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
