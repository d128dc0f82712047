// Device-side element and node arithmetic of the LagrangeLeapFrog step.
//
// Every function restates a reference expression in a form with fewer FP64
// instructions (GB300 issues about two FP64 instructions per clock per SM,
// so the FP64 instruction count, not HBM, bounds this step). The
// reformulations are exact in real arithmetic and differ from the
// reference's left-to-right evaluation only by rounding:
//  * the shape-function Jacobian columns (src/domain.jl:1964-1974) and the
//    monotonic-Q gradients (src/domain.jl:2244-2254) are the first-order
//    Walsh coefficients of the 8 corner values, taken through the four body
//    diagonals; power-of-two scale factors (0.125, 0.25, 8) are dropped where
//    they cancel or only scale a sign test, which is exact;
//  * the hourglass modes x8n*gamma (src/domain.jl:1510-1525) are the
//    second/third-order Walsh coefficients, found by a 3-stage butterfly or,
//    where the face diagonals exist anyway, as sums of four of them (face
//    diagonals join corners of one parity) plus the body diagonals;
//  * the node normals of a corner and its opposite corner are negatives of
//    each other (the face normals of a closed surface sum to zero);
//  * a face's area vector (sumElemFaceNormal, src/domain.jl:971-989) is
//    -(d1 x d2)/8 for the face's two diagonals d1, d2;
//  * voluDer (src/domain.jl:1178-1211) only ever sums the 12 hex edges, so
//    the 36 edge sums are formed once per element;
//  * the velocity-gradient trace (src/domain.jl:2023-2081, 2156-2158) is
//    trace(C^T W(v)) / det, with C the cofactors of the Jacobian and W(v) the
//    Walsh coefficients of the velocities;
//  * reciprocals of one element share a division (recip3), square roots are
//    x * rsqrt(x), and the hourglass coefficient's 1/cbrt is a float seed
//    with one Householder step (inv_cbrt): a division costs about 5 FP64
//    instructions, sqrt about 9 and the library rcbrt about 18.
// Products are contracted into FMAs.
#pragma once

#include <math.h>

#include "lulesh_internal.h"

namespace lulesh {

#define LDG(p) __ldg(p)

// Index guard of the checked build (-DLULESH_CHECK, a debug build the tests
// run small cases with): an index outside [0, n) records ST_INDEX in the
// problem's status word and is replaced by 0, so the access stays in bounds.
// A normal build passes the index through.
#ifdef LULESH_CHECK
#define LULESH_IDX(i, n, st) \
  (((unsigned)(i) < (unsigned)(n)) ? (i) : (atomicOr(&(st)->status, ST_INDEX), 0))
#else
#define LULESH_IDX(i, n, st) (i)
#endif

// gamma[n][m] of calcFBHourglassForceForElems, src/domain.jl:1490-1499.
__device__ __forceinline__ double gamma_nm(int n, int m) {
  // column m is the Walsh function eta*zeta, xi*zeta, xi*eta, xi*eta*zeta
  // over the corner signs xi = (-,+,+,-,-,+,+,-), eta = (-,-,+,+,-,-,+,+),
  // zeta = (-,-,-,-,+,+,+,+).
  const int xs = ((n == 1) | (n == 2) | (n == 5) | (n == 6)) ? 1 : -1;
  const int es = ((n == 2) | (n == 3) | (n == 6) | (n == 7)) ? 1 : -1;
  const int zs = (n >= 4) ? 1 : -1;
  const int v = (m == 0) ? es * zs : (m == 1) ? xs * zs : (m == 2) ? xs * es : xs * es * zs;
  return (double)v;
}

// First-order Walsh coefficients (xi, eta, zeta) of 8 corner values through
// the four body diagonals: 11 FP64 adds.
__device__ __forceinline__ void walsh1(const double v[8], double w[3]) {
  const double a = v[6] - v[0], b = v[5] - v[3], c = v[7] - v[1], d = v[4] - v[2];
  const double apb = a + b, cpd = c + d;
  w[0] = apb - cpd;
  w[1] = (a - b) + (c - d);
  w[2] = apb + cpd;
}

// First-order (w1: xi, eta, zeta) and higher-order (w2: eta*zeta, xi*zeta,
// xi*eta, xi*eta*zeta = the four hourglass modes) Walsh coefficients: 23 adds.
__device__ __forceinline__ void walsh7(const double v[8], double w1[3], double w2[4]) {
  const double sa = v[0] + v[1], da = v[1] - v[0];
  const double sb = v[3] + v[2], db = v[2] - v[3];
  const double sc = v[4] + v[5], dc = v[5] - v[4];
  const double sd = v[7] + v[6], dd = v[6] - v[7];
  const double ss1 = sa + sb, sd1 = sb - sa, ds1 = da + db, dd1 = db - da;
  const double ss2 = sc + sd, sd2 = sd - sc, ds2 = dc + dd, dd2 = dd - dc;
  w1[0] = ds1 + ds2;
  w1[1] = sd1 + sd2;
  w1[2] = ss2 - ss1;
  w2[0] = sd2 - sd1;
  w2[1] = ds2 - ds1;
  w2[2] = dd1 + dd2;
  w2[3] = dd2 - dd1;
}

__device__ __forceinline__ void cross(double ax, double ay, double az, double bx, double by,
                                      double bz, double& cx, double& cy, double& cz) {
  cx = fma(ay, bz, -az * by);
  cy = fma(az, bx, -ax * bz);
  cz = fma(ax, by, -ay * bx);
}

// Integer-pipe helpers for exact tests on FP64 values (keeps DSETP off the
// scarce FP64 pipe). Valid for non-NaN inputs.
__device__ __forceinline__ bool le_zero(double a) {  // a <= 0.0
  return __double_as_longlong(a) <= 0;  // +0 -> 0, -0 and negatives -> sign bit
}
__device__ __forceinline__ bool gt_zero(double a) {  // a > 0.0
  return __double_as_longlong(a) > 0;
}
__device__ __forceinline__ bool abs_lt(double a, double c) {  // |a| < c for c >= 0
  return (unsigned long long)(__double_as_longlong(a) & 0x7FFFFFFFFFFFFFFFll) <
         (unsigned long long)__double_as_longlong(c);
}

// Integer-pipe comparison key of a non-NaN double (fkey_bits): a < b exactly
// when fkey(a) < fkey(b), -0 equal to +0. A DSETP takes an FP64 pipe slot;
// the key and a 64-bit integer compare take a few integer instructions, of
// which the FP64-bound kernels have plenty to spare.
__device__ __forceinline__ long long fkey(double x) { return fkey_bits(__double_as_longlong(x)); }
__device__ __forceinline__ bool lt_zero(double a) { return fkey(a) < 0; }  // a < 0.0
__device__ __forceinline__ bool is_zero(double a) {                         // a == 0.0
  return (__double_as_longlong(a) & 0x7FFFFFFFFFFFFFFFll) == 0;
}
// max of two non-negative doubles (+0 included) by their bit patterns
__device__ __forceinline__ double max_nonneg(double a, double b) {
  const long long x = __double_as_longlong(a), y = __double_as_longlong(b);
  return __longlong_as_double(x > y ? x : y);
}

// x^(-1/3) for x > 0 in six FP64 instructions: a single-precision seed y0
// refined by one second-order Householder step. With e = 1 - x y0^3 the
// exact value is y0 (1 - e)^(-1/3) = y0 (1 + e/3 + 2e^2/9 + 14e^3/81 + ...);
// the seed's |e| is below 2^-21, so the dropped terms are below 2^-64 and the
// result is within about one ulp (y0^2 is exact, y0^3 and 1 - x y0^3 are
// rounded once). Outside [1e-30, 1e30] (beyond the seed's float range) the
// library rcbrt is used; the range test runs on the integer pipe.
__device__ __forceinline__ double inv_cbrt(double x) {
  const long long b = __double_as_longlong(x);
  if (b < 0x39B4484BFEEBC2A0ll || b > 0x46293E5939A08CEAll) return rcbrt(x);  // 1e-30, 1e30
  const double y0 = (double)rcbrtf((float)x);
  const double y2 = y0 * y0;
  const double e = fma(-x, y2 * y0, 1.0);
  return fma(y0, e * fma(e, 2.0 / 9.0, 1.0 / 3.0), y0);
}

// True when |v| is a normal finite double (exponent field neither 0 nor all
// ones), tested on the integer pipe.
__device__ __forceinline__ bool normal_finite(double v) {
  const unsigned long long m = (unsigned long long)__double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFull;
  return m - 0x0010000000000000ull < 0x7FE0000000000000ull;
}

// 1/a and 1/b from one division, r = 1/(a b): 1/a = r b, 1/b = r a; the
// two quotients one by one when a b is not a normal finite double.
__device__ __forceinline__ void recip2(double a, double b, double& ia, double& ib) {
  const double ab = a * b;
  if (normal_finite(ab)) {
    const double r = 1.0 / ab;
    ia = r * b;
    ib = r * a;
  } else {
    ia = 1.0 / a;
    ib = 1.0 / b;
  }
}

// 1/a, 1/b, 1/c from one division: r = 1/(a b c), 1/c = r (a b),
// 1/a = (r c) b, 1/b = (r c) a; each result is within a few ulps of the
// quotient. When a b or a b c is not a normal finite double (a state far
// outside the physical ranges, or a zero operand) the three quotients are
// formed one by one, so the results are those of the divisions. The range
// test runs on the integer pipe.
__device__ __forceinline__ void recip3(double a, double b, double c, double& ia, double& ib, double& ic) {
  const double ab = a * b, abc = ab * c;
  if (normal_finite(ab) && normal_finite(abc)) {
    const double r = 1.0 / abc;
    const double rc = r * c;
    ic = r * ab;
    ia = rc * b;
    ib = rc * a;
  } else {
    ia = 1.0 / a;
    ib = 1.0 / b;
    ic = 1.0 / c;
  }
}

// timeIncrement!, src/domain.jl:920-961, shared by the host API and the
// device run loop.
__host__ __device__ inline void time_increment(double& time, double& deltatime, long long& cycle,
                                               double dtcourant, double dthydro,
                                               const Params& prm) {
  double targetdt = prm.stoptime - time;
  if (prm.dtfixed <= 0.0 && cycle != 0) {
    const double olddt = deltatime;
    double gnewdt = (double)INFINITY;  // typemax(Float64)
    if (dtcourant < gnewdt) gnewdt = dtcourant / 2.0;
    if (dthydro < gnewdt) gnewdt = dthydro * 2.0 / 3.0;
    double newdt = gnewdt;
    const double ratio = newdt / olddt;
    if (ratio >= 1.0) {
      if (ratio < prm.deltatimemultlb) newdt = olddt;
      else if (ratio > prm.deltatimemultub) newdt = olddt * prm.deltatimemultub;
    }
    // Julia min: NaN-propagating
    if (newdt != newdt) {
    } else if (prm.dtmax != prm.dtmax) {
      newdt = prm.dtmax;
    } else if (prm.dtmax < newdt) {
      newdt = prm.dtmax;
    }
    deltatime = newdt;
  }
  if (deltatime < targetdt && targetdt < 4.0 * deltatime / 3.0) targetdt = 2.0 * deltatime / 3.0;
  if (targetdt < deltatime) deltatime = targetdt;
  time = time + deltatime;
  cycle += 1;
}

}  // namespace lulesh
