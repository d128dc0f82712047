// LULESH oracle: a CPU restatement of JuliaLabs/LULESH.jl's single-rank
// Sedov setup and LagrangeLeapFrog timestep, used ONLY as test infrastructure
// (parity reference, CPU baseline timing, golden-fixture generator). The product
// library never links, loads or calls anything in this directory.
//
// Parity status: UNPINNED against the Julia reference itself. The reference
// ships no golden vectors or known-answer tests (test/runtests.jl:33-50 only
// checks the exit status of examples/benchmark.jl), and Julia is not available
// to run it. This file restates the reference's arithmetic expression by
// expression, in the reference's evaluation order, with 0-based indices and
// the raw index values the Julia Domain stores. Build with
// -ffp-contract=off: Julia does not contract a*b+c into an FMA.
//
// Three behaviours of the reference are reproduced by default (mode FAITHFUL)
// and can be corrected (mode LULESH2):
//   * src/domain.jl:1042-1055 (calcElemNodeNormals, face 5) adds areaY to
//     pfy[1] twice and never adds areaZ to pfz[1];
//   * src/domain.jl:1213-1256 (calcElemVolumeDerivative) stores the volume
//     derivative of node 3 in node 1's slot and that of node 1 in node 3's;
//   * src/domain.jl:2349 (calcMonotonicQRegionForElems) reads
//     delv_xi[lxip[i]] without the +1 every other neighbour access has, so
//     interior elements use their own delv_xi as the xi-plus neighbour.
//
// The Julia `@simd` node-gather loops (src/domain.jl:1118, :1684) permit
// reassociation; this restatement sums sequentially in nodeElemCornerList
// order. Julia's cbrt is its own implementation; this file calls the C
// library's cbrt. Both can differ from the reference in the last bits.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>
#include <string>
#include <vector>

namespace lulesh_oracle {

// Boundary-condition bit masks, src/bc.jl:3-30.
enum : uint32_t {
  XI_M = 0x00007, XI_M_SYMM = 0x00001, XI_M_FREE = 0x00002, XI_M_COMM = 0x00004,
  XI_P = 0x00038, XI_P_SYMM = 0x00008, XI_P_FREE = 0x00010, XI_P_COMM = 0x00020,
  ETA_M = 0x001c0, ETA_M_SYMM = 0x00040, ETA_M_FREE = 0x00080, ETA_M_COMM = 0x00100,
  ETA_P = 0x00e00, ETA_P_SYMM = 0x00200, ETA_P_FREE = 0x00400, ETA_P_COMM = 0x00800,
  ZETA_M = 0x07000, ZETA_M_SYMM = 0x01000, ZETA_M_FREE = 0x02000, ZETA_M_COMM = 0x04000,
  ZETA_P = 0x38000, ZETA_P_SYMM = 0x08000, ZETA_P_FREE = 0x10000, ZETA_P_COMM = 0x20000,
};

// Status codes; the same numbering the product's C ABI uses.
enum Status : int {
  OK = 0,
  ERR_VOLUME = 1,   // any of the reference's "Volume Error" raises
  ERR_QSTOP = 2,    // "QStopError", src/domain.jl:2580
  ERR_BAD_BC = 3,   // error("Error") on an invalid BC mask, src/domain.jl:2343
};

// Which reference error site raised (finer than Status).
enum VolumeSite : int {
  SITE_NONE = 0,
  SITE_EARLY = 1,      // integrateStressForElems, src/domain.jl:1104
  SITE_HOURGLASS = 2,  // calcHourglassControlForElems, :1727
  SITE_MID = 3,        // calcVolumeForceForElems, :1758
  SITE_KINEMATICS = 4, // calcKinematicsForElems, :2118
  SITE_LAGRANGE = 5,   // calcLagrangeElements, :2169
  SITE_MATERIAL = 6,   // applyMaterialPropertiesForElems, :2905
  SITE_UPDATE = 7,     // updateVolumesForElems, :2926
};

// Mode is a bit set of corrections to the reference's behaviour. FAITHFUL (no
// bits) reproduces the reference; LULESH2 (all bits) is the corrected method.
enum Mode : int {
  FAITHFUL = 0,
  FIX_NORMALS = 1,   // calcElemNodeNormals face 5, src/domain.jl:1046-1055
  FIX_VOLUDER = 2,   // calcElemVolumeDerivative slots, src/domain.jl:1253-1255
  FIX_LXIP = 4,      // xi-plus neighbour index, src/domain.jl:2349
  LULESH2 = 7,
};

template <class T> inline double val(const T& a) { return (double)a; }

// abs(x) for the scalar type (sign flip keeps derivatives for dual numbers).
inline double jabs(double a) { return std::fabs(a); }
template <class T> inline T jabs(const T& a) { return val(a) < 0.0 ? -a : a; }

// Julia's Base.max / Base.min for IEEE floats (NaN-propagating, -0 < +0).
template <class T> inline T jmax(const T& x, const T& y) {
  double xv = val(x), yv = val(y);
  bool pick_y = (yv > xv) || (std::signbit(yv) < std::signbit(xv));
  if (pick_y) return std::isnan(xv) ? x : y;
  return std::isnan(yv) ? y : x;
}
template <class T> inline T jmin(const T& x, const T& y) {
  double xv = val(x), yv = val(y);
  bool pick_y = (yv < xv) || (std::signbit(yv) > std::signbit(xv));
  if (pick_y) return std::isnan(xv) ? x : y;
  return std::isnan(yv) ? y : x;
}

// Problem description (LuleshProblem, src/LULESH.jl:31-49, single rank).
struct Problem {
  int nx = 30;        // elements per edge
  int nr = 11;        // regions
  int balance = 1;
  int cost = 1;
  int mode = FAITHFUL;
  uint64_t region_seed = 0;  // Random.seed!(myRank); myRank = 0
};

template <class T>
struct Domain {
  // sizes
  int64_t sizeX = 0, numElem = 0, numNode = 0;
  int mode = FAITHFUL;
  // element-centred
  std::vector<int64_t> matElemlist, nodelist, lxim, lxip, letam, letap, lzetam, lzetap;
  std::vector<uint32_t> elemBC;
  std::vector<T> e, p, q, ql, qq, v, volo, delv, vdov, arealg, ss, elemMass;
  std::vector<T> vnew, delv_xi, delv_eta, delv_zeta, delx_xi, delx_eta, delx_zeta, dxx, dyy, dzz;
  // node-centred
  std::vector<T> x, y, z, xd, yd, zd, xdd, ydd, zdd, fx, fy, fz, nodalMass;
  std::vector<int64_t> symmX, symmY, symmZ;
  std::vector<int64_t> nodeElemCount, nodeElemStart, nodeElemCornerList;
  // parameters (src/domain.jl:663-701)
  T dtfixed, deltatimemultlb, deltatimemultub, stoptime, dtmax;
  int64_t cycle = 0;
  T dthydro, dtcourant;
  T time, deltatime;
  T u_cut, hgcoef, qstop, monoq_max_slope, monoq_limiter_mult, e_cut, p_cut, ss4o3,
      q_cut, v_cut, qlc_monoq, qqc_monoq, qqc, eosvmax, eosvmin, pmin, emin, dvovmax, refdens;
  // regions (src/domain.jl:338-465)
  int numReg = 1, balance = 1, cost = 1;
  std::vector<int64_t> regElemSize, regCSR, regReps, regNumList, regElemlist, regSorted;
  // last error site (diagnostics only)
  int error_site = SITE_NONE;
  int64_t error_index = -1;
  // scratch reused between calls (the reference allocates these every step)
  std::vector<T> fx_elem, fy_elem, fz_elem, determ, dvdx, dvdy, dvdz, x8n, y8n, z8n, sigxx;
};

// ---------------------------------------------------------------------------
// Geometry helpers
// ---------------------------------------------------------------------------

// calcElemVolume, src/utils.jl:36-116.
template <class T>
inline T calcElemVolume(const T x[8], const T y[8], const T z[8]) {
  auto tp = [](const T& x1, const T& y1, const T& z1, const T& x2, const T& y2, const T& z2,
               const T& x3, const T& y3, const T& z3) -> T {
    return ((x1 * ((y2 * z3) - (z2 * y3)) + x2 * ((z1 * y3) - (y1 * z3))) +
            x3 * ((y1 * z2) - (z1 * y2)));
  };
  const T twelveth = T(1.0) / T(12.0);
  T dx61 = x[6] - x[1], dy61 = y[6] - y[1], dz61 = z[6] - z[1];
  T dx70 = x[7] - x[0], dy70 = y[7] - y[0], dz70 = z[7] - z[0];
  T dx63 = x[6] - x[3], dy63 = y[6] - y[3], dz63 = z[6] - z[3];
  T dx20 = x[2] - x[0], dy20 = y[2] - y[0], dz20 = z[2] - z[0];
  T dx50 = x[5] - x[0], dy50 = y[5] - y[0], dz50 = z[5] - z[0];
  T dx64 = x[6] - x[4], dy64 = y[6] - y[4], dz64 = z[6] - z[4];
  T dx31 = x[3] - x[1], dy31 = y[3] - y[1], dz31 = z[3] - z[1];
  T dx72 = x[7] - x[2], dy72 = y[7] - y[2], dz72 = z[7] - z[2];
  T dx43 = x[4] - x[3], dy43 = y[4] - y[3], dz43 = z[4] - z[3];
  T dx57 = x[5] - x[7], dy57 = y[5] - y[7], dz57 = z[5] - z[7];
  T dx14 = x[1] - x[4], dy14 = y[1] - y[4], dz14 = z[1] - z[4];
  T dx25 = x[2] - x[5], dy25 = y[2] - y[5], dz25 = z[2] - z[5];
  T volume = (tp(dx31 + dx72, dx63, dx20, dy31 + dy72, dy63, dy20, dz31 + dz72, dz63, dz20) +
              tp(dx43 + dx57, dx64, dx70, dy43 + dy57, dy64, dy70, dz43 + dz57, dz64, dz70)) +
             tp(dx14 + dx25, dx61, dx50, dy14 + dy25, dy61, dy50, dz14 + dz25, dz61, dz50);
  volume = volume * twelveth;
  return volume;
}

// calcElemShapeFunctionDerivatives, src/domain.jl:1932-2021. b[c][d], d = x,y,z.
template <class T>
inline T calcElemShapeFunctionDerivatives(const T x[8], const T y[8], const T z[8], T b[8][3]) {
  const T x0 = x[0], x1 = x[1], x2 = x[2], x3 = x[3], x4 = x[4], x5 = x[5], x6 = x[6], x7 = x[7];
  const T y0 = y[0], y1 = y[1], y2 = y[2], y3 = y[3], y4 = y[4], y5 = y[5], y6 = y[6], y7 = y[7];
  const T z0 = z[0], z1 = z[1], z2 = z[2], z3 = z[3], z4 = z[4], z5 = z[5], z6 = z[6], z7 = z[7];
  const T c = T(0.125);
  T fjxxi = c * ((((x6 - x0) + (x5 - x3)) - (x7 - x1)) - (x4 - x2));
  T fjxet = c * ((((x6 - x0) - (x5 - x3)) + (x7 - x1)) - (x4 - x2));
  T fjxze = c * ((((x6 - x0) + (x5 - x3)) + (x7 - x1)) + (x4 - x2));
  T fjyxi = c * ((((y6 - y0) + (y5 - y3)) - (y7 - y1)) - (y4 - y2));
  T fjyet = c * ((((y6 - y0) - (y5 - y3)) + (y7 - y1)) - (y4 - y2));
  T fjyze = c * ((((y6 - y0) + (y5 - y3)) + (y7 - y1)) + (y4 - y2));
  T fjzxi = c * ((((z6 - z0) + (z5 - z3)) - (z7 - z1)) - (z4 - z2));
  T fjzet = c * ((((z6 - z0) - (z5 - z3)) + (z7 - z1)) - (z4 - z2));
  T fjzze = c * ((((z6 - z0) + (z5 - z3)) + (z7 - z1)) + (z4 - z2));

  T cjxxi = (fjyet * fjzze) - (fjzet * fjyze);
  T cjxet = (-(fjyxi * fjzze)) + (fjzxi * fjyze);
  T cjxze = (fjyxi * fjzet) - (fjzxi * fjyet);
  T cjyxi = (-(fjxet * fjzze)) + (fjzet * fjxze);
  T cjyet = (fjxxi * fjzze) - (fjzxi * fjxze);
  T cjyze = (-(fjxxi * fjzet)) + (fjzxi * fjxet);
  T cjzxi = (fjxet * fjyze) - (fjyet * fjxze);
  T cjzet = (-(fjxxi * fjyze)) + (fjyxi * fjxze);
  T cjzze = (fjxxi * fjyet) - (fjyxi * fjxet);

  if (b) {
    b[0][0] = ((-cjxxi) - cjxet) - cjxze;
    b[1][0] = (cjxxi - cjxet) - cjxze;
    b[2][0] = (cjxxi + cjxet) - cjxze;
    b[3][0] = ((-cjxxi) + cjxet) - cjxze;
    b[4][0] = -b[2][0]; b[5][0] = -b[3][0]; b[6][0] = -b[0][0]; b[7][0] = -b[1][0];
    b[0][1] = ((-cjyxi) - cjyet) - cjyze;
    b[1][1] = (cjyxi - cjyet) - cjyze;
    b[2][1] = (cjyxi + cjyet) - cjyze;
    b[3][1] = ((-cjyxi) + cjyet) - cjyze;
    b[4][1] = -b[2][1]; b[5][1] = -b[3][1]; b[6][1] = -b[0][1]; b[7][1] = -b[1][1];
    b[0][2] = ((-cjzxi) - cjzet) - cjzze;
    b[1][2] = (cjzxi - cjzet) - cjzze;
    b[2][2] = (cjzxi + cjzet) - cjzze;
    b[3][2] = ((-cjzxi) + cjzet) - cjzze;
    b[4][2] = -b[2][2]; b[5][2] = -b[3][2]; b[6][2] = -b[0][2]; b[7][2] = -b[1][2];
  }
  return T(8.0) * (((fjxet * cjxet) + (fjyet * cjyet)) + (fjzet * cjzet));
}

// sumElemFaceNormal, src/domain.jl:971-989.
template <class T>
inline void sumElemFaceNormal(const T& x0, const T& y0, const T& z0, const T& x1, const T& y1,
                              const T& z1, const T& x2, const T& y2, const T& z2, const T& x3,
                              const T& y3, const T& z3, T& areaX, T& areaY, T& areaZ) {
  const T RHALF = T(0.5), RQTR = T(0.25);
  T bisectX0 = RHALF * (((x3 + x2) - x1) - x0);
  T bisectY0 = RHALF * (((y3 + y2) - y1) - y0);
  T bisectZ0 = RHALF * (((z3 + z2) - z1) - z0);
  T bisectX1 = RHALF * (((x2 + x1) - x3) - x0);
  T bisectY1 = RHALF * (((y2 + y1) - y3) - y0);
  T bisectZ1 = RHALF * (((z2 + z1) - z3) - z0);
  areaX = RQTR * ((bisectY0 * bisectZ1) - (bisectZ0 * bisectY1));
  areaY = RQTR * ((bisectZ0 * bisectX1) - (bisectX0 * bisectZ1));
  areaZ = RQTR * ((bisectX0 * bisectY1) - (bisectY0 * bisectX1));
}

// calcElemNodeNormals, src/domain.jl:991-1067. B[c][d]. mode FAITHFUL keeps
// the face-5 accumulation exactly as the reference writes it.
template <class T>
inline void calcElemNodeNormals(const T x[8], const T y[8], const T z[8], T B[8][3], int mode) {
  T pfx[8], pfy[8], pfz[8];
  for (int i = 0; i < 8; ++i) pfx[i] = pfy[i] = pfz[i] = T(0.0);
  T ax, ay, az;
  auto add = [&](const int* nodes, int n) {
    for (int i = 0; i < n; ++i) {
      pfx[nodes[i]] = pfx[nodes[i]] + ax;
      pfy[nodes[i]] = pfy[nodes[i]] + ay;
      pfz[nodes[i]] = pfz[nodes[i]] + az;
    }
  };
  // face 1: nodes 0,1,2,3
  sumElemFaceNormal(x[0], y[0], z[0], x[1], y[1], z[1], x[2], y[2], z[2], x[3], y[3], z[3], ax, ay, az);
  { const int n[4] = {0, 1, 2, 3}; add(n, 4); }
  // face 2: nodes 0,4,5,1
  sumElemFaceNormal(x[0], y[0], z[0], x[4], y[4], z[4], x[5], y[5], z[5], x[1], y[1], z[1], ax, ay, az);
  { const int n[4] = {0, 1, 4, 5}; add(n, 4); }
  // face 3: nodes 1,5,6,2
  sumElemFaceNormal(x[1], y[1], z[1], x[5], y[5], z[5], x[6], y[6], z[6], x[2], y[2], z[2], ax, ay, az);
  { const int n[4] = {1, 2, 5, 6}; add(n, 4); }
  // face 4: nodes 2,6,7,3
  sumElemFaceNormal(x[2], y[2], z[2], x[6], y[6], z[6], x[7], y[7], z[7], x[3], y[3], z[3], ax, ay, az);
  { const int n[4] = {2, 3, 6, 7}; add(n, 4); }
  // face 5: nodes 3,7,4,0
  sumElemFaceNormal(x[3], y[3], z[3], x[7], y[7], z[7], x[4], y[4], z[4], x[0], y[0], z[0], ax, ay, az);
  if (!(mode & FIX_NORMALS)) {
    // src/domain.jl:1046-1055, statement by statement.
    pfx[0] = pfx[0] + ax;
    pfx[3] = pfx[3] + ax; pfx[4] = pfx[4] + ax;
    pfx[7] = pfx[7] + ax;
    pfy[0] = pfy[0] + ay;
    pfy[3] = pfy[3] + ay; pfy[4] = pfy[4] + ay;
    pfy[7] = pfy[7] + ay;
    pfy[0] = pfy[0] + ay;
    pfz[3] = pfz[3] + az; pfz[4] = pfz[4] + az;
    pfz[7] = pfz[7] + az;
  } else {
    const int n[4] = {0, 3, 4, 7}; add(n, 4);
  }
  // face 6: nodes 4,7,6,5
  sumElemFaceNormal(x[4], y[4], z[4], x[7], y[7], z[7], x[6], y[6], z[6], x[5], y[5], z[5], ax, ay, az);
  { const int n[4] = {4, 5, 6, 7}; add(n, 4); }
  for (int i = 0; i < 8; ++i) { B[i][0] = pfx[i]; B[i][1] = pfy[i]; B[i][2] = pfz[i]; }
}

// voluDer, src/domain.jl:1178-1211.
template <class T>
inline void voluDer(const T& x0, const T& x1, const T& x2, const T& x3, const T& x4, const T& x5,
                    const T& y0, const T& y1, const T& y2, const T& y3, const T& y4, const T& y5,
                    const T& z0, const T& z1, const T& z2, const T& z3, const T& z4, const T& z5,
                    T& dvdx, T& dvdy, T& dvdz) {
  dvdx = (((((y1 + y2) * (z0 + z1) - (y0 + y1) * (z1 + z2)) + (y0 + y4) * (z3 + z4)) -
           (y3 + y4) * (z0 + z4)) - (y2 + y5) * (z3 + z5)) + (y3 + y5) * (z2 + z5);
  dvdy = (((((-(x1 + x2)) * (z0 + z1) + (x0 + x1) * (z1 + z2)) - (x0 + x4) * (z3 + z4)) +
           (x3 + x4) * (z0 + z4)) + (x2 + x5) * (z3 + z5)) - (x3 + x5) * (z2 + z5);
  dvdz = (((((-(y1 + y2)) * (x0 + x1) + (y0 + y1) * (x1 + x2)) - (y0 + y4) * (x3 + x4)) +
           (y3 + y4) * (x0 + x4)) + (y2 + y5) * (x3 + x5)) - (y3 + y5) * (x2 + x5);
  const T twelfth = T(1.0) / T(12.0);
  dvdx = dvdx * twelfth;
  dvdy = dvdy * twelfth;
  dvdz = dvdz * twelfth;
}

// calcElemVolumeDerivative, src/domain.jl:1213-1256 (0-based node permutations).
// The n-th voluDer call below is the volume derivative with respect to node
// owner[n]. The reference stores call n in slot n (src/domain.jl:1253-1255),
// so slots 1 and 3 hold the derivatives of nodes 3 and 1 (mode FAITHFUL);
// mode LULESH2 stores each derivative in its own node's slot.
template <class T>
inline void calcElemVolumeDerivative(const T x[8], const T y[8], const T z[8], T dvdx[8], T dvdy[8],
                                     T dvdz[8], int mode = FAITHFUL) {
  static const int perm[8][6] = {{1, 2, 3, 4, 5, 7}, {0, 1, 2, 7, 4, 6}, {3, 0, 1, 6, 7, 5},
                                 {2, 3, 0, 5, 6, 4}, {7, 6, 5, 0, 3, 1}, {4, 7, 6, 1, 0, 2},
                                 {5, 4, 7, 2, 1, 3}, {6, 5, 4, 3, 2, 0}};
  static const int owner[8] = {0, 3, 2, 1, 4, 5, 6, 7};
  for (int n = 0; n < 8; ++n) {
    const int* q = perm[n];
    const int slot = (mode & FIX_VOLUDER) ? owner[n] : n;
    voluDer(x[q[0]], x[q[1]], x[q[2]], x[q[3]], x[q[4]], x[q[5]], y[q[0]], y[q[1]], y[q[2]],
            y[q[3]], y[q[4]], y[q[5]], z[q[0]], z[q[1]], z[q[2]], z[q[3]], z[q[4]], z[q[5]],
            dvdx[slot], dvdy[slot], dvdz[slot]);
  }
}

// areaFace, src/domain.jl:1874-1891.
template <class T>
inline T areaFace(const T& x0, const T& x1, const T& x2, const T& x3, const T& y0, const T& y1,
                  const T& y2, const T& y3, const T& z0, const T& z1, const T& z2, const T& z3) {
  T fx = (x2 - x0) - (x3 - x1);
  T fy = (y2 - y0) - (y3 - y1);
  T fz = (z2 - z0) - (z3 - z1);
  T gx = (x2 - x0) + (x3 - x1);
  T gy = (y2 - y0) + (y3 - y1);
  T gz = (z2 - z0) + (z3 - z1);
  T fg = ((fx * gx) + (fy * gy)) + (fz * gz);
  return ((((fx * fx) + (fy * fy)) + (fz * fz)) * (((gx * gx) + (gy * gy)) + (gz * gz))) - fg * fg;
}

// calcElemCharacteristicLength, src/domain.jl:1893-1930.
template <class T>
inline T calcElemCharacteristicLength(const T x[8], const T y[8], const T z[8], const T& volume) {
  using std::sqrt;
  T charLength = T(0.0);
  static const int f[6][4] = {{0, 1, 2, 3}, {4, 5, 6, 7}, {0, 1, 5, 4},
                              {1, 2, 6, 5}, {2, 3, 7, 6}, {3, 0, 4, 7}};
  for (int i = 0; i < 6; ++i) {
    const int* q = f[i];
    T a = areaFace(x[q[0]], x[q[1]], x[q[2]], x[q[3]], y[q[0]], y[q[1]], y[q[2]], y[q[3]],
                   z[q[0]], z[q[1]], z[q[2]], z[q[3]]);
    charLength = jmax(a, charLength);
  }
  return (T(4.0) * volume) / sqrt(charLength);
}

// calcElemVelocityGradient, src/domain.jl:2023-2081 (only d1..d3 are kept by
// calcKinematicsForElems).
template <class T>
inline void calcElemVelocityGradient(const T xv[8], const T yv[8], const T zv[8], const T b[8][3],
                                     const T& detJ, T& d1, T& d2, T& d3) {
  T inv_detJ = T(1.0) / detJ;
  d1 = inv_detJ * ((((b[0][0] * (xv[0] - xv[6])) + (b[1][0] * (xv[1] - xv[7]))) +
                    (b[2][0] * (xv[2] - xv[4]))) + (b[3][0] * (xv[3] - xv[5])));
  d2 = inv_detJ * ((((b[0][1] * (yv[0] - yv[6])) + (b[1][1] * (yv[1] - yv[7]))) +
                    (b[2][1] * (yv[2] - yv[4]))) + (b[3][1] * (yv[3] - yv[5])));
  d3 = inv_detJ * ((((b[0][2] * (zv[0] - zv[6])) + (b[1][2] * (zv[1] - zv[7]))) +
                    (b[2][2] * (zv[2] - zv[4]))) + (b[3][2] * (zv[3] - zv[5])));
}

// ---------------------------------------------------------------------------
// Setup: Domain(prob), src/domain.jl:467-771 and helpers (single rank).
// ---------------------------------------------------------------------------

// createRegionIndexSets!, src/domain.jl:338-465. Julia's rand(Int) stream is
// not reproducible without Julia; std::mt19937_64 output reinterpreted as a
// signed Int64 is used in its place with the same bin structure (including
// the negative remainders Julia's rem produces). Regions never change results.
template <class T>
inline void createRegionIndexSets(Domain<T>& d, int nr, int b, uint64_t seed) {
  d.numReg = nr;
  d.balance = b;
  const int64_t numElem = d.numElem;
  std::mt19937_64 rng(seed);
  auto randInt = [&]() -> int64_t { return (int64_t)rng(); };
  std::vector<int64_t> regElemSize(nr, 0);
  d.regNumList.assign(numElem, 0);
  d.regElemlist.assign(numElem, 0);
  d.regCSR.assign(nr, 0);
  d.regReps.assign(nr, 0);
  d.regSorted.assign(nr, 0);
  int64_t nextIndex = 0;
  const int64_t myRank = 0;
  if (nr == 1) {
    while (nextIndex < numElem) { d.regNumList[nextIndex] = 1; nextIndex++; }
    regElemSize[0] = 0;
  } else {
    int64_t lastReg = -1, runto = 0, costDenominator = 0;
    std::vector<int64_t> regBinEnd(nr);
    for (int i = 1; i <= nr; ++i) {
      regElemSize[i - 1] = 0;
      int64_t pw = 1;
      for (int k = 0; k < b; ++k) pw *= i;
      costDenominator += pw;
      regBinEnd[i - 1] = costDenominator;
    }
    while (nextIndex < numElem) {
      int64_t regionVar = randInt() % costDenominator;
      int64_t i = 0;
      while (regionVar >= regBinEnd[i]) i++;
      int64_t regionNum = ((i + myRank) % nr) + 1;
      while (regionNum == lastReg) {
        regionVar = randInt() % costDenominator;
        i = 0;
        while (regionVar >= regBinEnd[i]) i++;
        regionNum = ((i + myRank) % nr) + 1;
      }
      int64_t binSize = randInt() % 1000;
      int64_t elements;
      if (binSize < 773) elements = randInt() % 15 + 1;
      else if (binSize < 937) elements = randInt() % 16 + 16;
      else if (binSize < 970) elements = randInt() % 32 + 32;
      else if (binSize < 974) elements = randInt() % 64 + 64;
      else if (binSize < 978) elements = randInt() % 128 + 128;
      else if (binSize < 981) elements = randInt() % 256 + 256;
      else elements = randInt() % 1537 + 512;
      runto = elements + nextIndex;
      while (nextIndex < runto && nextIndex < numElem) {
        d.regNumList[nextIndex] = regionNum;
        nextIndex++;
      }
      lastReg = regionNum;
    }
  }
  for (int64_t i = 0; i < numElem; ++i) regElemSize[d.regNumList[i] - 1] += 1;
  for (int r = 1; r <= nr; ++r) {
    int64_t rep;
    if (r < nr / 2) rep = 1;
    else if (r < (nr - (nr + 15) / 20)) rep = 1 + d.cost;
    else rep = 10 * (1 + d.cost);
    d.regReps[r - 1] = rep;
  }
  // sortRegions, src/domain.jl:313-336 (inner bound numReg-i-1 as written).
  {
    std::vector<int64_t> regIndex(nr);
    for (int v = 0; v < nr; ++v) regIndex[v] = v + 1;
    for (int i = 1; i <= nr - 1; ++i) {
      for (int j = 1; j <= nr - i - 1; ++j) {
        if (d.regReps[j - 1] < d.regReps[j]) {
          std::swap(d.regReps[j - 1], d.regReps[j]);
          std::swap(regElemSize[j - 1], regElemSize[j]);
          std::swap(regIndex[j - 1], regIndex[j]);
        }
      }
    }
    for (int i = 1; i <= nr; ++i) d.regSorted[regIndex[i - 1] - 1] = i;
  }
  d.regCSR[0] = 0;
  for (int i = 2; i <= nr; ++i) d.regCSR[i - 1] = d.regCSR[i - 2] + regElemSize[i - 2];
  for (int64_t i = 1; i <= numElem; ++i) {
    int64_t r = d.regSorted[d.regNumList[i - 1] - 1];
    d.regElemlist[d.regCSR[r - 1]] = i;
    d.regCSR[r - 1] += 1;
  }
  d.regElemSize = regElemSize;
}

template <class T>
inline void buildDomain(Domain<T>& d, const Problem& prob) {
  const int64_t nx = prob.nx;
  const int64_t edgeElems = nx, edgeNodes = nx + 1;
  d.mode = prob.mode;
  d.sizeX = edgeElems;
  d.numElem = edgeElems * edgeElems * edgeElems;
  d.numNode = edgeNodes * edgeNodes * edgeNodes;
  const int64_t E = d.numElem, N = d.numNode;

  auto zeros = [](std::vector<T>& a, int64_t n) { a.assign(n, T(0.0)); };
  for (auto* a : {&d.e, &d.p, &d.q, &d.ql, &d.qq, &d.v, &d.volo, &d.delv, &d.vdov, &d.arealg,
                  &d.ss, &d.elemMass, &d.vnew, &d.delv_xi, &d.delv_eta, &d.delv_zeta,
                  &d.delx_xi, &d.delx_eta, &d.delx_zeta, &d.dxx, &d.dyy, &d.dzz})
    zeros(*a, E);
  for (auto* a : {&d.x, &d.y, &d.z, &d.xd, &d.yd, &d.zd, &d.xdd, &d.ydd, &d.zdd, &d.fx, &d.fy,
                  &d.fz, &d.nodalMass})
    zeros(*a, N);
  d.v.assign(E, T(1.0));

  // buildMesh!, src/domain.jl:117-174 (single rank: colLoc = rowLoc = planeLoc = 0, tp = 1)
  const int64_t meshEdgeElems = nx;
  int64_t nidx = 0;
  for (int64_t plane = 0; plane < edgeNodes; ++plane) {
    T tz = T(1.125 * (double)plane) / T((double)meshEdgeElems);
    for (int64_t row = 0; row < edgeNodes; ++row) {
      T ty = T(1.125 * (double)row) / T((double)meshEdgeElems);
      for (int64_t col = 0; col < edgeNodes; ++col) {
        T tx = T(1.125 * (double)col) / T((double)meshEdgeElems);
        d.x[nidx] = tx; d.y[nidx] = ty; d.z[nidx] = tz;
        nidx++;
      }
    }
  }
  d.nodelist.assign(8 * E, 0);
  int64_t zidx = 0;
  nidx = 0;
  for (int64_t plane = 0; plane < edgeElems; ++plane) {
    for (int64_t row = 0; row < edgeElems; ++row) {
      for (int64_t col = 0; col < edgeElems; ++col) {
        int64_t* nl = &d.nodelist[8 * zidx];
        nl[0] = nidx;
        nl[1] = nidx + 1;
        nl[2] = nidx + edgeNodes + 1;
        nl[3] = nidx + edgeNodes;
        nl[4] = nidx + edgeNodes * edgeNodes;
        nl[5] = nidx + edgeNodes * edgeNodes + 1;
        nl[6] = nidx + edgeNodes * edgeNodes + edgeNodes + 1;
        nl[7] = nidx + edgeNodes * edgeNodes + edgeNodes;
        zidx++;
        nidx++;
      }
      nidx++;
    }
    nidx += edgeNodes;
  }

  // symmetry nodesets, src/domain.jl:579-608 and setupSymmetryPlanes :773-791
  const int64_t nbc = edgeNodes * edgeNodes;
  d.symmX.assign(nbc, 0); d.symmY.assign(nbc, 0); d.symmZ.assign(nbc, 0);
  nidx = 0;
  for (int64_t i = 0; i < edgeNodes; ++i) {
    int64_t planeInc = i * edgeNodes * edgeNodes, rowInc = i * edgeNodes;
    for (int64_t j = 0; j < edgeNodes; ++j) {
      d.symmZ[nidx] = rowInc + j;
      d.symmY[nidx] = planeInc + j;
      d.symmX[nidx] = planeInc + j * edgeNodes;
      nidx++;
    }
  }

  // node -> element-corner CSR, src/domain.jl:614-654 (corner values 1-based)
  d.nodeElemCount.assign(N, 0);
  for (int64_t i = 0; i < E; ++i)
    for (int j = 0; j < 8; ++j) d.nodeElemCount[d.nodelist[8 * i + j]] += 1;
  d.nodeElemStart.assign(N, 0);
  for (int64_t i = 1; i < N; ++i) d.nodeElemStart[i] = d.nodeElemStart[i - 1] + d.nodeElemCount[i - 1];
  d.nodeElemCornerList.assign(d.nodeElemStart[N - 1] + d.nodeElemCount[N - 1], 0);
  std::fill(d.nodeElemCount.begin(), d.nodeElemCount.end(), 0);
  for (int64_t i = 0; i < E; ++i) {
    for (int j = 0; j < 8; ++j) {
      int64_t m = d.nodelist[8 * i + j];
      int64_t k = 8 * i + j + 1;
      int64_t offset = d.nodeElemStart[m] + d.nodeElemCount[m];
      d.nodeElemCornerList[offset] = k;
      d.nodeElemCount[m] += 1;
    }
  }

  d.matElemlist.resize(E);
  for (int64_t i = 0; i < E; ++i) d.matElemlist[i] = i + 1;

  d.dthydro = T(1e20);
  d.dtcourant = T(1e20);
  d.time = T(0.0);
  d.dtfixed = T(-1.0e-6);
  d.deltatimemultlb = T(1.1);
  d.deltatimemultub = T(1.2);
  d.stoptime = T(1.0e-2);
  d.dtmax = T(1.0e-2);
  d.cycle = 0;
  d.e_cut = T(1.0e-7);
  d.p_cut = T(1.0e-7);
  d.q_cut = T(1.0e-7);
  d.u_cut = T(1.0e-7);
  d.v_cut = T(1.0e-10);
  d.hgcoef = T(3.0);
  d.ss4o3 = T(4.0 / 3.0);
  d.qstop = T(1.0e+12);
  d.monoq_max_slope = T(1.0);
  d.monoq_limiter_mult = T(2.0);
  d.qlc_monoq = T(0.5);
  d.qqc_monoq = T(2.0 / 3.0);
  d.qqc = T(2.0);
  d.pmin = T(0.0);
  d.emin = T(-1.0e+15);
  d.dvovmax = T(0.1);
  d.eosvmax = T(1.0e+9);
  d.eosvmin = T(1.0e-9);
  d.refdens = T(1.0);

  // volumes and masses, src/domain.jl:709-731
  for (int64_t i = 0; i < E; ++i) {
    T xl[8], yl[8], zl[8];
    for (int l = 0; l < 8; ++l) {
      int64_t g = d.nodelist[8 * i + l];
      xl[l] = d.x[g]; yl[l] = d.y[g]; zl[l] = d.z[g];
    }
    T volume = calcElemVolume(xl, yl, zl);
    d.volo[i] = volume;
    d.elemMass[i] = volume;
    for (int j = 0; j < 8; ++j) {
      int64_t g = d.nodelist[8 * i + j];
      d.nodalMass[g] = d.nodalMass[g] + volume / T(8.0);
    }
  }

  // energy deposit and initial dt, src/domain.jl:738-749
  const double ebase = 3.948746e+7;
  const double scale = (double)(nx * 1) / 45.0;
  const double einit = ebase * scale * scale * scale;
  d.e[0] = T(einit);
  {
    using std::cbrt; using std::sqrt;
    d.deltatime = (T(0.5) * cbrt(d.volo[0])) / sqrt(T(2.0 * einit));
  }

  d.cost = prob.cost;
  createRegionIndexSets(d, prob.nr, prob.balance, prob.region_seed);

  // setupElementConnectivities, src/domain.jl:793-820 (raw Julia values)
  d.lxim.assign(E, 0); d.lxip.assign(E, 0); d.letam.assign(E, 0); d.letap.assign(E, 0);
  d.lzetam.assign(E, 0); d.lzetap.assign(E, 0);
  d.lxim[0] = 1;
  for (int64_t i = 1; i <= E - 1; ++i) { d.lxim[i] = i - 1; d.lxip[i - 1] = i; }
  d.lxip[E - 1] = E - 1;
  for (int64_t i = 0; i < edgeElems; ++i) { d.letam[i] = i; d.letap[E - edgeElems + i] = i; }
  for (int64_t i = edgeElems; i <= E - 1; ++i) { d.letam[i] = i - edgeElems; d.letap[i - edgeElems] = i; }
  const int64_t e2 = edgeElems * edgeElems;
  for (int64_t i = 0; i < e2; ++i) { d.lzetam[i] = i; d.lzetap[E - e2 + i] = E - e2 + i; }
  for (int64_t i = e2; i <= E - 1; ++i) { d.lzetam[i] = i - e2; d.lzetap[i - e2] = i; }

  // setupBoundaryConditions, src/domain.jl:822-916 (single rank: no COMM faces)
  d.elemBC.assign(E, 0);
  for (int64_t i = 0; i < edgeElems; ++i) {
    int64_t planeInc = i * e2, rowInc = i * edgeElems;
    for (int64_t j = 0; j < edgeElems; ++j) {
      d.elemBC[rowInc + j] |= ZETA_M_SYMM;
      d.elemBC[rowInc + j + E - e2] |= ZETA_P_FREE;
      d.elemBC[planeInc + j] |= ETA_M_SYMM;
      d.elemBC[planeInc + j + e2 - edgeElems] |= ETA_P_FREE;
      d.elemBC[planeInc + j * edgeElems] |= XI_M_SYMM;
      d.elemBC[planeInc + j * edgeElems + edgeElems - 1] |= XI_P_FREE;
    }
  }

  d.fx_elem.assign(8 * E, T(0.0)); d.fy_elem.assign(8 * E, T(0.0)); d.fz_elem.assign(8 * E, T(0.0));
  d.determ.assign(E, T(0.0));
  d.dvdx.assign(8 * E, T(0.0)); d.dvdy.assign(8 * E, T(0.0)); d.dvdz.assign(8 * E, T(0.0));
  d.x8n.assign(8 * E, T(0.0)); d.y8n.assign(8 * E, T(0.0)); d.z8n.assign(8 * E, T(0.0));
  d.sigxx.assign(E, T(0.0));
}

// ---------------------------------------------------------------------------
// timeIncrement!, src/domain.jl:920-961
// ---------------------------------------------------------------------------
template <class T>
inline void timeIncrement(Domain<T>& d) {
  T targetdt = d.stoptime - d.time;
  if (val(d.dtfixed) <= 0.0 && d.cycle != 0) {
    T olddt = d.deltatime;
    T gnewdt = T(INFINITY);  // typemax(Float64)
    T newdt = T(0.0);
    if (val(d.dtcourant) < val(gnewdt)) gnewdt = d.dtcourant / T(2.0);
    if (val(d.dthydro) < val(gnewdt)) gnewdt = d.dthydro * T(2.0) / T(3.0);
    newdt = gnewdt;  // comm_min at one rank
    T ratio = newdt / olddt;
    if (val(ratio) >= 1.0) {
      if (val(ratio) < val(d.deltatimemultlb)) newdt = olddt;
      else if (val(ratio) > val(d.deltatimemultub)) newdt = olddt * d.deltatimemultub;
    }
    newdt = jmin(newdt, d.dtmax);
    d.deltatime = newdt;
  }
  if (val(d.deltatime) < val(targetdt) && val(targetdt) < val(T(4.0) * d.deltatime / T(3.0)))
    targetdt = T(2.0) * d.deltatime / T(3.0);
  if (val(targetdt) < val(d.deltatime)) d.deltatime = targetdt;
  d.time = d.time + d.deltatime;
  d.cycle += 1;
}

// ---------------------------------------------------------------------------
// lagrangeNodal, src/domain.jl:963-1872
// ---------------------------------------------------------------------------
template <class T>
inline void gatherNodal(const Domain<T>& d, const std::vector<T>& src, int64_t k, T out[8]) {
  for (int i = 0; i < 8; ++i) out[i] = src[d.nodelist[8 * k + i]];
}

#ifdef _OPENMP
#define ORA_PARFOR _Pragma("omp parallel for schedule(static)")
#else
#define ORA_PARFOR
#endif

// integrateStressForElems, src/domain.jl:1087-1128. Returns status.
template <class T>
inline int integrateStressForElems(Domain<T>& d) {
  const int64_t E = d.numElem, N = d.numNode;
  int64_t bad = -1;
  ORA_PARFOR
  for (int64_t k = 0; k < E; ++k) {
    T xl[8], yl[8], zl[8];
    gatherNodal(d, d.x, k, xl); gatherNodal(d, d.y, k, yl); gatherNodal(d, d.z, k, zl);
    T detJ = calcElemShapeFunctionDerivatives<T>(xl, yl, zl, nullptr);
    d.determ[k] = detJ;
    if (val(detJ) <= 0.0) {
#ifdef _OPENMP
#pragma omp critical
#endif
      { if (bad < 0 || k < bad) bad = k; }
    }
    T B[8][3];
    calcElemNodeNormals(xl, yl, zl, B, d.mode);
    // sumElemStressesToNodeForces, src/domain.jl:1069-1084; sig = -p - q
    T sig = (-d.p[k]) - d.q[k];
    for (int c = 0; c < 8; ++c) {
      d.fx_elem[8 * k + c] = (-sig) * B[c][0];
      d.fy_elem[8 * k + c] = (-sig) * B[c][1];
      d.fz_elem[8 * k + c] = (-sig) * B[c][2];
    }
  }
  if (bad >= 0) { d.error_site = SITE_EARLY; d.error_index = bad; return ERR_VOLUME; }
  ORA_PARFOR
  for (int64_t g = 0; g < N; ++g) {
    int64_t count = d.nodeElemCount[g], start = d.nodeElemStart[g];
    T fx = T(0.0), fy = T(0.0), fz = T(0.0);
    for (int64_t i = 0; i < count; ++i) {
      int64_t el = d.nodeElemCornerList[start + i] - 1;
      fx = fx + d.fx_elem[el];
      fy = fy + d.fy_elem[el];
      fz = fz + d.fz_elem[el];
    }
    d.fx[g] = fx; d.fy[g] = fy; d.fz[g] = fz;
  }
  return OK;
}

// calcFBHourglassForceForElems + calcElemFBHourglassForce,
// src/domain.jl:1258-1694.
template <class T>
inline void calcFBHourglassForceForElems(Domain<T>& d, const T& hourg) {
  using std::cbrt;
  const int64_t E = d.numElem, N = d.numNode;
  static const double gamma[8][4] = {{1, 1, 1, -1}, {1, -1, -1, 1}, {-1, -1, 1, -1}, {-1, 1, -1, 1},
                                     {-1, -1, 1, 1}, {-1, 1, -1, -1}, {1, 1, 1, 1}, {1, -1, -1, -1}};
  ORA_PARFOR
  for (int64_t i2 = 0; i2 < E; ++i2) {
    const int64_t i3 = 8 * i2;
    T volinv = T(1.0) / d.determ[i2];
    T hg[8][4];
    for (int m = 0; m < 4; ++m) {
      T hx = d.x8n[i3] * T(gamma[0][m]), hy = d.y8n[i3] * T(gamma[0][m]), hz = d.z8n[i3] * T(gamma[0][m]);
      for (int n = 1; n < 8; ++n) {
        hx = hx + d.x8n[i3 + n] * T(gamma[n][m]);
        hy = hy + d.y8n[i3 + n] * T(gamma[n][m]);
        hz = hz + d.z8n[i3 + n] * T(gamma[n][m]);
      }
      for (int n = 0; n < 8; ++n)
        hg[n][m] = T(gamma[n][m]) -
                   volinv * (((d.dvdx[i3 + n] * hx) + (d.dvdy[i3 + n] * hy)) + (d.dvdz[i3 + n] * hz));
    }
    T ss1 = d.ss[i2], mass1 = d.elemMass[i2];
    T volume13 = cbrt(d.determ[i2]);
    T xd1[8], yd1[8], zd1[8];
    gatherNodal(d, d.xd, i2, xd1); gatherNodal(d, d.yd, i2, yd1); gatherNodal(d, d.zd, i2, zd1);
    T coefficient = ((((-hourg) * T(0.01)) * ss1) * mass1) / volume13;
    const T* vel[3] = {xd1, yd1, zd1};
    std::vector<T>* out[3] = {&d.fx_elem, &d.fy_elem, &d.fz_elem};
    for (int dim = 0; dim < 3; ++dim) {
      const T* vv = vel[dim];
      T h[4];
      for (int m = 0; m < 4; ++m) {
        T s = hg[0][m] * vv[0];
        for (int n = 1; n < 8; ++n) s = s + hg[n][m] * vv[n];
        h[m] = s;
      }
      for (int n = 0; n < 8; ++n)
        (*out[dim])[i3 + n] =
            coefficient * ((((hg[n][0] * h[0]) + (hg[n][1] * h[1])) + (hg[n][2] * h[2])) + (hg[n][3] * h[3]));
    }
  }
  ORA_PARFOR
  for (int64_t g = 0; g < N; ++g) {
    int64_t count = d.nodeElemCount[g], start = d.nodeElemStart[g];
    T fx = T(0.0), fy = T(0.0), fz = T(0.0);
    for (int64_t i = 0; i < count; ++i) {
      int64_t el = d.nodeElemCornerList[start + i] - 1;
      fx = fx + d.fx_elem[el];
      fy = fy + d.fy_elem[el];
      fz = fz + d.fz_elem[el];
    }
    d.fx[g] = d.fx[g] + fx; d.fy[g] = d.fy[g] + fy; d.fz[g] = d.fz[g] + fz;
  }
}

// calcHourglassControlForElems, src/domain.jl:1696-1736.
template <class T>
inline int calcHourglassControlForElems(Domain<T>& d, const T& hgcoef) {
  const int64_t E = d.numElem;
  int64_t bad = -1;
  ORA_PARFOR
  for (int64_t i = 0; i < E; ++i) {
    T x1[8], y1[8], z1[8];
    gatherNodal(d, d.x, i, x1); gatherNodal(d, d.y, i, y1); gatherNodal(d, d.z, i, z1);
    T pfx[8], pfy[8], pfz[8];
    calcElemVolumeDerivative(x1, y1, z1, pfx, pfy, pfz, d.mode);
    for (int ii = 0; ii < 8; ++ii) {
      int64_t jj = 8 * i + ii;
      d.dvdx[jj] = pfx[ii]; d.dvdy[jj] = pfy[ii]; d.dvdz[jj] = pfz[ii];
      d.x8n[jj] = x1[ii]; d.y8n[jj] = y1[ii]; d.z8n[jj] = z1[ii];
    }
    d.determ[i] = d.volo[i] * d.v[i];
    if (val(d.v[i]) <= 0.0) {
#ifdef _OPENMP
#pragma omp critical
#endif
      { if (bad < 0 || i < bad) bad = i; }
    }
  }
  if (bad >= 0) { d.error_site = SITE_HOURGLASS; d.error_index = bad; return ERR_VOLUME; }
  if (val(hgcoef) > 0.0) calcFBHourglassForceForElems(d, hgcoef);
  return OK;
}

// calcForceForNodes + calcVolumeForceForElems, src/domain.jl:1738-1779.
template <class T>
inline int calcForceForNodes(Domain<T>& d) {
  const int64_t N = d.numNode, E = d.numElem;
  for (int64_t g = 0; g < N; ++g) { d.fx[g] = T(0.0); d.fy[g] = T(0.0); d.fz[g] = T(0.0); }
  int st = integrateStressForElems(d);
  if (st) return st;
  for (int64_t i = 0; i < E; ++i)
    if (val(d.determ[i]) <= 0.0) { d.error_site = SITE_MID; d.error_index = i; return ERR_VOLUME; }
  return calcHourglassControlForElems(d, d.hgcoef);
}

// lagrangeNodal, src/domain.jl:1781-1872 (communication is a no-op at one rank).
template <class T>
inline int lagrangeNodal(Domain<T>& d) {
  const int64_t N = d.numNode;
  T delt = d.deltatime;
  T u_cut = d.u_cut;
  int st = calcForceForNodes(d);
  if (st) return st;
  ORA_PARFOR
  for (int64_t i = 0; i < N; ++i) {
    d.xdd[i] = d.fx[i] / d.nodalMass[i];
    d.ydd[i] = d.fy[i] / d.nodalMass[i];
    d.zdd[i] = d.fz[i] / d.nodalMass[i];
  }
  const int64_t numNodeBC = (d.sizeX + 1) * (d.sizeX + 1);
  for (int64_t i = 0; i < numNodeBC; ++i) d.xdd[d.symmX[i]] = T(0.0);
  for (int64_t i = 0; i < numNodeBC; ++i) d.ydd[d.symmY[i]] = T(0.0);
  for (int64_t i = 0; i < numNodeBC; ++i) d.zdd[d.symmZ[i]] = T(0.0);
  ORA_PARFOR
  for (int64_t i = 0; i < N; ++i) {
    using std::fabs;
    T xdtmp = d.xd[i] + d.xdd[i] * delt;
    if (fabs(val(xdtmp)) < val(u_cut)) xdtmp = T(0.0);
    d.xd[i] = xdtmp;
    T ydtmp = d.yd[i] + d.ydd[i] * delt;
    if (fabs(val(ydtmp)) < val(u_cut)) ydtmp = T(0.0);
    d.yd[i] = ydtmp;
    T zdtmp = d.zd[i] + d.zdd[i] * delt;
    if (fabs(val(zdtmp)) < val(u_cut)) zdtmp = T(0.0);
    d.zd[i] = zdtmp;
  }
  ORA_PARFOR
  for (int64_t i = 0; i < N; ++i) {
    d.x[i] = d.x[i] + d.xd[i] * delt;
    d.y[i] = d.y[i] + d.yd[i] * delt;
    d.z[i] = d.z[i] + d.zd[i] * delt;
  }
  return OK;
}

// ---------------------------------------------------------------------------
// lagrangeElements, src/domain.jl:2099-2962
// ---------------------------------------------------------------------------

// calcKinematicsForElems, src/domain.jl:2099-2147.
template <class T>
inline int calcKinematicsForElems(Domain<T>& d, const T& dt) {
  const int64_t E = d.numElem;
  int64_t bad = -1;
  ORA_PARFOR
  for (int64_t k = 0; k < E; ++k) {
    T xl[8], yl[8], zl[8];
    gatherNodal(d, d.x, k, xl); gatherNodal(d, d.y, k, yl); gatherNodal(d, d.z, k, zl);
    T volume = calcElemVolume(xl, yl, zl);
    T relativeVolume = volume / d.volo[k];
    d.vnew[k] = relativeVolume;
    if (val(relativeVolume) <= 0.0) {
#ifdef _OPENMP
#pragma omp critical
#endif
      { if (bad < 0 || k < bad) bad = k; }
    }
    d.delv[k] = relativeVolume - d.v[k];
    d.arealg[k] = calcElemCharacteristicLength(xl, yl, zl, volume);
    T xv[8], yv[8], zv[8];
    gatherNodal(d, d.xd, k, xv); gatherNodal(d, d.yd, k, yv); gatherNodal(d, d.zd, k, zv);
    T dt2 = T(0.5) * dt;
    for (int j = 0; j < 8; ++j) {
      xl[j] = xl[j] - dt2 * xv[j];
      yl[j] = yl[j] - dt2 * yv[j];
      zl[j] = zl[j] - dt2 * zv[j];
    }
    T B[8][3];
    T detJ = calcElemShapeFunctionDerivatives(xl, yl, zl, B);
    T d1, d2, d3;
    calcElemVelocityGradient(xv, yv, zv, B, detJ, d1, d2, d3);
    d.dxx[k] = d1; d.dyy[k] = d2; d.dzz[k] = d3;
  }
  if (bad >= 0) { d.error_site = SITE_KINEMATICS; d.error_index = bad; return ERR_VOLUME; }
  return OK;
}

// calcLagrangeElements, src/domain.jl:2149-2173.
template <class T>
inline int calcLagrangeElements(Domain<T>& d, const T& delt) {
  const int64_t E = d.numElem;
  if (E > 0) {
    int st = calcKinematicsForElems(d, delt);
    if (st) return st;
    for (int64_t k = 0; k < E; ++k) {
      T vdov = (d.dxx[k] + d.dyy[k]) + d.dzz[k];
      T vdovthird = vdov / T(3.0);
      d.vdov[k] = vdov;
      d.dxx[k] = d.dxx[k] - vdovthird;
      d.dyy[k] = d.dyy[k] - vdovthird;
      d.dzz[k] = d.dzz[k] - vdovthird;
      if (val(d.vnew[k]) <= 0.0) { d.error_site = SITE_LAGRANGE; d.error_index = k; return ERR_VOLUME; }
    }
  }
  return OK;
}

// calcMonotonicQGradientsForElems, src/domain.jl:2175-2320.
template <class T>
inline void calcMonotonicQGradientsForElems(Domain<T>& d) {
  using std::sqrt;
  const T ptiny = T(1.e-36);
  const int64_t E = d.numElem;
  auto sum4 = [](const T& a, const T& b, const T& c, const T& e) -> T { return ((a + b) + c) + e; };
  ORA_PARFOR
  for (int64_t i = 0; i < E; ++i) {
    T x[8], y[8], z[8], xv[8], yv[8], zv[8];
    gatherNodal(d, d.x, i, x); gatherNodal(d, d.y, i, y); gatherNodal(d, d.z, i, z);
    gatherNodal(d, d.xd, i, xv); gatherNodal(d, d.yd, i, yv); gatherNodal(d, d.zd, i, zv);
    T vol = d.volo[i] * d.vnew[i];
    T norm = T(1.0) / (vol + ptiny);
    T dxj = T(-0.25) * (sum4(x[0], x[1], x[5], x[4]) - sum4(x[3], x[2], x[6], x[7]));
    T dyj = T(-0.25) * (sum4(y[0], y[1], y[5], y[4]) - sum4(y[3], y[2], y[6], y[7]));
    T dzj = T(-0.25) * (sum4(z[0], z[1], z[5], z[4]) - sum4(z[3], z[2], z[6], z[7]));
    T dxi = T(0.25) * (sum4(x[1], x[2], x[6], x[5]) - sum4(x[0], x[3], x[7], x[4]));
    T dyi = T(0.25) * (sum4(y[1], y[2], y[6], y[5]) - sum4(y[0], y[3], y[7], y[4]));
    T dzi = T(0.25) * (sum4(z[1], z[2], z[6], z[5]) - sum4(z[0], z[3], z[7], z[4]));
    T dxk = T(0.25) * (sum4(x[4], x[5], x[6], x[7]) - sum4(x[0], x[1], x[2], x[3]));
    T dyk = T(0.25) * (sum4(y[4], y[5], y[6], y[7]) - sum4(y[0], y[1], y[2], y[3]));
    T dzk = T(0.25) * (sum4(z[4], z[5], z[6], z[7]) - sum4(z[0], z[1], z[2], z[3]));

    // zeta: i cross j
    T ax = (dyi * dzj) - (dzi * dyj);
    T ay = (dzi * dxj) - (dxi * dzj);
    T az = (dxi * dyj) - (dyi * dxj);
    d.delx_zeta[i] = vol / sqrt((((ax * ax) + (ay * ay)) + (az * az)) + ptiny);
    ax = ax * norm; ay = ay * norm; az = az * norm;
    T dxv = T(0.25) * (sum4(xv[4], xv[5], xv[6], xv[7]) - sum4(xv[0], xv[1], xv[2], xv[3]));
    T dyv = T(0.25) * (sum4(yv[4], yv[5], yv[6], yv[7]) - sum4(yv[0], yv[1], yv[2], yv[3]));
    T dzv = T(0.25) * (sum4(zv[4], zv[5], zv[6], zv[7]) - sum4(zv[0], zv[1], zv[2], zv[3]));
    d.delv_zeta[i] = ((ax * dxv) + (ay * dyv)) + (az * dzv);

    // xi: j cross k
    ax = (dyj * dzk) - (dzj * dyk);
    ay = (dzj * dxk) - (dxj * dzk);
    az = (dxj * dyk) - (dyj * dxk);
    d.delx_xi[i] = vol / sqrt((((ax * ax) + (ay * ay)) + (az * az)) + ptiny);
    ax = ax * norm; ay = ay * norm; az = az * norm;
    dxv = T(0.25) * (sum4(xv[1], xv[2], xv[6], xv[5]) - sum4(xv[0], xv[3], xv[7], xv[4]));
    dyv = T(0.25) * (sum4(yv[1], yv[2], yv[6], yv[5]) - sum4(yv[0], yv[3], yv[7], yv[4]));
    dzv = T(0.25) * (sum4(zv[1], zv[2], zv[6], zv[5]) - sum4(zv[0], zv[3], zv[7], zv[4]));
    d.delv_xi[i] = ((ax * dxv) + (ay * dyv)) + (az * dzv);

    // eta: k cross i
    ax = (dyk * dzi) - (dzk * dyi);
    ay = (dzk * dxi) - (dxk * dzi);
    az = (dxk * dyi) - (dyk * dxi);
    d.delx_eta[i] = vol / sqrt((((ax * ax) + (ay * ay)) + (az * az)) + ptiny);
    ax = ax * norm; ay = ay * norm; az = az * norm;
    dxv = T(-0.25) * (sum4(xv[0], xv[1], xv[5], xv[4]) - sum4(xv[3], xv[2], xv[6], xv[7]));
    dyv = T(-0.25) * (sum4(yv[0], yv[1], yv[5], yv[4]) - sum4(yv[3], yv[2], yv[6], yv[7]));
    dzv = T(-0.25) * (sum4(zv[0], zv[1], zv[5], zv[4]) - sum4(zv[3], zv[2], zv[6], zv[7]));
    d.delv_eta[i] = ((ax * dxv) + (ay * dyv)) + (az * dzv);
  }
}

// One limiter direction of calcMonotonicQRegionForElems, src/domain.jl:2330-2376.
template <class T>
inline T monoqPhi(const T& delv_self, const T& delvm_in, const T& delvp_in, const T& ptiny,
                  const T& monoq_limiter_mult, const T& monoq_max_slope) {
  T norm = T(1.0) / (delv_self + ptiny);
  T delvm = delvm_in * norm;
  T delvp = delvp_in * norm;
  T phi = T(0.5) * (delvm + delvp);
  delvm = delvm * monoq_limiter_mult;
  delvp = delvp * monoq_limiter_mult;
  if (val(delvm) < val(phi)) phi = delvm;
  if (val(delvp) < val(phi)) phi = delvp;
  if (val(phi) < 0.0) phi = T(0.0);
  if (val(phi) > val(monoq_max_slope)) phi = monoq_max_slope;
  return phi;
}

// calcMonotonicQRegionForElems, src/domain.jl:2322-2513. Returns status.
template <class T>
inline int calcMonotonicQRegionForElems(Domain<T>& d, const T& qlc_monoq, const T& qqc_monoq,
                                        const T& monoq_limiter_mult, const T& monoq_max_slope,
                                        const T& ptiny, int64_t elength) {
  int64_t bad = -1;
  ORA_PARFOR
  for (int64_t ielem = 0; ielem < elength; ++ielem) {
    const int64_t i = d.matElemlist[ielem] - 1;
    const uint32_t bcMask = d.elemBC[i];
    bool badbc = false;
    auto neigh = [&](const std::vector<T>& dv, uint32_t mask, uint32_t symm, uint32_t freeb,
                     uint32_t comm, int64_t idx) -> T {
      uint32_t c = bcMask & mask;
      if (c == 0 || c == comm) return dv[idx];
      if (c == symm) return dv[i];
      if (c == freeb) return T(0.0);
      badbc = true;
      return T(0.0);
    };
    // xi-plus neighbour: FAITHFUL indexes delv_xi with the raw lxip value
    // (1-based array, no +1), i.e. 0-based lxip-1.
    int64_t ixp = (d.mode & FIX_LXIP) ? d.lxip[i] : d.lxip[i] - 1;
    T delvm = neigh(d.delv_xi, XI_M, XI_M_SYMM, XI_M_FREE, XI_M_COMM, d.lxim[i]);
    T delvp = neigh(d.delv_xi, XI_P, XI_P_SYMM, XI_P_FREE, XI_P_COMM, ixp);
    T phixi = monoqPhi(d.delv_xi[i], delvm, delvp, ptiny, monoq_limiter_mult, monoq_max_slope);
    delvm = neigh(d.delv_eta, ETA_M, ETA_M_SYMM, ETA_M_FREE, ETA_M_COMM, d.letam[i]);
    delvp = neigh(d.delv_eta, ETA_P, ETA_P_SYMM, ETA_P_FREE, ETA_P_COMM, d.letap[i]);
    T phieta = monoqPhi(d.delv_eta[i], delvm, delvp, ptiny, monoq_limiter_mult, monoq_max_slope);
    delvm = neigh(d.delv_zeta, ZETA_M, ZETA_M_SYMM, ZETA_M_FREE, ZETA_M_COMM, d.lzetam[i]);
    delvp = neigh(d.delv_zeta, ZETA_P, ZETA_P_SYMM, ZETA_P_FREE, ZETA_P_COMM, d.lzetap[i]);
    T phizeta = monoqPhi(d.delv_zeta[i], delvm, delvp, ptiny, monoq_limiter_mult, monoq_max_slope);
    if (badbc) {
#ifdef _OPENMP
#pragma omp critical
#endif
      { if (bad < 0 || i < bad) bad = i; }
    }
    T qlin, qquad;
    if (val(d.vdov[i]) > 0.0) {
      qlin = T(0.0);
      qquad = T(0.0);
    } else {
      T delvxxi = d.delv_xi[i] * d.delx_xi[i];
      T delvxeta = d.delv_eta[i] * d.delx_eta[i];
      T delvxzeta = d.delv_zeta[i] * d.delx_zeta[i];
      if (val(delvxxi) > 0.0) delvxxi = T(0.0);
      if (val(delvxeta) > 0.0) delvxeta = T(0.0);
      if (val(delvxzeta) > 0.0) delvxzeta = T(0.0);
      T rho = d.elemMass[i] / (d.volo[i] * d.vnew[i]);
      qlin = ((-qlc_monoq) * rho) *
             (((delvxxi * (T(1.0) - phixi)) + (delvxeta * (T(1.0) - phieta))) +
              (delvxzeta * (T(1.0) - phizeta)));
      qquad = (qqc_monoq * rho) *
              ((((delvxxi * delvxxi) * (T(1.0) - phixi * phixi)) +
                ((delvxeta * delvxeta) * (T(1.0) - phieta * phieta))) +
               ((delvxzeta * delvxzeta) * (T(1.0) - phizeta * phizeta)));
    }
    d.qq[i] = qquad;
    d.ql[i] = qlin;
  }
  if (bad >= 0) { d.error_index = bad; return ERR_BAD_BC; }
  return OK;
}

// calcQForElems, src/domain.jl:2541-2583.
template <class T>
inline int calcQForElems(Domain<T>& d) {
  const int64_t E = d.numElem;
  calcMonotonicQGradientsForElems(d);
  if (E > 0) {
    int st = calcMonotonicQRegionForElems(d, d.qlc_monoq, d.qqc_monoq, d.monoq_limiter_mult,
                                          d.monoq_max_slope, T(1e-36), E);
    if (st) return st;
  }
  if (E != 0) {
    for (int64_t i = 0; i < E; ++i)
      if (val(d.q[i]) > val(d.qstop)) { d.error_index = i; return ERR_QSTOP; }
  }
  return OK;
}

// calcPressureForElems, src/domain.jl:2585-2614, for one element.
template <class T>
inline void calcPressure(T& p_new, T& bvc, T& pbvc, const T& e_old, const T& compression,
                         const T& vnewc, const T& pmin, const T& p_cut, const T& eosvmax) {
  using std::fabs;
  const T c1s = T(2.0) / T(3.0);
  bvc = c1s * (compression + T(1.0));
  pbvc = c1s;
  p_new = bvc * e_old;
  if (fabs(val(p_new)) < val(p_cut)) p_new = T(0.0);
  if (val(vnewc) >= val(eosvmax)) p_new = T(0.0);
  if (val(p_new) < val(pmin)) p_new = pmin;
}

// evalEOSForElems + calcEnergyForElems + calcSoundSpeedForElems,
// src/domain.jl:2617-2857, for one element (every loop in the reference is
// elementwise, so fusing the loops per element does not change any result).
template <class T>
inline void evalEOSElem(Domain<T>& d, int64_t zidx, const T& vnewc_in) {
  using std::fabs; using std::sqrt;
  const T e_cut = d.e_cut, p_cut = d.p_cut, q_cut = d.q_cut;
  const T eosvmax = d.eosvmax, eosvmin = d.eosvmin, pmin = d.pmin, emin = d.emin, rho0 = d.refdens;
  const T TINY1 = T(0.111111e-36), TINY3 = T(0.333333e-18), SIXTH = T(1.0) / T(6.0);
  const T vnewc = vnewc_in;
  T e_old = d.e[zidx], delvc = d.delv[zidx], p_old = d.p[zidx], q_old = d.q[zidx];
  T compression = T(1.0) / vnewc - T(1.0);
  T vchalf = vnewc - delvc * T(0.5);
  T compHalfStep = (T(1.0) / vchalf) - T(1.0);
  if (val(eosvmin) != 0.0 && val(vnewc) <= val(eosvmin)) compHalfStep = compression;
  if (val(eosvmax) != 0.0 && val(vnewc) >= val(eosvmax)) {
    p_old = T(0.0); compression = T(0.0); compHalfStep = T(0.0);
  }
  T qq = d.qq[zidx], ql = d.ql[zidx], work = T(0.0);

  // calcEnergyForElems
  T p_new, e_new, q_new, bvc, pbvc, pHalfStep;
  e_new = (e_old - ((T(0.5) * delvc) * (p_old + q_old))) + (T(0.5) * work);
  if (val(e_new) < val(emin)) e_new = emin;
  calcPressure(pHalfStep, bvc, pbvc, e_new, compHalfStep, vnewc, pmin, p_cut, eosvmax);
  T vhalf = T(1.0) / (T(1.0) + compHalfStep);
  if (val(delvc) > 0.0) {
    q_new = T(0.0);
  } else {
    T ssc = ((pbvc * e_new) + (((vhalf * vhalf) * bvc) * pHalfStep)) / rho0;
    if (val(ssc) <= val(TINY1)) ssc = TINY3; else ssc = sqrt(ssc);
    q_new = (ssc * ql) + qq;
  }
  e_new = e_new + ((T(0.5) * delvc) * ((T(3.0) * (p_old + q_old)) - (T(4.0) * (pHalfStep + q_new))));
  e_new = e_new + (T(0.5) * work);
  if (fabs(val(e_new)) < val(e_cut)) e_new = T(0.0);
  if (val(e_new) < val(emin)) e_new = emin;
  calcPressure(p_new, bvc, pbvc, e_new, compression, vnewc, pmin, p_cut, eosvmax);
  T q_tilde;
  if (val(delvc) > 0.0) {
    q_tilde = T(0.0);
  } else {
    T ssc = ((pbvc * e_new) + (((vnewc * vnewc) * bvc) * p_new)) / rho0;
    if (val(ssc) <= val(TINY1)) ssc = TINY3; else ssc = sqrt(ssc);
    q_tilde = (ssc * ql) + qq;
  }
  e_new = e_new - (((((T(7.0) * (p_old + q_old)) - (T(8.0) * (pHalfStep + q_new))) + (p_new + q_tilde)) *
                    delvc) * SIXTH);
  if (fabs(val(e_new)) < val(e_cut)) e_new = T(0.0);
  if (val(e_new) < val(emin)) e_new = emin;
  calcPressure(p_new, bvc, pbvc, e_new, compression, vnewc, pmin, p_cut, eosvmax);
  if (val(delvc) <= 0.0) {
    T ssc = ((pbvc * e_new) + (((vnewc * vnewc) * bvc) * p_new)) / rho0;
    if (val(ssc) <= val(TINY1)) ssc = TINY3; else ssc = sqrt(ssc);
    q_new = (ssc * ql) + qq;
    if (fabs(val(q_new)) < val(q_cut)) q_new = T(0.0);
  }
  d.p[zidx] = p_new;
  d.e[zidx] = e_new;
  d.q[zidx] = q_new;
  // calcSoundSpeedForElems
  T ssTmp = ((pbvc * e_new) + (((vnewc * vnewc) * bvc) * p_new)) / rho0;
  if (val(ssTmp) <= val(TINY1)) ssTmp = TINY3; else ssTmp = sqrt(ssTmp);
  d.ss[zidx] = ssTmp;
}

// applyMaterialPropertiesForElems, src/domain.jl:2860-2910.
template <class T>
inline int applyMaterialPropertiesForElems(Domain<T>& d) {
  const int64_t length = d.numElem;
  if (length == 0) return OK;
  const T eosvmin = d.eosvmin, eosvmax = d.eosvmax;
  std::vector<T> vnewc(length);
  for (int64_t i = 0; i < length; ++i) {
    T vc = d.vnew[d.matElemlist[i] - 1];
    if (val(eosvmin) != 0.0 && val(vc) < val(eosvmin)) vc = eosvmin;
    if (val(eosvmax) != 0.0 && val(vc) > val(eosvmax)) vc = eosvmax;
    vnewc[i] = vc;
  }
  for (int64_t i = 0; i < length; ++i) {
    T vc = d.v[d.matElemlist[i] - 1];
    if (val(eosvmin) != 0.0 && val(vc) < val(eosvmin)) vc = eosvmin;
    if (val(eosvmax) != 0.0 && val(vc) > val(eosvmax)) vc = eosvmax;
    if (val(vc) <= 0.0) { d.error_site = SITE_MATERIAL; d.error_index = i; return ERR_VOLUME; }
  }
  ORA_PARFOR
  for (int64_t i = 0; i < length; ++i) evalEOSElem(d, d.matElemlist[i] - 1, vnewc[i]);
  return OK;
}

// updateVolumesForElems, src/domain.jl:2912-2930.
template <class T>
inline int updateVolumesForElems(Domain<T>& d) {
  using std::fabs;
  const int64_t E = d.numElem;
  for (int64_t i = 0; i < E; ++i) {
    T tmpV = d.vnew[i];
    if (fabs(val(tmpV) - 1.0) < val(d.v_cut)) tmpV = T(1.0);
    d.v[i] = tmpV;
    if (val(tmpV) <= 0.0) { d.error_site = SITE_UPDATE; d.error_index = i; return ERR_VOLUME; }
  }
  return OK;
}

template <class T>
inline int lagrangeElements(Domain<T>& d) {
  T delt = d.deltatime;
  int st = calcLagrangeElements(d, delt);
  if (st) return st;
  st = calcQForElems(d);
  if (st) return st;
  st = applyMaterialPropertiesForElems(d);
  if (st) return st;
  return updateVolumesForElems(d);
}

// calcCourantConstraintForElems + calcHydroConstraintForElems,
// src/domain.jl:2964-3064.
template <class T>
inline void calcTimeConstraintsForElems(Domain<T>& d) {
  using std::sqrt; using std::fabs;
  const int64_t length = d.numElem;
  {
    T dtcourant = T(1.0e+20);
    int64_t courant_elem = -1;
    T qqc2 = (T(64.0) * d.qqc) * d.qqc;
    for (int64_t i = 0; i < length; ++i) {
      int64_t indx = d.matElemlist[i] - 1;
      T dtf = d.ss[indx] * d.ss[indx];
      if (val(d.vdov[indx]) < 0.0)
        dtf = dtf + ((((qqc2 * d.arealg[indx]) * d.arealg[indx]) * d.vdov[indx]) * d.vdov[indx]);
      dtf = sqrt(dtf);
      dtf = d.arealg[indx] / dtf;
      if (val(d.vdov[indx]) != 0.0 && val(dtf) < val(dtcourant)) {
        dtcourant = dtf;
        courant_elem = indx;
      }
    }
    if (courant_elem != -1) d.dtcourant = dtcourant;
  }
  {
    T dthydro = T(1.0e+20);
    int64_t hydro_elem = -1;
    for (int64_t i = 0; i < length; ++i) {
      int64_t indx = d.matElemlist[i] - 1;
      if (val(d.vdov[indx]) != 0.0) {
        T dtdvov = d.dvovmax / (jabs(d.vdov[indx]) + T(1.e-20));
        if (val(dthydro) > val(dtdvov)) { dthydro = dtdvov; hydro_elem = indx; }
      }
    }
    if (hydro_elem != -1) d.dthydro = dthydro;
  }
}

// lagrangeLeapFrog, src/domain.jl:3067-3080.
template <class T>
inline int lagrangeLeapFrog(Domain<T>& d) {
  d.error_site = SITE_NONE;
  d.error_index = -1;
  int st = lagrangeNodal(d);
  if (st) return st;
  st = lagrangeElements(d);
  if (st) return st;
  calcTimeConstraintsForElems(d);
  return OK;
}

// verifyAndWriteFinalOutput's symmetry check, src/utils.jl:124-158.
template <class T>
inline void symmetryCheck(const Domain<T>& d, double out[3]) {
  const int64_t nx = d.sizeX;
  double MaxAbsDiff = 0.0, MaxRelDiff = 0.0, TotalAbsDiff = 0.0;
  for (int64_t j = 1; j <= nx; ++j) {
    for (int64_t k = j + 1; k <= nx; ++k) {
      double a = val(d.e[(j - 1) * nx + k - 1]), b = val(d.e[(k - 1) * nx + j - 1]);
      double AbsDiff = std::fabs(a - b);
      TotalAbsDiff += AbsDiff;
      if (MaxAbsDiff < AbsDiff) MaxAbsDiff = AbsDiff;
      double RelDiff = AbsDiff / b;
      if (MaxRelDiff < RelDiff) MaxRelDiff = RelDiff;
    }
  }
  out[0] = MaxAbsDiff; out[1] = TotalAbsDiff; out[2] = MaxRelDiff;
}

}  // namespace lulesh_oracle
