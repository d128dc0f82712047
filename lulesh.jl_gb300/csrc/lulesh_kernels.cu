// The LagrangeLeapFrog step as four sm_103a kernels (one thread per element
// or node, FP64 throughout):
//   k_force      calcVolumeForceForElems: stress integration + FB hourglass,
//                one 8-corner force triple per element corner
//                (src/domain.jl:963-1762)
//   k_node       deterministic corner-force gather in nodeElemCornerList
//                order + acceleration, symmetry BCs, velocity and position
//                (src/domain.jl:1112-1127, 1676-1693, 1781-1838)
//   k_kinematics calcKinematicsForElems + calcLagrangeElements +
//                calcMonotonicQGradientsForElems (src/domain.jl:2099-2320)
//   k_material   calcMonotonicQRegionForElems + qstop check +
//                applyMaterialPropertiesForElems/evalEOSForElems +
//                updateVolumesForElems + Courant/hydro dt minima
//                (src/domain.jl:2322-3064)
// plus k_time_increment (timeIncrement!, src/domain.jl:920-961) for the
// device-resident run loop.
#include "lulesh_device.cuh"
#include "lulesh_kernels.h"

namespace lulesh {

// Each kernel stops at once when an earlier kernel of the step (or of the
// device run loop) recorded an error or finished the run, as the reference
// stops at its first raised error.
__device__ __forceinline__ bool step_off(const DevState* st) {
  return (*(volatile const unsigned int*)&st->status) != 0u || (*(volatile const int*)&st->done) != 0;
}

// ---------------------------------------------------------------------------
// Element geometry at one set of positions
// ---------------------------------------------------------------------------
// The force kernel of a cycle sees the positions the kinematics kernel of
// the cycle before it saw. So the kinematics kernel (or k_geometry, at the
// start of a run and after the host changed the positions) forms what the
// force kernel needs from the positions alone and stores it in d.nextGeo
// ([kGeoSlots][E]), and the force kernel loads it instead of forming it
// again. Both sides use the functions below, so a stored value is bitwise
// the one the force kernel would form (the taping force kernel still forms
// them, for its tape).
//
// d.nextGeo slots: 0..23 the volume derivatives of corner n, coordinate k
// (8k + n, in corner order); 24..35 the hourglass modes of coordinate k
// (24 + 4k + m, before the 1/(12 determ) scale); 36..47 the node normals of
// corners 0..3 (36 + 4k + n, before node 0's quirk and the stress scale);
// 48 and 49 face 0 + face 1's z normal and face 4's y normal (node 0's
// quirk); 50 the Jacobian determinant of the detJ check.

// The 12 face diagonals, two per face in calcElemNodeNormals' argument order
// p2 - p0, p3 - p1 (src/domain.jl:991-1067). Face f: (2,0,3,1) (5,0,1,4)
// (6,1,2,5) (7,2,3,6) (4,3,0,7) (6,4,5,7), so g = d20 d31 d50 d14 d61 d25
// d72 d36 d43 d07 d64 d57.
__device__ __forceinline__ void face_diagonals(const double x[8], const double y[8], const double z[8],
                                               double g[12][3]) {
  constexpr int pa[12] = {2, 3, 5, 1, 6, 2, 7, 3, 4, 0, 6, 5};
  constexpr int pb[12] = {0, 1, 0, 4, 1, 5, 2, 6, 3, 7, 4, 7};
#pragma unroll
  for (int q = 0; q < 12; ++q) {
    g[q][0] = x[pa[q]] - x[pb[q]];
    g[q][1] = y[pa[q]] - y[pb[q]];
    g[q][2] = z[pa[q]] - z[pb[q]];
  }
}

// Walsh coefficients of the positions: w[k] = the Jacobian columns (xi, eta,
// zeta) of coordinate k, hm[k] = its hourglass modes (eta*zeta, xi*zeta,
// xi*eta, xi*eta*zeta; src/domain.jl:1510-1525 without the gamma sums).
// Face diagonals join corners of one parity, so the three even modes are
// sums of four of them: eta*zeta = (d64 - d57) - (d20 + d31), xi*zeta =
// (d07 + d61) - (d43 + d25), xi*eta = (d07 + d61) + (d43 + d25); w and
// xi*eta*zeta come from the four body diagonals a = p6 - p0, b = p5 - p3,
// c = p7 - p1, d = p4 - p2: (a+b) - (c+d), (a-b) + (c-d), (a+b) + (c+d) and
// (a-b) - (c-d). 19 adds per coordinate instead of a 23-add butterfly.
__device__ __forceinline__ void position_walsh(const double x[8], const double y[8], const double z[8],
                                               const double g[12][3], double w[3][3], double hm[3][4]) {
  const double* P[3] = {x, y, z};
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const double* v = P[k];
    const double a = v[6] - v[0], b = v[5] - v[3], c = v[7] - v[1], dd = v[4] - v[2];
    const double apb = a + b, cpd = c + dd, amb = a - b, cmd = c - dd;
    w[k][0] = apb - cpd;
    w[k][1] = amb + cmd;
    w[k][2] = apb + cpd;
    hm[k][3] = amb - cmd;
    hm[k][0] = (g[10][k] - g[11][k]) - (g[0][k] + g[1][k]);
    const double pp = g[9][k] + g[4][k], qq = g[8][k] + g[5][k];
    hm[k][1] = pp - qq;
    hm[k][2] = pp + qq;
  }
}

// integrateStressForElems' detJ <= 0 check (src/domain.jl:1101-1105): the
// sign of 8*(fjxet*cjxet + fjyet*cjyet + fjzet*cjzet) (src/domain.jl:2019),
// with the eta cofactor column c = W_zeta x W_xi (also the monotonic-Q
// gradient's eta direction).
__device__ __forceinline__ void eta_cofactors(const double w[3][3], double c[3]) {
  cross(w[0][2], w[1][2], w[2][2], w[0][0], w[1][0], w[2][0], c[0], c[1], c[2]);
}
__device__ __forceinline__ double jacobian_det(const double w[3][3], const double c[3]) {
  return fma(w[0][1], c[0], fma(w[1][1], c[1], w[2][1] * c[2]));
}
__device__ __forceinline__ double jacobian_det(const double w[3][3]) {
  double c[3];
  eta_cofactors(w, c);
  return jacobian_det(w, c);
}

// Face f's area vector times -8: the cross product of its two diagonals.
__device__ __forceinline__ void face_normal(const double g[12][3], int f, double n[3]) {
  cross(g[2 * f][0], g[2 * f][1], g[2 * f][2], g[2 * f + 1][0], g[2 * f + 1][1], g[2 * f + 1][2], n[0], n[1], n[2]);
}

// Node normals (calcElemNodeNormals, src/domain.jl:991-1067) of corners 0..3
// as sums of their three faces' cross products (true B = -Bc/8); node 0
// without its quirk, for which pz01 and ny4 are returned. The six face
// normals are the area vectors of a closed surface and sum to zero, and
// opposite corners touch complementary faces (node 0: faces 0,1,4; node 6:
// 2,3,5), so corners 6, 7, 4, 5 are minus corners 0, 1, 2, 3 and face 5's
// normal is never needed.
__device__ __forceinline__ void node_normals(const double n[6][3], double B[3][4], double& pz01, double& ny4) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const double p01 = n[0][k] + n[1][k];
    B[k][0] = p01 + n[4][k];
    B[k][1] = p01 + n[2][k];
    B[k][2] = (n[0][k] + n[2][k]) + n[3][k];
    B[k][3] = (n[0][k] + n[3][k]) + n[4][k];
    if (k == 2) pz01 = p01;
  }
  ny4 = n[4][1];
}

// calcElemVolume's three triple products U.(V x W) of face diagonals
// (src/utils.jl:36-116): (d31+d72).(d63 x d20), (d43+d57).(d64 x d70),
// (d14+d25).(d61 x d50); U[t] and the gradients V x W, W x U, U x V.
__device__ __forceinline__ void volume_terms(const double g[12][3], double U[3][3], double gU[3][3], double gV[3][3],
                                             double gW[3][3]) {
  auto grads = [&](int t, const double V[3], const double W[3]) {
    cross(V[0], V[1], V[2], W[0], W[1], W[2], gU[t][0], gU[t][1], gU[t][2]);
    cross(W[0], W[1], W[2], U[t][0], U[t][1], U[t][2], gV[t][0], gV[t][1], gV[t][2]);
    cross(U[t][0], U[t][1], U[t][2], V[0], V[1], V[2], gW[t][0], gW[t][1], gW[t][2]);
  };
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    U[0][k] = g[1][k] + g[6][k];
    U[1][k] = g[8][k] + g[11][k];
    U[2][k] = g[3][k] + g[5][k];
  }
  const double V1[3] = {-g[7][0], -g[7][1], -g[7][2]};
  grads(0, V1, g[0]);
  const double W2[3] = {-g[9][0], -g[9][1], -g[9][2]};
  grads(1, g[10], W2);
  grads(2, g[4], g[2]);
}

// calcElemVolumeDerivative (src/domain.jl:1178-1256), times 12, in corner
// order: its voluDer values are the gradient of 12*volume, the triple
// products' gradients scattered to their corners (U1 = +3 -1 +7 -2,
// V1 = +6 -3, W1 = +2 -0; U2 = +4 -3 +5 -7, V2 = +6 -4, W2 = +7 -0;
// U3 = +1 -4 +2 -5, V3 = +6 -1, W3 = +5 -0). The reference's n-th call
// stores node owner[n]'s derivative in slot n (slots 1 and 3 exchanged)
// unless corrected; the force kernel applies that when it reads them.
__device__ __forceinline__ void volume_derivatives(const double gU[3][3], const double gV[3][3],
                                                   const double gW[3][3], double gr[3][8]) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    // corners 1 and 2, 3 and 7, 4 and 5 share a difference of the U gradients
    const double t12 = gU[2][k] - gU[0][k], t37 = gU[0][k] - gU[1][k], t45 = gU[1][k] - gU[2][k];
    gr[k][0] = -((gW[0][k] + gW[1][k]) + gW[2][k]);
    gr[k][1] = t12 - gV[2][k];
    gr[k][2] = t12 + gW[0][k];
    gr[k][3] = t37 - gV[0][k];
    gr[k][4] = t45 - gV[1][k];
    gr[k][5] = t45 + gW[2][k];
    gr[k][6] = (gV[0][k] + gV[1][k]) + gV[2][k];
    gr[k][7] = t37 + gW[1][k];
  }
}

__device__ __forceinline__ void store_geometry(double* geo, int E, int e, const double gr[3][8], const double hm[3][4],
                                               const double B[3][4], double pz01, double ny4, double det) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
#pragma unroll
    for (int n = 0; n < 8; ++n) geo[(8 * k + n) * E + e] = gr[k][n];
#pragma unroll
    for (int m = 0; m < 4; ++m) geo[(24 + 4 * k + m) * E + e] = hm[k][m];
#pragma unroll
    for (int n = 0; n < 4; ++n) geo[(36 + 4 * k + n) * E + e] = B[k][n];
  }
  geo[48 * E + e] = pz01;
  geo[49 * E + e] = ny4;
  geo[50 * E + e] = det;
}

// The force tape's face normals 0..4 of these positions (slots 48 + f,
// 54 + f, 60 + f), read by the hourglass transpose.
__device__ __forceinline__ void tape_force_normals(double* tape, int E, int e, const double n[6][3]) {
#pragma unroll
  for (int f = 0; f < 5; ++f) {
    tape[(48 + f) * E + e] = n[f][0];
    tape[(54 + f) * E + e] = n[f][1];
    tape[(60 + f) * E + e] = n[f][2];
  }
}

// The face diagonals of these positions (slot 3q + k of a [36][E] buffer):
// at the start of a taped segment, for the position transpose of the run's
// first cycle (every other cycle's is fused into the kinematics transpose of
// the cycle before, which reads the kinematics tape).
__device__ __forceinline__ void tape_diagonals(double* diag, int E, int e, const double g[12][3]) {
#pragma unroll
  for (int q = 0; q < 12; ++q)
#pragma unroll
    for (int k = 0; k < 3; ++k) diag[(3 * q + k) * E + e] = g[q][k];
}

// The force kernel's geometry of one element's positions, formed by the same
// calls in the same order as k_geometry and k_kinematics, so the values are
// bitwise those they store.
__device__ __forceinline__ void force_geometry(const double x[8], const double y[8], const double z[8],
                                               double gr[3][8], double hm[3][4], double B[3][4], double& pz01,
                                               double& ny4, double& det) {
  double g[12][3], w[3][3], n[6][3], U[3][3], gU[3][3], gV[3][3], gW[3][3];
  face_diagonals(x, y, z, g);
  position_walsh(x, y, z, g, w, hm);
#pragma unroll
  for (int f = 0; f < 5; ++f) face_normal(g, f, n[f]);
  node_normals(n, B, pz01, ny4);
  volume_terms(g, U, gU, gV, gW);
  volume_derivatives(gU, gV, gW, gr);
  det = jacobian_det(w);
}

// The stored geometry of the current positions (see above): at the start of
// a run, after the host changed the positions, and for the ensemble's reset;
// in a taped run also the first cycle's face diagonals and normals.
__global__ void __launch_bounds__(kMaxElemBlock) k_geometry(DevDomain d) {
  const int E = d.E;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= E) return;
  double x[8], y[8], z[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    const int nd = LULESH_IDX(LDG(&d.nodelist[c * E + e]), d.N, d.st);
    x[c] = LDG(&d.x[nd]); y[c] = LDG(&d.y[nd]); z[c] = LDG(&d.z[nd]);
  }
  double g[12][3], w[3][3], hm[3][4], n[6][3], B[3][4], pz01, ny4;
  double U[3][3], gU[3][3], gV[3][3], gW[3][3], gr[3][8];
  face_diagonals(x, y, z, g);
  position_walsh(x, y, z, g, w, hm);
#pragma unroll
  for (int f = 0; f < 5; ++f) face_normal(g, f, n[f]);
  node_normals(n, B, pz01, ny4);
  volume_terms(g, U, gU, gV, gW);
  volume_derivatives(gU, gV, gW, gr);
  store_geometry(d.nextGeo, E, e, gr, hm, B, pz01, ny4, jacobian_det(w));
  if (d.tapeGeoNext) tape_force_normals(d.tapeGeoNext, E, e, n);
  if (d.tapeDiag) tape_diagonals(d.tapeDiag, E, e, g);
}

// ---------------------------------------------------------------------------
// k_force
// ---------------------------------------------------------------------------
// The geometry of the cycle's positions is loaded from d.nextGeo, or, with
// GEO_INLINE (the other fusion split, chosen by the autotuner), formed here
// from the positions (k_kinematics then stores none); the taping variant
// loads it and adds the volume derivatives, scaled modes and mode sums to
// the force tape (the diagonals and normals are there already).
template <int MODE, bool ENS, bool TAPE, bool GEO_INLINE>
__global__ void __launch_bounds__(kMaxElemBlock) k_force(DevDomain d, Params prm) {
  const int E = d.E;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= E) return;
  const int inst = ENS ? LULESH_IDX(LDG(&d.elemInst[e]), d.ninst, d.st) : 0;
  DevState* const st = d.st + inst;
  if (step_off(st)) return;
  const double hgcoef = ENS ? LDG(&d.instHg[inst]) : prm.hgcoef;

  int nd[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) nd[c] = LULESH_IDX(LDG(&d.nodelist[c * E + e]), d.N, st);

  double gr[3][8], hm[3][4], B[3][4], pz01, ny4, det;
  if (GEO_INLINE) {
    double x[8], y[8], z[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) { x[c] = LDG(&d.x[nd[c]]); y[c] = LDG(&d.y[nd[c]]); z[c] = LDG(&d.z[nd[c]]); }
    force_geometry(x, y, z, gr, hm, B, pz01, ny4, det);
  } else {
    const double* geo = d.nextGeo;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
#pragma unroll
      for (int n = 0; n < 8; ++n) gr[k][n] = LDG(&geo[(8 * k + n) * E + e]);
#pragma unroll
      for (int m = 0; m < 4; ++m) hm[k][m] = LDG(&geo[(24 + 4 * k + m) * E + e]);
#pragma unroll
      for (int n = 0; n < 4; ++n) B[k][n] = LDG(&geo[(36 + 4 * k + n) * E + e]);
    }
    pz01 = LDG(&geo[48 * E + e]);
    ny4 = LDG(&geo[49 * E + e]);
    det = LDG(&geo[50 * E + e]);
  }
  if (le_zero(det)) atomicOr(&st->status, ST_EARLY);

  // the reference's slots of the volume derivatives: node 3's in slot 1 and
  // node 1's in slot 3 unless corrected
  double dvx[8], dvy[8], dvz[8];
#pragma unroll
  for (int n = 0; n < 8; ++n) {
    const int src = (MODE & 2) ? n : (n == 1 ? 3 : n == 3 ? 1 : n);
    dvx[n] = gr[0][src]; dvy[n] = gr[1][src]; dvz[n] = gr[2][src];
  }

  // stress: f = (-sig) * B = (sig/8) * Bc with sig = -p - q; corners 4..7
  // are minus corners 2, 3, 0, 1, formed before node 0's quirk
  const double s8 = ((-LDG(&d.p[e])) - LDG(&d.q[e])) * 0.125;
  double SB[3][4];
#pragma unroll
  for (int k = 0; k < 3; ++k)
#pragma unroll
    for (int n = 0; n < 4; ++n) SB[k][n] = s8 * B[k][n];
  double q0y = SB[1][0], q0z = SB[2][0];
  if (!(MODE & 1)) {
    // src/domain.jl:1050-1055: node 1 takes face 5's areaY twice, no areaZ
    q0y = s8 * (B[1][0] + ny4);
    q0z = s8 * pz01;
  }
  // s8*Bc of corner n, component k (n and k are constants after unrolling, so
  // the sign folds into the instruction that consumes it)
  auto bstress = [&](int k, int n) -> double {
    if (n == 0) return k == 0 ? SB[0][0] : k == 1 ? q0y : q0z;
    if (n < 4) return SB[k][n];
    return -SB[k][n == 4 ? 2 : n == 5 ? 3 : n == 6 ? 0 : 1];
  };

  // calcHourglassControlForElems (src/domain.jl:1696-1736): determ = volo*v.
  const double v = LDG(&d.v[e]);
  const double determ = LDG(&d.volo[e]) * v;
  if (le_zero(v)) atomicOr(&st->status, ST_HOURGLASS);

  double fx[8], fy[8], fz[8];
  if (gt_zero(hgcoef)) {
    // hourgam (src/domain.jl:1527-1549) with volinv/12 folded into the modes
    // determ^(-1/3) serves the coefficient, its cube the modes' 1/(12 determ)
    const double rc = inv_cbrt(determ);
    const double vi12 = (rc * rc) * (rc * (1.0 / 12.0));
    double hmx[4], hmy[4], hmz[4];
#pragma unroll
    for (int m = 0; m < 4; ++m) { hmx[m] = hm[0][m] * vi12; hmy[m] = hm[1][m] * vi12; hmz[m] = hm[2][m] * vi12; }
    if (TAPE) {
#pragma unroll
      for (int n = 0; n < 8; ++n) {
        d.tapeGeo[n * E + e] = dvx[n];
        d.tapeGeo[(8 + n) * E + e] = dvy[n];
        d.tapeGeo[(16 + n) * E + e] = dvz[n];
      }
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        d.tapeGeo[(24 + m) * E + e] = hmx[m];
        d.tapeGeo[(28 + m) * E + e] = hmy[m];
        d.tapeGeo[(32 + m) * E + e] = hmz[m];
      }
    }
    double hg[8][4];
#pragma unroll
    for (int n = 0; n < 8; ++n)
#pragma unroll
      for (int m = 0; m < 4; ++m)
        hg[n][m] = fma(-dvz[n], hmz[m], fma(-dvy[n], hmy[m], fma(-dvx[n], hmx[m], gamma_nm(n, m))));

    // coefficient = -hgcoef*0.01*ss*mass/cbrt(determ) (src/domain.jl:1605)
    const double coef = ((-hgcoef * 0.01) * LDG(&d.ss[e])) * LDG(&d.elemMass[e]) * rc;

    // calcElemFBHourglassForce (src/domain.jl:1258-1460), one velocity
    // component at a time to bound register use.
    const double* vel[3] = {d.xd, d.yd, d.zd};
    double* fo[3] = {fx, fy, fz};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      double vv[8];
#pragma unroll
      for (int c = 0; c < 8; ++c) vv[c] = LDG(&vel[k][nd[c]]);
      double h[4];
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        double s = hg[0][m] * vv[0];
#pragma unroll
        for (int n = 1; n < 8; ++n) s = fma(hg[n][m], vv[n], s);
        if (TAPE) d.tapeGeo[(36 + 4 * k + m) * E + e] = s;
        h[m] = coef * s;
      }
#pragma unroll
      for (int n = 0; n < 8; ++n) {
        fo[k][n] = fma(hg[n][0], h[0], fma(hg[n][1], h[1], fma(hg[n][2], h[2], fma(hg[n][3], h[3], bstress(k, n)))));
      }
    }
  } else {
#pragma unroll
    for (int n = 0; n < 8; ++n) { fx[n] = bstress(0, n); fy[n] = bstress(1, n); fz[n] = bstress(2, n); }
  }
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    d.fcx[c * E + e] = fx[c];
    d.fcy[c * E + e] = fy[c];
    d.fcz[c * E + e] = fz[c];
  }
}

// ---------------------------------------------------------------------------
// k_node
// ---------------------------------------------------------------------------
template <bool AUX, bool ENS>
__global__ void __launch_bounds__(kMaxNodeBlock) k_node(DevDomain d, Params prm) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.N) return;
  DevState* const st = d.st + (ENS ? LULESH_IDX(LDG(&d.nodeInst[i]), d.ninst, d.st) : 0);
  if (step_off(st)) return;
  const double dt = st->deltatime;
  const int s = LDG(&d.nodeElemStart[i]);
  int t = LDG(&d.nodeElemStart[i + 1]);
#ifdef LULESH_CHECK
  // the node's corner range must lie within the corner list; an empty one reads nothing
  if (s < 0 || t < s || t > d.nCornerList) { atomicOr(&st->status, ST_INDEX); t = s; }
#endif
  double fx = 0.0, fy = 0.0, fz = 0.0;
  if (s < t) {
    const int c0 = LULESH_IDX(LDG(&d.cornerList[s]), d.nCornerSlot, st);
    fx = LDG(&d.fcx[c0]); fy = LDG(&d.fcy[c0]); fz = LDG(&d.fcz[c0]);
    for (int j = s + 1; j < t; ++j) {
      const int c = LULESH_IDX(LDG(&d.cornerList[j]), d.nCornerSlot, st);
      fx += LDG(&d.fcx[c]); fy += LDG(&d.fcy[c]); fz += LDG(&d.fcz[c]);
    }
  }
  const double im = LDG(&d.inv_nodalMass[i]);
  double ax = fx * im, ay = fy * im, az = fz * im;
  const unsigned bc = d.nodeBC[i];
  if (bc & 1u) ax = 0.0;
  if (bc & 2u) ay = 0.0;
  if (bc & 4u) az = 0.0;
  double xd = fma(ax, dt, d.xd[i]);
  double yd = fma(ay, dt, d.yd[i]);
  double zd = fma(az, dt, d.zd[i]);
  if (abs_lt(xd, prm.u_cut)) xd = 0.0;
  if (abs_lt(yd, prm.u_cut)) yd = 0.0;
  if (abs_lt(zd, prm.u_cut)) zd = 0.0;
  d.xd[i] = xd; d.yd[i] = yd; d.zd[i] = zd;
  d.x[i] = fma(xd, dt, d.x[i]);
  d.y[i] = fma(yd, dt, d.y[i]);
  d.z[i] = fma(zd, dt, d.z[i]);
  if (AUX) {
    d.fx[i] = fx; d.fy[i] = fy; d.fz[i] = fz;
    d.xdd[i] = ax; d.ydd[i] = ay; d.zdd[i] = az;
  }
}

// ---------------------------------------------------------------------------
// k_kinematics
// ---------------------------------------------------------------------------
// GEO: also store the next force kernel's geometry of these positions
// (d.nextGeo); without it (the GEO_INLINE split) k_force forms it itself.
template <bool AUX, bool ENS, bool TAPE, bool GEO>
__global__ void __launch_bounds__(kMaxElemBlock) k_kinematics(DevDomain d, Params prm) {
  const int E = d.E;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= E) return;
  DevState* const st = d.st + (ENS ? LULESH_IDX(LDG(&d.elemInst[e]), d.ninst, d.st) : 0);
  if (step_off(st)) return;
  const double dt = st->deltatime;

  int nd[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) nd[c] = LULESH_IDX(LDG(&d.nodelist[c * E + e]), d.N, st);
  double x[8], y[8], z[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    x[c] = LDG(&d.x[nd[c]]);
    y[c] = LDG(&d.y[nd[c]]);
    z[c] = LDG(&d.z[nd[c]]);
  }

  // calcElemVolume (src/utils.jl:36-116) and calcElemCharacteristicLength
  // (src/domain.jl:1874-1930) from the face diagonals; the next force
  // kernel's geometry of these positions is stored too.
  double volume, charLength = 0.0;
  double w[3][3];  // first-order Walsh vectors (xi, eta, zeta) of x, y, z
  double cet[3];   // W_zeta x W_xi
  {
    double g[12][3], hm[3][4], n[6][3], U[3][3], gU[3][3], gV[3][3], gW[3][3];
    face_diagonals(x, y, z, g);
    position_walsh(x, y, z, g, w, hm);
    volume_terms(g, U, gU, gV, gW);
    auto triple_t = [&](int t) { return fma(U[t][0], gU[t][0], fma(U[t][1], gU[t][1], U[t][2] * gU[t][2])); };
    volume = ((triple_t(0) + triple_t(1)) + triple_t(2)) * (1.0 / 12.0);
#pragma unroll
    for (int f = 0; f < 6; ++f) face_normal(g, f, n[f]);
    if (TAPE) {
      // the 12 diagonals in the order d61 d70 d63 d20 d50 d64 d31 d72 d43 d57
      // d14 d25 (force-order index, sign) and the V x W factors
      constexpr int gi[12] = {4, 9, 7, 0, 2, 10, 1, 6, 8, 11, 3, 5};
      constexpr int gs[12] = {1, -1, -1, 1, 1, 1, 1, 1, 1, 1, 1, 1};
#pragma unroll
      for (int q = 0; q < 12; ++q)
#pragma unroll
        for (int k = 0; k < 3; ++k) d.tapeKin[(45 + 3 * q + k) * E + e] = gs[q] < 0 ? -g[gi[q]][k] : g[gi[q]][k];
#pragma unroll
      for (int t = 0; t < 3; ++t)
#pragma unroll
        for (int k = 0; k < 3; ++k) d.tapeKin[(81 + 3 * t + k) * E + e] = gU[t][k];
    }
    // areaFace (src/domain.jl:1874-1891): with f, g = a -/+ b for the face
    // diagonals a, b, |f|^2|g|^2 - (f.g)^2 = |f x g|^2 = 4 |a x b|^2; the 4
    // is folded into arealg below. The reference's faces in order are the
    // force order's 0, 5, 1, 2, 3, 4, the last two with reversed diagonals
    // (so minus those cross products).
    int fidx = 0;
    double fcx = 0.0, fcy = 0.0, fcz = 0.0;  // the largest face's cross product (TAPE)
    constexpr int ff[6] = {0, 5, 1, 2, 3, 4};
#pragma unroll
    for (int q = 0; q < 6; ++q) {
      const double* c = n[ff[q]];
      // area4 >= +0 and charLength too: their bit patterns order them
      const double area4 = fma(c[0], c[0], fma(c[1], c[1], c[2] * c[2]));
      if (TAPE && (q == 0 || __double_as_longlong(area4) > __double_as_longlong(charLength))) {
        const bool neg = q >= 4;
        fidx = q;
        fcx = neg ? -c[0] : c[0]; fcy = neg ? -c[1] : c[1]; fcz = neg ? -c[2] : c[2];
      }
      charLength = max_nonneg(area4, charLength);
    }
    if (TAPE) {
      d.tapeFlags[e] = (unsigned long long)fidx << TF_FACE_SHIFT;
      d.tapeKin[41 * E + e] = fcx; d.tapeKin[42 * E + e] = fcy; d.tapeKin[43 * E + e] = fcz;
      // the next cycle's face normals, for its hourglass transpose
      if (d.tapeGeoNext) tape_force_normals(d.tapeGeoNext, E, e, n);
    }
    if (GEO) {
      double B[3][4], pz01, ny4, gr[3][8];
      node_normals(n, B, pz01, ny4);
      volume_derivatives(gU, gV, gW, gr);
      eta_cofactors(w, cet);
      store_geometry(d.nextGeo, E, e, gr, hm, B, pz01, ny4, jacobian_det(w, cet));
    } else {
      eta_cofactors(w, cet);
    }
  }
  const double* wx = w[0];
  const double* wy = w[1];
  const double* wz = w[2];
  const double vnew = volume * LDG(&d.inv_volo[e]);
  if (le_zero(vnew)) atomicOr(&st->status, ST_KINEMATICS);
  d.vnew[e] = vnew;
  d.delv[e] = vnew - LDG(&d.v[e]);
  // 4*volume/sqrt(max area) with area = 4*area4
  {
    const double rcl = rsqrt(charLength);
    d.arealg[e] = (2.0 * volume) * rcl;
    if (TAPE) d.tapeKin[44 * E + e] = rcl;
  }

  // Velocity gradient trace at the half-step position (src/domain.jl:2128-2158)
  double vxw[3], vyw[3], vzw[3];
  {
    double v8[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) v8[c] = LDG(&d.xd[nd[c]]);
    walsh1(v8, vxw);
#pragma unroll
    for (int c = 0; c < 8; ++c) v8[c] = LDG(&d.yd[nd[c]]);
    walsh1(v8, vyw);
#pragma unroll
    for (int c = 0; c < 8; ++c) v8[c] = LDG(&d.zd[nd[c]]);
    walsh1(v8, vzw);
  }
  if (TAPE) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      d.tapeKin[a * E + e] = wx[a]; d.tapeKin[(3 + a) * E + e] = wy[a]; d.tapeKin[(6 + a) * E + e] = wz[a];
      d.tapeKin[(9 + a) * E + e] = vxw[a]; d.tapeKin[(12 + a) * E + e] = vyw[a]; d.tapeKin[(15 + a) * E + e] = vzw[a];
    }
  }
  // 1/det of the velocity gradient and 1/(64 vol + 64 ptiny) of the Q
  // gradients come from one division
  const double volq = LDG(&d.volo[e]) * vnew;
  const double q64 = fma(64.0, volq, 64.0 * 1.e-36);
  double inv, norm64;
  {
    const double dt2 = -0.5 * dt;
    double F[3][3];  // F[k][a]: coordinate k, direction a (xi, eta, zeta)
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      F[0][a] = fma(dt2, vxw[a], wx[a]);
      F[1][a] = fma(dt2, vyw[a], wy[a]);
      F[2][a] = fma(dt2, vzw[a], wz[a]);
    }
    // cofactors (src/domain.jl:1976-1987)
    const double Cxxi = fma(F[1][1], F[2][2], -(F[2][1] * F[1][2]));
    const double Cxet = fma(F[2][0], F[1][2], -(F[1][0] * F[2][2]));
    const double Cxze = fma(F[1][0], F[2][1], -(F[2][0] * F[1][1]));
    const double Cyxi = fma(F[2][1], F[0][2], -(F[0][1] * F[2][2]));
    const double Cyet = fma(F[0][0], F[2][2], -(F[2][0] * F[0][2]));
    const double Cyze = fma(F[2][0], F[0][1], -(F[0][0] * F[2][1]));
    const double Czxi = fma(F[0][1], F[1][2], -(F[1][1] * F[0][2]));
    const double Czet = fma(F[1][0], F[0][2], -(F[0][0] * F[1][2]));
    const double Czze = fma(F[0][0], F[1][1], -(F[1][0] * F[0][1]));
    const double det = fma(F[0][1], Cxet, fma(F[1][1], Cyet, F[2][1] * Czet));
    const double d1 = fma(Cxxi, vxw[0], fma(Cxet, vxw[1], Cxze * vxw[2]));
    const double d2 = fma(Cyxi, vyw[0], fma(Cyet, vyw[1], Cyze * vyw[2]));
    const double d3 = fma(Czxi, vzw[0], fma(Czet, vzw[1], Czze * vzw[2]));
    recip2(det, q64, inv, norm64);
    const double vdov = ((d1 + d2) + d3) * inv;
    d.vdov[e] = vdov;
    if (TAPE) {
      // cofactor columns C_xi, C_eta, C_zeta (x, y, z each), then 1/det
      const double cof[9] = {Cxxi, Cyxi, Czxi, Cxet, Cyet, Czet, Cxze, Cyze, Czze};
#pragma unroll
      for (int q = 0; q < 9; ++q) d.tapeKin[(18 + q) * E + e] = cof[q];
      d.tapeKin[27 * E + e] = inv;
    }
    if (AUX) {
      const double third = vdov / 3.0;
      d.dxx[e] = d1 * inv - third;
      d.dyy[e] = d2 * inv - third;
      d.dzz[e] = d3 * inv - third;
    }
  }

  // calcMonotonicQGradientsForElems (src/domain.jl:2175-2320). With the
  // reference's dxi = W_xi/4 etc.: delx = 16*vol/sqrt(|A|^2 + 256*ptiny) and
  // delv = norm/64 * (A . W(v)) for the cross product A of two Walsh vectors.
  {
    const double ptiny = 1.e-36;
    const double vol = volq;
    const double vol16 = 16.0 * vol;
    double ax, ay, az, rs;
    // taped per direction d (xi, eta, zeta): the cross product A and 1/|A|
    auto tape_a = [&](int dir) {
      if (TAPE) {
        d.tapeKin[(28 + 3 * dir) * E + e] = ax; d.tapeKin[(29 + 3 * dir) * E + e] = ay;
        d.tapeKin[(30 + 3 * dir) * E + e] = az; d.tapeKin[(37 + dir) * E + e] = rs;
      }
    };
    if (TAPE) d.tapeKin[40 * E + e] = norm64;
    // zeta: xi x eta
    cross(wx[0], wy[0], wz[0], wx[1], wy[1], wz[1], ax, ay, az);
    rs = rsqrt(fma(ax, ax, fma(ay, ay, fma(az, az, 256.0 * ptiny))));
    d.delx_zeta[e] = vol16 * rs;
    d.delv_zeta[e] = norm64 * fma(ax, vxw[2], fma(ay, vyw[2], az * vzw[2]));
    tape_a(2);
    // xi: eta x zeta
    cross(wx[1], wy[1], wz[1], wx[2], wy[2], wz[2], ax, ay, az);
    rs = rsqrt(fma(ax, ax, fma(ay, ay, fma(az, az, 256.0 * ptiny))));
    d.delx_xi[e] = vol16 * rs;
    d.delv_xi[e] = norm64 * fma(ax, vxw[0], fma(ay, vyw[0], az * vzw[0]));
    tape_a(0);
    // eta: zeta x xi (formed for the detJ check)
    ax = cet[0]; ay = cet[1]; az = cet[2];
    rs = rsqrt(fma(ax, ax, fma(ay, ay, fma(az, az, 256.0 * ptiny))));
    d.delx_eta[e] = vol16 * rs;
    d.delv_eta[e] = norm64 * fma(ax, vxw[1], fma(ay, vyw[1], az * vzw[1]));
    tape_a(1);
  }
}

// ---------------------------------------------------------------------------
// k_material
// ---------------------------------------------------------------------------

// One limiter direction, src/domain.jl:2330-2376. `src` reports which value
// the result is (PHI_*), for the adjoint's tape.
__device__ __forceinline__ double monoq_phi(double norm, double dm, double dp, const Params& prm, int& src,
                                            double& t_norm, double& t_dm, double& t_dp) {
  // norm = 1 / (delv + ptiny) of this direction
  dm *= norm;
  dp *= norm;
  t_norm = norm; t_dm = dm; t_dp = dp;  // kept for the adjoint's tape
  double phi = 0.5 * (dm + dp);
  src = PHI_MEAN;
  dm *= prm.monoq_limiter_mult;
  dp *= prm.monoq_limiter_mult;
  // the comparisons on the integer keys (fkey), with IEEE's outcomes
  long long kphi = fkey(phi);
  const long long km = fkey(dm), kp = fkey(dp);
  if (km < kphi) { phi = dm; kphi = km; src = PHI_M; }
  if (kp < kphi) { phi = dp; kphi = kp; src = PHI_P; }
  if (kphi < 0) { phi = 0.0; kphi = 0; src = PHI_ZERO; }
  if (kphi > prm.k_max_slope) { phi = prm.monoq_max_slope; src = PHI_MAX; }
  return phi;
}

// Neighbour value for one face of the limiter (the four BC cases).
__device__ __forceinline__ double monoq_neighbour(const double* dv, unsigned mask, unsigned bits,
                                                  unsigned symm, unsigned freeb, unsigned comm,
                                                  int idx, int self, int E, bool& bad) {
  const unsigned c = mask & bits;
  if (c == 0u || c == comm) {
    if (idx < 0 || idx >= E) { bad = true; return 0.0; }
    return LDG(&dv[idx]);
  }
  if (c == symm) return LDG(&dv[self]);
  if (c == freeb) return 0.0;
  bad = true;
  return 0.0;
}

__device__ __forceinline__ void block_min2(unsigned long long a, unsigned long long b,
                                           unsigned long long* ga, unsigned long long* gb) {
  __shared__ unsigned long long sa[32], sb[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long ta = __shfl_xor_sync(0xffffffffu, a, o);
    const unsigned long long tb = __shfl_xor_sync(0xffffffffu, b, o);
    a = ta < a ? ta : a;
    b = tb < b ? tb : b;
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) { sa[w] = a; sb[w] = b; }
  __syncthreads();
  if (w == 0) {
    const int nw = blockDim.x >> 5;
    a = l < nw ? sa[l] : kInfBits;
    b = l < nw ? sb[l] : kInfBits;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long ta = __shfl_xor_sync(0xffffffffu, a, o);
      const unsigned long long tb = __shfl_xor_sync(0xffffffffu, b, o);
      a = ta < a ? ta : a;
      b = tb < b ? tb : b;
    }
    if (l == 0) {
      if (a != kInfBits) atomicMin(ga, a);
      if (b != kInfBits) atomicMin(gb, b);
    }
  }
}

// Per-instance minima of an ensemble: a warp whose elements all belong to one
// instance reduces first; a warp straddling two instances (or the ragged
// tail) falls back to one atomic per thread. Every lane must call this.
__device__ __forceinline__ void warp_min2_by_instance(unsigned long long a, unsigned long long b, int inst,
                                                      DevState* st) {
  const unsigned full = 0xffffffffu;
  const int inst0 = __shfl_sync(full, inst, 0);
  if (__all_sync(full, inst == inst0)) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long ta = __shfl_xor_sync(full, a, o);
      const unsigned long long tb = __shfl_xor_sync(full, b, o);
      a = ta < a ? ta : a;
      b = tb < b ? tb : b;
    }
    if ((threadIdx.x & 31) == 0) {
      if (a != kInfBits) atomicMin(&st[inst0].acc_courant, a);
      if (b != kInfBits) atomicMin(&st[inst0].acc_hydro, b);
    }
  } else {
    if (a != kInfBits) atomicMin(&st[inst].acc_courant, a);
    if (b != kInfBits) atomicMin(&st[inst].acc_hydro, b);
  }
}

// An empty register move the compiler cannot see through: a value passed
// through it must be recomputed from it.
__device__ __forceinline__ void opaque(double& x) { asm volatile("" : "+d"(x)); }

// REGION: threads take elements in region order (d.regOrder) so that a warp
// runs one region's rep count; each element's EOS is evaluated that many times.
template <int MODE, bool AUX, bool ENS, bool TAPE, bool REGION>
__global__ void __launch_bounds__(kMaxElemBlock) k_material(DevDomain d, Params prm) {
  const int E = d.E;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = REGION ? (t < E ? LULESH_IDX(LDG(&d.regOrder[t]), E, d.st) : E) : t;
  // every thread of the block takes part in the dt reduction
  unsigned long long courant = kInfBits, hydro = kInfBits;
  const int inst = (ENS && i < E) ? LULESH_IDX(LDG(&d.elemInst[i]), d.ninst, d.st) : 0;
  DevState* const st = d.st + inst;
  const bool live = (i < E) && !step_off(st);
  if (live) {
    unsigned int err = 0u;
    unsigned long long fl = 0ull;  // branch record (TAPE only)
    // ---- calcMonotonicQRegionForElems, src/domain.jl:2322-2513 ----
    const unsigned mask = LDG(&d.elemBC[i]);
    const double dvxi = LDG(&d.delv_xi[i]), dveta = LDG(&d.delv_eta[i]), dvzeta = LDG(&d.delv_zeta[i]);
    bool bad = false;
    int src0, src1, src2;
    // xi-plus: the reference indexes delv_xi[lxip[i]] without +1 (:2349)
    const int ixp = (MODE & 4) ? LDG(&d.lxip[i]) : LDG(&d.lxip[i]) - 1;
    const int Eg = d.Eg;  // neighbour reads may reach the ghost slots of a block-partitioned mesh
    double dm = monoq_neighbour(d.delv_xi, mask, XI_M, XI_M_SYMM, XI_M_FREE, XI_M_COMM, LDG(&d.lxim[i]), i, Eg, bad);
    double dp = monoq_neighbour(d.delv_xi, mask, XI_P, XI_P_SYMM, XI_P_FREE, XI_P_COMM, ixp, i, Eg, bad);
    double tl[9];  // limiter terms per direction: norm, dm/norm, dp/norm (TAPE)
    // the three 1/(delv + ptiny) from one division
    double inx, iny, inz;
    recip3(dvxi + 1.e-36, dveta + 1.e-36, dvzeta + 1.e-36, inx, iny, inz);
    const double phixi = monoq_phi(inx, dm, dp, prm, src0, tl[0], tl[3], tl[6]);
    dm = monoq_neighbour(d.delv_eta, mask, ETA_M, ETA_M_SYMM, ETA_M_FREE, ETA_M_COMM, LDG(&d.letam[i]), i, Eg, bad);
    dp = monoq_neighbour(d.delv_eta, mask, ETA_P, ETA_P_SYMM, ETA_P_FREE, ETA_P_COMM, LDG(&d.letap[i]), i, Eg, bad);
    const double phieta = monoq_phi(iny, dm, dp, prm, src1, tl[1], tl[4], tl[7]);
    dm = monoq_neighbour(d.delv_zeta, mask, ZETA_M, ZETA_M_SYMM, ZETA_M_FREE, ZETA_M_COMM, LDG(&d.lzetam[i]), i, Eg, bad);
    dp = monoq_neighbour(d.delv_zeta, mask, ZETA_P, ZETA_P_SYMM, ZETA_P_FREE, ZETA_P_COMM, LDG(&d.lzetap[i]), i, Eg, bad);
    const double phizeta = monoq_phi(inz, dm, dp, prm, src2, tl[2], tl[5], tl[8]);
    if (bad) err |= ST_BAD_BC;
    // d.tapeMat slot q of this element (TAPE only)
    auto tm = [&](int q, double v) { if (TAPE) d.tapeMat[q * E + i] = v; };
    if (TAPE) {
      fl |= (unsigned long long)(src0 | (src1 << 3) | (src2 << 6));
#pragma unroll
      for (int q = 0; q < 9; ++q) tm(q, tl[q]);
    }

    const double vdov = LDG(&d.vdov[i]);
    const double vnew = LDG(&d.vnew[i]);
    const double delvc_in = LDG(&d.delv[i]);

    // ---- applyMaterialPropertiesForElems' clamp, src/domain.jl:2860-2910 ----
    // (the threshold tests of this kernel compare integer keys, fkey)
    double vnewc_in = vnew;
    long long kvn = fkey(vnew);
    bool clamped = false;
    if (prm.has_eosvmin && kvn < prm.k_eosvmin) {
      vnewc_in = prm.eosvmin; kvn = prm.k_eosvmin; clamped = true;
      if (TAPE) fl |= TF_VNEW_MIN;
    }
    if (prm.has_eosvmax && kvn > prm.k_eosvmax) {
      vnewc_in = prm.eosvmax; clamped = true;
      if (TAPE) fl |= TF_VNEW_MAX;
    }
    // 1/vnewc, 1/vchalf (vchalf = vnewc - delvc/2 > 0) and the hydro
    // constraint's 1/(|vdov| + 1e-20) from one division
    const double w_hydro = fabs(vdov) + 1.e-20;
    double inv_vnewc_in, inv_vchalf_in, inv_w;
    recip3(vnewc_in, fma(delvc_in, -0.5, vnewc_in), w_hydro, inv_vnewc_in, inv_vchalf_in, inv_w);
    const double inv_vnew = clamped ? 1.0 / vnew : inv_vnewc_in;
    double qlin, qquad;
    if (gt_zero(vdov)) {
      qlin = 0.0;
      qquad = 0.0;
      if (TAPE) {
        fl |= TF_QZERO;
#pragma unroll
        for (int q = 9; q < 14; ++q) tm(q, 0.0);
      }
    } else {
      double dxxi = dvxi * LDG(&d.delx_xi[i]);
      double dxeta = dveta * LDG(&d.delx_eta[i]);
      double dxzeta = dvzeta * LDG(&d.delx_zeta[i]);
      if (gt_zero(dxxi)) { dxxi = 0.0; if (TAPE) fl |= TF_DXCLAMP0; }
      if (gt_zero(dxeta)) { dxeta = 0.0; if (TAPE) fl |= TF_DXCLAMP0 << 1; }
      if (gt_zero(dxzeta)) { dxzeta = 0.0; if (TAPE) fl |= TF_DXCLAMP0 << 2; }
      // rho = elemMass / (volo vnew), from the reciprocals of volo and vnew
      const double rho = (LDG(&d.elemMass[i]) * LDG(&d.inv_volo[i])) * inv_vnew;
      const double s1sum = fma(dxxi, 1.0 - phixi, fma(dxeta, 1.0 - phieta, dxzeta * (1.0 - phizeta)));
      const double s2sum = fma(dxxi * dxxi, fma(-phixi, phixi, 1.0),
                               fma(dxeta * dxeta, fma(-phieta, phieta, 1.0), (dxzeta * dxzeta) * fma(-phizeta, phizeta, 1.0)));
      qlin = (-prm.qlc_monoq * rho) * s1sum;
      qquad = (prm.qqc_monoq * rho) * s2sum;
      tm(9, rho); tm(10, qlin); tm(11, qquad); tm(12, s1sum); tm(13, s2sum);
    }
    if (AUX) { d.ql[i] = qlin; d.qq[i] = qquad; }

    // ---- qstop check on the old q, src/domain.jl:2567-2582 ----
    const double q_old_in = d.q[i];
    if (fkey(q_old_in) > prm.k_qstop) err |= ST_QSTOP;

    // ---- applyMaterialPropertiesForElems' volume check ----
    {
      double vc = LDG(&d.v[i]);
      long long kvc = fkey(vc);
      if (prm.has_eosvmin && kvc < prm.k_eosvmin) { vc = prm.eosvmin; kvc = prm.k_eosvmin; }
      if (prm.has_eosvmax && kvc > prm.k_eosvmax) vc = prm.eosvmax;
      if (le_zero(vc)) err |= ST_MATERIAL;
    }

    // ---- evalEOSForElems + calcEnergyForElems + calcSoundSpeedForElems,
    //      src/domain.jl:2617-2857, per element ----
    // The region cost model (LULESH 2.0's rep loop in EvalEOSForElems, which
    // the reference computes in regReps but never applies) evaluates the
    // energy update `reps` times with identical inputs; the inputs pass
    // through an opaque register move each time so no evaluation is folded
    // away, and the last one is kept. Results do not depend on reps.
    const int reps = REGION ? LDG(&d.posReps[t]) : 1;
    const double e_old_in = d.e[i];
    const double p_old_in = d.p[i];
    const double c1s = 2.0 / 3.0;
    const double inv_rho0 = prm.inv_refdens;
    double e_out = 0.0, p_out = 0.0, vv_out = 0.0;
    bool compress_out = false;
    // TINY-guarded sound-speed square root (src/domain.jl:2655-2659, 2738-2742)
    auto tiny_sqrt = [&](double ssc, unsigned long long bit) -> double {
      // ssc <= 0.111111e-36 (a positive threshold: the signed bit patterns order)
      if (__double_as_longlong(ssc) <= 0x3842E7910CC4BCABll) { if (TAPE) fl |= bit; return 0.333333e-18; }
      return ssc * rsqrt(ssc);
    };
#pragma unroll 1
    for (int rep = 0; rep < reps; ++rep) {
    double delvc = delvc_in, e_old = e_old_in, p_old = p_old_in, q_old = q_old_in, vnewc = vnewc_in;
    if (REGION) { opaque(delvc); opaque(e_old); opaque(p_old); opaque(q_old); opaque(vnewc); }
    const double vchalf = fma(delvc, -0.5, vnewc);
    // the rep passes form the reciprocals anew from their opaque inputs
    double inv_vnewc = inv_vnewc_in, inv_vchalf = inv_vchalf_in;
    if (REGION) { double iw; recip3(vnewc, vchalf, w_hydro, inv_vnewc, inv_vchalf, iw); }
    // compression = 1/vnewc - 1 and compHalfStep = 1/vchalf - 1 enter only as
    // bvc = c1s (1 + compression) and bvc_half = c1s (1 + compHalfStep):
    // bv and bvh are those factors over c1s for the branch taken
    const long long kv = fkey(vnewc);
    const bool at_vmin = prm.has_eosvmin && kv <= prm.k_eosvmin;  // eosvmin != 0 && vnewc <= eosvmin
    const bool vmax_hit = kv >= prm.k_eosvmax;                     // vnewc >= eosvmax
    const bool at_vmax = prm.has_eosvmax && vmax_hit;
    double bv = inv_vnewc, bvh = inv_vchalf;
    if (at_vmin) { bvh = bv; if (TAPE) fl |= TF_HALF_EQ_COMP; }
    if (at_vmax) {
      p_old = 0.0; bv = 1.0; bvh = 1.0;
      if (TAPE) fl |= TF_VMAX_HIT;
    }
    // calcPressureForElems (src/domain.jl:2585-2614) for one element; the
    // cut / pmin outcomes go to the tape bits given
    auto pressure = [&](double enew, double bvc, unsigned long long cut_bit, unsigned long long min_bit) -> double {
      double pn = bvc * enew;
      if (abs_lt(pn, prm.p_cut)) { pn = 0.0; if (TAPE) fl |= cut_bit; }
      if (vmax_hit) pn = 0.0;
      if (fkey(pn) < prm.k_pmin) { pn = prm.pmin; if (TAPE) fl |= min_bit; }
      return pn;
    };
    const double pq_old = p_old + q_old;
    // 0.5 delvc and pHalfStep + q_new serve both energy updates (the negated
    // and scaled forms are exact, so the values are those of separate products)
    const double hdv = 0.5 * delvc;
    double e_new = fma(-hdv, pq_old, e_old);
    if (fkey(e_new) < prm.k_emin) { e_new = prm.emin; if (TAPE) fl |= TF_E1_MIN; }
    const double bvc_half = c1s * bvh;
    const double pHalfStep = pressure(e_new, bvc_half, TF_PH_CUT, TF_PH_MIN);
    // vhalf = 1 / (1 + compHalfStep): vchalf, vnewc or 1 by the branch taken
    const double vhalf = at_vmax ? 1.0 : at_vmin ? vnewc : vchalf;
    const bool compress = !gt_zero(delvc);   // delvc <= 0 (non-NaN)
    if (TAPE && compress) fl |= TF_COMPRESS;
    tm(14, bv); tm(15, bvh); tm(16, e_new); tm(17, pHalfStep); tm(18, vhalf);
    double q_new = 0.0;
    if (compress) {
      const double ssc = fma(c1s, e_new, ((vhalf * vhalf) * bvc_half) * pHalfStep) * inv_rho0;
      const double s1 = tiny_sqrt(ssc, TF_S1_TINY);
      q_new = fma(s1, qlin, qquad);
      tm(19, s1); tm(28, ssc);
    } else {
      tm(19, 0.0); tm(28, 0.0);
    }
    tm(20, q_new);
    const double sh = pHalfStep + q_new;
    e_new = fma(hdv, fma(3.0, pq_old, -4.0 * sh), e_new);
    if (abs_lt(e_new, prm.e_cut)) { e_new = 0.0; if (TAPE) fl |= TF_E2_CUT; }
    if (fkey(e_new) < prm.k_emin) { e_new = prm.emin; if (TAPE) fl |= TF_E2_MIN; }
    const double bvc = c1s * bv;
    double p_new = pressure(e_new, bvc, TF_PN1_CUT, TF_PN1_MIN);
    const double vv_bvc = (vnewc * vnewc) * bvc;
    tm(21, e_new); tm(22, p_new);
    double q_tilde = 0.0;
    if (compress) {
      const double ssc = fma(c1s, e_new, vv_bvc * p_new) * inv_rho0;
      const double s2 = tiny_sqrt(ssc, TF_S2_TINY);
      q_tilde = fma(s2, qlin, qquad);
      tm(23, s2); tm(29, ssc);
    } else {
      tm(23, 0.0); tm(29, 0.0);
    }
    tm(24, q_tilde);
    e_new = e_new - ((fma(7.0, pq_old, -8.0 * sh) + (p_new + q_tilde)) * delvc) * (1.0 / 6.0);
    if (abs_lt(e_new, prm.e_cut)) { e_new = 0.0; if (TAPE) fl |= TF_E3_CUT; }
    if (fkey(e_new) < prm.k_emin) { e_new = prm.emin; if (TAPE) fl |= TF_E3_MIN; }
    p_new = pressure(e_new, bvc, TF_PN2_CUT, TF_PN2_MIN);
    e_out = e_new; p_out = p_new; vv_out = vv_bvc; compress_out = compress;
    }  // rep loop
    const double e_new = e_out, p_new = p_out, vv_bvc = vv_out;
    const bool compress = compress_out;
    double q_new = 0.0;
    // the last q evaluation and the sound speed share one expression
    const double ssc3 = fma(c1s, e_new, vv_bvc * p_new) * inv_rho0;
    const double ss_new = tiny_sqrt(ssc3, TF_SS_TINY);
    tm(25, e_new); tm(26, p_new); tm(27, ss_new); tm(30, ssc3);
    if (compress) {
      q_new = fma(ss_new, qlin, qquad);
      if (abs_lt(q_new, prm.q_cut)) { q_new = 0.0; if (TAPE) fl |= TF_Q_CUT; }
    }
    d.p[i] = p_new;
    d.e[i] = e_new;
    d.q[i] = q_new;
    d.ss[i] = ss_new;

    // ---- updateVolumesForElems, src/domain.jl:2912-2930 ----
    double tmpV = vnew;
    if (abs_lt(tmpV - 1.0, prm.v_cut)) { tmpV = 1.0; if (TAPE) fl |= TF_V_SNAP; }
    d.v[i] = tmpV;
    if (le_zero(tmpV)) err |= ST_UPDATE;

    // ---- Courant and hydro constraints, src/domain.jl:2964-3054 ----
    double dtc = __longlong_as_double((long long)kInfBits), dth = dtc;
    if (!is_zero(vdov)) {
      const double arealg = LDG(&d.arealg[i]);
      double dtf = ss_new * ss_new;
      if (lt_zero(vdov)) dtf = fma(prm.qqc2x64 * (arealg * arealg), vdov * vdov, dtf);
      dtc = arealg * rsqrt(dtf);
      dth = prm.dvovmax * inv_w;
      courant = (unsigned long long)__double_as_longlong(dtc);
      hydro = (unsigned long long)__double_as_longlong(dth);
    }
    if (TAPE) {
      d.tapeFlags[i] |= fl;  // k_kinematics stored the face bits of this cycle
      d.tapeDtc[i] = dtc;
      d.tapeDth[i] = dth;
    }
    if (err) atomicOr(&st->status, err);
  }
  if (ENS) warp_min2_by_instance(courant, hydro, inst, d.st);
  else block_min2(courant, hydro, &d.st->acc_courant, &d.st->acc_hydro);
}

// ---------------------------------------------------------------------------
// Halo copies of a block-partitioned mesh (the single-GPU form of commSBN and
// commMonoQ, src/comm.jl:776, 1127): each ghost slot takes the value of the
// corner force or element its owning block computed.
// ---------------------------------------------------------------------------
__global__ void k_halo_corners(DevDomain d) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  const int base = 8 * d.E;
  if (g >= d.nCornerSlot - base) return;
  if (step_off(d.st)) return;
  const int s = LULESH_IDX(LDG(&d.haloCornerSrc[g]), base, d.st);
  d.fcx[base + g] = d.fcx[s];
  d.fcy[base + g] = d.fcy[s];
  d.fcz[base + g] = d.fcz[s];
}

__global__ void k_halo_delv(DevDomain d) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= d.Eg - d.E) return;
  if (step_off(d.st)) return;
  const int s = LULESH_IDX(LDG(&d.haloDelvSrc[g]), d.E, d.st);
  d.delv_xi[d.E + g] = d.delv_xi[s];
  d.delv_eta[d.E + g] = d.delv_eta[s];
  d.delv_zeta[d.E + g] = d.delv_zeta[s];
}

// ---------------------------------------------------------------------------
// k_time_increment (device run loop): one thread per problem
// ---------------------------------------------------------------------------
__device__ void advance_time(DevState* st, const Params& prm) {
  if (st->done) return;
  if (st->status) { st->done = 1; return; }
  // fold the previous step's minima (src/domain.jl:3012-3014, 3050-3052)
  if (dt_registers(st->acc_courant)) st->dtcourant = __longlong_as_double((long long)st->acc_courant);
  if (dt_registers(st->acc_hydro)) st->dthydro = __longlong_as_double((long long)st->acc_hydro);
  st->acc_courant = kInfBits;
  st->acc_hydro = kInfBits;
  // examples/benchmark.jl:82-98: while time < stoptime ... break if cycle >= num_iters
  if (!(st->time < prm.stoptime) || (!st->first && st->cycle >= st->num_iters)) { st->done = 1; return; }
  st->first = 0;
  double time = st->time, dt = st->deltatime;
  long long cycle = st->cycle;
  time_increment(time, dt, cycle, st->dtcourant, st->dthydro, prm);
  st->time = time;
  st->deltatime = dt;
  st->cycle = cycle;
}

__global__ void k_time_increment(DevState* st, int n, Params prm) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) advance_time(st + k, prm);
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
// An ensemble (d.elemInst set) runs the ENS instantiations, which read each
// element's or node's instance; the plain path runs ENS = false.
void launch_geometry(const DevDomain& d, cudaStream_t s) {
  const int bs = 128;
  k_geometry<<<(d.E + bs - 1) / bs, bs, 0, s>>>(d);
}

void launch_force(const DevDomain& d, const Params& prm, const Tuning& t, cudaStream_t s) {
  const int bs = t.force;
  const int grid = (d.E + bs - 1) / bs;
  const bool ens = d.elemInst != nullptr;
  const bool inl = t.geo != 0 && !d.tapeGeo;  // the taping kernels always use the stored geometry
#define LULESH_FORCE(M)                                                                            \
  (ens ? (inl ? k_force<M, true, false, true><<<grid, bs, 0, s>>>(d, prm)                          \
              : k_force<M, true, false, false><<<grid, bs, 0, s>>>(d, prm))                        \
       : d.tapeGeo ? k_force<M, false, true, false><<<grid, bs, 0, s>>>(d, prm)                    \
                   : (inl ? k_force<M, false, false, true><<<grid, bs, 0, s>>>(d, prm)              \
                          : k_force<M, false, false, false><<<grid, bs, 0, s>>>(d, prm)))
  switch (d.mode & 3) {
    case 0: LULESH_FORCE(0); break;
    case 1: LULESH_FORCE(1); break;
    case 2: LULESH_FORCE(2); break;
    default: LULESH_FORCE(3); break;
  }
#undef LULESH_FORCE
}

void launch_node(const DevDomain& d, const Params& prm, bool aux, const Tuning& t, cudaStream_t s) {
  if (d.haloCornerSrc) {
    const int n = d.nCornerSlot - 8 * d.E;
    k_halo_corners<<<(n + 255) / 256, 256, 0, s>>>(d);
  }
  const int bs = t.node;
  const int grid = (d.N + bs - 1) / bs;
  if (d.nodeInst) k_node<false, true><<<grid, bs, 0, s>>>(d, prm);
  else if (aux) k_node<true, false><<<grid, bs, 0, s>>>(d, prm);
  else k_node<false, false><<<grid, bs, 0, s>>>(d, prm);
}

void launch_kinematics(const DevDomain& d, const Params& prm, bool aux, const Tuning& t, cudaStream_t s) {
  const int bs = t.kin;
  const int grid = (d.E + bs - 1) / bs;
  const bool geo = t.geo == 0;
  if (d.elemInst) {
    if (geo) k_kinematics<false, true, false, true><<<grid, bs, 0, s>>>(d, prm);
    else k_kinematics<false, true, false, false><<<grid, bs, 0, s>>>(d, prm);
  } else if (d.tapeFlags) {
    k_kinematics<false, false, true, true><<<grid, bs, 0, s>>>(d, prm);
  } else if (aux) {
    if (geo) k_kinematics<true, false, false, true><<<grid, bs, 0, s>>>(d, prm);
    else k_kinematics<true, false, false, false><<<grid, bs, 0, s>>>(d, prm);
  } else {
    if (geo) k_kinematics<false, false, false, true><<<grid, bs, 0, s>>>(d, prm);
    else k_kinematics<false, false, false, false><<<grid, bs, 0, s>>>(d, prm);
  }
}

void launch_material(const DevDomain& d, const Params& prm, bool aux, const Tuning& t, cudaStream_t s) {
  if (d.haloDelvSrc) {
    const int n = d.Eg - d.E;
    k_halo_delv<<<(n + 255) / 256, 256, 0, s>>>(d);
  }
  const int bs = t.mat;
  const int grid = (d.E + bs - 1) / bs;
  const bool fix = (d.mode & 4) != 0;
  const bool region = d.regOrder != nullptr;
#define LULESH_MAT(M, AUX, ENS, TAPE, REGION) k_material<M, AUX, ENS, TAPE, REGION><<<grid, bs, 0, s>>>(d, prm)
  if (d.elemInst) {
    if (fix) LULESH_MAT(4, false, true, false, false);
    else LULESH_MAT(0, false, true, false, false);
  } else if (d.tapeFlags) {
    if (fix) LULESH_MAT(4, false, false, true, false);
    else LULESH_MAT(0, false, false, true, false);
  } else if (region) {
    if (fix) { if (aux) LULESH_MAT(4, true, false, false, true); else LULESH_MAT(4, false, false, false, true); }
    else { if (aux) LULESH_MAT(0, true, false, false, true); else LULESH_MAT(0, false, false, false, true); }
  } else if (fix) {
    if (aux) LULESH_MAT(4, true, false, false, false);
    else LULESH_MAT(4, false, false, false, false);
  } else {
    if (aux) LULESH_MAT(0, true, false, false, false);
    else LULESH_MAT(0, false, false, false, false);
  }
#undef LULESH_MAT
}

void launch_time_increment(DevState* st, int n, const Params& prm, cudaStream_t s) {
  k_time_increment<<<(n + 127) / 128, 128, 0, s>>>(st, n, prm);
}

}  // namespace lulesh
