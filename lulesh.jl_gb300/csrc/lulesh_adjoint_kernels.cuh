// Reverse-mode adjoint kernels of the LagrangeLeapFrog step.
//
// Each kernel is the hand-written transpose (vector-Jacobian product) of one
// forward kernel of lulesh_kernels.cu, in the same formulation (Walsh
// coefficients, face-diagonal cross products, edge sums). Forward values are
// recomputed from the cycle's tape (start state, end positions/velocities,
// accelerations, kinematics outputs); every branch (cut-offs, clamps, limiter
// cases, the characteristic-length face, velocity snaps) is read from the
// tape the taping forward kernels wrote, so the derivative is that of the
// branches actually taken. Node sums are transposed into per-corner buffers
// and gathered back in nodeElemCornerList order; neighbour reads of the Q
// limiter are transposed into per-face slots and gathered through an inverse
// neighbour list: no atomics, so gradients are bitwise reproducible.
#pragma once

#include <climits>

#include "lulesh_device.cuh"

namespace lulesh {

constexpr int kAdjBlock = 128;

// Scalars of one recorded cycle: timeIncrement!'s inputs and output, and the
// elements that attained the Courant and hydro minima (INT_MAX: none).
struct CycleRec {
  double time_prev, dt_prev, dtc_in, dth_in, dt;
  long long cycle_prev;
  int active_c, active_h, argmin_c, argmin_h;
};

// Adjoints of the Domain scalars carried from cycle to cycle.
struct AdjScal {
  double Ltime, Ldt, Ldtc, Ldth, Lhg;
};

// The 11 state fields (x y z xd yd zd e p q v ss) of one stored state.
struct StateSet {
  double* f[11];
};

struct AdjDev {
  int E, N;
  // constants of the problem
  const int* nodelist;        // [8][E]
  const int* nodeElemStart;   // N+1
  const int* cornerList;      // 8E, values c*E + e
  const unsigned char* nodeBC;
  const double *inv_nodalMass, *volo, *inv_volo, *elemMass;
  const unsigned* elemBC;
  const int *lxim, *lxip, *letam, *letap, *lzetam, *lzetap;
  const int *nbStart, *nbList;  // inverse neighbour lists (entries slot*E + j)
  // cycle start state S0 and end positions/velocities S1
  const double *x0, *y0, *z0, *xd0, *yd0, *zd0, *e0, *p0, *q0, *v0, *ss0;
  const double *x1, *y1, *z1, *xd1, *yd1, *zd1, *p1, *q1;
  // tape of the cycle
  const double *ax, *ay, *az;                 // accelerations (N)
  const double *vnew, *delv, *arealg, *vdov;  // kinematics outputs (E)
  const double *dvl[3], *dxl[3];              // delv_{xi,eta,zeta}, delx_{xi,eta,zeta}
  const unsigned long long* flags;
  const double* geo;                          // [66][E] force-kernel tape (dv, hms, S, N)
  const double* diag0;                        // [36][E] face diagonals at the run's start (first cycle)
  const double* kin;                          // [90][E] kinematics-kernel tape
  const double* mat;                          // [31][E] material-kernel tape
  // adjoints of the state (in place: S1 on entry, S0 on exit)
  double *lx, *ly, *lz, *lxd, *lyd, *lzd;     // N
  double *le, *lp, *lq, *lss, *lv;            // E
  // adjoints of intermediate quantities
  double *lfx, *lfy, *lfz;                    // N
  double *lvnew, *ldelv, *larealg, *lvdov;    // E
  double *ldv[3], *ldx[3];                    // E
  double* lnb;                                // [6][E]: limiter neighbour slots
  double *cX, *cV;                            // [3][8][E] kinematics corner buffers
  double *fX, *fV;                            // [3][8][E] force corner buffers: the first cycle's position
                                              // transpose; each cycle's hourglass velocity corners
  double *part_dt, *part_dtn, *part_hg;       // per-block partial sums (kinematics, node, force)
  double *sLdv, *sLhm;                        // [3][8][E], [3][4][E]: hourglass -> geometry
  double* sLU;                                // [5][3][E]: the stress force's face terms (hourglass -> geometry)
};

// Deterministic block sum (fixed tree order); thread 0 writes the block's sum.
__device__ __forceinline__ void block_sum_to(double v, double* out) {
  __shared__ double sh[kAdjBlock];
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int s = kAdjBlock / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = sh[0];
}

struct V3 {
  double x, y, z;
};
__device__ __forceinline__ V3 v3(double x, double y, double z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 vcross(const V3& a, const V3& b) {
  V3 c;
  cross(a.x, a.y, a.z, b.x, b.y, b.z, c.x, c.y, c.z);
  return c;
}
__device__ __forceinline__ double vdot(const V3& a, const V3& b) { return fma(a.x, b.x, fma(a.y, b.y, a.z * b.z)); }
__device__ __forceinline__ void vaxpy(V3& y, double a, const V3& x) {
  y.x = fma(a, x.x, y.x); y.y = fma(a, x.y, y.y); y.z = fma(a, x.z, y.z);
}
__device__ __forceinline__ void vadd(V3& y, const V3& x) { y.x += x.x; y.y += x.y; y.z += x.z; }

// Resolved limiter neighbour: the element whose delv is read (self for a
// symmetry face or the reference's self-reading xi-plus index), -1 for a free
// face.
__device__ __forceinline__ int limiter_index(unsigned mask, unsigned bits, unsigned symm, unsigned freeb,
                                             unsigned comm, int idx, int self, int E) {
  const unsigned c = mask & bits;
  if (c == 0u || c == comm) return (idx >= 0 && idx < E) ? idx : -1;
  if (c == symm) return self;
  return -1;
}

// ---------------------------------------------------------------------------
// ka_material: transpose of k_material (Q limiter, EOS, volume update,
// Courant and hydro candidates).
// ---------------------------------------------------------------------------
template <int MODE>
__global__ void __launch_bounds__(kAdjBlock, 4) ka_material(AdjDev a, Params prm, double irho0, const CycleRec* rec,
                                                          const AdjScal* sc) {
  const int E = a.E;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= E) return;
  // the cycle's Courant/hydro minima pass their adjoint to the element that
  // attained them
  const int argmin_c = rec->argmin_c, argmin_h = rec->argmin_h;
  const double lam_c = rec->active_c ? sc->Ldtc : 0.0, lam_h = rec->active_h ? sc->Ldth : 0.0;
  const unsigned long long fl = a.flags[i];
  const unsigned mask = a.elemBC[i];
  // neighbour resolution exactly as the forward kernel
  int im[3], ip[3];
  im[0] = limiter_index(mask, XI_M, XI_M_SYMM, XI_M_FREE, XI_M_COMM, a.lxim[i], i, E);
  ip[0] = limiter_index(mask, XI_P, XI_P_SYMM, XI_P_FREE, XI_P_COMM, (MODE & 4) ? a.lxip[i] : a.lxip[i] - 1, i, E);
  im[1] = limiter_index(mask, ETA_M, ETA_M_SYMM, ETA_M_FREE, ETA_M_COMM, a.letam[i], i, E);
  ip[1] = limiter_index(mask, ETA_P, ETA_P_SYMM, ETA_P_FREE, ETA_P_COMM, a.letap[i], i, E);
  im[2] = limiter_index(mask, ZETA_M, ZETA_M_SYMM, ZETA_M_FREE, ZETA_M_COMM, a.lzetam[i], i, E);
  ip[2] = limiter_index(mask, ZETA_P, ZETA_P_SYMM, ZETA_P_FREE, ZETA_P_COMM, a.lzetap[i], i, E);

  // forward values from the material kernel's tape (slots: see tapeMat)
  auto tm = [&](int q) { return a.mat[q * E + i]; };
  double self[3], norm[3], tdm[3], tdp[3], phi[3], delx[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    self[d] = a.dvl[d][i];
    norm[d] = tm(d);
    tdm[d] = tm(3 + d);  // minus neighbour's delv * norm
    tdp[d] = tm(6 + d);  // plus neighbour's delv * norm
    const int src = (int)((fl >> (3 * d)) & 7ull);
    phi[d] = src == PHI_MEAN ? 0.5 * (tdm[d] + tdp[d])
           : src == PHI_M ? tdm[d] * prm.monoq_limiter_mult
           : src == PHI_P ? tdp[d] * prm.monoq_limiter_mult
           : src == PHI_ZERO ? 0.0 : prm.monoq_max_slope;
    delx[d] = a.dxl[d][i];
  }
  const double vdov = a.vdov[i], vnew = a.vnew[i];
  const double delvc = a.delv[i], arealg = a.arealg[i];
  const bool vmin_c = (fl & TF_VNEW_MIN) != 0, vmax_c = (fl & TF_VNEW_MAX) != 0;
  const double vnewc = vmin_c ? prm.eosvmin : vmax_c ? prm.eosvmax : vnew;
  const bool vmax_hit = (fl & TF_VMAX_HIT) != 0, half_eq = (fl & TF_HALF_EQ_COMP) != 0;
  // bv = 1 + compression and bvh = 1 + compHalfStep as the forward formed
  // them: 1/vnewc and 1/vchalf on the branches where they are reciprocals
  const double bv = tm(14), bvh = tm(15);
  const double inv_vnewc = vmax_hit ? 1.0 / vnewc : bv;
  const double inv_vnew = (vnewc == vnew) ? inv_vnewc : 1.0 / vnew;
  const double inv_vchalf = (vmax_hit || half_eq) ? 0.0 : bvh;
  const bool qzero = (fl & TF_QZERO) != 0;
  double dx[3] = {0.0, 0.0, 0.0};
  const double rho = tm(9), qlin = tm(10), qquad = tm(11), s1sum = tm(12), s2sum = tm(13);
  if (!qzero) {
#pragma unroll
    for (int d = 0; d < 3; ++d) dx[d] = (fl & (TF_DXCLAMP0 << d)) ? 0.0 : self[d] * delx[d];
  }
  const double p_old = vmax_hit ? 0.0 : a.p0[i], q_old = a.q0[i];
  const double c1s = 2.0 / 3.0;  // irho0 = 1 / refdens
  const double pq = p_old + q_old;
  const bool e1min = (fl & TF_E1_MIN) != 0;
  const double e1 = tm(16), pH = tm(17), vhalf = tm(18);
  const double bvc_h = c1s * bvh;
  const bool pH_on = !vmax_hit && !(fl & (TF_PH_CUT | TF_PH_MIN));
  const bool comp = (fl & TF_COMPRESS) != 0;
  const bool s1t = (fl & TF_S1_TINY) != 0, s2t = (fl & TF_S2_TINY) != 0, sst = (fl & TF_SS_TINY) != 0;
  // each square root s = sqrt(c) comes with h = 0.5 / s = 0.5 rsqrt(c)
  const double s1 = tm(19), qn1 = tm(20);
  const double h1 = (comp && !s1t) ? 0.5 * rsqrt(tm(28)) : 0.0;
  const bool e2fix = (fl & (TF_E2_CUT | TF_E2_MIN)) != 0;
  const double k2 = fma(3.0, pq, -4.0 * (pH + qn1));
  const double e2 = tm(21), pn1 = tm(22);
  const double bvc = c1s * bv;
  const bool pn1_on = !vmax_hit && !(fl & (TF_PN1_CUT | TF_PN1_MIN));
  const double vv_bvc = (vnewc * vnewc) * bvc;
  const double s2 = tm(23), qt = tm(24);
  const double h2 = (comp && !s2t) ? 0.5 * rsqrt(tm(29)) : 0.0;
  const double k3 = fma(7.0, pq, -8.0 * (pH + qn1)) + (pn1 + qt);
  const bool e3fix = (fl & (TF_E3_CUT | TF_E3_MIN)) != 0;
  const double e3 = tm(25), pn2 = tm(26), ss = tm(27);
  const bool pn2_on = !vmax_hit && !(fl & (TF_PN2_CUT | TF_PN2_MIN));
  const double hs = sst ? 0.0 : 0.5 * rsqrt(tm(30));

  // ---------------- reverse ----------------
  double Le3 = a.le[i], Lpn2 = a.lp[i], Lq = a.lq[i], Lss = a.lss[i], Lv1 = a.lv[i];
  double Lvnew = 0.0, Larealg = 0.0, Lvdov = 0.0, Ldelvc = 0.0;
  // Courant and hydro candidates (only the arg-min element carries a seed)
  if (i == argmin_c && vdov != 0.0) {
    const double qqc2 = (64.0 * prm.qqc) * prm.qqc;
    double dtf = ss * ss;
    if (vdov < 0.0) dtf = fma(qqc2 * (arealg * arealg), vdov * vdov, dtf);
    const double rs = rsqrt(dtf);
    Larealg += lam_c * rs;
    const double Ldtf = lam_c * arealg * (-0.5) * rs * rs * rs;
    Lss += 2.0 * ss * Ldtf;
    if (vdov < 0.0) {
      Larealg += Ldtf * 2.0 * qqc2 * arealg * vdov * vdov;
      Lvdov += Ldtf * 2.0 * qqc2 * arealg * arealg * vdov;
    }
  }
  if (i == argmin_h && vdov != 0.0) {
    const double den = fabs(vdov) + 1.e-20;
    Lvdov += lam_h * (-prm.dvovmax / (den * den)) * (vdov < 0.0 ? -1.0 : 1.0);
  }
  if (!(fl & TF_V_SNAP)) Lvnew += Lv1;
  double Lqlin = 0.0, Lqquad = 0.0;
  // final q = ss*qlin + qquad
  if (comp && !(fl & TF_Q_CUT)) { Lss += Lq * qlin; Lqlin += Lq * ss; Lqquad += Lq; }
  double Lvv = 0.0, Lbvc = 0.0, Le2 = 0.0, Lpn1 = 0.0, Lpq = 0.0, LpH = 0.0, Lqn1 = 0.0, Lqt = 0.0;
  // ss = sqrt(ssc3)
  if (!sst) {
    const double Lssc = Lss * hs * irho0;
    Le3 += Lssc * c1s;
    Lvv += Lssc * pn2;
    Lpn2 += Lssc * vv_bvc;
  }
  if (pn2_on) { Lbvc += Lpn2 * e3; Le3 += Lpn2 * bvc; }
  if (!e3fix) {
    Le2 += Le3;
    const double Lk = -Le3 * delvc * (1.0 / 6.0);
    Ldelvc += -Le3 * k3 * (1.0 / 6.0);
    Lpq += 7.0 * Lk; LpH += -8.0 * Lk; Lqn1 += -8.0 * Lk; Lpn1 += Lk; Lqt += Lk;
  }
  if (comp) {
    Lqlin += Lqt * s2; Lqquad += Lqt;
    if (!s2t) {
      const double Lssc = Lqt * qlin * h2 * irho0;
      Le2 += Lssc * c1s;
      Lvv += Lssc * pn1;
      Lpn1 += Lssc * vv_bvc;
    }
  }
  double Lvnewc = 2.0 * vnewc * bvc * Lvv;
  Lbvc += Lvv * (vnewc * vnewc);
  if (pn1_on) { Lbvc += Lpn1 * e2; Le2 += Lpn1 * bvc; }
  double Le1 = 0.0;
  if (!e2fix) {
    Le1 += Le2;
    Ldelvc += Le2 * 0.5 * k2;
    Lpq += Le2 * 1.5 * delvc;
    LpH += -2.0 * delvc * Le2;
    Lqn1 += -2.0 * delvc * Le2;
  }
  double Lchs = 0.0, Lbvch = 0.0;
  if (comp) {
    Lqlin += Lqn1 * s1; Lqquad += Lqn1;
    if (!s1t) {
      const double Lssc = Lqn1 * qlin * h1 * irho0;
      Le1 += Lssc * c1s;
      const double Lvhalf = Lssc * 2.0 * vhalf * bvc_h * pH;
      Lbvch += Lssc * (vhalf * vhalf) * pH;
      LpH += Lssc * (vhalf * vhalf) * bvc_h;
      Lchs += -Lvhalf * vhalf * vhalf;
    }
  }
  if (pH_on) { Lbvch += LpH * e1; Le1 += LpH * bvc_h; }
  Lchs += Lbvch * c1s;
  double Le_old = 0.0;
  if (!e1min) {
    Le_old += Le1;
    Ldelvc += -0.5 * pq * Le1;
    Lpq += -0.5 * delvc * Le1;
  }
  double Lcomp = Lbvc * c1s;
  const double Lp_old = vmax_hit ? 0.0 : Lpq;
  const double Lq_old = Lpq;
  if (!vmax_hit) {
    if (half_eq) Lcomp += Lchs;
    else {
      const double Lvch = -Lchs * (inv_vchalf * inv_vchalf);
      Lvnewc += Lvch;
      Ldelvc += -0.5 * Lvch;
    }
    Lvnewc += -Lcomp * (inv_vnewc * inv_vnewc);
  }
  if (!vmin_c && !vmax_c) Lvnew += Lvnewc;
  // qlin / qquad
  double Lself[3] = {0.0, 0.0, 0.0}, Ldx[3] = {0.0, 0.0, 0.0};
  double Lphi[3] = {0.0, 0.0, 0.0};
  if (!qzero) {
    const double Lrho = Lqlin * (-prm.qlc_monoq) * s1sum + Lqquad * prm.qqc_monoq * s2sum;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const double Ldxd = Lqlin * (-prm.qlc_monoq * rho) * (1.0 - phi[d]) +
                          Lqquad * (prm.qqc_monoq * rho) * 2.0 * dx[d] * fma(-phi[d], phi[d], 1.0);
      Lphi[d] = Lqlin * (prm.qlc_monoq * rho) * dx[d] + Lqquad * (-prm.qqc_monoq * rho) * dx[d] * dx[d] * 2.0 * phi[d];
      if (!(fl & (TF_DXCLAMP0 << d))) { Lself[d] += Ldxd * delx[d]; Ldx[d] += Ldxd * self[d]; }
    }
    Lvnew += -Lrho * rho * inv_vnew;
  }
  // limiter
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const int src = (int)((fl >> (3 * d)) & 7ull);
    double Ldm = 0.0, Ldp = 0.0;
    if (src == PHI_MEAN) { Ldm = 0.5 * Lphi[d]; Ldp = 0.5 * Lphi[d]; }
    else if (src == PHI_M) Ldm = prm.monoq_limiter_mult * Lphi[d];
    else if (src == PHI_P) Ldp = prm.monoq_limiter_mult * Lphi[d];
    const double Lm = Ldm * norm[d], Lp = Ldp * norm[d];
    // norm = 1/(self + ptiny): d(mv norm)/dself = -(mv norm) norm
    Lself[d] += -fma(Ldm, tdm[d], Ldp * tdp[d]) * norm[d];
    double sm = 0.0, sp = 0.0;
    if (im[d] == i) Lself[d] += Lm; else if (im[d] >= 0) sm = Lm;
    if (ip[d] == i) Lself[d] += Lp; else if (ip[d] >= 0) sp = Lp;
    a.lnb[(2 * d) * E + i] = sm;
    a.lnb[(2 * d + 1) * E + i] = sp;
    a.ldv[d][i] = Lself[d];
    a.ldx[d][i] = Ldx[d];
  }
  a.lvdov[i] = Lvdov;
  a.lvnew[i] = Lvnew;
  a.ldelv[i] = Ldelvc;
  a.larealg[i] = Larealg;
  // adjoints of the cycle's start state from the material update
  a.le[i] = Le_old;
  a.lp[i] = Lp_old;
  a.lq[i] = Lq_old;
  a.lss[i] = 0.0;
  a.lv[i] = 0.0;
}

// Transpose of walsh1: adds dL/dv of the 8 corner values for the adjoints
// Lw of the three coefficients (through the body diagonals, 14 adds).
__device__ __forceinline__ void walsh1_t(const double Lw[3], double L[8]) {
  const double p = Lw[0] + Lw[2], q = Lw[2] - Lw[0];
  const double La = p + Lw[1], Lb = p - Lw[1], Lc = q + Lw[1], Ld = q - Lw[1];
  L[6] += La; L[0] -= La;
  L[5] += Lb; L[3] -= Lb;
  L[7] += Lc; L[1] -= Lc;
  L[4] += Ld; L[2] -= Ld;
}

// Transpose of the hourglass mode transform: out[n] = sum_m gamma[n][m] t[m]
// (12 adds).
__device__ __forceinline__ void walsh_modes_t(const double t[4], double out[8]) {
  const double cm = t[2] - t[3], cp = t[2] + t[3];
  const double s = t[0] + t[1], d = t[0] - t[1];
  out[0] = s + cm; out[1] = d - cm; out[2] = cm - s; out[3] = -d - cm;
  out[4] = cp - s; out[5] = -d - cp; out[6] = s + cp; out[7] = d - cp;
}

// ---------------------------------------------------------------------------
// ka_kinematics: transpose of k_kinematics (volume, characteristic length,
// velocity-gradient trace, monotonic-Q gradients), into the corner buffers.
// The cycle's end positions are the next cycle's start positions, so the
// position transpose of the next cycle's k_force (what force_geo_t does for
// the first cycle) joins it here, from what that cycle's ka_hourglass left:
// its modes' transpose starts the position corners, its volume-derivative
// Hessian-vector product merges with this cycle's volume gradient, and its
// stress terms add to the same face-diagonal adjoints, scattered once.
// ---------------------------------------------------------------------------
template <int MODE>
__global__ void __launch_bounds__(kAdjBlock, 3) ka_kinematics(AdjDev a, const CycleRec* rec) {
  const int E = a.E;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  const double dt = rec->dt;
  double Ldt = 0.0;
  if (e < E) {
    // forward values from the kinematics kernel's tape (slots: see tapeKin)
    auto tk = [&](int q) { return a.kin[q * E + e]; };

    const double vnew = a.vnew[e], volo = a.volo[e];
    double Lvnew = a.lvnew[e] + a.ldelv[e];
    a.lv[e] -= a.ldelv[e];  // delv = vnew - v
    // Walsh vectors of positions and velocities
    V3 W[3], VW[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      W[d] = v3(tk(d), tk(3 + d), tk(6 + d));
      VW[d] = v3(tk(9 + d), tk(12 + d), tk(15 + d));
    }
    V3 LW[3] = {v3(0, 0, 0), v3(0, 0, 0), v3(0, 0, 0)}, LVW[3] = {v3(0, 0, 0), v3(0, 0, 0), v3(0, 0, 0)};
    // ---- monotonic-Q gradients ----
    {
      const double vol = volo * vnew;
      const double norm64 = tk(40);  // 1/(64 vol + 64 ptiny)
      double Lvol = 0.0, Lnorm64 = 0.0;
      // limiter reads of this element's delv by its neighbours (inverse
      // neighbour list, fixed order) join its own delv adjoints
      double Ldvs[3] = {a.ldv[0][e], a.ldv[1][e], a.ldv[2][e]};
      for (int j = a.nbStart[e]; j < a.nbStart[e + 1]; ++j) {
        const int ent = a.nbList[j];
        const int dir = (ent / E) >> 1;
        const double v = a.lnb[ent];
        if (dir == 0) Ldvs[0] += v;
        else if (dir == 1) Ldvs[1] += v;
        else Ldvs[2] += v;
      }
      // direction d uses A = P x Q and velocity vector VW[d]
      const int Pi[3] = {1, 2, 0}, Qi[3] = {2, 0, 1};
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const V3 P = W[Pi[d]], Q = W[Qi[d]];
        const V3 A = v3(tk(28 + 3 * d), tk(29 + 3 * d), tk(30 + 3 * d));  // P x Q
        const double rs = tk(37 + d);  // 1/sqrt(|A|^2 + 256 ptiny)
        const double Ldx = a.ldx[d][e], Ldv = Ldvs[d];
        Lvol += Ldx * 16.0 * rs;
        const double Ls2 = Ldx * 16.0 * vol * (-0.5) * rs * rs * rs;
        V3 LA = v3(2.0 * A.x * Ls2, 2.0 * A.y * Ls2, 2.0 * A.z * Ls2);
        const double dot = vdot(A, VW[d]);
        Lnorm64 += Ldv * dot;
        vaxpy(LA, Ldv * norm64, VW[d]);
        vaxpy(LVW[d], Ldv * norm64, A);
        vadd(LW[Pi[d]], vcross(Q, LA));
        vadd(LW[Qi[d]], vcross(LA, P));
      }
      Lvol += Lnorm64 * (-64.0 * norm64 * norm64);
      Lvnew += Lvol * volo;
    }
    // ---- velocity-gradient trace at the half step ----
    {
      const double dt2 = -0.5 * dt;
      V3 F[3];
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        F[d] = v3(fma(dt2, VW[d].x, W[d].x), fma(dt2, VW[d].y, W[d].y), fma(dt2, VW[d].z, W[d].z));
      }
      // cofactor columns C0 = F1 x F2, C1 = F2 x F0, C2 = F0 x F1 and 1/det
      const V3 C0 = v3(tk(18), tk(19), tk(20)), C1 = v3(tk(21), tk(22), tk(23)), C2 = v3(tk(24), tk(25), tk(26));
      const double inv = tk(27);
      const double vdov = a.vdov[e];
      const double Ls = a.lvdov[e] * inv;
      const double Ldet = -a.lvdov[e] * vdov * inv;
      V3 LC[3];
      LC[0] = v3(Ls * VW[0].x, Ls * VW[0].y, Ls * VW[0].z);
      LC[1] = v3(Ls * VW[1].x, Ls * VW[1].y, Ls * VW[1].z);
      LC[2] = v3(Ls * VW[2].x, Ls * VW[2].y, Ls * VW[2].z);
      vaxpy(LVW[0], Ls, C0);
      vaxpy(LVW[1], Ls, C1);
      vaxpy(LVW[2], Ls, C2);
      vaxpy(LC[1], Ldet, F[1]);
      V3 LF[3] = {v3(0, 0, 0), v3(0, 0, 0), v3(0, 0, 0)};
      vaxpy(LF[1], Ldet, C1);
      // C0 = F1 x F2, C1 = F2 x F0, C2 = F0 x F1
      vadd(LF[1], vcross(F[2], LC[0])); vadd(LF[2], vcross(LC[0], F[1]));
      vadd(LF[2], vcross(F[0], LC[1])); vadd(LF[0], vcross(LC[1], F[2]));
      vadd(LF[0], vcross(F[1], LC[2])); vadd(LF[1], vcross(LC[2], F[0]));
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        vadd(LW[d], LF[d]);
        vaxpy(LVW[d], dt2, LF[d]);
        Ldt += -0.5 * vdot(LF[d], VW[d]);
      }
    }
    // Walsh transposes; the position corners start from the next cycle's
    // hourglass-mode transpose Gamma^T dL/dhm
    double LX[3][8], LV[3][8];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      double t[4];
#pragma unroll
      for (int m = 0; m < 4; ++m) t[m] = a.sLhm[(k * 4 + m) * E + e];
      walsh_modes_t(t, LX[k]);
#pragma unroll
      for (int c = 0; c < 8; ++c) LV[k][c] = 0.0;
    }
    {
      const double lwx[3] = {LW[0].x, LW[1].x, LW[2].x}, lwy[3] = {LW[0].y, LW[1].y, LW[2].y},
                   lwz[3] = {LW[0].z, LW[1].z, LW[2].z};
      walsh1_t(lwx, LX[0]); walsh1_t(lwy, LX[1]); walsh1_t(lwz, LX[2]);
      const double lvx[3] = {LVW[0].x, LVW[1].x, LVW[2].x}, lvy[3] = {LVW[0].y, LVW[1].y, LVW[2].y},
                   lvz[3] = {LVW[0].z, LVW[1].z, LVW[2].z};
      walsh1_t(lvx, LV[0]); walsh1_t(lvy, LV[1]); walsh1_t(lvz, LV[2]);
    }
    // the velocity corners, plus the hourglass velocity corners of the cycle
    // after this one
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
      for (int c = 0; c < 8; ++c) a.cV[(k * 8 + c) * E + e] = LV[k][c] + a.fV[(k * 8 + c) * E + e];
    // ---- volume and characteristic length, and the position transpose of
    //      the next cycle's k_force (same positions, same face diagonals) ----
    {
      // the 12 diagonals of the new positions are on the tape in the order
      // d61 d70 d63 d20 d50 d64 d31 d72 d43 d57 d14 d25
      auto dg = [&](int q) { return v3(tk(45 + 3 * q), tk(46 + 3 * q), tk(47 + 3 * q)); };
      const double volume = vnew * volo;  // vnew = volume / volo
      // characteristic length from the face the tape recorded: its diagonals
      // fa, fb (kinematics face order (d20, d31) (d64, d57) (d50, d14)
      // (d61, d25) (d72, d63) (d43, d70))
      const int f = (int)((a.flags[e] >> TF_FACE_SHIFT) & 7ull);
      const int qa = f == 0 ? 3 : f == 1 ? 5 : f == 2 ? 4 : f == 3 ? 0 : f == 4 ? 7 : 8;
      const int qb = f == 0 ? 6 : f == 1 ? 9 : f == 2 ? 10 : f == 3 ? 11 : f == 4 ? 2 : 1;
      const V3 nf = v3(tk(41), tk(42), tk(43));  // fa x fb
      const double rsc = tk(44);                  // 1/|fa x fb|
      const double Lar = a.larealg[e];
      double Lvolume = Lar * 2.0 * rsc + Lvnew * a.inv_volo[e];
      const double Lcl = Lar * 2.0 * volume * (-0.5) * rsc * rsc * rsc;
      const V3 Ln = v3(2.0 * nf.x * Lcl, 2.0 * nf.y * Lcl, 2.0 * nf.z * Lcl);
      const V3 Lfa = vcross(dg(qb), Ln), Lfb = vcross(Ln, dg(qa));
      const double Lv12 = Lvolume * (1.0 / 12.0);
      // The next cycle's force kernel used the gradient of 12*volume (its
      // voluDer, dv): G = dL/ddv (zero before the first transposed cycle;
      // the faithful slots 1 and 3 swapped back) makes its transpose the
      // Hessian-vector product of the same triple products along G. With
      // this cycle's Lv12 * gradient: dL/dU = Lv12 (V x W) + dV x W + V x dW,
      // dL/dV = W x (Lv12 U + dU) + dW x U, dL/dW = (Lv12 U + dU) x V + U x dV,
      // dU, dV, dW the differences of G along U, V, W (V x W is taped).
      double G[3][8];
#pragma unroll
      for (int j = 0; j < 3; ++j)
#pragma unroll
        for (int c = 0; c < 8; ++c) G[j][c] = a.sLdv[(j * 8 + c) * E + e];
      if (!(MODE & 2)) {
#pragma unroll
        for (int j = 0; j < 3; ++j) { const double t = G[j][1]; G[j][1] = G[j][3]; G[j][3] = t; }
      }
      auto gd = [&](int p, int q) { return v3(G[0][p] - G[0][q], G[1][p] - G[1][q], G[2][p] - G[2][q]); };
      auto triple_t = [&](const V3& U, const V3& V, const V3& W, const V3& gUt, const V3& dU, const V3& dV,
                          const V3& dW, V3& LUa, V3& LUb, V3& LVd, V3& LWd) {
        V3 A = dU; vaxpy(A, Lv12, U);
        V3 gU = vcross(dV, W); vadd(gU, vcross(V, dW)); vaxpy(gU, Lv12, gUt);
        V3 gV = vcross(W, A); vadd(gV, vcross(dW, U));
        V3 gW = vcross(A, V); vadd(gW, vcross(U, dV));
        vadd(LUa, gU); vadd(LUb, gU); vadd(LVd, gV); vadd(LWd, gW);
      };
      // The next cycle's stress force: face f's normal d1 x d2 (its
      // diagonals, force order: faces (d20, d31) (d50, d14) (d61, d25)
      // (d72, d36) (d43, d07), d36 = -d63, d07 = -d70) with LN = s8 LU_f
      // gives d1 the adjoint d2 x LN and d2 the adjoint LN x d1; s8 from
      // this cycle's end state.
      const double s8 = ((-a.p1[e]) - a.q1[e]) * 0.125;
      auto LN = [&](int fc) {
        return v3(s8 * a.sLU[(fc * 3) * E + e], s8 * a.sLU[(fc * 3 + 1) * E + e], s8 * a.sLU[(fc * 3 + 2) * E + e]);
      };
      auto put = [&](const V3& L, int p, int q) {
        LX[0][p] += L.x; LX[1][p] += L.y; LX[2][p] += L.z;
        LX[0][q] -= L.x; LX[1][q] -= L.y; LX[2][q] -= L.z;
      };
      const V3 z0 = v3(0, 0, 0);
      // Each triple product's four diagonals take adjoints from it, from two
      // or one of the stress faces and possibly the characteristic face, and
      // from nothing else: three disjoint groups, each scattered once.
      {  // (d31 + d72).(d63 x d20), faces 0 and 3, characteristic faces 0 and 4
        const V3 d63 = dg(2), d20 = dg(3), d31 = dg(6), d72 = dg(7);
        V3 L63 = z0, L20 = z0, L31 = z0, L72 = z0;
        V3 U = d31; vadd(U, d72);
        V3 dU = gd(3, 1); vadd(dU, gd(7, 2));
        triple_t(U, d63, d20, v3(tk(81), tk(82), tk(83)), dU, gd(6, 3), gd(2, 0), L31, L72, L63, L20);
        { const V3 n = LN(0); vadd(L20, vcross(d31, n)); vadd(L31, vcross(n, d20)); }
        { const V3 n = LN(3); vadd(L72, vcross(n, d63)); vadd(L63, vcross(d72, n)); }
        if (f == 0) { vadd(L20, Lfa); vadd(L31, Lfb); }
        else if (f == 4) { vadd(L72, Lfa); vadd(L63, Lfb); }
        put(L63, 6, 3); put(L20, 2, 0); put(L31, 3, 1); put(L72, 7, 2);
      }
      {  // (d43 + d57).(d64 x d70), face 4, characteristic faces 1 and 5
        const V3 d70 = dg(1), d64 = dg(5), d43 = dg(8), d57 = dg(9);
        V3 L70 = z0, L64 = z0, L43 = z0, L57 = z0;
        V3 U = d43; vadd(U, d57);
        V3 dU = gd(4, 3); vadd(dU, gd(5, 7));
        triple_t(U, d64, d70, v3(tk(84), tk(85), tk(86)), dU, gd(6, 4), gd(7, 0), L43, L57, L64, L70);
        { const V3 n = LN(4); vadd(L43, vcross(n, d70)); vadd(L70, vcross(d43, n)); }
        if (f == 1) { vadd(L64, Lfa); vadd(L57, Lfb); }
        else if (f == 5) { vadd(L43, Lfa); vadd(L70, Lfb); }
        put(L70, 7, 0); put(L64, 6, 4); put(L43, 4, 3); put(L57, 5, 7);
      }
      {  // (d14 + d25).(d61 x d50), faces 1 and 2, characteristic faces 2 and 3
        const V3 d61 = dg(0), d50 = dg(4), d14 = dg(10), d25 = dg(11);
        V3 L61 = z0, L50 = z0, L14 = z0, L25 = z0;
        V3 U = d14; vadd(U, d25);
        V3 dU = gd(1, 4); vadd(dU, gd(2, 5));
        triple_t(U, d61, d50, v3(tk(87), tk(88), tk(89)), dU, gd(6, 1), gd(5, 0), L14, L25, L61, L50);
        { const V3 n = LN(1); vadd(L50, vcross(d14, n)); vadd(L14, vcross(n, d50)); }
        { const V3 n = LN(2); vadd(L61, vcross(d25, n)); vadd(L25, vcross(n, d61)); }
        if (f == 2) { vadd(L50, Lfa); vadd(L14, Lfb); }
        else if (f == 3) { vadd(L61, Lfa); vadd(L25, Lfb); }
        put(L61, 6, 1); put(L50, 5, 0); put(L14, 1, 4); put(L25, 2, 5);
      }
    }
    // the position corners
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
      for (int c = 0; c < 8; ++c) a.cX[(k * 8 + c) * E + e] = LX[k][c];
  }
  block_sum_to(Ldt, a.part_dt);
}

// Sums the force corner buffers into node adjoints (added to what is there):
// the last step of a reverse sweep (each cycle's ka_node gathers the previous
// transposed cycle's force corners itself).
__global__ void __launch_bounds__(kAdjBlock) ka_gather_corners(AdjDev a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.N) return;
  const int s = a.nodeElemStart[i], t = a.nodeElemStart[i + 1];
  const long long E8 = 8ll * a.E;
  double gx = 0, gy = 0, gz = 0, hx = 0, hy = 0, hz = 0;
  for (int j = s; j < t; ++j) {
    const int c = a.cornerList[j];
    gx += a.fX[c]; gy += a.fX[E8 + c]; gz += a.fX[2 * E8 + c];
    hx += a.fV[c]; hy += a.fV[E8 + c]; hz += a.fV[2 * E8 + c];
  }
  a.lx[i] += gx; a.ly[i] += gy; a.lz[i] += gz;
  a.lxd[i] += hx; a.lyd[i] += hy; a.lzd[i] += hz;
}

// ---------------------------------------------------------------------------
// ka_node: transpose of k_node (position and velocity update with the
// velocity snap, acceleration = force / mass with the symmetry BCs).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kAdjBlock) ka_node(AdjDev a, const CycleRec* rec) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const double dt = rec->dt;
  double Ldt = 0.0;
  if (i < a.N) {
    const unsigned bc = a.nodeBC[i];
    const double im = a.inv_nodalMass[i];
    double* Lx[3] = {a.lx, a.ly, a.lz};
    double* Lxd[3] = {a.lxd, a.lyd, a.lzd};
    double* Lf[3] = {a.lfx, a.lfy, a.lfz};
    const double* xd1[3] = {a.xd1, a.yd1, a.zd1};
    const double* acc[3] = {a.ax, a.ay, a.az};
    // the end-state adjoints gather this cycle's kinematics transpose and
    // (added per corner by ka_kinematics) the force transpose of the cycle
    // after this one
    double gx[3] = {0.0, 0.0, 0.0}, gv[3] = {0.0, 0.0, 0.0};
    {
      const int s = a.nodeElemStart[i], t = a.nodeElemStart[i + 1];
      const long long E8 = 8ll * a.E;
      for (int j = s; j < t; ++j) {
        const int c = a.cornerList[j];
#pragma unroll
        for (int k = 0; k < 3; ++k) { gx[k] += a.cX[k * E8 + c]; gv[k] += a.cV[k * E8 + c]; }
      }
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const double lxn = Lx[k][i] + gx[k];
      const double v1 = xd1[k][i];
      double lv = (Lxd[k][i] + gv[k]) + lxn * dt;   // x1 = x0 + xd1*dt
      Ldt += lxn * v1;
      double lf = 0.0;
      if (v1 == 0.0) {
        lv = 0.0;                        // snapped to zero (|v| < u_cut)
      } else {
        const double acc_k = acc[k][i];
        Ldt += lv * acc_k;               // xd1 = xd0 + a*dt
        if (!(bc & (1u << k))) lf = lv * dt * im;
      }
      Lx[k][i] = lxn;
      Lxd[k][i] = lv;
      Lf[k][i] = lf;
    }
  }
  block_sum_to(Ldt, a.part_dtn);
}

// ---------------------------------------------------------------------------
// Transpose of k_force, in two kernels: ka_hourglass (the FB hourglass force
// onto the velocities, ss, v, hgcoef and the two geometric factors) and
// ka_force_geo (the stress force and those geometric factors onto the
// positions).
// ---------------------------------------------------------------------------

// The 8 volume derivatives (times 12) of one coordinate pair, in the forward
// kernel's slot order: dv_x uses (ey, ez), dv_y (ex, ez), dv_z (ey, ex) with
// the sign pattern of each.
template <int MODE>
__device__ __forceinline__ void volu_der(const double ex[12], const double ey[12], const double ez[12],
                                         double dv[3][8]) {
  constexpr int pe[8][6] = {{5, 3, 4, 8, 7, 9}, {3, 0, 2, 9, 6, 11}, {0, 1, 7, 11, 4, 10},
                            {1, 5, 6, 10, 2, 8}, {10, 11, 7, 1, 4, 0}, {11, 9, 2, 0, 6, 3},
                            {9, 8, 4, 3, 7, 5}, {8, 10, 6, 5, 2, 1}};
  constexpr int owner[8] = {0, 3, 2, 1, 4, 5, 6, 7};
#pragma unroll
  for (int n = 0; n < 8; ++n) {
    const int p12 = pe[n][0], p01 = pe[n][1], p04 = pe[n][2], p34 = pe[n][3], p25 = pe[n][4], p35 = pe[n][5];
    const int slot = (MODE & 2) ? owner[n] : n;
    dv[0][slot] = fma(ey[p12], ez[p01], fma(-ey[p01], ez[p12], fma(ey[p04], ez[p34],
                  fma(-ey[p34], ez[p04], fma(-ey[p25], ez[p35], ey[p35] * ez[p25])))));
    dv[1][slot] = fma(-ex[p12], ez[p01], fma(ex[p01], ez[p12], fma(-ex[p04], ez[p34],
                  fma(ex[p34], ez[p04], fma(ex[p25], ez[p35], -(ex[p35] * ez[p25]))))));
    dv[2][slot] = fma(-ey[p12], ex[p01], fma(ey[p01], ex[p12], fma(-ey[p04], ex[p34],
                  fma(ey[p34], ex[p04], fma(ey[p25], ex[p35], -(ey[p35] * ex[p25]))))));
  }
}

// Hourglass transpose. With hg[n][m] = gamma[n][m] - sum_j dv_j[n] hms_j[m]
// (hms = the modes over 12*determ), S_k = hg^T V_k, T_k = hg^T lf_k (lf the
// force adjoints) and coef the hourglass coefficient, the forward force is
// F_k = coef hg S_k and its transpose needs only
//   dL/dV_k   = coef hg T_k,
//   dL/ddv_j  = -coef sum_k (lf_k (S_k . hms_j) + V_k (T_k . hms_j)),
//   dL/dhms_j = -coef sum_k (S_k (lf_k . dv_j) + T_k (V_k . dv_j)),
//   dL/dcoef  = sum_k S_k . T_k,
// where hg^T u = Gamma(u) - sum_j hms_j (dv_j . u): 3x3 dot-product tables
// replace the 8x4 matrices hg and dL/dhg. Three blocks per SM (168
// registers, a few spilled) run faster than two without spills: the
// transpose is partly latency-bound at 48^3.
template <int MODE>
__global__ void __launch_bounds__(kAdjBlock, 3) ka_hourglass(AdjDev a, double hgcoef) {
  const int E = a.E;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  double Lhg_coef = 0.0;
  if (e < E) {
    int nd[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) nd[c] = a.nodelist[c * E + e];
    if (!(hgcoef > 0.0)) {
#pragma unroll
      for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int c = 0; c < 8; ++c) { a.fV[(k * 8 + c) * E + e] = 0.0; a.sLdv[(k * 8 + c) * E + e] = 0.0; }
#pragma unroll
      for (int k = 0; k < 12; ++k) a.sLhm[k * E + e] = 0.0;
    } else {
      const double* Vp[3] = {a.xd0, a.yd0, a.zd0};
      const double* Lf[3] = {a.lfx, a.lfy, a.lfz};
      // the forward kernel's volume derivatives and scaled modes, from the tape
      double hms[3][4], dv[3][8];
#pragma unroll
      for (int j = 0; j < 3; ++j)
#pragma unroll
        for (int c = 0; c < 8; ++c) dv[j][c] = a.geo[(j * 8 + c) * E + e];
#pragma unroll
      for (int j = 0; j < 3; ++j)
#pragma unroll
        for (int m = 0; m < 4; ++m) hms[j][m] = a.geo[(24 + j * 4 + m) * E + e];
      const double determ = a.volo[e] * a.v0[e];
      const double inv_det = 1.0 / determ;
      const double vi12 = inv_det * (1.0 / 12.0);
      const double ss = a.ss0[e], mass = a.elemMass[e];
      const double r = inv_cbrt(determ);
      const double c0 = -hgcoef * 0.01;
      const double coef = ((c0 * ss) * mass) * r;
      // S_k (taped), D[k][j] = V_k . dv_j and T_k, C[k][j] = lf_k . dv_j
      double S[3][4], T[3][4], D[3][3], C[3][3];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        double u[8], w2[4], w1[3];
#pragma unroll
        for (int m = 0; m < 4; ++m) S[k][m] = a.geo[(36 + 4 * k + m) * E + e];
#pragma unroll
        for (int c = 0; c < 8; ++c) u[c] = Vp[k][nd[c]];
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          double s = dv[j][0] * u[0];
#pragma unroll
          for (int c = 1; c < 8; ++c) s = fma(dv[j][c], u[c], s);
          D[k][j] = s;
        }
#pragma unroll
        for (int c = 0; c < 8; ++c) u[c] = Lf[k][nd[c]];
        walsh7(u, w1, w2);
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          double s = dv[j][0] * u[0];
#pragma unroll
          for (int c = 1; c < 8; ++c) s = fma(dv[j][c], u[c], s);
          C[k][j] = s;
        }
#pragma unroll
        for (int m = 0; m < 4; ++m)
          T[k][m] = fma(-hms[2][m], C[k][2], fma(-hms[1][m], C[k][1], fma(-hms[0][m], C[k][0], w2[m])));
      }
      double Lcoef = 0.0;
#pragma unroll
      for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int m = 0; m < 4; ++m) Lcoef = fma(S[k][m], T[k][m], Lcoef);
      // A[k][j] = S_k . hms_j, B[k][j] = T_k . hms_j
      double A[3][3], B[3][3];
#pragma unroll
      for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          A[k][j] = fma(S[k][0], hms[j][0], fma(S[k][1], hms[j][1], fma(S[k][2], hms[j][2], S[k][3] * hms[j][3])));
          B[k][j] = fma(T[k][0], hms[j][0], fma(T[k][1], hms[j][1], fma(T[k][2], hms[j][2], T[k][3] * hms[j][3])));
        }
      // dL/dhms_j = -coef P_j with P_j[m] the dot products below; dL/dhm_j =
      // vi12 dL/dhms_j (hms = vi12 hm); dL/dvi12 = sum_j dL/dhms_j . hms_j / vi12
      double Pvi = 0.0;  // sum_j P_j . hms_j
      {
        const double ncv = -coef * vi12;
#pragma unroll
        for (int j = 0; j < 3; ++j)
#pragma unroll
          for (int m = 0; m < 4; ++m) {
            const double P = fma(S[0][m], C[0][j], fma(S[1][m], C[1][j], fma(S[2][m], C[2][j],
                             fma(T[0][m], D[0][j], fma(T[1][m], D[1][j], T[2][m] * D[2][j])))));
            Pvi = fma(P, hms[j][m], Pvi);
            a.sLhm[(j * 4 + m) * E + e] = ncv * P;
          }
      }
      const double Lvi12 = -coef * Pvi;
      // the coefficient folded into the tables: nA = -coef A, nB = -coef B
      double nA[3][3], nB[3][3];
#pragma unroll
      for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int j = 0; j < 3; ++j) { nA[k][j] = -coef * A[k][j]; nB[k][j] = -coef * B[k][j]; }
      // dL/dV_k = coef (Gamma^T T_k - sum_j dv_j B[k][j]) = Gamma^T (coef T_k) + sum_j dv_j nB[k][j]
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        double cT[4], q[8];
#pragma unroll
        for (int m = 0; m < 4; ++m) cT[m] = coef * T[k][m];
        walsh_modes_t(cT, q);
#pragma unroll
        for (int c = 0; c < 8; ++c)
          a.fV[(k * 8 + c) * E + e] = fma(dv[2][c], nB[k][2], fma(dv[1][c], nB[k][1], fma(dv[0][c], nB[k][0], q[c])));
      }
      // dL/ddv_j = -coef sum_k (lf_k A[k][j] + V_k B[k][j]) = sum_k (lf_k nA[k][j] + V_k nB[k][j])
      {
        double Ldv[3][8];
#pragma unroll
        for (int j = 0; j < 3; ++j)
#pragma unroll
          for (int c = 0; c < 8; ++c) Ldv[j][c] = 0.0;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
#pragma unroll
          for (int c = 0; c < 8; ++c) {
            const double lf = Lf[k][nd[c]], vv = Vp[k][nd[c]];
#pragma unroll
            for (int j = 0; j < 3; ++j) Ldv[j][c] = fma(lf, nA[k][j], fma(vv, nB[k][j], Ldv[j][c]));
          }
        }
#pragma unroll
        for (int j = 0; j < 3; ++j)
#pragma unroll
          for (int c = 0; c < 8; ++c) a.sLdv[(j * 8 + c) * E + e] = Ldv[j][c];
      }
      // coef = c0 ss mass determ^(-1/3), vi12 = 1/(12 determ), determ = volo v
      a.lss[e] += Lcoef * c0 * mass * r;
      Lhg_coef = Lcoef * (-0.01) * ss * mass * r;
      const double Ldeterm = (Lcoef * c0 * ss * mass * (-1.0 / 3.0) * r - Lvi12) * inv_det;
      a.lv[e] += Ldeterm * a.volo[e];
    }
    // stress part of the force, f = s8 * B with s8 = (-p - q)/8. The forward
    // forms B0..B3 from faces 0-4 (node n's three face cross products) and
    // the opposite corners as B6 = -B0, B7 = -B1, B4 = -B2, B5 = -B3 (the face
    // normals of a closed surface sum to zero), so face 5 carries no adjoint:
    // sum_n lf_n . B_n = sum_f N_f . LU_f. The face terms LU go to sLU for
    // the position transpose; p and q get -1/8 sum_f N_f . LU_f here, before
    // the material transpose of the cycle before reads them.
    {
      const double* Lf[3] = {a.lfx, a.lfy, a.lfz};
      // face normals 0..4 (the forward's cross products, from the tape)
      V3 N[5];
#pragma unroll
      for (int f = 0; f < 5; ++f) N[f] = v3(a.geo[(48 + f) * E + e], a.geo[(54 + f) * E + e], a.geo[(60 + f) * E + e]);
      auto lfv = [&](int n) { return v3(Lf[0][nd[n]], Lf[1][nd[n]], Lf[2][nd[n]]); };
      // w_n = lf_n - lf_opposite(n) for the corners 0..3 (opposites 6, 7, 4, 5)
      const V3 lf0 = lfv(0);
      V3 w0 = lf0, w1 = lfv(1), w2 = lfv(2), w3 = lfv(3);
      {
        const V3 o0 = lfv(6), o1 = lfv(7), o2 = lfv(4), o3 = lfv(5);
        w0.x -= o0.x; w0.y -= o0.y; w0.z -= o0.z;
        w1.x -= o1.x; w1.y -= o1.y; w1.z -= o1.z;
        w2.x -= o2.x; w2.y -= o2.y; w2.z -= o2.z;
        w3.x -= o3.x; w3.y -= o3.y; w3.z -= o3.z;
      }
      // corners 0..3 touch faces {0,1,4} {0,1,2} {0,2,3} {0,3,4}
      V3 w01 = w0; vadd(w01, w1);
      V3 w23 = w2; vadd(w23, w3);
      V3 LU[5];
      LU[0] = w01; vadd(LU[0], w23);
      LU[1] = w01;
      LU[2] = w1; vadd(LU[2], w2);
      LU[3] = w23;
      LU[4] = w0; vadd(LU[4], w3);
      if (!(MODE & 1)) {
        // src/domain.jl:1050-1055: node 1 (corner 0) takes face 5's areaY twice
        // and no areaZ; its opposite corner has the plain sum
        LU[4].y += lf0.y;
        LU[4].z -= lf0.z;
      }
      double Ls8 = 0.0;
#pragma unroll
      for (int f = 0; f < 5; ++f) {
        Ls8 += vdot(N[f], LU[f]);
        a.sLU[(f * 3) * E + e] = LU[f].x;
        a.sLU[(f * 3 + 1) * E + e] = LU[f].y;
        a.sLU[(f * 3 + 2) * E + e] = LU[f].z;
      }
      const double Lpq = -0.125 * Ls8;
      a.lp[e] += Lpq;
      a.lq[e] += Lpq;
    }
  }
  block_sum_to(Lhg_coef, a.part_hg);
}

// Position transpose of one element's k_force, added into LX:
//  * the hourglass modes: Gamma^T of dL/dhm;
//  * the volume derivatives: the forward's dv is the gradient of 12*volume
//    (calcElemVolume's three triple products U.(V x W) of face diagonals), so
//    the transpose of G -> sum <G, dv> is the Hessian-vector product of those
//    triple products along G (the faithful slots 1 and 3 swapped back);
//  * the stress force f_n = s8 B_n with B_n the node's face-diagonal cross
//    products, through the face terms LU (see ka_hourglass).
// All three use the 12 face diagonals of the element (force order d20 d31
// d50 d14 d61 d25 d72 d36 d43 d07 d64 d57); the hourglass transpose of the
// same cycle left dL/dhm, dL/ddv and LU in sLhm, sLdv and sLU.
template <int MODE>
__device__ __forceinline__ void force_geo_t(const AdjDev& a, int e, const V3 dgs[12], double s8, double LX[3][8]) {
  const int E = a.E;
  const V3 d20 = dgs[0], d31 = dgs[1], d50 = dgs[2], d14 = dgs[3], d61 = dgs[4], d25 = dgs[5];
  const V3 d72 = dgs[6], d36 = dgs[7], d43 = dgs[8], d07 = dgs[9], d64 = dgs[10], d57 = dgs[11];
  // hourglass modes hm_k = Gamma(X_k)
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    double t[4], q[8];
#pragma unroll
    for (int m = 0; m < 4; ++m) t[m] = a.sLhm[(k * 4 + m) * E + e];
    walsh_modes_t(t, q);
#pragma unroll
    for (int c = 0; c < 8; ++c) LX[k][c] = q[c];
  }
  auto add = [&](int c, const V3& v) { LX[0][c] += v.x; LX[1][c] += v.y; LX[2][c] += v.z; };
  auto sub = [&](int c, const V3& v) { LX[0][c] -= v.x; LX[1][c] -= v.y; LX[2][c] -= v.z; };
  // volume derivatives: Hessian-vector product of the triple products
  {
    double G[3][8];
#pragma unroll
    for (int j = 0; j < 3; ++j)
#pragma unroll
      for (int c = 0; c < 8; ++c) G[j][c] = a.sLdv[(j * 8 + c) * E + e];
    if (!(MODE & 2)) {
      // the faithful forward stores node 3's derivative in slot 1 and node 1's in slot 3
#pragma unroll
      for (int j = 0; j < 3; ++j) { const double t = G[j][1]; G[j][1] = G[j][3]; G[j][3] = t; }
    }
    auto gd = [&](int p, int q) { return v3(G[0][p] - G[0][q], G[1][p] - G[1][q], G[2][p] - G[2][q]); };
    auto hvp = [&](const V3& U, const V3& V, const V3& W, const V3& dU, const V3& dV, const V3& dW,
                   int u0, int u1, int u2, int u3, int v0, int v1, int w0, int w1) {
      V3 gU = vcross(dV, W); vadd(gU, vcross(V, dW));
      V3 gV = vcross(W, dU); vadd(gV, vcross(dW, U));
      V3 gW = vcross(dU, V); vadd(gW, vcross(U, dV));
      add(u0, gU); sub(u1, gU); add(u2, gU); sub(u3, gU);
      add(v0, gV); sub(v1, gV);
      add(w0, gW); sub(w1, gW);
    };
    // 12*volume = (d31 + d72).(d63 x d20) + (d43 + d57).(d64 x d70) + (d14 + d25).(d61 x d50)
    {
      V3 U = d31; vadd(U, d72);
      V3 dU = gd(3, 1); vadd(dU, gd(7, 2));
      const V3 V = v3(-d36.x, -d36.y, -d36.z);
      hvp(U, V, d20, dU, gd(6, 3), gd(2, 0), 3, 1, 7, 2, 6, 3, 2, 0);
    }
    {
      V3 U = d43; vadd(U, d57);
      V3 dU = gd(4, 3); vadd(dU, gd(5, 7));
      const V3 W = v3(-d07.x, -d07.y, -d07.z);
      hvp(U, d64, W, dU, gd(6, 4), gd(7, 0), 4, 3, 5, 7, 6, 4, 7, 0);
    }
    {
      V3 U = d14; vadd(U, d25);
      V3 dU = gd(1, 4); vadd(dU, gd(2, 5));
      hvp(U, d61, d50, dU, gd(6, 1), gd(5, 0), 1, 4, 2, 5, 6, 1, 5, 0);
    }
  }
  // stress part: with N_f = d1 x d2 for (d1, d2) = (p0 - p1, p2 - p3) of the
  // face's corners, sum_n lf_n . f_n = s8 sum_f N_f . LU_f
  {
    V3 LU[5];
#pragma unroll
    for (int f = 0; f < 5; ++f) LU[f] = v3(a.sLU[(f * 3) * E + e], a.sLU[(f * 3 + 1) * E + e], a.sLU[(f * 3 + 2) * E + e]);
    auto face_t = [&](int f, const V3& d1, const V3& d2, int p0, int p1, int p2, int p3) {
      const V3 LN = v3(s8 * LU[f].x, s8 * LU[f].y, s8 * LU[f].z);
      const V3 L1 = vcross(d2, LN), L2 = vcross(LN, d1);
      add(p0, L1); sub(p1, L1); add(p2, L2); sub(p3, L2);
    };
    face_t(0, d20, d31, 2, 0, 3, 1);
    face_t(1, d50, d14, 5, 0, 1, 4);
    face_t(2, d61, d25, 6, 1, 2, 5);
    face_t(3, d72, d36, 7, 2, 3, 6);
    face_t(4, d43, d07, 4, 3, 0, 7);
  }
}

// The position transpose of the first cycle's k_force (the other cycles'
// is part of ka_kinematics of the cycle before), from the face diagonals
// taped at the segment's start (diag0), into the force corner buffer that
// ka_gather_corners sums.
template <int MODE>
__global__ void __launch_bounds__(kAdjBlock, 3) ka_force_geo(AdjDev a) {
  const int E = a.E;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= E) return;
  V3 dgs[12];
#pragma unroll
  for (int q = 0; q < 12; ++q) dgs[q] = v3(a.diag0[(3 * q) * E + e], a.diag0[(3 * q + 1) * E + e], a.diag0[(3 * q + 2) * E + e]);
  const double s8 = ((-a.p0[e]) - a.q0[e]) * 0.125;
  double LX[3][8];
  force_geo_t<MODE>(a, e, dgs, s8, LX);
#pragma unroll
  for (int k = 0; k < 3; ++k)
#pragma unroll
    for (int c = 0; c < 8; ++c) a.fX[(k * 8 + c) * E + e] = LX[k][c];
}

// Sum of `n` partials in a fixed order by one block of BS threads; every
// thread gets it.
template <int BS>
__device__ double block_fixed_sum(const double* part, int n) {
  __shared__ double sh[BS];
  double s = 0.0;
  for (int j = threadIdx.x; j < n; j += BS) s += part[j];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = BS / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  const double r = sh[0];
  __syncthreads();
  return r;
}

// Sums `n` partials in a fixed order (one block).
__global__ void __launch_bounds__(kAdjBlock) ka_sum(const double* part, int n, double* out) {
  const double s = block_fixed_sum<kAdjBlock>(part, n);
  if (threadIdx.x == 0) *out = s;
}

// Transpose of timeIncrement! (src/domain.jl:920-961) for the recorded
// inputs: Ldt is the adjoint of the new deltatime; adds to the adjoints of
// the previous time, deltatime, dtcourant and dthydro along the branch taken.
__host__ __device__ inline void time_increment_reverse(const CycleRec& r, const Params& prm, double Ldt,
                                                       double& Ltime, double& Ldt_prev, double& Ldtc,
                                                       double& Ldth) {
  double targetdt = prm.stoptime - r.time_prev;
  double dt_pre = r.dt_prev;
  int which = 0, rb = 0;
  bool mb = false;
  const bool adaptive = prm.dtfixed <= 0.0 && r.cycle_prev != 0;
  if (adaptive) {
    const double olddt = r.dt_prev;
    double gnewdt = (double)INFINITY;
    if (r.dtc_in < gnewdt) { gnewdt = r.dtc_in / 2.0; which = 1; }
    if (r.dth_in < gnewdt) { gnewdt = r.dth_in * 2.0 / 3.0; which = 2; }
    double newdt = gnewdt;
    const double ratio = newdt / olddt;
    if (ratio >= 1.0) {
      if (ratio < prm.deltatimemultlb) { newdt = olddt; rb = 1; }
      else if (ratio > prm.deltatimemultub) { newdt = olddt * prm.deltatimemultub; rb = 2; }
    }
    if (!(newdt != newdt) && (prm.dtmax != prm.dtmax || prm.dtmax < newdt)) { newdt = prm.dtmax; mb = true; }
    dt_pre = newdt;
  }
  bool t1 = false;
  if (dt_pre < targetdt && targetdt < 4.0 * dt_pre / 3.0) { targetdt = 2.0 * dt_pre / 3.0; t1 = true; }
  const bool t2 = targetdt < dt_pre;
  double Lpre = 0.0;
  if (t2) {
    if (t1) Lpre += (2.0 / 3.0) * Ldt;
    else Ltime += -Ldt;  // dt = stoptime - time
  } else {
    Lpre += Ldt;
  }
  if (!adaptive) { Ldt_prev += Lpre; return; }
  if (mb) return;
  if (rb == 1) { Ldt_prev += Lpre; return; }
  if (rb == 2) { Ldt_prev += prm.deltatimemultub * Lpre; return; }
  if (which == 1) Ldtc += 0.5 * Lpre;
  else if (which == 2) Ldth += (2.0 / 3.0) * Lpre;
}

// Closes the transpose of one cycle (one block): sums the kernels' partial
// adjoints of dt and hgcoef in a fixed order (each thread its strided share
// of all three, a warp tree, then the warps in order), then transposes
// time += dt and timeIncrement! on the carried scalar adjoints.
constexpr int kCloseBlock = 256;
__global__ void __launch_bounds__(kCloseBlock) ka_cycle_close(AdjDev a, int ge, int gn, const CycleRec* rec,
                                                               AdjScal* sc, Params prm) {
  double t_kin = 0.0, t_node = 0.0, t_hg = 0.0;
  for (int j = threadIdx.x; j < ge; j += kCloseBlock) { t_kin += a.part_dt[j]; t_hg += a.part_hg[j]; }
  for (int j = threadIdx.x; j < gn; j += kCloseBlock) t_node += a.part_dtn[j];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    t_kin += __shfl_down_sync(0xffffffffu, t_kin, o);
    t_node += __shfl_down_sync(0xffffffffu, t_node, o);
    t_hg += __shfl_down_sync(0xffffffffu, t_hg, o);
  }
  __shared__ double wsum[3][kCloseBlock / 32];
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) { wsum[0][w] = t_kin; wsum[1][w] = t_node; wsum[2][w] = t_hg; }
  __syncthreads();
  if (threadIdx.x != 0) return;
  double s_kin = wsum[0][0], s_node = wsum[1][0], s_hg = wsum[2][0];
#pragma unroll
  for (int k = 1; k < kCloseBlock / 32; ++k) { s_kin += wsum[0][k]; s_node += wsum[1][k]; s_hg += wsum[2][k]; }
  const CycleRec r = *rec;
  AdjScal v = *sc;
  v.Lhg += s_hg;
  // a minimum the cycle did not reach leaves the scalar as it was
  double Ldtc_prev = r.active_c ? 0.0 : v.Ldtc, Ldth_prev = r.active_h ? 0.0 : v.Ldth;
  // time_n = time_{n-1} + dt_n
  const double Ldt_tot = v.Ldt + (s_kin + s_node) + v.Ltime;
  double Ldt_prev = 0.0;
  time_increment_reverse(r, prm, Ldt_tot, v.Ltime, Ldt_prev, Ldtc_prev, Ldth_prev);
  v.Ldt = Ldt_prev;
  v.Ldtc = Ldtc_prev;
  v.Ldth = Ldth_prev;
  *sc = v;
}

// Copies the 11 state fields (node fields n < N, element fields n < E).
// A field whose destination is null is not copied (a tape set's per-cycle
// states keep only the fields the transposes read).
__device__ __forceinline__ void copy_state_at(int i, const StateSet& src, const StateSet& dst, int E, int N) {
  if (i < N) {
#pragma unroll
    for (int k = 0; k < 6; ++k)
      if (dst.f[k]) dst.f[k][i] = src.f[k][i];
  }
  if (i < E) {
#pragma unroll
    for (int k = 6; k < 11; ++k)
      if (dst.f[k]) dst.f[k][i] = src.f[k][i];
  }
}

__global__ void __launch_bounds__(kAdjBlock) ka_copy_state(StateSet src, StateSet dst, int E, int N) {
  copy_state_at(blockIdx.x * blockDim.x + threadIdx.x, src, dst, E, N);
}

// Start of a taped cycle: every thread copies the cycle's start state to its
// slot; thread 0 folds the previous cycle's minima, records timeIncrement!'s
// inputs, advances time and records the new dt. A run that has reached
// stoptime (the examples/benchmark.jl loop condition) or an earlier error
// makes the cycle a no-op (done / status, which the step kernels check).
__global__ void __launch_bounds__(kAdjBlock) ka_tape_begin(StateSet src, StateSet dst, int E, int N, DevState* st,
                                                            CycleRec* rec, Params prm) {
  copy_state_at(blockIdx.x * blockDim.x + threadIdx.x, src, dst, E, N);
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (st->status != 0u || st->done) return;
  if (dt_registers(st->acc_courant)) st->dtcourant = __longlong_as_double((long long)st->acc_courant);
  if (dt_registers(st->acc_hydro)) st->dthydro = __longlong_as_double((long long)st->acc_hydro);
  st->acc_courant = kInfBits;
  st->acc_hydro = kInfBits;
  if (!(st->time < prm.stoptime)) { st->done = 1; return; }
  CycleRec r;
  r.time_prev = st->time;
  r.dt_prev = st->deltatime;
  r.dtc_in = st->dtcourant;
  r.dth_in = st->dthydro;
  r.cycle_prev = st->cycle;
  double time = st->time, dt = st->deltatime;
  long long cycle = st->cycle;
  time_increment(time, dt, cycle, st->dtcourant, st->dthydro, prm);
  st->time = time;
  st->deltatime = dt;
  st->cycle = cycle;
  r.dt = dt;
  r.active_c = r.active_h = 0;
  r.argmin_c = r.argmin_h = INT_MAX;
  *rec = r;
}

// End of a taped cycle: which minima the cycle reached, and the smallest
// element index attaining each (the element the reference's strict-less-than
// scan keeps, src/domain.jl:3003-3008 and :3041-3046).
__global__ void __launch_bounds__(kAdjBlock) ka_tape_close(const double* dtc, const double* dth, int E,
                                                            const DevState* st, CycleRec* rec) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned long long bc = st->acc_courant, bh = st->acc_hydro;
  if (i == 0) {
    rec->active_c = dt_registers(bc);
    rec->active_h = dt_registers(bh);
  }
  if (i >= E) return;
  if (dt_registers(bc) && (unsigned long long)__double_as_longlong(dtc[i]) == bc) atomicMin(&rec->argmin_c, i);
  if (dt_registers(bh) && (unsigned long long)__double_as_longlong(dth[i]) == bh) atomicMin(&rec->argmin_h, i);
}

// Loss seed and value: L = sum_e w_e e + sum_n 0.5 w_n |u|^2 with
// w_e = mask*elemMass, w_n = mask*nodalMass (masks from the reference mesh).
__global__ void __launch_bounds__(kAdjBlock) ka_loss_elem(const double* we, const double* e, int E, double* le,
                                                           double* part) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double s = 0.0;
  if (i < E) {
    s = we[i] * e[i];
    if (le) le[i] = we[i];
  }
  block_sum_to(s, part);
}

__global__ void __launch_bounds__(kAdjBlock) ka_loss_node(const double* wn, const double* xd, const double* yd,
                                                           const double* zd, int N, double* lxd, double* lyd,
                                                           double* lzd, double* part) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double s = 0.0;
  if (i < N) {
    const double w = wn[i], u = xd[i], v = yd[i], z = zd[i];
    s = 0.5 * w * fma(u, u, fma(v, v, z * z));
    if (lxd) { lxd[i] = w * u; lyd[i] = w * v; lzd[i] = w * z; }
  }
  block_sum_to(s, part);
}

}  // namespace lulesh
