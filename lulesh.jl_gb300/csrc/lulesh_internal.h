// Internal structures of the GB300 LagrangeLeapFrog library.
#pragma once

#include <cstdint>
#include <cstring>
#include <cuda_runtime.h>

namespace lulesh {

// Boundary-condition masks, src/bc.jl:3-30.
enum : uint32_t {
  XI_M = 0x00007, XI_M_SYMM = 0x00001, XI_M_FREE = 0x00002, XI_M_COMM = 0x00004,
  XI_P = 0x00038, XI_P_SYMM = 0x00008, XI_P_FREE = 0x00010, XI_P_COMM = 0x00020,
  ETA_M = 0x001c0, ETA_M_SYMM = 0x00040, ETA_M_FREE = 0x00080, ETA_M_COMM = 0x00100,
  ETA_P = 0x00e00, ETA_P_SYMM = 0x00200, ETA_P_FREE = 0x00400, ETA_P_COMM = 0x00800,
  ZETA_M = 0x07000, ZETA_M_SYMM = 0x01000, ZETA_M_FREE = 0x02000, ZETA_M_COMM = 0x04000,
  ZETA_P = 0x38000, ZETA_P_SYMM = 0x08000, ZETA_P_FREE = 0x10000, ZETA_P_COMM = 0x20000,
};

// Status bits OR-ed by the kernels into DevState::status; the host maps the
// first set bit (reference order) to a lulesh_status / lulesh_site.
enum : uint32_t {
  ST_EARLY = 1u << 0,       // detJ <= 0, src/domain.jl:1104
  ST_HOURGLASS = 1u << 1,   // v <= 0, src/domain.jl:1727
  ST_KINEMATICS = 1u << 2,  // vnew <= 0, src/domain.jl:2118
  ST_BAD_BC = 1u << 3,      // invalid elemBC, src/domain.jl:2343
  ST_QSTOP = 1u << 4,       // q > qstop, src/domain.jl:2567-2580
  ST_MATERIAL = 1u << 5,    // clamped v <= 0, src/domain.jl:2905
  ST_UPDATE = 1u << 6,      // new v <= 0, src/domain.jl:2926
  ST_INDEX = 1u << 7,       // checked build (LULESH_CHECK): an index outside its range
};

// Which value a monotonic-Q limiter returned (src/domain.jl:2357-2376).
enum : int { PHI_MEAN = 0, PHI_M = 1, PHI_P = 2, PHI_ZERO = 3, PHI_MAX = 4 };

// Branch record of one element's step, written by the taping forward kernels
// and read by the adjoint so it differentiates exactly the branches taken.
enum : unsigned long long {
  TF_PHI_SHIFT = 0,            // 3 bits per direction (xi, eta, zeta): PHI_*
  TF_QZERO = 1ull << 9,        // vdov > 0: ql = qq = 0
  TF_DXCLAMP0 = 1ull << 10,    // delv_d * delx_d > 0 clamped to 0 (d = 0, 1, 2: bits 10-12)
  TF_VNEW_MIN = 1ull << 13,    // vnewc clamped to eosvmin
  TF_VNEW_MAX = 1ull << 14,    // vnewc clamped to eosvmax
  TF_HALF_EQ_COMP = 1ull << 15,  // compHalfStep = compression (vnewc <= eosvmin)
  TF_VMAX_HIT = 1ull << 16,    // vnewc >= eosvmax: pressures 0, p_old/compressions 0
  TF_E1_MIN = 1ull << 17,      // first energy clamped to emin
  TF_PH_CUT = 1ull << 18,      // half-step pressure: |p| < p_cut -> 0
  TF_PH_MIN = 1ull << 19,      // half-step pressure clamped to pmin
  TF_COMPRESS = 1ull << 20,    // delvc <= 0: q terms active
  TF_S1_TINY = 1ull << 21,     // half-step sound speed took the TINY branch
  TF_E2_CUT = 1ull << 22, TF_E2_MIN = 1ull << 23,
  TF_PN1_CUT = 1ull << 24, TF_PN1_MIN = 1ull << 25,
  TF_S2_TINY = 1ull << 26,
  TF_E3_CUT = 1ull << 27, TF_E3_MIN = 1ull << 28,
  TF_PN2_CUT = 1ull << 29, TF_PN2_MIN = 1ull << 30,
  TF_SS_TINY = 1ull << 31,
  TF_Q_CUT = 1ull << 32,       // final q: |q| < q_cut -> 0
  TF_V_SNAP = 1ull << 33,      // |vnew - 1| < v_cut: v = 1
  TF_FACE_SHIFT = 40,          // 3 bits: face whose area set the characteristic length
};

// Per-problem parameters passed by value to every kernel.
struct Params {
  double u_cut, hgcoef, qstop, monoq_max_slope, monoq_limiter_mult, e_cut, p_cut, q_cut, v_cut;
  double qlc_monoq, qqc_monoq, qqc, eosvmax, eosvmin, pmin, emin, dvovmax, refdens;
  double dtfixed, deltatimemultlb, deltatimemultub, stoptime, dtmax;
  // formed once on the host by finish_params: 1 / refdens, 64 qqc^2, the comparison
  // keys (fkey) of the thresholds the element kernels test against, and
  // whether eosvmin / eosvmax are set (nonzero)
  double inv_refdens, qqc2x64;
  long long k_qstop, k_max_slope, k_eosvmin, k_eosvmax, k_pmin, k_emin;
  int has_eosvmin, has_eosvmax;
};

// Order-preserving integer key of a non-NaN double given its bit pattern:
// a < b exactly when fkey(a) < fkey(b), and -0 and +0 share the key 0, as
// IEEE comparison has them. Negative values map to minus their magnitude.
__host__ __device__ inline long long fkey_bits(long long b) {
  return b < 0 ? (long long)(0x8000000000000000ull - (unsigned long long)b) : b;
}

inline long long fkey_host(double x) {
  long long b;
  memcpy(&b, &x, sizeof b);
  return fkey_bits(b);
}

inline void finish_params(Params& p) {
  p.inv_refdens = 1.0 / p.refdens;
  p.qqc2x64 = (64.0 * p.qqc) * p.qqc;
  p.k_qstop = fkey_host(p.qstop);
  p.k_max_slope = fkey_host(p.monoq_max_slope);
  p.k_eosvmin = fkey_host(p.eosvmin);
  p.k_eosvmax = fkey_host(p.eosvmax);
  p.k_pmin = fkey_host(p.pmin);
  p.k_emin = fkey_host(p.emin);
  p.has_eosvmin = p.eosvmin != 0.0;
  p.has_eosvmax = p.eosvmax != 0.0;
}

// Device-resident step state. acc_* are running minima (bit patterns of
// non-negative doubles, so an unsigned min is the FP min) filled by the
// material kernel and folded into dtcourant/dthydro by timeIncrement.
struct DevState {
  double time, deltatime, dtcourant, dthydro;
  long long cycle;
  unsigned long long acc_courant, acc_hydro;
  unsigned int status;
  int done;             // device run loop: 1 once stoptime/num_iters/error is reached
  long long num_iters;   // device run loop: stop once cycle >= num_iters (after the first)
  long long first;       // device run loop: 1 before the first cycle of a run call
};

constexpr unsigned long long kInfBits = 0x7FF0000000000000ull;

// The Courant and hydro scans start at 1.0e+20 and keep a candidate only if it
// is strictly below (src/domain.jl:2966, 3003-3014, 3022, 3041-3052): a cycle
// registers a new dtcourant/dthydro only when its minimum lies below 1e20.
// kDtRegisterBits is the bit pattern of 1.0e+20; for non-negative doubles
// (and NaNs, whose patterns lie above +inf) the unsigned order is the FP order.
constexpr unsigned long long kDtRegisterBits = 0x4415AF1D78B58C40ull;
__host__ __device__ inline bool dt_registers(unsigned long long acc) { return acc < kDtRegisterBits; }

// doubles per element of DevDomain::nextGeo
constexpr int kGeoSlots = 51;

// Pointers of one problem's device fields. Element arrays have E entries,
// node arrays N; corner arrays 8E in corner-major order (c*E + e).
// A block-partitioned mesh adds ghost slots: the delv arrays hold Eg >= E
// entries, the corner-force arrays nCornerSlot >= 8E and the corner list
// nCornerList >= 8E; haloDelvSrc / haloCornerSrc give the element or
// corner-force slot each ghost slot copies before the kernel that reads it.
struct DevDomain {
  int E, N, nx;
  int mode;
  int Eg, nCornerSlot, nCornerList;
  const int* haloDelvSrc;    // Eg - E entries (null without ghosts)
  const int* haloCornerSrc;  // nCornerSlot - 8E entries (null without ghosts)
  // nodes
  double *x, *y, *z, *xd, *yd, *zd;
  double *nodalMass, *inv_nodalMass;
  double *xdd, *ydd, *zdd, *fx, *fy, *fz;     // kept only with keep_aux
  unsigned char* nodeBC;                      // bit0 symmX, bit1 symmY, bit2 symmZ
  int *nodeElemStart;                         // N+1
  int *cornerList;                            // 8E, values c*E + e
  // elements
  int* nodelist;                              // [8][E]
  double *e, *p, *q, *v, *volo, *inv_volo, *elemMass, *ss;
  double *ql, *qq, *vnew, *delv, *arealg, *vdov;
  double *delv_xi, *delv_eta, *delv_zeta, *delx_xi, *delx_eta, *delx_zeta;
  double *dxx, *dyy, *dzz;                    // kept only with keep_aux
  unsigned int* elemBC;
  int *lxim, *lxip, *letam, *letap, *lzetam, *lzetap;
  // region batching (cost model only)
  int* regElemlist0;                          // E, 0-based element ids grouped by region
  int* regOfSlot;                             // E, region rep count per slot
  // the force kernel's geometry of the current positions, [kGeoSlots][E]
  // (formed by the kinematics kernel of the cycle before, or by k_geometry)
  double* nextGeo;
  // taped runs: the next cycle's force tape, where the kinematics kernel (or
  // k_geometry) writes the face normals of these positions, and at the start
  // of a taped segment the buffer k_geometry writes their face diagonals to
  double* tapeGeoNext;
  double* tapeDiag;
  // corner forces [8][E]
  double *fcx, *fcy, *fcz;
  // step state: one entry, or one per instance of an ensemble
  DevState* st;
  // ensemble only: instance of every element and node, per-instance hgcoef
  const int* elemInst;
  const int* nodeInst;
  const double* instHg;
  int ninst;
  // region cost model (null unless region_reps): elements in region order and
  // the EOS evaluation count of each position's region
  const int* regOrder;
  const int* posReps;
  // adjoint taping (null unless recording): branch flags and each element's
  // Courant and hydro dt candidates (+inf where vdov == 0)
  unsigned long long* tapeFlags;
  double* tapeDtc;
  double* tapeDth;
  // [66][E]: the force kernel's volume derivatives dv_j[n] (24, node
  // order), hourglass modes over 12*determ (12), mode sums S_k[m] of the
  // velocities (12) and face-diagonal cross products (x, y, z of the 6
  // faces: 18; faces 0..4 written)
  double* tapeGeo;
  // [90][E]: the kinematics kernel's Walsh vectors of positions (9) and
  // velocities (9), cofactor columns (9), 1/det (1), monotonic-Q cross
  // products (9) with their reciprocal norms (3), 1/(64 vol) (1), the largest
  // face's diagonal cross product (3) and rsqrt of its square norm (1), the
  // 12 diagonals d61 d70 d63 d20 d50 d64 d31 d72 d43 d57 d14 d25 of the new
  // positions (36) and the V x W factors of the three volume triple products (9)
  double* tapeKin;
  // [31][E]: the material kernel's limiter terms (norm, scaled neighbours:
  // 9), Q terms (rho, qlin, qquad, and their two sums: 5) and EOS values
  // (1 + compression, 1 + compHalfStep, e1, pHalf, vhalf, s1, q1, e2, p1, s2,
  // q2, e3, p2, ss: 14; the three squared sound speeds: 3)
  double* tapeMat;
};

}  // namespace lulesh
