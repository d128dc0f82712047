// Reverse-mode adjoint of the LagrangeLeapFrog run (C ABI: lulesh_adj_*).
//
// gradient(num_cycles):
//   1. forward sweep from the handle's current state, saving the state and
//      the Domain scalars every `checkpoint_every` cycles;
//   2. the objective at the final state (energy within a radius of the
//      origin, or caller-given linear weights) seeds the adjoint state;
//   3. reverse sweep, segment by segment: restore the segment's checkpoint,
//      recompute its cycles with the taping kernels (start states, the
//      kinematics outputs, accelerations, branch flags, dt candidates), then
//      transpose the cycles in reverse with the ka_* kernels. The dt control
//      (timeIncrement!, the Courant and hydro minima) is transposed on the
//      host from the recorded scalars: the minima pass their adjoint to the
//      element that attained them.
// The handle is left at its final state. Every derivative is that of the
// branches the forward run took.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <new>
#include <vector>

#include "../../include/lulesh_gb300.h"
#include "lulesh_adjoint_kernels.cuh"
#include "lulesh_device.cuh"
#include "lulesh_handle.h"

using namespace lulesh;

namespace {

int acuda(cudaError_t e) {
  if (e == cudaSuccess) return LULESH_OK;
  std::fprintf(stderr, "liblulesh_gb300 (adjoint): CUDA error %s\n", cudaGetErrorString(e));
  return LULESH_ERR_CUDA;
}
#define ACK(call) do { int rc_ = acuda(call); if (rc_) return rc_; } while (0)

constexpr int kStateFields = 11;  // x y z xd yd zd (node), e p q v ss (element)
const int32_t kStateIds[kStateFields] = {LULESH_F_X, LULESH_F_Y, LULESH_F_Z, LULESH_F_XD, LULESH_F_YD,
                                         LULESH_F_ZD, LULESH_F_E, LULESH_F_P, LULESH_F_Q, LULESH_F_V,
                                         LULESH_F_SS};

struct StateBuf {
  double* f[kStateFields];
};

struct CycleTape {
  double *ax, *ay, *az;
  double *vnew, *delv, *arealg, *vdov, *dv[3], *dx[3];
  unsigned long long* flags;
  double *dtc, *dth;
};

struct ScalarRec {
  double time_prev, dt_prev, dtc_in, dth_in;
  long long cycle_prev;
  double dt, time;
  bool active_c, active_h;
  int argmin_c, argmin_h;
};

struct Scalars5 {
  double time, dt, dtc, dth;
  long long cycle;
};

double** state_ptr(DevDomain& d, int k) {
  double** p[kStateFields] = {&d.x, &d.y, &d.z, &d.xd, &d.yd, &d.zd, &d.e, &d.p, &d.q, &d.v, &d.ss};
  return p[k];
}

}  // namespace

struct lulesh_adjoint {
  lulesh_domain* dom = nullptr;
  double radius = 0.3;
  int K = 20;
  int E = 0, N = 0;
  std::vector<void*> allocs;
  std::vector<StateBuf> slots;   // K+1 states of the current segment
  std::vector<CycleTape> tape;   // K cycles
  std::vector<StateBuf> ckpts;   // segment start states
  std::vector<Scalars5> ckpt_scalars;
  StateBuf final_state{};
  double *we = nullptr, *wn = nullptr;  // objective weights
  int *nbStart = nullptr, *nbList = nullptr;
  double *fx_s = nullptr, *fy_s = nullptr, *fz_s = nullptr;  // force scratch of taped cycles
  AdjDev ad{};
  double* scal = nullptr;  // device: sums of partials
  int* argmin = nullptr;
  std::map<int32_t, double*> seeds;  // linear-objective weights per state field
  std::vector<ScalarRec> rec;
};

static int dmalloc(lulesh_adjoint* a, void** p, size_t bytes) {
  if (cudaMalloc(p, bytes ? bytes : 8) != cudaSuccess) { cudaGetLastError(); return LULESH_ERR_MEMORY; }
  a->allocs.push_back(*p);
  return LULESH_OK;
}
template <class T>
static int dalloc(lulesh_adjoint* a, T** p, size_t n) {
  return dmalloc(a, reinterpret_cast<void**>(p), n * sizeof(T));
}

static int alloc_state(lulesh_adjoint* a, StateBuf& s) {
  for (int k = 0; k < kStateFields; ++k) {
    int rc = dalloc(a, &s.f[k], k < 6 ? a->N : a->E);
    if (rc) return rc;
  }
  return LULESH_OK;
}

static int copy_state_from_domain(lulesh_adjoint* a, StateBuf& s) {
  for (int k = 0; k < kStateFields; ++k)
    ACK(cudaMemcpyAsync(s.f[k], *state_ptr(a->dom->dd, k), (k < 6 ? a->N : a->E) * sizeof(double),
                        cudaMemcpyDeviceToDevice, a->dom->stream));
  return LULESH_OK;
}

static int copy_state_to_domain(lulesh_adjoint* a, const StateBuf& s) {
  for (int k = 0; k < kStateFields; ++k)
    ACK(cudaMemcpyAsync(*state_ptr(a->dom->dd, k), s.f[k], (k < 6 ? a->N : a->E) * sizeof(double),
                        cudaMemcpyDeviceToDevice, a->dom->stream));
  return LULESH_OK;
}

static Scalars5 get_scalars(const lulesh_domain* d) {
  return Scalars5{d->sc[LULESH_S_TIME], d->sc[LULESH_S_DELTATIME], d->sc[LULESH_S_DTCOURANT],
                  d->sc[LULESH_S_DTHYDRO], (long long)d->sc[LULESH_S_CYCLE]};
}
static void set_scalars(lulesh_domain* d, const Scalars5& s) {
  d->sc[LULESH_S_TIME] = s.time;
  d->sc[LULESH_S_DELTATIME] = s.dt;
  d->sc[LULESH_S_DTCOURANT] = s.dtc;
  d->sc[LULESH_S_DTHYDRO] = s.dth;
  d->sc[LULESH_S_CYCLE] = (double)s.cycle;
}

// One cycle driven from the host (timeIncrement! on the host, the step on the
// device) exactly as lulesh_time_increment + lulesh_lagrange_leapfrog; with a
// tape, the kinematics outputs, accelerations, flags and dt candidates of the
// cycle go to it and the arg-min elements are found.
static int forward_cycle(lulesh_adjoint* a, const CycleTape* tp, ScalarRec* r) {
  lulesh_domain* d = a->dom;
  const Params prm = make_params(d);
  cudaStream_t s = d->stream;
  ScalarRec rec{};
  rec.time_prev = d->sc[LULESH_S_TIME];
  rec.dt_prev = d->sc[LULESH_S_DELTATIME];
  rec.dtc_in = d->sc[LULESH_S_DTCOURANT];
  rec.dth_in = d->sc[LULESH_S_DTHYDRO];
  rec.cycle_prev = (long long)d->sc[LULESH_S_CYCLE];
  {
    double time = rec.time_prev, dt = rec.dt_prev;
    long long cycle = rec.cycle_prev;
    time_increment(time, dt, cycle, rec.dtc_in, rec.dth_in, prm);
    d->sc[LULESH_S_TIME] = time;
    d->sc[LULESH_S_DELTATIME] = dt;
    d->sc[LULESH_S_CYCLE] = (double)cycle;
    rec.dt = dt;
    rec.time = time;
  }
  state_to_device_mirror(d);
  ACK(cudaMemcpyAsync(d->dd.st, d->hst, sizeof(DevState), cudaMemcpyHostToDevice, s));
  DevDomain td = d->dd;
  bool aux = d->params.keep_aux != 0;
  if (tp) {
    td.vnew = tp->vnew; td.delv = tp->delv; td.arealg = tp->arealg; td.vdov = tp->vdov;
    td.delv_xi = tp->dv[0]; td.delv_eta = tp->dv[1]; td.delv_zeta = tp->dv[2];
    td.delx_xi = tp->dx[0]; td.delx_eta = tp->dx[1]; td.delx_zeta = tp->dx[2];
    td.xdd = tp->ax; td.ydd = tp->ay; td.zdd = tp->az;
    td.fx = a->fx_s; td.fy = a->fy_s; td.fz = a->fz_s;
    td.tapeFlags = tp->flags; td.tapeDtc = tp->dtc; td.tapeDth = tp->dth;
    aux = true;  // the node kernel stores the accelerations
  }
  launch_force(td, prm, d->tuning, s);
  launch_node(td, prm, aux, d->tuning, s);
  launch_kinematics(td, prm, false, d->tuning, s);
  launch_material(td, prm, false, d->tuning, s);
  ACK(cudaGetLastError());
  ACK(cudaMemcpyAsync(d->hst, d->dd.st, sizeof(DevState), cudaMemcpyDeviceToHost, s));
  ACK(cudaStreamSynchronize(s));
  const unsigned long long accc = d->hst->acc_courant, acch = d->hst->acc_hydro;
  state_from_device_mirror(d);
  if (d->status) return d->status;
  rec.active_c = accc != kInfBits;
  rec.active_h = acch != kInfBits;
  rec.argmin_c = rec.argmin_h = -1;
  if (tp) {
    const int grid = (a->E + kAdjBlock - 1) / kAdjBlock;
    int init[2] = {INT_MAX, INT_MAX};
    ACK(cudaMemcpyAsync(a->argmin, init, sizeof(init), cudaMemcpyHostToDevice, s));
    if (rec.active_c) ka_argmin<<<grid, kAdjBlock, 0, s>>>(tp->dtc, a->E, accc, a->argmin);
    if (rec.active_h) ka_argmin<<<grid, kAdjBlock, 0, s>>>(tp->dth, a->E, acch, a->argmin + 1);
    int got[2];
    ACK(cudaMemcpyAsync(got, a->argmin, sizeof(got), cudaMemcpyDeviceToHost, s));
    ACK(cudaStreamSynchronize(s));
    rec.argmin_c = rec.active_c ? got[0] : -1;
    rec.argmin_h = rec.active_h ? got[1] : -1;
  }
  if (r) *r = rec;
  return LULESH_OK;
}

// Transpose of timeIncrement! (src/domain.jl:920-961) for the recorded
// inputs: Ldt is the adjoint of the new deltatime; adds to the adjoints of
// the previous time, deltatime, dtcourant and dthydro along the branch taken.
static void time_increment_reverse(const ScalarRec& r, const Params& prm, double Ldt, double& Ltime,
                                   double& Ldt_prev, double& Ldtc, double& Ldth) {
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
    if (!(newdt != newdt) && prm.dtmax < newdt) { newdt = prm.dtmax; mb = true; }
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

static void set_cycle_pointers(lulesh_adjoint* a, const StateBuf& s0, const StateBuf& s1, const CycleTape& t) {
  AdjDev& ad = a->ad;
  ad.x0 = s0.f[0]; ad.y0 = s0.f[1]; ad.z0 = s0.f[2]; ad.xd0 = s0.f[3]; ad.yd0 = s0.f[4]; ad.zd0 = s0.f[5];
  ad.e0 = s0.f[6]; ad.p0 = s0.f[7]; ad.q0 = s0.f[8]; ad.v0 = s0.f[9]; ad.ss0 = s0.f[10];
  ad.x1 = s1.f[0]; ad.y1 = s1.f[1]; ad.z1 = s1.f[2]; ad.xd1 = s1.f[3]; ad.yd1 = s1.f[4]; ad.zd1 = s1.f[5];
  ad.ax = t.ax; ad.ay = t.ay; ad.az = t.az;
  ad.vnew = t.vnew; ad.delv = t.delv; ad.arealg = t.arealg; ad.vdov = t.vdov;
  for (int k = 0; k < 3; ++k) { ad.dvl[k] = t.dv[k]; ad.dxl[k] = t.dx[k]; }
  ad.flags = t.flags;
}

// Transpose of one recorded cycle: the adjoint state goes from the cycle's
// end to its start; returns the kernels' adjoint of dt and of hgcoef.
static int reverse_cycle(lulesh_adjoint* a, const ScalarRec& r, int argmin_c, double lam_c, int argmin_h,
                         double lam_h, double* Ldt_k, double* Lhg_k) {
  lulesh_domain* d = a->dom;
  cudaStream_t s = d->stream;
  const Params prm = make_params(d);
  const int ge = (a->E + kAdjBlock - 1) / kAdjBlock, gn = (a->N + kAdjBlock - 1) / kAdjBlock;
  const int mode = d->dd.mode;
  if (mode & 4) ka_material<4><<<ge, kAdjBlock, 0, s>>>(a->ad, prm, argmin_c, lam_c, argmin_h, lam_h);
  else ka_material<0><<<ge, kAdjBlock, 0, s>>>(a->ad, prm, argmin_c, lam_c, argmin_h, lam_h);
  ka_nb_gather<<<ge, kAdjBlock, 0, s>>>(a->ad);
  ka_kinematics<<<ge, kAdjBlock, 0, s>>>(a->ad, r.dt);
  ka_gather_corners<<<gn, kAdjBlock, 0, s>>>(a->ad);
  ka_node<<<gn, kAdjBlock, 0, s>>>(a->ad, r.dt);
  const double hg = d->sc[LULESH_S_HGCOEF];
  switch (mode & 3) {
    case 0: ka_force<0><<<ge, kAdjBlock, 0, s>>>(a->ad, hg); break;
    case 1: ka_force<1><<<ge, kAdjBlock, 0, s>>>(a->ad, hg); break;
    case 2: ka_force<2><<<ge, kAdjBlock, 0, s>>>(a->ad, hg); break;
    default: ka_force<3><<<ge, kAdjBlock, 0, s>>>(a->ad, hg); break;
  }
  ka_gather_corners<<<gn, kAdjBlock, 0, s>>>(a->ad);
  ka_sum<<<1, kAdjBlock, 0, s>>>(a->ad.part_dt, ge, a->scal);
  ka_sum<<<1, kAdjBlock, 0, s>>>(a->ad.part_dtn, gn, a->scal + 1);
  ka_sum<<<1, kAdjBlock, 0, s>>>(a->ad.part_hg, ge, a->scal + 2);
  ACK(cudaGetLastError());
  double h[3];
  ACK(cudaMemcpyAsync(h, a->scal, sizeof(h), cudaMemcpyDeviceToHost, s));
  ACK(cudaStreamSynchronize(s));
  *Ldt_k = h[0] + h[1];
  *Lhg_k = h[2];
  return LULESH_OK;
}

static double* adj_field(lulesh_adjoint* a, int32_t f) {
  AdjDev& ad = a->ad;
  switch (f) {
    case LULESH_F_X: return ad.lx;
    case LULESH_F_Y: return ad.ly;
    case LULESH_F_Z: return ad.lz;
    case LULESH_F_XD: return ad.lxd;
    case LULESH_F_YD: return ad.lyd;
    case LULESH_F_ZD: return ad.lzd;
    case LULESH_F_E: return ad.le;
    case LULESH_F_P: return ad.lp;
    case LULESH_F_Q: return ad.lq;
    case LULESH_F_V: return ad.lv;
    case LULESH_F_SS: return ad.lss;
    default: return nullptr;
  }
}

static int field_index(int32_t f) {
  for (int k = 0; k < kStateFields; ++k)
    if (kStateIds[k] == f) return k;
  return -1;
}

// The objective at the domain's current state; with `seed` the adjoint state
// is set to its gradient.
static int objective(lulesh_adjoint* a, bool seed, double* loss) {
  lulesh_domain* d = a->dom;
  cudaStream_t s = d->stream;
  AdjDev& ad = a->ad;
  const int ge = (a->E + kAdjBlock - 1) / kAdjBlock, gn = (a->N + kAdjBlock - 1) / kAdjBlock;
  if (seed) {
    for (int k = 0; k < kStateFields; ++k) {
      double* lam = adj_field(a, kStateIds[k]);
      ACK(cudaMemsetAsync(lam, 0, (k < 6 ? a->N : a->E) * sizeof(double), s));
    }
  }
  double total = 0.0;
  if (a->seeds.empty()) {
    ka_loss_elem<<<ge, kAdjBlock, 0, s>>>(a->we, d->dd.e, a->E, seed ? ad.le : nullptr, ad.part_dt);
    ka_sum<<<1, kAdjBlock, 0, s>>>(ad.part_dt, ge, a->scal);
    ka_loss_node<<<gn, kAdjBlock, 0, s>>>(a->wn, d->dd.xd, d->dd.yd, d->dd.zd, a->N, seed ? ad.lxd : nullptr,
                                           seed ? ad.lyd : nullptr, seed ? ad.lzd : nullptr, ad.part_dtn);
    ka_sum<<<1, kAdjBlock, 0, s>>>(ad.part_dtn, gn, a->scal + 1);
    double h[2];
    ACK(cudaMemcpyAsync(h, a->scal, sizeof(h), cudaMemcpyDeviceToHost, s));
    ACK(cudaStreamSynchronize(s));
    total = h[0] + h[1];
  } else {
    for (auto& kv : a->seeds) {
      const int k = field_index(kv.first);
      const int n = k < 6 ? a->N : a->E;
      const int g = (n + kAdjBlock - 1) / kAdjBlock;
      ka_loss_elem<<<g, kAdjBlock, 0, s>>>(kv.second, *state_ptr(d->dd, k), n, seed ? adj_field(a, kv.first) : nullptr,
                                           ad.part_dt);
      ka_sum<<<1, kAdjBlock, 0, s>>>(ad.part_dt, g, a->scal);
      double h;
      ACK(cudaMemcpyAsync(&h, a->scal, sizeof(h), cudaMemcpyDeviceToHost, s));
      ACK(cudaStreamSynchronize(s));
      total += h;
    }
  }
  if (loss) *loss = total;
  return LULESH_OK;
}

extern "C" {

int lulesh_adj_create(lulesh_domain* dom, double radius, int32_t checkpoint_every, lulesh_adjoint** out) {
  if (!dom || !out || checkpoint_every < 1 || !(radius >= 0.0)) return LULESH_ERR_ARGUMENT;
  *out = nullptr;
  ACK(cudaSetDevice(dom->params.device));
  lulesh_adjoint* a = new (std::nothrow) lulesh_adjoint();
  if (!a) return LULESH_ERR_MEMORY;
  a->dom = dom;
  a->radius = radius;
  a->K = checkpoint_every;
  a->E = (int)dom->E;
  a->N = (int)dom->N;
  const int E = a->E, N = a->N, K = a->K;
  auto fail = [&](int rc) { lulesh_adj_destroy(a); return rc; };
  int rc;
  a->slots.resize(K + 1);
  for (auto& s : a->slots)
    if ((rc = alloc_state(a, s))) return fail(rc);
  a->tape.resize(K);
  for (auto& t : a->tape) {
    if ((rc = dalloc(a, &t.ax, N)) || (rc = dalloc(a, &t.ay, N)) || (rc = dalloc(a, &t.az, N)) ||
        (rc = dalloc(a, &t.vnew, E)) || (rc = dalloc(a, &t.delv, E)) || (rc = dalloc(a, &t.arealg, E)) ||
        (rc = dalloc(a, &t.vdov, E)) || (rc = dalloc(a, &t.flags, E)) || (rc = dalloc(a, &t.dtc, E)) ||
        (rc = dalloc(a, &t.dth, E)))
      return fail(rc);
    for (int k = 0; k < 3; ++k)
      if ((rc = dalloc(a, &t.dv[k], E)) || (rc = dalloc(a, &t.dx[k], E))) return fail(rc);
  }
  if ((rc = alloc_state(a, a->final_state))) return fail(rc);
  AdjDev& ad = a->ad;
  const int ge = (E + kAdjBlock - 1) / kAdjBlock, gn = (N + kAdjBlock - 1) / kAdjBlock;
  if ((rc = dalloc(a, &ad.lx, N)) || (rc = dalloc(a, &ad.ly, N)) || (rc = dalloc(a, &ad.lz, N)) ||
      (rc = dalloc(a, &ad.lxd, N)) || (rc = dalloc(a, &ad.lyd, N)) || (rc = dalloc(a, &ad.lzd, N)) ||
      (rc = dalloc(a, &ad.lfx, N)) || (rc = dalloc(a, &ad.lfy, N)) || (rc = dalloc(a, &ad.lfz, N)) ||
      (rc = dalloc(a, &ad.le, E)) || (rc = dalloc(a, &ad.lp, E)) || (rc = dalloc(a, &ad.lq, E)) ||
      (rc = dalloc(a, &ad.lss, E)) || (rc = dalloc(a, &ad.lv, E)) || (rc = dalloc(a, &ad.lvnew, E)) ||
      (rc = dalloc(a, &ad.ldelv, E)) || (rc = dalloc(a, &ad.larealg, E)) || (rc = dalloc(a, &ad.lvdov, E)) ||
      (rc = dalloc(a, &ad.lnb, 6 * (size_t)E)) || (rc = dalloc(a, &ad.cX, 24 * (size_t)E)) ||
      (rc = dalloc(a, &ad.cV, 24 * (size_t)E)) || (rc = dalloc(a, &ad.part_dt, std::max(ge, gn))) ||
      (rc = dalloc(a, &ad.part_dtn, gn)) || (rc = dalloc(a, &ad.part_hg, ge)) || (rc = dalloc(a, &a->scal, 4)) ||
      (rc = dalloc(a, &a->argmin, 2)) || (rc = dalloc(a, &a->we, E)) || (rc = dalloc(a, &a->wn, N)) ||
      (rc = dalloc(a, &a->fx_s, N)) || (rc = dalloc(a, &a->fy_s, N)) || (rc = dalloc(a, &a->fz_s, N)))
    return fail(rc);
  for (int k = 0; k < 3; ++k)
    if ((rc = dalloc(a, &ad.ldv[k], E)) || (rc = dalloc(a, &ad.ldx[k], E))) return fail(rc);
  const DevDomain& dd = dom->dd;
  ad.E = E; ad.N = N;
  ad.nodelist = dd.nodelist; ad.nodeElemStart = dd.nodeElemStart; ad.cornerList = dd.cornerList;
  ad.nodeBC = dd.nodeBC; ad.inv_nodalMass = dd.inv_nodalMass; ad.volo = dd.volo; ad.inv_volo = dd.inv_volo;
  ad.elemMass = dd.elemMass; ad.elemBC = dd.elemBC;
  ad.lxim = dd.lxim; ad.lxip = dd.lxip; ad.letam = dd.letam; ad.letap = dd.letap;
  ad.lzetam = dd.lzetam; ad.lzetap = dd.lzetap;

  // host copies of what the inverse neighbour lists and weights need
  cudaStream_t s = dom->stream;
  std::vector<unsigned> bc(E);
  std::vector<int> nb[6];
  int* srcs[6] = {dd.lxim, dd.lxip, dd.letam, dd.letap, dd.lzetam, dd.lzetap};
  for (int k = 0; k < 6; ++k) nb[k].resize(E);
  std::vector<double> emass(E), nmass(N);
  if (cudaMemcpyAsync(bc.data(), dd.elemBC, E * sizeof(unsigned), cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return fail(LULESH_ERR_CUDA);
  for (int k = 0; k < 6; ++k)
    if (cudaMemcpyAsync(nb[k].data(), srcs[k], E * sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess)
      return fail(LULESH_ERR_CUDA);
  if (cudaMemcpyAsync(emass.data(), dd.elemMass, E * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaMemcpyAsync(nmass.data(), dd.nodalMass, N * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return fail(LULESH_ERR_CUDA);
  // inverse neighbour lists: element k collects slot (2d + side)*E + j of
  // every element j whose limiter reads k's delv (self reads excluded)
  {
    const unsigned bits[6] = {XI_M, XI_P, ETA_M, ETA_P, ZETA_M, ZETA_P};
    const unsigned symm[6] = {XI_M_SYMM, XI_P_SYMM, ETA_M_SYMM, ETA_P_SYMM, ZETA_M_SYMM, ZETA_P_SYMM};
    const unsigned comm[6] = {XI_M_COMM, XI_P_COMM, ETA_M_COMM, ETA_P_COMM, ZETA_M_COMM, ZETA_P_COMM};
    std::vector<int> count(E + 1, 0);
    std::vector<std::pair<int, int>> ent;  // (target k, entry)
    for (int j = 0; j < E; ++j)
      for (int sl = 0; sl < 6; ++sl) {
        const unsigned c = bc[j] & bits[sl];
        int idx = nb[sl][j];
        if (sl == 1 && !(dd.mode & 4)) idx -= 1;  // the reference's xi-plus index
        int k = -1;
        if (c == 0u || c == comm[sl]) k = (idx >= 0 && idx < E) ? idx : -1;
        else if (c == symm[sl]) k = j;
        if (k >= 0 && k != j) ent.emplace_back(k, sl * E + j);
      }
    std::stable_sort(ent.begin(), ent.end(), [](const std::pair<int, int>& p, const std::pair<int, int>& q) {
      return p.first < q.first;
    });
    std::vector<int> start(E + 1, 0), list(ent.size());
    for (auto& p : ent) start[p.first + 1] += 1;
    for (int k = 0; k < E; ++k) start[k + 1] += start[k];
    for (size_t t = 0; t < ent.size(); ++t) list[t] = ent[t].second;
    if ((rc = dalloc(a, &a->nbStart, E + 1)) || (rc = dalloc(a, &a->nbList, std::max<size_t>(1, list.size()))))
      return fail(rc);
    if (cudaMemcpy(a->nbStart, start.data(), (E + 1) * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess ||
        (!list.empty() && cudaMemcpy(a->nbList, list.data(), list.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess))
      return fail(LULESH_ERR_CUDA);
    ad.nbStart = a->nbStart;
    ad.nbList = a->nbList;
  }
  // objective weights: mass of the elements whose reference-mesh centroid and
  // of the nodes whose reference position lies within `radius` of the origin
  {
    const int nx = dom->params.nx, en = nx + 1;
    const double h = 1.125 / nx, r2 = radius * radius;
    std::vector<double> w(E), v(N);
    for (int pl = 0; pl < nx; ++pl)
      for (int row = 0; row < nx; ++row)
        for (int col = 0; col < nx; ++col) {
          const double cx = (col + 0.5) * h, cy = (row + 0.5) * h, cz = (pl + 0.5) * h;
          const int e = (pl * nx + row) * nx + col;
          w[e] = (cx * cx + cy * cy + cz * cz < r2) ? emass[e] : 0.0;
        }
    for (int pl = 0; pl < en; ++pl)
      for (int row = 0; row < en; ++row)
        for (int col = 0; col < en; ++col) {
          const double px = col * h, py = row * h, pz = pl * h;
          const int n = (pl * en + row) * en + col;
          v[n] = (px * px + py * py + pz * pz < r2) ? nmass[n] : 0.0;
        }
    if (cudaMemcpy(a->we, w.data(), E * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(a->wn, v.data(), N * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess)
      return fail(LULESH_ERR_CUDA);
  }
  *out = a;
  return LULESH_OK;
}

int lulesh_adj_destroy(lulesh_adjoint* a) {
  if (!a) return LULESH_ERR_ARGUMENT;
  cudaSetDevice(a->dom->params.device);
  cudaStreamSynchronize(a->dom->stream);
  for (void* p : a->allocs) cudaFree(p);
  delete a;
  return LULESH_OK;
}

int lulesh_adj_set_seed(lulesh_adjoint* a, int32_t field, const double* w, int64_t count) {
  if (!a || !w) return LULESH_ERR_ARGUMENT;
  const int k = field_index(field);
  if (k < 0 || count != (k < 6 ? a->N : a->E)) return LULESH_ERR_ARGUMENT;
  double*& dst = a->seeds[field];
  if (!dst) {
    int rc = dalloc(a, &dst, count);
    if (rc) { a->seeds.erase(field); return rc; }
  }
  ACK(cudaMemcpy(dst, w, count * sizeof(double), cudaMemcpyHostToDevice));
  return LULESH_OK;
}

int lulesh_adj_clear_seeds(lulesh_adjoint* a) {
  if (!a) return LULESH_ERR_ARGUMENT;
  a->seeds.clear();  // the buffers stay in allocs and are freed with the handle
  return LULESH_OK;
}

int lulesh_adj_loss(lulesh_adjoint* a, double* loss) {
  if (!a || !loss) return LULESH_ERR_ARGUMENT;
  ACK(cudaSetDevice(a->dom->params.device));
  return objective(a, false, loss);
}

int lulesh_adj_gradient(lulesh_adjoint* a, int64_t num_cycles, lulesh_adj_result* res) {
  if (!a || num_cycles < 1) return LULESH_ERR_ARGUMENT;
  lulesh_domain* d = a->dom;
  ACK(cudaSetDevice(d->params.device));
  cudaStream_t s = d->stream;
  const int K = a->K;
  lulesh_adj_result out{};
  int rc;
  // ---- forward sweep with checkpoints (stops early at stoptime, as the
  // examples/benchmark.jl loop does) ----
  auto t0 = std::chrono::steady_clock::now();
  int64_t done = 0;
  int nseg = 0;
  auto running = [&]() { return done < num_cycles && d->sc[LULESH_S_TIME] < d->sc[LULESH_S_STOPTIME]; };
  while (running()) {
    if ((int)a->ckpts.size() == nseg) {
      a->ckpts.emplace_back();
      if ((rc = alloc_state(a, a->ckpts.back()))) { a->ckpts.pop_back(); return rc; }
    }
    if ((int)a->ckpt_scalars.size() == nseg) a->ckpt_scalars.emplace_back();
    if ((rc = copy_state_from_domain(a, a->ckpts[nseg]))) return rc;
    a->ckpt_scalars[nseg] = get_scalars(d);
    ++nseg;
    for (int j = 0; j < K && running(); ++j, ++done)
      if ((rc = forward_cycle(a, nullptr, nullptr))) { out.status = rc; if (res) *res = out; return rc; }
  }
  out.cycles = done;
  out.checkpoints = nseg;
  ACK(cudaStreamSynchronize(s));
  auto t1 = std::chrono::steady_clock::now();
  if ((rc = objective(a, true, &out.loss))) return rc;
  if ((rc = copy_state_from_domain(a, a->final_state))) return rc;
  const Scalars5 final_sc = get_scalars(d);
  // ---- reverse sweep ----
  const Params prm = make_params(d);
  double Ltime = 0.0, Ldt = 0.0, Ldtc = 0.0, Ldth = 0.0, Lhg = 0.0;
  a->rec.resize(K);
  for (int k = nseg - 1; k >= 0; --k) {
    if ((rc = copy_state_to_domain(a, a->ckpts[k]))) return rc;
    set_scalars(d, a->ckpt_scalars[k]);
    const int n = (int)std::min<int64_t>(K, done - (int64_t)k * K);
    for (int j = 0; j < n; ++j) {
      if ((rc = copy_state_from_domain(a, a->slots[j]))) return rc;
      if ((rc = forward_cycle(a, &a->tape[j], &a->rec[j]))) return rc;
    }
    if ((rc = copy_state_from_domain(a, a->slots[n]))) return rc;
    for (int j = n - 1; j >= 0; --j) {
      const ScalarRec& r = a->rec[j];
      // the cycle's Courant/hydro minima feed the element that attained them
      const double lam_c = r.active_c ? Ldtc : 0.0, lam_h = r.active_h ? Ldth : 0.0;
      double Ldtc_prev = r.active_c ? 0.0 : Ldtc, Ldth_prev = r.active_h ? 0.0 : Ldth;
      set_cycle_pointers(a, a->slots[j], a->slots[j + 1], a->tape[j]);
      double Ldt_k = 0.0, Lhg_k = 0.0;
      if ((rc = reverse_cycle(a, r, r.argmin_c, lam_c, r.argmin_h, lam_h, &Ldt_k, &Lhg_k))) return rc;
      Lhg += Lhg_k;
      // time_n = time_{n-1} + dt_n, then timeIncrement!'s transpose
      double Ldt_tot = Ldt + Ldt_k + Ltime;
      double Ldt_prev = 0.0;
      time_increment_reverse(r, prm, Ldt_tot, Ltime, Ldt_prev, Ldtc_prev, Ldth_prev);
      Ldt = Ldt_prev;
      Ldtc = Ldtc_prev;
      Ldth = Ldth_prev;
    }
  }
  if ((rc = copy_state_to_domain(a, a->final_state))) return rc;
  set_scalars(d, final_sc);
  ACK(cudaStreamSynchronize(s));
  auto t2 = std::chrono::steady_clock::now();
  out.grad_hgcoef = Lhg;
  out.forward_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
  out.reverse_ms = std::chrono::duration<double, std::milli>(t2 - t1).count();
  out.status = LULESH_OK;
  if (res) *res = out;
  return LULESH_OK;
}

int lulesh_adj_get_gradient(lulesh_adjoint* a, int32_t field, double* host, int64_t count) {
  if (!a || !host) return LULESH_ERR_ARGUMENT;
  const int k = field_index(field);
  if (k < 0 || count != (k < 6 ? a->N : a->E)) return LULESH_ERR_ARGUMENT;
  ACK(cudaSetDevice(a->dom->params.device));
  ACK(cudaMemcpy(host, adj_field(a, field), count * sizeof(double), cudaMemcpyDeviceToHost));
  return LULESH_OK;
}

}  // extern "C"
