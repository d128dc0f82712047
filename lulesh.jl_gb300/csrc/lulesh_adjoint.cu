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
//      device from the recorded scalars: the minima pass their adjoint to the
//      element that attained them.
// The forward sweep runs as lulesh_run does (CUDA graphs, dt on the device);
// the recompute and the transpose of a segment are queued without any host
// synchronisation. With two tape sets (when they fit), segment k-1 is
// recomputed on a second stream while segment k is transposed: the FP64-bound
// forward kernels fill the SMs the latency-bound transposes leave idle.
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
#include "lulesh_trace.h"

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
  double* geo;  // [66][E] force-kernel tape
  double* kin;  // [90][E] kinematics-kernel tape
  double* mat;  // [31][E] material-kernel tape
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

// What one segment's recompute leaves for its transpose: the K+1 states, the
// K cycles' tape and their device records.
struct TapeSet {
  std::vector<StateBuf> slots;
  std::vector<CycleTape> tape;
  CycleRec* rec = nullptr;
  double* diag0 = nullptr;  // [36][E]: the face diagonals at the segment's start
  bool ready = false;
};

struct lulesh_adjoint {
  lulesh_domain* dom = nullptr;
  double radius = 0.3;
  int K = 20;
  int E = 0, N = 0;
  std::vector<void*> allocs;
  TapeSet sets[2];               // set 1 only for the overlapped sweep with two tapes
  std::vector<void*> set1_allocs;
  // reverse sweep: 0 sequential, 1 overlapped (two tapes where they fit, else
  // one), 2 overlapped on one tape
  int overlap = 1;
  cudaStream_t rstream = nullptr;  // recompute stream of the overlapped sweep
  cudaStream_t tstream = nullptr;  // transpose stream of the overlapped sweep (high priority)
  cudaEvent_t ev_start = nullptr, ev_done = nullptr;
  cudaEvent_t ev_ready[2] = {nullptr, nullptr}, ev_free[2] = {nullptr, nullptr};
  std::vector<cudaEvent_t> ev_slot;  // one tape: tape slot j released by the transpose
  std::vector<StateBuf> ckpts;   // segment start states
  std::vector<int> seg_len;      // cycles of each segment
  DevState* ckpt_st = nullptr;   // device: step state at each checkpoint
  int ckpt_st_cap = 0;
  StateBuf final_state{};
  double *we = nullptr, *wn = nullptr;  // objective weights
  int *nbStart = nullptr, *nbList = nullptr;
  double *fx_s = nullptr, *fy_s = nullptr, *fz_s = nullptr;  // force scratch of taped cycles
  AdjDev ad{};
  double* scal = nullptr;       // device: sums of partials (objective)
  AdjScal* dsc = nullptr;       // device: carried scalar adjoints
  std::map<int32_t, double*> seeds;  // linear-objective weights per state field
  // graph of K forward cycles for the checkpointed sweep, with what it bakes in
  cudaGraphExec_t fwd_graph = nullptr;
  Params fwd_prm{};
  Tuning fwd_tuning{};
  bool fwd_aux = false;
  // graphs of one full segment's recompute (into set X) and transpose (of
  // set X), with what they bake in
  cudaGraphExec_t rec_graph[2] = {nullptr, nullptr}, tr_graph[2] = {nullptr, nullptr};
  Params rev_prm{};
  Tuning rev_tuning{};
};

static int dmalloc_to(std::vector<void*>& list, void** p, size_t bytes) {
  if (cudaMalloc(p, bytes ? bytes : 8) != cudaSuccess) { cudaGetLastError(); return LULESH_ERR_MEMORY; }
  list.push_back(*p);
  return LULESH_OK;
}
static int dmalloc(lulesh_adjoint* a, void** p, size_t bytes) { return dmalloc_to(a->allocs, p, bytes); }
template <class T>
static int dalloc(lulesh_adjoint* a, T** p, size_t n) {
  return dmalloc(a, reinterpret_cast<void**>(p), n * sizeof(T));
}
template <class T>
static int dalloc_to(std::vector<void*>& list, T** p, size_t n) {
  return dmalloc_to(list, reinterpret_cast<void**>(p), n * sizeof(T));
}

static int alloc_state_to(lulesh_adjoint* a, std::vector<void*>& list, StateBuf& s) {
  for (int k = 0; k < kStateFields; ++k) {
    int rc = dalloc_to(list, &s.f[k], k < 6 ? a->N : a->E);
    if (rc) return rc;
  }
  return LULESH_OK;
}
static int alloc_state(lulesh_adjoint* a, StateBuf& s) { return alloc_state_to(a, a->allocs, s); }

// A tape set's per-cycle state: only the fields the transposes read (the
// velocities, p, q, v, ss); positions and energy stay null, and the state
// copies skip them.
static int alloc_slot_state(lulesh_adjoint* a, std::vector<void*>& list, StateBuf& s) {
  for (int k = 0; k < kStateFields; ++k) {
    s.f[k] = nullptr;
    if (k <= 2 || k == 6) continue;  // x y z e
    int rc = dalloc_to(list, &s.f[k], k < 6 ? a->N : a->E);
    if (rc) return rc;
  }
  return LULESH_OK;
}

// The K+1 states, K cycles of tape and K records of one tape set.
static int alloc_set(lulesh_adjoint* a, std::vector<void*>& list, TapeSet& t) {
  const int E = a->E, N = a->N, K = a->K;
  int rc;
  t.slots.assign(K + 1, StateBuf{});
  for (auto& st : t.slots)
    if ((rc = alloc_slot_state(a, list, st))) return rc;
  t.tape.assign(K, CycleTape{});
  for (auto& c : t.tape) {
    if ((rc = dalloc_to(list, &c.ax, N)) || (rc = dalloc_to(list, &c.ay, N)) || (rc = dalloc_to(list, &c.az, N)) ||
        (rc = dalloc_to(list, &c.vnew, E)) || (rc = dalloc_to(list, &c.delv, E)) ||
        (rc = dalloc_to(list, &c.arealg, E)) || (rc = dalloc_to(list, &c.vdov, E)) ||
        (rc = dalloc_to(list, &c.flags, E)) || (rc = dalloc_to(list, &c.dtc, E)) || (rc = dalloc_to(list, &c.dth, E)) ||
        (rc = dalloc_to(list, &c.geo, 66 * (size_t)E)) || (rc = dalloc_to(list, &c.kin, 90 * (size_t)E)) ||
        (rc = dalloc_to(list, &c.mat, 31 * (size_t)E)))
      return rc;
    for (int k = 0; k < 3; ++k)
      if ((rc = dalloc_to(list, &c.dv[k], E)) || (rc = dalloc_to(list, &c.dx[k], E))) return rc;
  }
  if ((rc = dalloc_to(list, &t.rec, K)) || (rc = dalloc_to(list, &t.diag0, 36 * (size_t)E))) return rc;
  t.ready = true;
  return LULESH_OK;
}

static void free_set1(lulesh_adjoint* a) {
  if (a->rec_graph[1]) { cudaGraphExecDestroy(a->rec_graph[1]); a->rec_graph[1] = nullptr; }
  if (a->tr_graph[1]) { cudaGraphExecDestroy(a->tr_graph[1]); a->tr_graph[1] = nullptr; }
  for (void* p : a->set1_allocs) cudaFree(p);
  a->set1_allocs.clear();
  a->sets[1] = TapeSet{};
}

// The streams and events of an overlapped reverse sweep; false (sequential
// sweep) when they cannot be made. The transposes are the sweep's critical
// path, so their stream takes the device's highest priority: the block
// scheduler gives them the SMs first and the recompute fills what they leave
// idle (partial waves, latency-bound phases).
static bool ensure_streams(lulesh_adjoint* a) {
  if (!a->rstream && cudaStreamCreateWithFlags(&a->rstream, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    a->rstream = nullptr;
    return false;
  }
  if (!a->tstream) {
    int least = 0, greatest = 0;
    if (cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess ||
        cudaStreamCreateWithPriority(&a->tstream, cudaStreamNonBlocking, greatest) != cudaSuccess) {
      cudaGetLastError();
      a->tstream = nullptr;
      return false;
    }
  }
  cudaEvent_t* evs[6] = {&a->ev_start, &a->ev_done, &a->ev_ready[0], &a->ev_ready[1], &a->ev_free[0], &a->ev_free[1]};
  for (cudaEvent_t* e : evs)
    if (!*e && cudaEventCreateWithFlags(e, cudaEventDisableTiming) != cudaSuccess) {
      cudaGetLastError();
      *e = nullptr;
      return false;
    }
  return true;
}

// The second tape set; false when it does not fit.
static bool ensure_set1(lulesh_adjoint* a) {
  if (a->sets[1].ready) return true;
  if (alloc_set(a, a->set1_allocs, a->sets[1]) != LULESH_OK) {
    free_set1(a);
    return false;
  }
  return true;
}

// One event per tape slot, for the overlapped sweep on one tape.
static bool ensure_slot_events(lulesh_adjoint* a) {
  while ((int)a->ev_slot.size() < a->K) {
    cudaEvent_t e = nullptr;
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    a->ev_slot.push_back(e);
  }
  return true;
}

static StateSet domain_set(lulesh_adjoint* a) {
  StateSet t;
  for (int k = 0; k < kStateFields; ++k) t.f[k] = *state_ptr(a->dom->dd, k);
  return t;
}
static StateSet buf_set(const StateBuf& b) {
  StateSet t;
  for (int k = 0; k < kStateFields; ++k) t.f[k] = b.f[k];
  return t;
}
static void copy_state(lulesh_adjoint* a, const StateSet& src, const StateSet& dst, cudaStream_t s) {
  const int n = std::max(a->E, a->N);
  ka_copy_state<<<(n + kAdjBlock - 1) / kAdjBlock, kAdjBlock, 0, s>>>(src, dst, a->E, a->N);
}
static void copy_state_from_domain(lulesh_adjoint* a, StateBuf& b, cudaStream_t s) {
  copy_state(a, domain_set(a), buf_set(b), s);
}
static void copy_state_to_domain(lulesh_adjoint* a, const StateBuf& b, cudaStream_t s) {
  copy_state(a, buf_set(b), domain_set(a), s);
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

// The start of a taped segment: the force kernel's geometry of the current
// positions, with the first cycle's face normals on its tape and its face
// diagonals in the set's diag0.
static void tape_segment_begin(lulesh_adjoint* a, const CycleTape& first, double* diag0, cudaStream_t s) {
  DevDomain gd = a->dom->dd;
  gd.tapeGeoNext = first.geo;
  gd.tapeDiag = diag0;
  launch_geometry(gd, s);
}

// One taped cycle, queued on the stream: the start state to its slot and
// timeIncrement! on the device (recorded), the step kernels with the cycle's
// intermediate values, accelerations, branch flags and dt candidates going to
// the tape (the kinematics kernel also writes the next cycle's face normals
// to `next`, if there is one), then the arg-min elements of the
// Courant and hydro minima.
static void tape_cycle(lulesh_adjoint* a, StateBuf& slot, const CycleTape& tp, const CycleTape* next, CycleRec* rec,
                       cudaStream_t s) {
  lulesh_domain* d = a->dom;
  const Params prm = make_params(d);
  const int nmax = std::max(a->E, a->N);
  ka_tape_begin<<<(nmax + kAdjBlock - 1) / kAdjBlock, kAdjBlock, 0, s>>>(domain_set(a), buf_set(slot), a->E, a->N,
                                                                        d->dd.st, rec, prm);
  DevDomain td = d->dd;
  td.vnew = tp.vnew; td.delv = tp.delv; td.arealg = tp.arealg; td.vdov = tp.vdov;
  td.delv_xi = tp.dv[0]; td.delv_eta = tp.dv[1]; td.delv_zeta = tp.dv[2];
  td.delx_xi = tp.dx[0]; td.delx_eta = tp.dx[1]; td.delx_zeta = tp.dx[2];
  td.xdd = tp.ax; td.ydd = tp.ay; td.zdd = tp.az;
  td.fx = a->fx_s; td.fy = a->fy_s; td.fz = a->fz_s;
  td.tapeFlags = tp.flags; td.tapeDtc = tp.dtc; td.tapeDth = tp.dth; td.tapeGeo = tp.geo;
  td.tapeKin = tp.kin; td.tapeMat = tp.mat;
  td.tapeGeoNext = next ? next->geo : nullptr;
  launch_force(td, prm, d->tuning, s);
  launch_node(td, prm, true, d->tuning, s);  // aux: the node kernel stores the accelerations
  launch_kinematics(td, prm, false, d->tuning, s);
  launch_material(td, prm, false, d->tuning, s);
  const int ge = (a->E + kAdjBlock - 1) / kAdjBlock;
  ka_tape_close<<<ge, kAdjBlock, 0, s>>>(tp.dtc, tp.dth, a->E, d->dd.st, rec);
}

static void set_cycle_pointers(lulesh_adjoint* a, const StateBuf& s0, const StateBuf& s1, const CycleTape& t) {
  AdjDev& ad = a->ad;
  ad.x0 = s0.f[0]; ad.y0 = s0.f[1]; ad.z0 = s0.f[2]; ad.xd0 = s0.f[3]; ad.yd0 = s0.f[4]; ad.zd0 = s0.f[5];
  ad.e0 = s0.f[6]; ad.p0 = s0.f[7]; ad.q0 = s0.f[8]; ad.v0 = s0.f[9]; ad.ss0 = s0.f[10];
  ad.x1 = s1.f[0]; ad.y1 = s1.f[1]; ad.z1 = s1.f[2]; ad.xd1 = s1.f[3]; ad.yd1 = s1.f[4]; ad.zd1 = s1.f[5];
  ad.p1 = s1.f[7]; ad.q1 = s1.f[8];
  ad.ax = t.ax; ad.ay = t.ay; ad.az = t.az;
  ad.vnew = t.vnew; ad.delv = t.delv; ad.arealg = t.arealg; ad.vdov = t.vdov;
  for (int k = 0; k < 3; ++k) { ad.dvl[k] = t.dv[k]; ad.dxl[k] = t.dx[k]; }
  ad.flags = t.flags;
  ad.geo = t.geo;
  ad.kin = t.kin;
  ad.mat = t.mat;
}

// Transpose of one recorded cycle, queued on the stream: the adjoint state
// goes from the cycle's end to its start, and the carried scalar adjoints
// through timeIncrement!.
static void reverse_cycle(lulesh_adjoint* a, const CycleRec* rec, cudaStream_t s) {
  lulesh_domain* d = a->dom;
  const Params prm = make_params(d);
  const int ge = (a->E + kAdjBlock - 1) / kAdjBlock, gn = (a->N + kAdjBlock - 1) / kAdjBlock;
  const int mode = d->dd.mode;
  const double irho0 = 1.0 / prm.refdens;
  if (mode & 4) ka_material<4><<<ge, kAdjBlock, 0, s>>>(a->ad, prm, irho0, rec, a->dsc);
  else ka_material<0><<<ge, kAdjBlock, 0, s>>>(a->ad, prm, irho0, rec, a->dsc);
  const double hg = d->sc[LULESH_S_HGCOEF];
  // ka_kinematics also gathers the limiter's neighbour reads and does the
  // position transpose of the next cycle's k_force; ka_node gathers the
  // corners; ka_hourglass leaves this cycle's force terms for the
  // ka_kinematics of the cycle before (or ka_force_geo after the first cycle)
#define LULESH_KA_CYCLE(M)                                            \
  ka_kinematics<M><<<ge, kAdjBlock, 0, s>>>(a->ad, rec);              \
  ka_node<<<gn, kAdjBlock, 0, s>>>(a->ad, rec);                       \
  ka_hourglass<M><<<ge, kAdjBlock, 0, s>>>(a->ad, hg)
  switch (mode & 3) {
    case 0: LULESH_KA_CYCLE(0); break;
    case 1: LULESH_KA_CYCLE(1); break;
    case 2: LULESH_KA_CYCLE(2); break;
    default: LULESH_KA_CYCLE(3); break;
  }
#undef LULESH_KA_CYCLE
  ka_cycle_close<<<1, kCloseBlock, 0, s>>>(a->ad, ge, gn, rec, a->dsc, prm);
}

// Position transpose of the run's first cycle's k_force (the last one the
// reverse sweep reaches), into the force corner buffer.
static void first_cycle_force_geo(lulesh_adjoint* a, cudaStream_t s) {
  const int ge = (a->E + kAdjBlock - 1) / kAdjBlock;
  switch (a->dom->dd.mode & 3) {
    case 0: ka_force_geo<0><<<ge, kAdjBlock, 0, s>>>(a->ad); break;
    case 1: ka_force_geo<1><<<ge, kAdjBlock, 0, s>>>(a->ad); break;
    case 2: ka_force_geo<2><<<ge, kAdjBlock, 0, s>>>(a->ad); break;
    default: ka_force_geo<3><<<ge, kAdjBlock, 0, s>>>(a->ad); break;
  }
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
  // the adjoint kernels have no halo transposes: one block only
  if (dom->dd.haloDelvSrc || dom->dd.haloCornerSrc) return LULESH_ERR_ARGUMENT;
  *out = nullptr;
  ACK(cudaSetDevice(dom->params.device));
  lulesh_adjoint* a = new (std::nothrow) lulesh_adjoint();
  if (!a) return LULESH_ERR_MEMORY;
  a->dom = dom;
  a->radius = radius;
  a->K = checkpoint_every;
  a->E = (int)dom->E;
  a->N = (int)dom->N;
  const int E = a->E, N = a->N;
  auto fail = [&](int rc) { lulesh_adj_destroy(a); return rc; };
  int rc;
  if ((rc = alloc_set(a, a->allocs, a->sets[0]))) return fail(rc);
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
      (rc = dalloc(a, &ad.cV, 24 * (size_t)E)) || (rc = dalloc(a, &ad.fX, 24 * (size_t)E)) ||
      (rc = dalloc(a, &ad.fV, 24 * (size_t)E)) || (rc = dalloc(a, &ad.sLdv, 24 * (size_t)E)) ||
      (rc = dalloc(a, &ad.sLU, 15 * (size_t)E)) || (rc = dalloc(a, &ad.sLhm, 12 * (size_t)E)) ||
      (rc = dalloc(a, &ad.part_dt, std::max(ge, gn))) ||
      (rc = dalloc(a, &ad.part_dtn, gn)) || (rc = dalloc(a, &ad.part_hg, ge)) || (rc = dalloc(a, &a->scal, 4)) ||
      (rc = dalloc(a, &a->dsc, 1)) || (rc = dalloc(a, &a->we, E)) || (rc = dalloc(a, &a->wn, N)) ||
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
  if (a->fwd_graph) cudaGraphExecDestroy(a->fwd_graph);
  if (a->rec_graph[0]) cudaGraphExecDestroy(a->rec_graph[0]);
  if (a->tr_graph[0]) cudaGraphExecDestroy(a->tr_graph[0]);
  if (a->rstream) cudaStreamSynchronize(a->rstream);
  if (a->tstream) cudaStreamSynchronize(a->tstream);
  free_set1(a);
  for (cudaEvent_t e : {a->ev_start, a->ev_done, a->ev_ready[0], a->ev_ready[1], a->ev_free[0], a->ev_free[1]})
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : a->ev_slot) cudaEventDestroy(e);
  if (a->rstream) cudaStreamDestroy(a->rstream);
  if (a->tstream) cudaStreamDestroy(a->tstream);
  for (void* p : a->allocs) cudaFree(p);
  delete a;
  return LULESH_OK;
}

int lulesh_adj_set_overlap(lulesh_adjoint* a, int32_t mode) {
  if (!a || mode < 0 || mode > 2) return LULESH_ERR_ARGUMENT;
  ACK(cudaSetDevice(a->dom->params.device));
  ACK(cudaStreamSynchronize(a->dom->stream));
  if (a->rstream) ACK(cudaStreamSynchronize(a->rstream));
  if (a->tstream) ACK(cudaStreamSynchronize(a->tstream));
  a->overlap = mode;
  // the second tape is allocated by the next gradient that can use it
  if (mode != 1) free_set1(a);
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
  TraceRange trace("lulesh_adj_gradient");
  lulesh_domain* d = a->dom;
  ACK(cudaSetDevice(d->params.device));
  cudaStream_t s = d->stream;
  const int K = a->K;
  lulesh_adj_result out{};
  int rc;
  // ---- forward sweep with checkpoints ----
  // Segments of K cycles: each starts by copying the state and the device step
  // state to its checkpoint; the segments then run as captured graphs of
  // exactly K cycles (dt on the device; once time reaches stoptime, as in the
  // examples/benchmark.jl loop, the remaining cycles are no-ops), except the
  // last one (the last two when the sweep overlaps and has both tape sets),
  // which run taped so that the reverse sweep need not recompute them.
  // Nothing waits on the host until the sweep ends.
  auto t0 = std::chrono::steady_clock::now();
  const int nplan = (int)((num_cycles + K - 1) / K);
  const int last_len = (int)(num_cycles - (int64_t)(nplan - 1) * K);
  while ((int)a->ckpts.size() < nplan) {
    a->ckpts.emplace_back();
    if ((rc = alloc_state(a, a->ckpts.back()))) { a->ckpts.pop_back(); return rc; }
  }
  if (a->ckpt_st_cap < nplan) {
    DevState* p = nullptr;
    if ((rc = dalloc(a, &p, nplan))) return rc;
    a->ckpt_st = p;
    a->ckpt_st_cap = nplan;
  }
  const Params prm = make_params(d);
  const bool aux = d->params.keep_aux != 0;
  // The reverse sweep's plan: sequential (one tape, one stream), overlapped
  // with two tapes (segment k uses set k & 1), or overlapped on one tape
  // (consecutive segments store their cycles in opposite slot orders, so the
  // recompute of segment k-1 fills each slot as soon as the transpose of
  // segment k, which empties them in the same order, has released it).
  enum Plan { kSeq = 0, kTwo = 1, kOne = 2 };
  Plan plan = kSeq;
  if (nplan > 1 && a->overlap != 0 && ensure_streams(a)) {
    if (a->overlap == 1 && ensure_set1(a)) plan = kTwo;
    else if (ensure_slot_events(a)) plan = kOne;
  }
  const bool pipe = plan != kSeq, one = plan == kOne;
  auto set_of = [&](int k) -> TapeSet& { return a->sets[plan == kTwo ? (k & 1) : 0]; };
  // on one tape, segment k's cycle j goes to tape slot K-1-j and its start
  // state to state slot K-j when an odd number of segments follow it
  auto rev_of = [&](int k) { return one && ((nplan - 1 - k) & 1) != 0; };
  auto tslot = [&](bool rev, int j) { return rev ? K - 1 - j : j; };
  auto sslot = [&](bool rev, int j) { return rev ? K - j : j; };
  // segments k >= first_taped are taped by the forward sweep itself
  const int first_taped = nplan - (plan == kTwo ? std::min(2, nplan) : 1);
  if (nplan > 1 && (!a->fwd_graph || std::memcmp(&a->fwd_prm, &prm, sizeof(Params)) != 0 ||
                    std::memcmp(&a->fwd_tuning, &d->tuning, sizeof(Tuning)) != 0 || a->fwd_aux != aux)) {
    if (a->fwd_graph) cudaGraphExecDestroy(a->fwd_graph);
    a->fwd_graph = nullptr;
    cudaGraph_t g;
    ACK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    for (int j = 0; j < K; ++j) {
      launch_time_increment(d->dd.st, 1, prm, s);
      launch_force(d->dd, prm, d->tuning, s);
      launch_node(d->dd, prm, aux, d->tuning, s);
      launch_kinematics(d->dd, prm, aux, d->tuning, s);
      launch_material(d->dd, prm, aux, d->tuning, s);
    }
    ACK(cudaStreamEndCapture(s, &g));
    const cudaError_t ge = cudaGraphInstantiate(&a->fwd_graph, g, 0);
    cudaGraphDestroy(g);
    ACK(ge);
    a->fwd_prm = prm;
    a->fwd_tuning = d->tuning;
    a->fwd_aux = aux;
  }
  // Recompute R(k) (checkpoint k restored into the domain, its cycles taped
  // into set_of(k)) and transpose T(k) (the adjoint state through those
  // cycles, in reverse), in order k = nseg-1..0; segments the forward sweep
  // taped skip R. Sequential, R(k) runs right before T(k) on the domain's
  // stream. Overlapped, T runs on the high-priority transpose stream and R on
  // its own stream one segment ahead, and T(k) waits for R(k):
  //  * two tapes: R(k-1) is queued before T(k) and waits until T(k+1) has
  //    released its set;
  //  * one tape: R(k-1) is queued after T(k), whose cycles each release their
  //    tape slot (an event per slot); R(k-1) writes a slot (its tape, its
  //    start state, and the next cycle's face normals) only after that
  //    slot's event, and its end state after all of T(k).
  // The domain's stream joins both at the end. Full segments of the first
  // two plans run as captured graphs (one per set and phase, rebuilt when the
  // parameters they bake in change).
  cudaStream_t rs = pipe ? a->rstream : s;
  cudaStream_t tst = pipe ? a->tstream : s;
  auto queue_recompute = [&](TapeSet& ts, int n, bool rev, cudaStream_t st) -> int {
    if (one) ACK(cudaStreamWaitEvent(st, a->ev_slot[tslot(rev, 0)], 0));
    tape_segment_begin(a, ts.tape[tslot(rev, 0)], ts.diag0, st);
    for (int j = 0; j < n; ++j) {
      if (one && j + 1 < n) ACK(cudaStreamWaitEvent(st, a->ev_slot[tslot(rev, j + 1)], 0));
      tape_cycle(a, ts.slots[sslot(rev, j)], ts.tape[tslot(rev, j)], j + 1 < n ? &ts.tape[tslot(rev, j + 1)] : nullptr,
                 ts.rec + tslot(rev, j), st);
    }
    if (one) ACK(cudaStreamWaitEvent(st, a->ev_free[0], 0));
    copy_state_from_domain(a, ts.slots[sslot(rev, n)], st);
    return LULESH_OK;
  };
  auto queue_transpose = [&](TapeSet& ts, int n, bool rev, cudaStream_t st) -> int {
    for (int j = n - 1; j >= 0; --j) {
      set_cycle_pointers(a, ts.slots[sslot(rev, j)], ts.slots[sslot(rev, j + 1)], ts.tape[tslot(rev, j)]);
      reverse_cycle(a, ts.rec + tslot(rev, j), st);
      if (one) ACK(cudaEventRecord(a->ev_slot[tslot(rev, j)], st));
    }
    return LULESH_OK;
  };
  const int nsets = plan == kTwo ? 2 : 1;
  if (std::memcmp(&a->rev_prm, &prm, sizeof(Params)) != 0 || std::memcmp(&a->rev_tuning, &d->tuning, sizeof(Tuning)) != 0) {
    for (int x = 0; x < 2; ++x) {
      if (a->rec_graph[x]) { cudaGraphExecDestroy(a->rec_graph[x]); a->rec_graph[x] = nullptr; }
      if (a->tr_graph[x]) { cudaGraphExecDestroy(a->tr_graph[x]); a->tr_graph[x] = nullptr; }
    }
    a->rev_prm = prm;
    a->rev_tuning = d->tuning;
  }
  auto capture = [&](cudaGraphExec_t* out, cudaStream_t st, auto&& body) -> int {
    cudaGraph_t g;
    ACK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    const int brc = body();
    const cudaError_t ce = cudaStreamEndCapture(st, &g);
    if (brc) { if (ce == cudaSuccess) cudaGraphDestroy(g); return brc; }
    ACK(ce);
    const cudaError_t ge = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    ACK(ge);
    return LULESH_OK;
  };
  // graphs of full segments, built before the forward sweep, whose taped
  // full segments run them too
  const bool any_full = !one && (nplan > 1 || last_len == K);
  for (int x = 0; x < nsets && any_full; ++x) {
    TapeSet& ts = a->sets[x];
    if (!a->rec_graph[x] && (rc = capture(&a->rec_graph[x], rs, [&] { return queue_recompute(ts, K, false, rs); })))
      return rc;
    if (!a->tr_graph[x] && (rc = capture(&a->tr_graph[x], tst, [&] { return queue_transpose(ts, K, false, tst); })))
      return rc;
  }
  const int64_t c0 = (int64_t)d->sc[LULESH_S_CYCLE];
  state_to_device_mirror(d);  // no cycle limit: the segments count the cycles
  ACK(cudaMemcpyAsync(d->dd.st, d->hst, sizeof(DevState), cudaMemcpyHostToDevice, s));
  // the plain segments read the force geometry the kinematics kernel stores;
  // the taping kernels form their own, so after the gradient (the domain left
  // at the final state) it has to be formed again
  ensure_geometry(d);
  d->geo_valid = false;
  for (int k = 0; k < nplan; ++k) {
    copy_state_from_domain(a, a->ckpts[k], s);
    ACK(cudaMemcpyAsync(a->ckpt_st + k, d->dd.st, sizeof(DevState), cudaMemcpyDeviceToDevice, s));
    if (k < first_taped) {
      ACK(cudaGraphLaunch(a->fwd_graph, s));
    } else {
      const int n = k < nplan - 1 ? K : last_len;
      const int x = plan == kTwo ? (k & 1) : 0;
      if (!one && n == K) {
        ACK(cudaGraphLaunch(a->rec_graph[x], s));
      } else if ((rc = queue_recompute(set_of(k), n, rev_of(k), s))) {
        return rc;
      }
    }
  }
  ACK(cudaGetLastError());
  ACK(cudaMemcpyAsync(d->hst, d->dd.st, sizeof(DevState), cudaMemcpyDeviceToHost, s));
  ACK(cudaStreamSynchronize(s));
  state_from_device_mirror(d);
  const int64_t done = (int64_t)d->sc[LULESH_S_CYCLE] - c0;
  // segments that ran (a run that reached stoptime leaves later ones empty)
  a->seg_len.clear();
  for (int k = 0; k < nplan; ++k) {
    const int64_t cap = k < nplan - 1 ? K : last_len;
    const int64_t len = std::max<int64_t>(0, std::min<int64_t>(cap, done - (int64_t)k * K));
    if (len == 0) break;
    a->seg_len.push_back((int)len);
  }
  const int nseg = (int)a->seg_len.size();
  if (d->status) { out.status = d->status; out.cycles = done; if (res) *res = out; return d->status; }
  auto t1 = std::chrono::steady_clock::now();
  out.cycles = done;
  out.checkpoints = nseg;
  if ((rc = objective(a, true, &out.loss))) return rc;
  copy_state_from_domain(a, a->final_state, s);
  const Scalars5 final_sc = get_scalars(d);
  // ---- reverse sweep ----
  ACK(cudaMemsetAsync(a->dsc, 0, sizeof(AdjScal), s));
  // the force-transpose inputs the first transposed cycle's ka_kinematics
  // reads (no cycle after it): zero
  ACK(cudaMemsetAsync(a->ad.fV, 0, 24 * sizeof(double) * (size_t)a->E, s));
  ACK(cudaMemsetAsync(a->ad.sLdv, 0, 24 * sizeof(double) * (size_t)a->E, s));
  ACK(cudaMemsetAsync(a->ad.sLhm, 0, 12 * sizeof(double) * (size_t)a->E, s));
  ACK(cudaMemsetAsync(a->ad.sLU, 0, 15 * sizeof(double) * (size_t)a->E, s));
  auto recomputed = [&](int k) { return k < first_taped; };
  auto enqueue_R = [&](int k) -> int {
    const int x = plan == kTwo ? (k & 1) : 0, n = a->seg_len[k];
    if (plan == kTwo && k + 2 <= nseg - 1) ACK(cudaStreamWaitEvent(rs, a->ev_free[x], 0));
    copy_state_to_domain(a, a->ckpts[k], rs);
    ACK(cudaMemcpyAsync(d->dd.st, a->ckpt_st + k, sizeof(DevState), cudaMemcpyDeviceToDevice, rs));
    if (!one && n == K) ACK(cudaGraphLaunch(a->rec_graph[x], rs));
    else if (const int r = queue_recompute(a->sets[x], n, rev_of(k), rs)) return r;
    if (pipe) ACK(cudaEventRecord(a->ev_ready[x], rs));
    return LULESH_OK;
  };
  auto enqueue_T = [&](int k) -> int {
    const int x = plan == kTwo ? (k & 1) : 0, n = a->seg_len[k];
    if (pipe && recomputed(k)) ACK(cudaStreamWaitEvent(tst, a->ev_ready[x], 0));
    if (!one && n == K) ACK(cudaGraphLaunch(a->tr_graph[x], tst));
    else if (const int r = queue_transpose(a->sets[x], n, rev_of(k), tst)) return r;
    if (pipe) ACK(cudaEventRecord(a->ev_free[x], tst));
    return LULESH_OK;
  };
  if (pipe) {
    // both streams start once the objective and the final state are taken
    ACK(cudaEventRecord(a->ev_start, s));
    ACK(cudaStreamWaitEvent(rs, a->ev_start, 0));
    ACK(cudaStreamWaitEvent(tst, a->ev_start, 0));
    if (nseg > 0 && recomputed(nseg - 1) && (rc = enqueue_R(nseg - 1))) return rc;
  }
  for (int k = nseg - 1; k >= 0; --k) {
    if (plan == kSeq) {
      if (recomputed(k) && (rc = enqueue_R(k))) return rc;
      if ((rc = enqueue_T(k))) return rc;
    } else if (plan == kTwo) {
      if (k >= 1 && recomputed(k - 1) && (rc = enqueue_R(k - 1))) return rc;
      if ((rc = enqueue_T(k))) return rc;
    } else {
      if ((rc = enqueue_T(k))) return rc;
      if (k >= 1 && recomputed(k - 1) && (rc = enqueue_R(k - 1))) return rc;
    }
    ACK(cudaGetLastError());
  }
  if (pipe) {
    ACK(cudaEventRecord(a->ev_done, tst));
    ACK(cudaStreamWaitEvent(s, a->ev_done, 0));
  }
  // the first cycle's force transpose: its positions (segment 0's first
  // tape), then both force corner buffers onto the node adjoints; a run that
  // took no cycle has no tape and nothing to add
  if (nseg > 0) {
    TapeSet& t0 = set_of(0);
    const bool r0 = rev_of(0);
    set_cycle_pointers(a, t0.slots[sslot(r0, 0)], t0.slots[sslot(r0, 1)], t0.tape[tslot(r0, 0)]);
    a->ad.diag0 = t0.diag0;
    first_cycle_force_geo(a, s);
    ka_gather_corners<<<(a->N + kAdjBlock - 1) / kAdjBlock, kAdjBlock, 0, s>>>(a->ad);
  }
  copy_state_to_domain(a, a->final_state, s);
  AdjScal hsc;
  ACK(cudaMemcpyAsync(&hsc, a->dsc, sizeof(AdjScal), cudaMemcpyDeviceToHost, s));
  ACK(cudaStreamSynchronize(s));
  set_scalars(d, final_sc);
  state_to_device_mirror(d);
  ACK(cudaMemcpy(d->dd.st, d->hst, sizeof(DevState), cudaMemcpyHostToDevice));
  auto t2 = std::chrono::steady_clock::now();
  out.grad_hgcoef = hsc.Lhg;
  out.sweep = plan;
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
