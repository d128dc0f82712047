// Batched ensemble of independent Sedov problems (C ABI: lulesh_ens_*).
//
// Instances are packed into one element and one node index space (instance
// i owns elements [eoff[i], eoff[i+1]) and nodes [noff[i], noff[i+1])), with
// connectivity, neighbour and corner indices shifted into the packed space.
// The step kernels are the single-problem kernels in their ensemble
// instantiation: each thread reads its element's or node's instance for dt,
// status and hgcoef, and the dt minima are reduced per instance. A run is
// one launch of a captured CUDA graph of the whole run ([per-instance
// timeIncrement!, force, node, kinematics, material] per cycle; runs longer
// than kMaxGraphCycles launch it again until every instance has stopped);
// dt never leaves the device.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <random>
#include <thread>
#include <vector>

#include "../../include/lulesh_gb300.h"
#include "lulesh_arena.h"
#include "lulesh_device.cuh"
#include "lulesh_handle.h"
#include "lulesh_internal.h"
#include "lulesh_trace.h"
#include "lulesh_kernels.h"
#include "lulesh_setup.h"

using namespace lulesh;

namespace {

// a run's graph covers up to this many cycles; a longer run relaunches it
constexpr int kMaxGraphCycles = 512;

int cuda_rc(cudaError_t e) {
  if (e == cudaSuccess) return LULESH_OK;
  std::fprintf(stderr, "liblulesh_gb300 (ensemble): CUDA error %s\n", cudaGetErrorString(e));
  return LULESH_ERR_CUDA;
}
#define ECK(call) do { int rc_ = cuda_rc(call); if (rc_) return rc_; } while (0)

// The reference's parameters (src/domain.jl:663-701), shared by all instances.
Params reference_params() {
  Params p;
  std::memset(&p, 0, sizeof p);  // padding too: parameter sets are compared bytewise
  p.u_cut = 1.0e-7; p.hgcoef = 3.0; p.qstop = 1.0e+12; p.monoq_max_slope = 1.0;
  p.monoq_limiter_mult = 2.0; p.e_cut = 1.0e-7; p.p_cut = 1.0e-7; p.q_cut = 1.0e-7;
  p.v_cut = 1.0e-10; p.qlc_monoq = 0.5; p.qqc_monoq = 2.0 / 3.0; p.qqc = 2.0;
  p.eosvmax = 1.0e+9; p.eosvmin = 1.0e-9; p.pmin = 0.0; p.emin = -1.0e+15; p.dvovmax = 0.1;
  p.refdens = 1.0; p.dtfixed = -1.0e-6; p.deltatimemultlb = 1.1; p.deltatimemultub = 1.2;
  p.stoptime = 1.0e-2; p.dtmax = 1.0e-2;
  finish_params(p);
  return p;
}

void decode(unsigned bits, int32_t* status, int32_t* site) { lulesh::decode_status(bits, status, site); }

// The mutable per-run fields, snapshotted at creation for reset().
struct Mutable {
  double** dev;
  bool node;
};

}  // namespace

struct lulesh_ensemble {
  int n = 0, mode = 0, device = 0;
  std::vector<lulesh_instance> inst;
  std::vector<int64_t> eoff, noff;
  int64_t E = 0, N = 0;
  DevDomain dd{};
  Params prm{};
  Tuning tuning;
  void* arena = nullptr;
  void* snap = nullptr;  // initial x,y,z,xd,yd,zd (N each) and e,p,q,v,ss (E each)
  cudaStream_t stream = nullptr;
  DevState* hst = nullptr;  // pinned, n entries
  std::vector<DevState> init_state;
  cudaGraphExec_t graph = nullptr;
  int64_t graph_key = -1;
  bool geo_valid = false;  // dd.nextGeo holds the force geometry of the current positions
};

static double** mutable_node_fields(DevDomain& d, int k) {
  double** f[6] = {&d.x, &d.y, &d.z, &d.xd, &d.yd, &d.zd};
  return f[k];
}
static double** mutable_elem_fields(DevDomain& d, int k) {
  double** f[5] = {&d.e, &d.p, &d.q, &d.v, &d.ss};
  return f[k];
}

static int snapshot_copy(lulesh_ensemble* s, bool save) {
  char* p = static_cast<char*>(s->snap);
  const size_t nb = (size_t)s->N * sizeof(double), eb = (size_t)s->E * sizeof(double);
  for (int k = 0; k < 6; ++k, p += nb) {
    double* f = *mutable_node_fields(s->dd, k);
    ECK(cudaMemcpyAsync(save ? (void*)p : (void*)f, save ? (const void*)f : (const void*)p, nb,
                        cudaMemcpyDeviceToDevice, s->stream));
  }
  for (int k = 0; k < 5; ++k, p += eb) {
    double* f = *mutable_elem_fields(s->dd, k);
    ECK(cudaMemcpyAsync(save ? (void*)p : (void*)f, save ? (const void*)f : (const void*)p, eb,
                        cudaMemcpyDeviceToDevice, s->stream));
  }
  return LULESH_OK;
}

static int upload_states(lulesh_ensemble* s) {
  for (int i = 0; i < s->n; ++i) s->hst[i] = s->init_state[i];
  ECK(cudaMemcpyAsync(s->dd.st, s->hst, sizeof(DevState) * s->n, cudaMemcpyHostToDevice, s->stream));
  ECK(cudaStreamSynchronize(s->stream));
  return LULESH_OK;
}

static void drop_graph(lulesh_ensemble* s) {
  if (s->graph) cudaGraphExecDestroy(s->graph);
  s->graph = nullptr;
  s->graph_key = -1;
}

static void launch_cycle(lulesh_ensemble* s) {
  launch_time_increment(s->dd.st, s->n, s->prm, s->stream);
  launch_force(s->dd, s->prm, s->tuning, s->stream);
  launch_node(s->dd, s->prm, false, s->tuning, s->stream);
  launch_kinematics(s->dd, s->prm, false, s->tuning, s->stream);
  launch_material(s->dd, s->prm, false, s->tuning, s->stream);
}

extern "C" {

int lulesh_ens_partition(const lulesh_instance* in, int32_t n, int32_t parts, int32_t* part_of) {
  if (!in || !part_of || n < 0 || parts < 1) return LULESH_ERR_ARGUMENT;
  std::vector<int> order(n);
  for (int i = 0; i < n; ++i) {
    if (in[i].nx < 1) return LULESH_ERR_ARGUMENT;
    order[i] = i;
  }
  auto cost = [&](int i) { return (double)in[i].nx * in[i].nx * in[i].nx; };
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost(a) > cost(b); });
  std::vector<double> load(parts, 0.0);
  for (int i : order) {
    int best = 0;
    for (int p = 1; p < parts; ++p)
      if (load[p] < load[best]) best = p;
    part_of[i] = best;
    load[best] += cost(i);
  }
  return LULESH_OK;
}

int lulesh_ens_sedov_instances(uint64_t seed, int32_t n, int32_t nx_min, int32_t nx_max,
                               lulesh_instance* out) {
  if (!out || n < 1 || nx_min < 1 || nx_max < nx_min) return LULESH_ERR_ARGUMENT;
  std::mt19937_64 rng(seed);
  auto unit = [&]() { return (double)(rng() >> 11) * (1.0 / 9007199254740992.0); };  // [0, 1)
  for (int i = 0; i < n; ++i) {
    lulesh_instance& a = out[i];
    a.nx = nx_min + (int32_t)(rng() % (uint64_t)(nx_max - nx_min + 1));
    const double scale = (double)a.nx / 45.0;
    const double factor = std::exp(std::log(0.5) + unit() * (std::log(2.0) - std::log(0.5)));
    a.einit = 3.948746e+7 * scale * scale * scale * factor;
    a.hgcoef = 2.0 + 2.0 * unit();
    a.nr = (rng() & 1u) ? 11 : 1;
    a.balance = 1;
    a.cost = 1;
    a.region_seed = (uint64_t)i;
  }
  return LULESH_OK;
}

int lulesh_ens_create(const lulesh_instance* instances, int32_t n, int32_t mode, int32_t device,
                      lulesh_ensemble** out) {
  if (!instances || !out || n < 1 || mode < 0 || mode > 7) return LULESH_ERR_ARGUMENT;
  *out = nullptr;
  int64_t E = 0, N = 0;
  std::vector<int64_t> eoff(n + 1), noff(n + 1);
  for (int i = 0; i < n; ++i) {
    const lulesh_instance& a = instances[i];
    if (a.nx < 1 || a.nx > 640 || a.nr < 1 || a.balance < 0 || a.cost < 0 || !(a.hgcoef >= 0.0))
      return LULESH_ERR_ARGUMENT;
    eoff[i] = E;
    noff[i] = N;
    E += (int64_t)a.nx * a.nx * a.nx;
    N += (int64_t)(a.nx + 1) * (a.nx + 1) * (a.nx + 1);
  }
  eoff[n] = E;
  noff[n] = N;
  if (8 * E > INT_MAX || N > INT_MAX) return LULESH_ERR_ARGUMENT;  // 32-bit packed indices
  if (cudaSetDevice(device) != cudaSuccess) return LULESH_ERR_CUDA;

  lulesh_ensemble* s = new (std::nothrow) lulesh_ensemble();
  if (!s) return LULESH_ERR_MEMORY;
  s->n = n; s->mode = mode; s->device = device;
  s->inst.assign(instances, instances + n);
  s->eoff = eoff; s->noff = noff; s->E = E; s->N = N;
  s->prm = reference_params();
  auto fail = [&](int code) { lulesh_ens_destroy(s); return code; };

  DevDomain& dd = s->dd;
  const size_t bytes = layout(dd, nullptr, E, N, false, n);
  if (cudaMalloc(&s->arena, bytes) != cudaSuccess) { cudaGetLastError(); return fail(LULESH_ERR_MEMORY); }
  layout(dd, static_cast<char*>(s->arena), E, N, false, n);
  dd.E = (int)E; dd.N = (int)N; dd.nx = 0; dd.mode = mode;
  if (cudaMalloc(&s->snap, (6 * N + 5 * E) * sizeof(double)) != cudaSuccess) { cudaGetLastError(); return fail(LULESH_ERR_MEMORY); }
  if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) return fail(LULESH_ERR_CUDA);
  if (cudaMallocHost(&s->hst, sizeof(DevState) * n) != cudaSuccess) return fail(LULESH_ERR_CUDA);

  // host staging of the packed arrays, filled in parallel (instances own disjoint ranges)
  std::vector<double> x(N), y(N), z(N), mass(N), imass(N);
  std::vector<unsigned char> nbc(N, 0);
  std::vector<int> start(N + 1), corners(8 * E), nodelist(8 * E), ninst(N), einst(E);
  std::vector<double> volo(E), ivolo(E), emass(E), ones(E, 1.0), e0(E, 0.0), hg(n);
  std::vector<unsigned int> ebc(E);
  std::vector<int> lxim(E), lxip(E), letam(E), letap(E), lzetam(E), lzetap(E);
  s->init_state.resize(n);
  auto pack = [&](int i) {
    const lulesh_instance& a = s->inst[i];
    HostMesh m;
    build_mesh(m, a.nx, a.nr, a.balance, a.cost, a.region_seed, a.einit);
    const int64_t eo = eoff[i], no = noff[i], Ei = m.E, Ni = m.N;
    for (int64_t k = 0; k < Ni; ++k) {
      x[no + k] = m.x[k]; y[no + k] = m.y[k]; z[no + k] = m.z[k];
      mass[no + k] = m.nodalMass[k];
      imass[no + k] = 1.0 / m.nodalMass[k];
      start[no + k] = (int)(m.nodeElemStart[k] + 8 * eo);
      ninst[no + k] = i;
    }
    for (int v : m.symmX) nbc[no + v] |= 1u;
    for (int v : m.symmY) nbc[no + v] |= 2u;
    for (int v : m.symmZ) nbc[no + v] |= 4u;
    for (int64_t j = 0; j < 8 * Ei; ++j) {
      const int64_t val = m.cornerList[j], c = val / Ei, e = val % Ei;
      corners[8 * eo + j] = (int)(c * E + eo + e);
    }
    for (int64_t e = 0; e < Ei; ++e) {
      for (int c = 0; c < 8; ++c) nodelist[c * E + eo + e] = (int)(no + m.nodelist[8 * e + c]);
      volo[eo + e] = m.volo[e];
      ivolo[eo + e] = 1.0 / m.volo[e];
      emass[eo + e] = m.elemMass[e];
      ebc[eo + e] = m.elemBC[e];
      lxim[eo + e] = (int)(m.lxim[e] + eo); lxip[eo + e] = (int)(m.lxip[e] + eo);
      letam[eo + e] = (int)(m.letam[e] + eo); letap[eo + e] = (int)(m.letap[e] + eo);
      lzetam[eo + e] = (int)(m.lzetam[e] + eo); lzetap[eo + e] = (int)(m.lzetap[e] + eo);
      einst[eo + e] = i;
    }
    e0[eo] = m.einit;
    hg[i] = a.hgcoef;
    DevState& st = s->init_state[i];
    std::memset(&st, 0, sizeof(st));
    st.time = 0.0; st.deltatime = m.deltatime; st.dtcourant = 1e20; st.dthydro = 1e20; st.cycle = 0;
    st.acc_courant = kInfBits; st.acc_hydro = kInfBits; st.status = 0; st.done = 0; st.first = 1;
    st.num_iters = LLONG_MAX;
  };
  {
    const int workers = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    std::vector<std::thread> pool;
    for (int w = 0; w < workers; ++w)
      pool.emplace_back([&, w]() { for (int i = w; i < n; i += workers) pack(i); });
    for (auto& t : pool) t.join();
  }
  start[N] = (int)(8 * E);

  cudaStream_t st = s->stream;
  auto up = [&](void* dst, const void* src, size_t b) { return cudaMemcpyAsync(dst, src, b, cudaMemcpyHostToDevice, st); };
  cudaError_t err = cudaSuccess;
  const size_t nd = N * sizeof(double), ed = E * sizeof(double), ei = E * sizeof(int);
  if ((err = cudaMemsetAsync(s->arena, 0, bytes, st)) == cudaSuccess &&
      (err = up(dd.x, x.data(), nd)) == cudaSuccess && (err = up(dd.y, y.data(), nd)) == cudaSuccess &&
      (err = up(dd.z, z.data(), nd)) == cudaSuccess && (err = up(dd.nodalMass, mass.data(), nd)) == cudaSuccess &&
      (err = up(dd.inv_nodalMass, imass.data(), nd)) == cudaSuccess &&
      (err = up(dd.nodeBC, nbc.data(), N)) == cudaSuccess &&
      (err = up(dd.nodeElemStart, start.data(), (N + 1) * sizeof(int))) == cudaSuccess &&
      (err = up(dd.cornerList, corners.data(), 8 * ei)) == cudaSuccess &&
      (err = up(dd.nodelist, nodelist.data(), 8 * ei)) == cudaSuccess &&
      (err = up(dd.volo, volo.data(), ed)) == cudaSuccess && (err = up(dd.inv_volo, ivolo.data(), ed)) == cudaSuccess &&
      (err = up(dd.elemMass, emass.data(), ed)) == cudaSuccess && (err = up(dd.v, ones.data(), ed)) == cudaSuccess &&
      (err = up(dd.e, e0.data(), ed)) == cudaSuccess &&
      (err = up(dd.elemBC, ebc.data(), E * sizeof(unsigned))) == cudaSuccess &&
      (err = up(dd.lxim, lxim.data(), ei)) == cudaSuccess && (err = up(dd.lxip, lxip.data(), ei)) == cudaSuccess &&
      (err = up(dd.letam, letam.data(), ei)) == cudaSuccess && (err = up(dd.letap, letap.data(), ei)) == cudaSuccess &&
      (err = up(dd.lzetam, lzetam.data(), ei)) == cudaSuccess && (err = up(dd.lzetap, lzetap.data(), ei)) == cudaSuccess &&
      (err = up((void*)dd.elemInst, einst.data(), ei)) == cudaSuccess &&
      (err = up((void*)dd.nodeInst, ninst.data(), N * sizeof(int))) == cudaSuccess &&
      (err = up((void*)dd.instHg, hg.data(), n * sizeof(double))) == cudaSuccess)
    err = cudaStreamSynchronize(st);
  if (err != cudaSuccess) return fail(cuda_rc(err));
  int rc;
  if ((rc = snapshot_copy(s, true)) || (rc = upload_states(s))) return fail(rc);
  *out = s;
  return LULESH_OK;
}

int lulesh_ens_destroy(lulesh_ensemble* s) {
  if (!s) return LULESH_ERR_ARGUMENT;
  cudaSetDevice(s->device);
  if (s->stream) cudaStreamSynchronize(s->stream);
  drop_graph(s);
  if (s->hst) cudaFreeHost(s->hst);
  if (s->snap) cudaFree(s->snap);
  if (s->arena) cudaFree(s->arena);
  if (s->stream) cudaStreamDestroy(s->stream);
  delete s;
  return LULESH_OK;
}

int lulesh_ens_reset(lulesh_ensemble* s) {
  if (!s) return LULESH_ERR_ARGUMENT;
  ECK(cudaSetDevice(s->device));
  int rc = snapshot_copy(s, false);
  if (rc) return rc;
  s->geo_valid = false;
  return upload_states(s);
}

int lulesh_ens_run(lulesh_ensemble* s, int64_t num_iters) {
  if (!s) return LULESH_ERR_ARGUMENT;
  TraceRange trace("lulesh_ens_run");
  ECK(cudaSetDevice(s->device));
  cudaStream_t st = s->stream;
  // every instance becomes runnable again (first = 1): benchmark.jl semantics per instance
  ECK(cudaMemcpyAsync(s->hst, s->dd.st, sizeof(DevState) * s->n, cudaMemcpyDeviceToHost, st));
  ECK(cudaStreamSynchronize(st));
  int64_t budget = 1;
  for (int i = 0; i < s->n; ++i) {
    DevState& d = s->hst[i];
    if (dt_registers(d.acc_courant)) std::memcpy(&d.dtcourant, &d.acc_courant, 8);
    if (dt_registers(d.acc_hydro)) std::memcpy(&d.dthydro, &d.acc_hydro, 8);
    d.acc_courant = kInfBits;
    d.acc_hydro = kInfBits;
    if (d.status == 0u) d.done = 0;
    d.first = 1;
    d.num_iters = num_iters;
    budget = std::max<int64_t>(budget, num_iters - d.cycle);
  }
  ECK(cudaMemcpyAsync(s->dd.st, s->hst, sizeof(DevState) * s->n, cudaMemcpyHostToDevice, st));
  // the force kernel's stored geometry (an instance that stopped on an error
  // keeps its positions until a reset, which clears this)
  if (!s->geo_valid && s->tuning.geo == 0) {
    launch_geometry(s->dd, st);
    s->geo_valid = true;
  }
  // one graph of the whole run (up to kMaxGraphCycles cycles), kept for the
  // next run of the same length; the run limit lives in the device state and
  // cycles past an instance's stop are no-ops for it
  const int64_t glen = std::min<int64_t>(budget, kMaxGraphCycles);
  if (!s->graph || s->graph_key != glen) {
    drop_graph(s);
    cudaGraph_t g;
    ECK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    for (int64_t c = 0; c < glen; ++c) launch_cycle(s);
    ECK(cudaStreamEndCapture(st, &g));
    cudaError_t e = cudaGraphInstantiate(&s->graph, g, 0);
    cudaGraphDestroy(g);
    ECK(e);
    s->graph_key = glen;
  }
  int64_t launched = 0;
  for (;;) {
    ECK(cudaGraphLaunch(s->graph, st));
    launched += glen;
    ECK(cudaMemcpyAsync(s->hst, s->dd.st, sizeof(DevState) * s->n, cudaMemcpyDeviceToHost, st));
    ECK(cudaStreamSynchronize(st));
    bool all_done = true;
    for (int i = 0; i < s->n && all_done; ++i) all_done = s->hst[i].done != 0;
    if (all_done || launched >= budget) break;
  }
  if (s->tuning.geo != 0) s->geo_valid = false;  // the inline split stores no geometry
  for (int i = 0; i < s->n; ++i) {
    int32_t status, site;
    decode(s->hst[i].status, &status, &site);
    if (status) return status;
  }
  return LULESH_OK;
}

int lulesh_ens_sizes(const lulesh_ensemble* s, int32_t* n, int64_t* te, int64_t* tn) {
  if (!s) return LULESH_ERR_ARGUMENT;
  if (n) *n = s->n;
  if (te) *te = s->E;
  if (tn) *tn = s->N;
  return LULESH_OK;
}

int lulesh_ens_get_scalars(const lulesh_ensemble* s, int32_t i, lulesh_scalars* out) {
  if (!s || !out || i < 0 || i >= s->n) return LULESH_ERR_ARGUMENT;
  if (cudaSetDevice(s->device) != cudaSuccess) return LULESH_ERR_CUDA;
  DevState d;
  if (cudaMemcpy(&d, s->dd.st + i, sizeof(DevState), cudaMemcpyDeviceToHost) != cudaSuccess) return LULESH_ERR_CUDA;
  double dtc = d.dtcourant, dth = d.dthydro;
  if (dt_registers(d.acc_courant)) std::memcpy(&dtc, &d.acc_courant, 8);
  if (dt_registers(d.acc_hydro)) std::memcpy(&dth, &d.acc_hydro, 8);
  out->time = d.time;
  out->deltatime = d.deltatime;
  out->dtcourant = dtc;
  out->dthydro = dth;
  out->cycle = d.cycle;
  decode(d.status, &out->status, &out->site);
  return LULESH_OK;
}

static double* ens_field(lulesh_ensemble* s, int32_t f, bool* node) {
  DevDomain& d = s->dd;
  *node = f >= LULESH_F_X;
  switch (f) {
    case LULESH_F_E: return d.e;
    case LULESH_F_P: return d.p;
    case LULESH_F_Q: return d.q;
    case LULESH_F_V: return d.v;
    case LULESH_F_VOLO: return d.volo;
    case LULESH_F_DELV: return d.delv;
    case LULESH_F_VDOV: return d.vdov;
    case LULESH_F_AREALG: return d.arealg;
    case LULESH_F_SS: return d.ss;
    case LULESH_F_ELEMMASS: return d.elemMass;
    case LULESH_F_VNEW: return d.vnew;
    case LULESH_F_DELV_XI: return d.delv_xi;
    case LULESH_F_DELV_ETA: return d.delv_eta;
    case LULESH_F_DELV_ZETA: return d.delv_zeta;
    case LULESH_F_DELX_XI: return d.delx_xi;
    case LULESH_F_DELX_ETA: return d.delx_eta;
    case LULESH_F_DELX_ZETA: return d.delx_zeta;
    case LULESH_F_X: return d.x;
    case LULESH_F_Y: return d.y;
    case LULESH_F_Z: return d.z;
    case LULESH_F_XD: return d.xd;
    case LULESH_F_YD: return d.yd;
    case LULESH_F_ZD: return d.zd;
    case LULESH_F_NODALMASS: return d.nodalMass;
    default: return nullptr;
  }
}

int lulesh_ens_field_length(const lulesh_ensemble* s, int32_t i, int32_t f, int64_t* count) {
  if (!s || !count || i < 0 || i >= s->n) return LULESH_ERR_ARGUMENT;
  bool node;
  if (!ens_field(const_cast<lulesh_ensemble*>(s), f, &node)) return LULESH_ERR_ARGUMENT;
  *count = node ? s->noff[i + 1] - s->noff[i] : s->eoff[i + 1] - s->eoff[i];
  return LULESH_OK;
}

int lulesh_ens_download_field(lulesh_ensemble* s, int32_t i, int32_t f, void* host, int64_t count) {
  if (!s || !host || i < 0 || i >= s->n) return LULESH_ERR_ARGUMENT;
  bool node;
  double* p = ens_field(s, f, &node);
  if (!p) return LULESH_ERR_ARGUMENT;
  const int64_t off = node ? s->noff[i] : s->eoff[i];
  const int64_t len = node ? s->noff[i + 1] - off : s->eoff[i + 1] - off;
  if (count != len) return LULESH_ERR_ARGUMENT;
  ECK(cudaSetDevice(s->device));
  ECK(cudaMemcpyAsync(host, p + off, len * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  ECK(cudaStreamSynchronize(s->stream));
  return LULESH_OK;
}

int lulesh_ens_get_stream(lulesh_ensemble* s, void** stream) {
  if (!s || !stream) return LULESH_ERR_ARGUMENT;
  *stream = (void*)s->stream;
  return LULESH_OK;
}

int lulesh_ens_get_tuning(const lulesh_ensemble* s, lulesh_tuning* out) {
  if (!s || !out) return LULESH_ERR_ARGUMENT;
  out->force_block = s->tuning.force;
  out->node_block = s->tuning.node;
  out->kin_block = s->tuning.kin;
  out->mat_block = s->tuning.mat;
  out->geometry = s->tuning.geo;
  return LULESH_OK;
}

static bool valid_tuning(const lulesh_tuning* t) {
  auto elem_ok = [](int b) { return b == 64 || b == 128 || b == 256; };
  return t && elem_ok(t->force_block) && elem_ok(t->kin_block) && elem_ok(t->mat_block) &&
         (t->node_block == 128 || t->node_block == 256 || t->node_block == 512) &&
         (t->geometry == 0 || t->geometry == 1);
}

int lulesh_ens_set_tuning(lulesh_ensemble* s, const lulesh_tuning* t) {
  if (!s || !valid_tuning(t)) return LULESH_ERR_ARGUMENT;
  s->tuning.force = t->force_block;
  s->tuning.node = t->node_block;
  s->tuning.kin = t->kin_block;
  s->tuning.mat = t->mat_block;
  if (s->tuning.geo != t->geometry) s->geo_valid = false;
  s->tuning.geo = t->geometry;
  drop_graph(s);
  return LULESH_OK;
}

int lulesh_ens_autotune(lulesh_ensemble* s, int32_t cycles, lulesh_tuning* chosen) {
  if (!s) return LULESH_ERR_ARGUMENT;
  ECK(cudaSetDevice(s->device));
  // tune from the initial state, then return to it
  int rc = lulesh_ens_reset(s);
  if (rc) return rc;
  for (int i = 0; i < s->n; ++i) { s->hst[i] = s->init_state[i]; s->hst[i].first = 0; }
  ECK(cudaMemcpyAsync(s->dd.st, s->hst, sizeof(DevState) * s->n, cudaMemcpyHostToDevice, s->stream));
  launch_geometry(s->dd, s->stream);
  ECK(autotune_blocks(s->dd, s->prm, false, s->n, s->stream, cycles, s->tuning));
  drop_graph(s);
  if ((rc = lulesh_ens_reset(s))) return rc;
  return chosen ? lulesh_ens_get_tuning(s, chosen) : LULESH_OK;
}

}  // extern "C"
