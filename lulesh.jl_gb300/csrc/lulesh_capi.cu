// C ABI of the plain (single problem) path: see include/lulesh_gb300.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/lulesh_gb300.h"
#include "lulesh_internal.h"
#include "lulesh_kernels.h"
#include "lulesh_setup.h"
#include "lulesh_arena.h"
#include "lulesh_handle.h"
#include "lulesh_device.cuh"
#include "lulesh_trace.h"

using namespace lulesh;

namespace {

const char* const kKernelNames[kNumKernels] = {"k_time_increment", "k_force", "k_node",
                                               "k_kinematics", "k_material"};
constexpr int kGraphCycles = 16;   // cycles per captured graph
constexpr int kTimingCycles = 256; // cycles of kernel events held before a read-back
constexpr int kPollLaunches = 4;   // graph launches between host polls
constexpr int kPollCyclesTimed = 64;  // timed (graph-less) cycles between host polls

}  // namespace

static int cuda_fail(cudaError_t e) {
  if (e == cudaSuccess) return LULESH_OK;
  std::fprintf(stderr, "liblulesh_gb300: CUDA error %s\n", cudaGetErrorString(e));
  return LULESH_ERR_CUDA;
}
#define CK(call) do { int rc_ = cuda_fail(call); if (rc_) return rc_; } while (0)

Params lulesh::make_params(const lulesh_domain* d) {
  Params p;
  std::memset(&p, 0, sizeof p);  // padding too: parameter sets are compared bytewise
  p.u_cut = d->sc[LULESH_S_U_CUT];
  p.hgcoef = d->sc[LULESH_S_HGCOEF];
  p.qstop = d->sc[LULESH_S_QSTOP];
  p.monoq_max_slope = d->sc[LULESH_S_MONOQ_MAX_SLOPE];
  p.monoq_limiter_mult = d->sc[LULESH_S_MONOQ_LIMITER_MULT];
  p.e_cut = d->sc[LULESH_S_E_CUT];
  p.p_cut = d->sc[LULESH_S_P_CUT];
  p.q_cut = d->sc[LULESH_S_Q_CUT];
  p.v_cut = d->sc[LULESH_S_V_CUT];
  p.qlc_monoq = d->sc[LULESH_S_QLC_MONOQ];
  p.qqc_monoq = d->sc[LULESH_S_QQC_MONOQ];
  p.qqc = d->sc[LULESH_S_QQC];
  p.eosvmax = d->sc[LULESH_S_EOSVMAX];
  p.eosvmin = d->sc[LULESH_S_EOSVMIN];
  p.pmin = d->sc[LULESH_S_PMIN];
  p.emin = d->sc[LULESH_S_EMIN];
  p.dvovmax = d->sc[LULESH_S_DVOVMAX];
  p.refdens = d->sc[LULESH_S_REFDENS];
  p.dtfixed = d->sc[LULESH_S_DTFIXED];
  p.deltatimemultlb = d->sc[LULESH_S_DELTATIMEMULTLB];
  p.deltatimemultub = d->sc[LULESH_S_DELTATIMEMULTUB];
  p.stoptime = d->sc[LULESH_S_STOPTIME];
  p.dtmax = d->sc[LULESH_S_DTMAX];
  finish_params(p);
  return p;
}

// The stored force geometry is needed before a step of the stored split; the
// other split forms it in k_force and leaves d.nextGeo untouched (stale).
void lulesh::ensure_geometry(lulesh_domain* d) {
  if (d->geo_valid || d->tuning.geo != 0) return;
  launch_geometry(d->dd, d->stream);
  d->geo_valid = true;
}

// Maps kernel status bits to (status, site) in the reference's check order.
void lulesh::decode_status(unsigned bits, int32_t* status, int32_t* site) {
  *status = LULESH_OK;
  *site = LULESH_SITE_NONE;
  if (!bits) return;
  if (bits & ST_INDEX) { *status = LULESH_ERR_INDEX; return; }
  if (bits & ST_EARLY) { *status = LULESH_ERR_VOLUME; *site = LULESH_SITE_EARLY; return; }
  if (bits & ST_HOURGLASS) { *status = LULESH_ERR_VOLUME; *site = LULESH_SITE_HOURGLASS; return; }
  if (bits & ST_KINEMATICS) { *status = LULESH_ERR_VOLUME; *site = LULESH_SITE_KINEMATICS; return; }
  if (bits & ST_BAD_BC) { *status = LULESH_ERR_BAD_BC; return; }
  if (bits & ST_QSTOP) { *status = LULESH_ERR_QSTOP; return; }
  if (bits & ST_MATERIAL) { *status = LULESH_ERR_VOLUME; *site = LULESH_SITE_MATERIAL; return; }
  if (bits & ST_UPDATE) { *status = LULESH_ERR_VOLUME; *site = LULESH_SITE_UPDATE; return; }
}

void lulesh::state_to_device_mirror(lulesh_domain* d) {
  DevState* s = d->hst;
  s->time = d->sc[LULESH_S_TIME];
  s->deltatime = d->sc[LULESH_S_DELTATIME];
  s->dtcourant = d->sc[LULESH_S_DTCOURANT];
  s->dthydro = d->sc[LULESH_S_DTHYDRO];
  s->cycle = (long long)d->sc[LULESH_S_CYCLE];
  s->acc_courant = kInfBits;
  s->acc_hydro = kInfBits;
  s->status = 0u;
  s->done = 0;
  s->num_iters = LLONG_MAX;  // no cycle limit unless a run sets one
  s->first = 1;
}

void lulesh::state_from_device_mirror(lulesh_domain* d) {
  DevState* s = d->hst;
  d->sc[LULESH_S_TIME] = s->time;
  d->sc[LULESH_S_DELTATIME] = s->deltatime;
  double dtc = s->dtcourant, dth = s->dthydro;
  if (dt_registers(s->acc_courant)) { unsigned long long b = s->acc_courant; std::memcpy(&dtc, &b, 8); }
  if (dt_registers(s->acc_hydro)) { unsigned long long b = s->acc_hydro; std::memcpy(&dth, &b, 8); }
  d->sc[LULESH_S_DTCOURANT] = dtc;
  d->sc[LULESH_S_DTHYDRO] = dth;
  d->sc[LULESH_S_CYCLE] = (double)s->cycle;
  decode_status(s->status, &d->status, &d->site);
}

// ---------------------------------------------------------------------------
// device memory layout
// ---------------------------------------------------------------------------
// (the arena layout is shared with the ensemble: lulesh_arena.h)

template <class T>
static int h2d(T* dst, const T* src, size_t n, cudaStream_t s) {
  CK(cudaMemcpyAsync(dst, src, n * sizeof(T), cudaMemcpyHostToDevice, s));
  return LULESH_OK;
}
template <class T>
static int d2h(T* dst, const T* src, size_t n, cudaStream_t s) {
  CK(cudaMemcpyAsync(dst, src, n * sizeof(T), cudaMemcpyDeviceToHost, s));
  return LULESH_OK;
}

static void set_default_scalars(double* sc) {
  // src/domain.jl:663-701
  sc[LULESH_S_DTFIXED] = -1.0e-6;
  sc[LULESH_S_DELTATIMEMULTLB] = 1.1;
  sc[LULESH_S_DELTATIMEMULTUB] = 1.2;
  sc[LULESH_S_STOPTIME] = 1.0e-2;
  sc[LULESH_S_DTMAX] = 1.0e-2;
  sc[LULESH_S_DTHYDRO] = 1e20;
  sc[LULESH_S_DTCOURANT] = 1e20;
  sc[LULESH_S_TIME] = 0.0;
  sc[LULESH_S_DELTATIME] = 0.0;
  sc[LULESH_S_U_CUT] = 1.0e-7;
  sc[LULESH_S_HGCOEF] = 3.0;
  sc[LULESH_S_QSTOP] = 1.0e+12;
  sc[LULESH_S_MONOQ_MAX_SLOPE] = 1.0;
  sc[LULESH_S_MONOQ_LIMITER_MULT] = 2.0;
  sc[LULESH_S_E_CUT] = 1.0e-7;
  sc[LULESH_S_P_CUT] = 1.0e-7;
  sc[LULESH_S_SS4O3] = 4.0 / 3.0;
  sc[LULESH_S_Q_CUT] = 1.0e-7;
  sc[LULESH_S_V_CUT] = 1.0e-10;
  sc[LULESH_S_QLC_MONOQ] = 0.5;
  sc[LULESH_S_QQC_MONOQ] = 2.0 / 3.0;
  sc[LULESH_S_QQC] = 2.0;
  sc[LULESH_S_EOSVMAX] = 1.0e+9;
  sc[LULESH_S_EOSVMIN] = 1.0e-9;
  sc[LULESH_S_PMIN] = 0.0;
  sc[LULESH_S_EMIN] = -1.0e+15;
  sc[LULESH_S_DVOVMAX] = 0.1;
  sc[LULESH_S_REFDENS] = 1.0;
  sc[LULESH_S_CYCLE] = 0.0;
}

static int upload_node_bc(lulesh_domain* d) {
  std::vector<unsigned char> bc(d->N, 0);
  for (int v : d->symmX) if (v >= 0 && v < d->N) bc[v] |= 1u;
  for (int v : d->symmY) if (v >= 0 && v < d->N) bc[v] |= 2u;
  for (int v : d->symmZ) if (v >= 0 && v < d->N) bc[v] |= 4u;
  int rc = h2d(d->dd.nodeBC, bc.data(), bc.size(), d->stream);
  if (rc) return rc;
  CK(cudaStreamSynchronize(d->stream));
  return LULESH_OK;
}

static void drop_graph(lulesh_domain* d) {
  if (d->graph) cudaGraphExecDestroy(d->graph);
  d->graph = nullptr;
  d->graph_key = -1;
}

// ---------------------------------------------------------------------------
// step launch
// ---------------------------------------------------------------------------
static int collect_times(lulesh_domain* d) {
  if (d->ring_used == 0) return LULESH_OK;
  const int stride = kNumKernels + 1;
  CK(cudaEventSynchronize(d->ring[(d->ring_used - 1) * stride + kNumKernels]));
  for (int c = 0; c < d->ring_used; ++c)
    for (int k = 0; k < kNumKernels; ++k) {
      float ms = 0.f;
      CK(cudaEventElapsedTime(&ms, d->ring[c * stride + k], d->ring[c * stride + k + 1]));
      d->kernel_ms[k] += ms;
    }
  d->ring_used = 0;
  return LULESH_OK;
}

static int ensure_ring(lulesh_domain* d) {
  if (!d->ring.empty()) return LULESH_OK;
  d->ring.assign((size_t)kTimingCycles * (kNumKernels + 1), nullptr);
  for (auto& ev : d->ring) CK(cudaEventCreate(&ev));
  return LULESH_OK;
}

// Launches one cycle's kernels; with timing on, brackets each kernel with
// events from the ring (reading the ring back first when it is full).
static int launch_step(lulesh_domain* d, const Params& prm, bool with_time_increment, bool timed) {
  const bool aux = d->params.keep_aux != 0;
  cudaStream_t s = d->stream;
  cudaEvent_t* ev = nullptr;
  if (timed) {
    int rc = ensure_ring(d);
    if (rc) return rc;
    if (d->ring_used == kTimingCycles && (rc = collect_times(d))) return rc;
    ev = &d->ring[(size_t)d->ring_used * (kNumKernels + 1)];
    d->ring_used += 1;
  }
  if (ev) cudaEventRecord(ev[0], s);
  if (with_time_increment) {
    TraceRange r("timeIncrement!");
    launch_time_increment(d->dd.st, 1, prm, s);
  }
  if (ev) cudaEventRecord(ev[1], s);
  {
    TraceRange r("calcForceForNodes");
    launch_force(d->dd, prm, d->tuning, s);
  }
  if (ev) cudaEventRecord(ev[2], s);
  {
    TraceRange r("calcAccelerationForNodes .. calcPositionForNodes");
    launch_node(d->dd, prm, aux, d->tuning, s);
  }
  if (ev) cudaEventRecord(ev[3], s);
  {
    TraceRange r("calcLagrangeElements + calcMonotonicQGradientsForElems");
    launch_kinematics(d->dd, prm, aux, d->tuning, s);
  }
  if (ev) cudaEventRecord(ev[4], s);
  {
    TraceRange r("calcQForElems .. calcTimeConstraintsForElems");
    launch_material(d->dd, prm, aux, d->tuning, s);
  }
  if (ev) cudaEventRecord(ev[5], s);
  CK(cudaGetLastError());
  return LULESH_OK;
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

void lulesh_default_params(lulesh_params* p, int32_t nx) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->nx = nx;
  p->nr = 11;
  p->balance = 1;
  p->cost = 1;
  p->mode = LULESH_MODE_FAITHFUL;
  p->region_reps = 0;
  p->keep_aux = 0;
  p->device = 0;
  p->region_seed = 0;
}

const char* lulesh_status_string(int32_t status) {
  switch (status) {
    case LULESH_OK: return "ok";
    case LULESH_ERR_VOLUME: return "Volume Error";
    case LULESH_ERR_QSTOP: return "QStopError";
    case LULESH_ERR_BAD_BC: return "Error (invalid elemBC mask)";
    case LULESH_ERR_CUDA: return "CUDA error";
    case LULESH_ERR_TIMEOUT: return "device wait timed out";
    case LULESH_ERR_ARGUMENT: return "bad argument";
    case LULESH_ERR_MEMORY: return "device allocation failed";
    case LULESH_ERR_INDEX: return "index out of range (checked build)";
    default: return "unknown status";
  }
}

const char* lulesh_kernel_name(int32_t index) {
  return (index >= 0 && index < kNumKernels) ? kKernelNames[index] : "";
}

}  // extern "C"

// A handle for the mesh `m` (one block, or packed blocks with their halo plan).
static int create_domain(const lulesh_params* params, HostMesh& m, lulesh_domain** out) {
  const int nx = params->nx;
  CK(cudaSetDevice(params->device));
  lulesh_domain* d = new (std::nothrow) lulesh_domain();
  if (!d) return LULESH_ERR_MEMORY;
  d->params = *params;
  d->E = m.E;
  d->N = m.N;
  set_default_scalars(d->sc);
  d->sc[LULESH_S_DELTATIME] = m.deltatime;

  const bool aux = params->keep_aux != 0;
  DevDomain& dd = d->dd;
  const size_t bytes = layout(dd, nullptr, m.E, m.N, aux, 0, m.Eg, m.nCornerSlot, m.nCornerList);
  cudaError_t err = cudaMalloc(&d->arena, bytes);
  if (err != cudaSuccess) { delete d; cudaGetLastError(); return LULESH_ERR_MEMORY; }
  layout(dd, (char*)d->arena, m.E, m.N, aux, 0, m.Eg, m.nCornerSlot, m.nCornerList);
  dd.E = (int)m.E;
  dd.N = (int)m.N;
  dd.nx = nx;
  dd.mode = params->mode;
  int rc = LULESH_OK;
  auto fail = [&](int code) { lulesh_destroy(d); return code; };
  if ((err = cudaStreamCreateWithFlags(&d->stream, cudaStreamNonBlocking)) != cudaSuccess) return fail(cuda_fail(err));
  if ((err = cudaMallocHost(&d->hst, sizeof(DevState))) != cudaSuccess) return fail(cuda_fail(err));
  if ((err = cudaMemsetAsync(d->arena, 0, bytes, d->stream)) != cudaSuccess) return fail(cuda_fail(err));

  const int64_t E = m.E, N = m.N;
  cudaStream_t s = d->stream;
  // host staging that must outlive the async copies
  std::vector<int> nodelist_cm(8 * E), start(m.nodeElemStart);
  for (int64_t e = 0; e < E; ++e)
    for (int c = 0; c < 8; ++c) nodelist_cm[c * E + e] = m.nodelist[8 * e + c];
  std::vector<double> inv_volo(E), inv_mass(N), ones(E, 1.0), e0(E, 0.0);
  for (int64_t i = 0; i < E; ++i) inv_volo[i] = 1.0 / m.volo[i];
  for (int64_t i = 0; i < N; ++i) inv_mass[i] = 1.0 / m.nodalMass[i];
  e0[0] = m.einit;
  if ((rc = h2d(dd.x, m.x.data(), N, s)) || (rc = h2d(dd.y, m.y.data(), N, s)) ||
      (rc = h2d(dd.z, m.z.data(), N, s)) || (rc = h2d(dd.nodalMass, m.nodalMass.data(), N, s)) ||
      (rc = h2d(dd.inv_nodalMass, inv_mass.data(), N, s)) ||
      (rc = h2d(dd.nodeElemStart, start.data(), N + 1, s)) ||
      (rc = h2d(dd.cornerList, m.cornerList.data(), m.cornerList.size(), s)) ||
      (rc = h2d(dd.nodelist, nodelist_cm.data(), 8 * E, s)) ||
      (rc = h2d(dd.volo, m.volo.data(), E, s)) || (rc = h2d(dd.inv_volo, inv_volo.data(), E, s)) ||
      (rc = h2d(dd.elemMass, m.elemMass.data(), E, s)) || (rc = h2d(dd.v, ones.data(), E, s)) ||
      (rc = h2d(dd.e, e0.data(), E, s)) || (rc = h2d(dd.elemBC, m.elemBC.data(), E, s)) ||
      (rc = h2d(dd.lxim, m.lxim.data(), E, s)) || (rc = h2d(dd.lxip, m.lxip.data(), E, s)) ||
      (rc = h2d(dd.letam, m.letam.data(), E, s)) || (rc = h2d(dd.letap, m.letap.data(), E, s)) ||
      (rc = h2d(dd.lzetam, m.lzetam.data(), E, s)) || (rc = h2d(dd.lzetap, m.lzetap.data(), E, s)))
    return fail(rc);
  if (!m.haloDelvSrc.empty() && (rc = h2d(const_cast<int*>(dd.haloDelvSrc), m.haloDelvSrc.data(), m.haloDelvSrc.size(), s)))
    return fail(rc);
  if (!m.haloCornerSrc.empty() &&
      (rc = h2d(const_cast<int*>(dd.haloCornerSrc), m.haloCornerSrc.data(), m.haloCornerSrc.size(), s)))
    return fail(rc);
  d->blocks_per_edge = m.blocks_per_edge;
  d->elemGlobal = m.elemGlobal;
  d->nodeGlobal = m.nodeGlobal;
  d->haloCornerSrc = m.haloCornerSrc;
  d->symmX = m.symmX; d->symmY = m.symmY; d->symmZ = m.symmZ;
  d->regNumList = m.regNumList; d->regElemlist = m.regElemlist; d->regCSR = m.regCSR;
  d->regReps = m.regReps; d->regSorted = m.regSorted; d->regElemSize = m.regElemSize;
  if ((rc = upload_node_bc(d))) return fail(rc);
  if (d->params.region_reps) {
    // the region cost model: elements in region order (regElemlist, grouped by
    // sorted region) and each position's region rep count
    // (a block mesh brings both, block after block)
    std::vector<int> order(E), reps(E);
    if (!m.regionOrder.empty()) {
      order = m.regionOrder;
      reps = m.regionReps;
    } else {
      int64_t pos = 0;
      for (size_t r = 0; r < m.regElemSize.size(); ++r)
        for (int64_t k = 0; k < m.regElemSize[r]; ++k, ++pos) {
          order[pos] = (int)(m.regElemlist[pos] - 1);
          reps[pos] = (int)m.regReps[r];
        }
    }
    if ((err = cudaMalloc(&d->region_buf, 2 * (size_t)E * sizeof(int))) != cudaSuccess) {
      cudaGetLastError();
      d->region_buf = nullptr;
      return fail(LULESH_ERR_MEMORY);
    }
    int* ob = static_cast<int*>(d->region_buf);
    if ((err = cudaMemcpy(ob, order.data(), E * sizeof(int), cudaMemcpyHostToDevice)) != cudaSuccess ||
        (err = cudaMemcpy(ob + E, reps.data(), E * sizeof(int), cudaMemcpyHostToDevice)) != cudaSuccess)
      return fail(cuda_fail(err));
    dd.regOrder = ob;
    dd.posReps = ob + E;
  }
  state_to_device_mirror(d);
  if ((rc = h2d(dd.st, d->hst, 1, s))) return fail(rc);
  if ((err = cudaStreamSynchronize(s)) != cudaSuccess) return fail(cuda_fail(err));
  *out = d;
  return LULESH_OK;
}

static bool valid_params(const lulesh_params* p) {
  return p && p->nx >= 1 && p->nx <= 640 && p->nr >= 1 && p->balance >= 0 && p->cost >= 0 && p->mode >= 0 &&
         p->mode <= 7;
}

extern "C" {

int lulesh_create(const lulesh_params* params, lulesh_domain** out) {
  if (!params || !out) return LULESH_ERR_ARGUMENT;
  *out = nullptr;
  // 8*numElem must fit a 32-bit index
  if (!valid_params(params)) return LULESH_ERR_ARGUMENT;
  HostMesh m;
  try {
    build_mesh(m, params->nx, params->nr, params->balance, params->cost, params->region_seed);
  } catch (const std::bad_alloc&) {
    return LULESH_ERR_MEMORY;  // the host mesh did not fit
  }
  return create_domain(params, m, out);
}

// The packed block mesh of (nx*tp)^3 elements in tp^3 blocks; 0 or the error.
static int block_mesh(HostMesh& m, int nx, int tp, int nr, int balance, int cost, int mode, uint64_t seed) {
  if (tp < 1 || nx < 1 || (int64_t)nx * tp > 600) return LULESH_ERR_ARGUMENT;
  // every packed index must fit 31 bits: the corner list (at most 8 entries
  // per packed node) bounds the corner slots and ghost slots as well
  const int64_t en = nx + 1, packed_nodes = (int64_t)tp * tp * tp * en * en * en;
  if (8 * packed_nodes >= INT32_MAX) return LULESH_ERR_ARGUMENT;
  try {
    HostMesh g;
    build_mesh(g, nx * tp, 1, 1, 1, 0);
    build_block_mesh(m, g, nx, tp, mode);
    build_block_regions(m, nx, tp, nr, balance, cost, seed);
  } catch (const std::bad_alloc&) {
    return LULESH_ERR_MEMORY;
  }
  return LULESH_OK;
}

int lulesh_create_blocks(const lulesh_params* params, int32_t blocks_per_edge, lulesh_domain** out) {
  if (!params || !out) return LULESH_ERR_ARGUMENT;
  *out = nullptr;
  if (!valid_params(params)) return LULESH_ERR_ARGUMENT;
  HostMesh m;
  int rc = block_mesh(m, params->nx, blocks_per_edge, params->nr, params->balance, params->cost, params->mode,
                      params->region_seed);
  if (rc) return rc;
  return create_domain(params, m, out);
}

int lulesh_block_map(const lulesh_domain* d, int32_t* blocks_per_edge, int32_t* elem_global, int32_t* node_global) {
  if (!d) return LULESH_ERR_ARGUMENT;
  if (blocks_per_edge) *blocks_per_edge = d->blocks_per_edge;
  for (int64_t i = 0; elem_global && i < d->E; ++i) elem_global[i] = d->elemGlobal.empty() ? (int32_t)i : d->elemGlobal[i];
  for (int64_t i = 0; node_global && i < d->N; ++i) node_global[i] = d->nodeGlobal.empty() ? (int32_t)i : d->nodeGlobal[i];
  return LULESH_OK;
}

int lulesh_block_plan_sizes(int32_t nx, int32_t blocks_per_edge, int32_t mode, int64_t sizes[5]) {
  if (!sizes || mode < 0 || mode > 7) return LULESH_ERR_ARGUMENT;
  HostMesh m;
  int rc = block_mesh(m, nx, blocks_per_edge, 1, 1, 1, mode, 0);
  if (rc) return rc;
  sizes[0] = m.E;
  sizes[1] = m.N;
  sizes[2] = (int64_t)m.haloDelvSrc.size();
  sizes[3] = (int64_t)m.haloCornerSrc.size();
  sizes[4] = m.nCornerList;
  return LULESH_OK;
}

int lulesh_block_plan(int32_t nx, int32_t blocks_per_edge, int32_t mode, int32_t* elem_global, int32_t* node_global,
                      int32_t* halo_delv_src, int32_t* halo_delv_dst, int32_t* halo_corner_src,
                      int32_t* halo_corner_dst) {
  if (mode < 0 || mode > 7) return LULESH_ERR_ARGUMENT;
  HostMesh m;
  int rc = block_mesh(m, nx, blocks_per_edge, 1, 1, 1, mode, 0);
  if (rc) return rc;
  auto put = [](int32_t* dst, const std::vector<int>& v) {
    if (dst) std::copy(v.begin(), v.end(), dst);
  };
  put(elem_global, m.elemGlobal);
  put(node_global, m.nodeGlobal);
  put(halo_delv_src, m.haloDelvSrc);
  put(halo_delv_dst, m.haloDelvDst);
  put(halo_corner_src, m.haloCornerSrc);
  put(halo_corner_dst, m.haloCornerDst);
  return LULESH_OK;
}

int lulesh_destroy(lulesh_domain* d) {
  if (!d) return LULESH_ERR_ARGUMENT;
  cudaSetDevice(d->params.device);
  if (d->stream) cudaStreamSynchronize(d->stream);
  drop_graph(d);
  for (auto& ev : d->ring) if (ev) cudaEventDestroy(ev);
  if (d->hst) cudaFreeHost(d->hst);
  if (d->arena) cudaFree(d->arena);
  if (d->region_buf) cudaFree(d->region_buf);
  if (d->stream) cudaStreamDestroy(d->stream);
  delete d;
  return LULESH_OK;
}

int lulesh_sizes(const lulesh_domain* d, int64_t* ne, int64_t* nn) {
  if (!d) return LULESH_ERR_ARGUMENT;
  if (ne) *ne = d->E;
  if (nn) *nn = d->N;
  return LULESH_OK;
}

int lulesh_get_stream(lulesh_domain* d, void** stream) {
  if (!d || !stream) return LULESH_ERR_ARGUMENT;
  *stream = (void*)d->stream;
  return LULESH_OK;
}

int lulesh_time_increment(lulesh_domain* d) {
  if (!d) return LULESH_ERR_ARGUMENT;
  TraceRange trace("timeIncrement!");
  const Params prm = make_params(d);
  double time = d->sc[LULESH_S_TIME], dt = d->sc[LULESH_S_DELTATIME];
  long long cycle = (long long)d->sc[LULESH_S_CYCLE];
  time_increment(time, dt, cycle, d->sc[LULESH_S_DTCOURANT], d->sc[LULESH_S_DTHYDRO], prm);
  d->sc[LULESH_S_TIME] = time;
  d->sc[LULESH_S_DELTATIME] = dt;
  d->sc[LULESH_S_CYCLE] = (double)cycle;
  return LULESH_OK;
}

int lulesh_lagrange_leapfrog(lulesh_domain* d) {
  if (!d) return LULESH_ERR_ARGUMENT;
  TraceRange trace("lagrangeLeapFrog");
  CK(cudaSetDevice(d->params.device));
  const Params prm = make_params(d);
  state_to_device_mirror(d);
  int rc;
  if ((rc = h2d(d->dd.st, d->hst, 1, d->stream))) return rc;
  ensure_geometry(d);
  if ((rc = launch_step(d, prm, false, d->timing))) return rc;
  if ((rc = d2h(d->hst, d->dd.st, 1, d->stream))) return rc;
  CK(cudaStreamSynchronize(d->stream));
  if (d->timing && (rc = collect_times(d))) return rc;
  state_from_device_mirror(d);
  // a step that stopped early may leave the stored geometry behind the
  // positions; the inline split stores none
  if (d->status || d->tuning.geo != 0) d->geo_valid = false;
  return d->status;
}

int lulesh_run(lulesh_domain* d, int64_t num_iters, lulesh_scalars* out) {
  if (!d) return LULESH_ERR_ARGUMENT;
  TraceRange trace("lulesh_run");
  CK(cudaSetDevice(d->params.device));
  const Params prm = make_params(d);
  state_to_device_mirror(d);
  d->hst->num_iters = num_iters;
  int rc;
  cudaStream_t s = d->stream;
  if ((rc = h2d(d->dd.st, d->hst, 1, s))) return rc;
  ensure_geometry(d);
  // cycles the loop can still take: the first always runs, later ones while cycle < num_iters
  const int64_t cyc0 = d->cycle_i();
  const int64_t budget = std::max<int64_t>(1, num_iters - cyc0);
  if (d->timing) {
    // per-kernel events and no graph; the host polls the done flag every
    // kPollCyclesTimed cycles
    for (int64_t k = 0; k < budget; ++k) {
      if ((rc = launch_step(d, prm, true, true))) return rc;
      if ((k + 1) % kPollCyclesTimed == 0) {
        if ((rc = d2h(d->hst, d->dd.st, 1, s))) return rc;
        CK(cudaStreamSynchronize(s));
        if (d->hst->done) break;
      }
    }
    if ((rc = collect_times(d))) return rc;
  } else {
    // one graph = kGraphCycles cycles; rebuilt when a parameter it bakes in
    // changes (the run limit is read from the device state)
    if (!d->graph) {
      drop_graph(d);
      cudaGraph_t g;
      CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
      for (int c = 0; c < kGraphCycles; ++c) launch_step(d, prm, true, false);
      CK(cudaStreamEndCapture(s, &g));
      cudaError_t e = cudaGraphInstantiate(&d->graph, g, 0);
      cudaGraphDestroy(g);
      CK(e);
      d->graph_key = 0;
    }
    int64_t launched = 0;
    for (;;) {
      for (int k = 0; k < kPollLaunches && launched < budget; ++k) {
        CK(cudaGraphLaunch(d->graph, s));
        launched += kGraphCycles;
      }
      if ((rc = d2h(d->hst, d->dd.st, 1, s))) return rc;
      CK(cudaStreamSynchronize(s));
      if (d->hst->done || launched >= budget) break;
    }
  }
  if ((rc = d2h(d->hst, d->dd.st, 1, s))) return rc;
  CK(cudaStreamSynchronize(s));
  state_from_device_mirror(d);
  if (d->status || d->tuning.geo != 0) d->geo_valid = false;
  if (out) lulesh_get_scalars(d, out);
  return d->status;
}

int lulesh_get_scalars(const lulesh_domain* d, lulesh_scalars* out) {
  if (!d || !out) return LULESH_ERR_ARGUMENT;
  out->time = d->sc[LULESH_S_TIME];
  out->deltatime = d->sc[LULESH_S_DELTATIME];
  out->dtcourant = d->sc[LULESH_S_DTCOURANT];
  out->dthydro = d->sc[LULESH_S_DTHYDRO];
  out->cycle = (int64_t)d->sc[LULESH_S_CYCLE];
  out->status = d->status;
  out->site = d->site;
  return LULESH_OK;
}

int lulesh_get_scalar(const lulesh_domain* d, int32_t id, double* v) {
  if (!d || !v || id < 0 || id >= LULESH_S_COUNT) return LULESH_ERR_ARGUMENT;
  *v = d->sc[id];
  return LULESH_OK;
}

int lulesh_set_scalar(lulesh_domain* d, int32_t id, double v) {
  if (!d || id < 0 || id >= LULESH_S_COUNT) return LULESH_ERR_ARGUMENT;
  if (id == LULESH_S_CYCLE && (v < 0 || v != std::floor(v))) return LULESH_ERR_ARGUMENT;
  const bool state = id == LULESH_S_TIME || id == LULESH_S_DELTATIME || id == LULESH_S_DTCOURANT ||
                     id == LULESH_S_DTHYDRO || id == LULESH_S_CYCLE;
  // the other scalars are kernel parameters baked into the captured graph;
  // the step state is uploaded at the start of every call
  if (!state && !(d->sc[id] == v)) drop_graph(d);
  d->sc[id] = v;
  return LULESH_OK;
}

int lulesh_enable_timing(lulesh_domain* d, int32_t enable) {
  if (!d) return LULESH_ERR_ARGUMENT;
  d->timing = enable != 0;
  for (double& t : d->kernel_ms) t = 0.0;
  return LULESH_OK;
}

int lulesh_kernel_times(lulesh_domain* d, double* ms, int32_t max_kernels, int32_t* n) {
  if (!d || !ms) return LULESH_ERR_ARGUMENT;
  const int k = std::min<int32_t>(max_kernels, kNumKernels);
  for (int i = 0; i < k; ++i) { ms[i] = d->kernel_ms[i]; d->kernel_ms[i] = 0.0; }
  if (n) *n = kNumKernels;
  return LULESH_OK;
}

// ---- field I/O --------------------------------------------------------------

namespace {
enum Kind { F64_ELEM, F64_NODE, I64, U32 };
}

static double* f64_ptr(lulesh_domain* d, int32_t f, Kind* kind) {
  DevDomain& dd = d->dd;
  *kind = (f < LULESH_F_X) ? F64_ELEM : F64_NODE;
  switch (f) {
    case LULESH_F_E: return dd.e;
    case LULESH_F_P: return dd.p;
    case LULESH_F_Q: return dd.q;
    case LULESH_F_QL: return dd.ql;
    case LULESH_F_QQ: return dd.qq;
    case LULESH_F_V: return dd.v;
    case LULESH_F_VOLO: return dd.volo;
    case LULESH_F_DELV: return dd.delv;
    case LULESH_F_VDOV: return dd.vdov;
    case LULESH_F_AREALG: return dd.arealg;
    case LULESH_F_SS: return dd.ss;
    case LULESH_F_ELEMMASS: return dd.elemMass;
    case LULESH_F_VNEW: return dd.vnew;
    case LULESH_F_DELV_XI: return dd.delv_xi;
    case LULESH_F_DELV_ETA: return dd.delv_eta;
    case LULESH_F_DELV_ZETA: return dd.delv_zeta;
    case LULESH_F_DELX_XI: return dd.delx_xi;
    case LULESH_F_DELX_ETA: return dd.delx_eta;
    case LULESH_F_DELX_ZETA: return dd.delx_zeta;
    case LULESH_F_DXX: return dd.dxx;
    case LULESH_F_DYY: return dd.dyy;
    case LULESH_F_DZZ: return dd.dzz;
    case LULESH_F_X: return dd.x;
    case LULESH_F_Y: return dd.y;
    case LULESH_F_Z: return dd.z;
    case LULESH_F_XD: return dd.xd;
    case LULESH_F_YD: return dd.yd;
    case LULESH_F_ZD: return dd.zd;
    case LULESH_F_XDD: return dd.xdd;
    case LULESH_F_YDD: return dd.ydd;
    case LULESH_F_ZDD: return dd.zdd;
    case LULESH_F_FX: return dd.fx;
    case LULESH_F_FY: return dd.fy;
    case LULESH_F_FZ: return dd.fz;
    case LULESH_F_NODALMASS: return dd.nodalMass;
    default: return nullptr;
  }
}

static int64_t field_len(const lulesh_domain* d, int32_t f) {
  const int64_t E = d->E, N = d->N;
  if (f >= LULESH_F_E && f <= LULESH_F_DZZ) return E;
  if (f >= LULESH_F_X && f <= LULESH_F_NODALMASS) return N;
  switch (f) {
    case LULESH_F_NODELIST: return 8 * E;
    case LULESH_F_LXIM: case LULESH_F_LXIP: case LULESH_F_LETAM: case LULESH_F_LETAP:
    case LULESH_F_LZETAM: case LULESH_F_LZETAP: return E;
    case LULESH_F_SYMMX: return (int64_t)d->symmX.size();
    case LULESH_F_SYMMY: return (int64_t)d->symmY.size();
    case LULESH_F_SYMMZ: return (int64_t)d->symmZ.size();
    case LULESH_F_NODEELEMCOUNT: case LULESH_F_NODEELEMSTART: return N;
    case LULESH_F_NODEELEMCORNERLIST: return d->dd.nCornerList;
    case LULESH_F_MATELEMLIST: case LULESH_F_REGNUMLIST: case LULESH_F_REGELEMLIST: return E;
    case LULESH_F_REGCSR: case LULESH_F_REGREPS: case LULESH_F_REGSORTED: case LULESH_F_REGELEMSIZE:
      return d->params.nr;
    case LULESH_F_ELEMBC: return E;
    default: return -1;
  }
}

int lulesh_field_length(const lulesh_domain* d, int32_t f, int64_t* count) {
  if (!d || !count) return LULESH_ERR_ARGUMENT;
  const int64_t n = field_len(d, f);
  if (n < 0) return LULESH_ERR_ARGUMENT;
  *count = n;
  return LULESH_OK;
}

static int* neighbour_ptr(lulesh_domain* d, int32_t f) {
  switch (f) {
    case LULESH_F_LXIM: return d->dd.lxim;
    case LULESH_F_LXIP: return d->dd.lxip;
    case LULESH_F_LETAM: return d->dd.letam;
    case LULESH_F_LETAP: return d->dd.letap;
    case LULESH_F_LZETAM: return d->dd.lzetam;
    case LULESH_F_LZETAP: return d->dd.lzetap;
    default: return nullptr;
  }
}

int lulesh_download_field(lulesh_domain* d, int32_t f, void* host, int64_t count) {
  if (!d || !host) return LULESH_ERR_ARGUMENT;
  const int64_t n = field_len(d, f);
  if (n < 0 || count != n) return LULESH_ERR_ARGUMENT;
  CK(cudaSetDevice(d->params.device));
  cudaStream_t s = d->stream;
  const int64_t E = d->E, N = d->N;
  int rc;
  if (f < LULESH_F_NODELIST) {
    Kind k;
    double* p = f64_ptr(d, f, &k);
    if (!p) return LULESH_ERR_ARGUMENT;  // an aux field without keep_aux
    if ((rc = d2h((double*)host, p, n, s))) return rc;
    CK(cudaStreamSynchronize(s));
    return LULESH_OK;
  }
  int64_t* out = (int64_t*)host;
  if (f == LULESH_F_ELEMBC) {
    if ((rc = d2h((unsigned int*)host, d->dd.elemBC, n, s))) return rc;
    CK(cudaStreamSynchronize(s));
    return LULESH_OK;
  }
  if (int* nb = neighbour_ptr(d, f)) {
    std::vector<int> t(n);
    if ((rc = d2h(t.data(), nb, n, s))) return rc;
    CK(cudaStreamSynchronize(s));
    for (int64_t i = 0; i < n; ++i) out[i] = t[i];
    return LULESH_OK;
  }
  switch (f) {
    case LULESH_F_NODELIST: {
      std::vector<int> t(8 * E);
      if ((rc = d2h(t.data(), d->dd.nodelist, 8 * E, s))) return rc;
      CK(cudaStreamSynchronize(s));
      for (int64_t e = 0; e < E; ++e)
        for (int c = 0; c < 8; ++c) out[8 * e + c] = t[c * E + e];
      return LULESH_OK;
    }
    case LULESH_F_NODEELEMCOUNT:
    case LULESH_F_NODEELEMSTART: {
      std::vector<int> t(N + 1);
      if ((rc = d2h(t.data(), d->dd.nodeElemStart, N + 1, s))) return rc;
      CK(cudaStreamSynchronize(s));
      for (int64_t i = 0; i < N; ++i)
        out[i] = (f == LULESH_F_NODEELEMSTART) ? t[i] : t[i + 1] - t[i];
      return LULESH_OK;
    }
    case LULESH_F_NODEELEMCORNERLIST: {
      std::vector<int> t(n);
      if ((rc = d2h(t.data(), d->dd.cornerList, n, s))) return rc;
      CK(cudaStreamSynchronize(s));
      // Julia value: 1-based element-major corner k = 8*e + c + 1 (a ghost
      // slot of a block mesh gives the corner it copies)
      for (int64_t i = 0; i < n; ++i) {
        int64_t v = t[i];
        if (v >= 8 * E) v = d->haloCornerSrc[v - 8 * E];
        const int64_t c = v / E, e = v % E;
        out[i] = 8 * e + c + 1;
      }
      return LULESH_OK;
    }
    case LULESH_F_SYMMX: for (int64_t i = 0; i < n; ++i) out[i] = d->symmX[i]; return LULESH_OK;
    case LULESH_F_SYMMY: for (int64_t i = 0; i < n; ++i) out[i] = d->symmY[i]; return LULESH_OK;
    case LULESH_F_SYMMZ: for (int64_t i = 0; i < n; ++i) out[i] = d->symmZ[i]; return LULESH_OK;
    case LULESH_F_MATELEMLIST: for (int64_t i = 0; i < n; ++i) out[i] = i + 1; return LULESH_OK;
    case LULESH_F_REGNUMLIST: std::copy(d->regNumList.begin(), d->regNumList.end(), out); return LULESH_OK;
    case LULESH_F_REGELEMLIST: std::copy(d->regElemlist.begin(), d->regElemlist.end(), out); return LULESH_OK;
    case LULESH_F_REGCSR: std::copy(d->regCSR.begin(), d->regCSR.end(), out); return LULESH_OK;
    case LULESH_F_REGREPS: std::copy(d->regReps.begin(), d->regReps.end(), out); return LULESH_OK;
    case LULESH_F_REGSORTED: std::copy(d->regSorted.begin(), d->regSorted.end(), out); return LULESH_OK;
    case LULESH_F_REGELEMSIZE: std::copy(d->regElemSize.begin(), d->regElemSize.end(), out); return LULESH_OK;
    default: return LULESH_ERR_ARGUMENT;
  }
}

int lulesh_upload_field(lulesh_domain* d, int32_t f, const void* host, int64_t count) {
  if (!d || !host) return LULESH_ERR_ARGUMENT;
  const int64_t n = field_len(d, f);
  if (n < 0 || count != n) return LULESH_ERR_ARGUMENT;
  CK(cudaSetDevice(d->params.device));
  cudaStream_t s = d->stream;
  const int64_t E = d->E, N = d->N;
  int rc;
  // the force kernel's stored geometry depends on the positions and the connectivity
  if (f == LULESH_F_X || f == LULESH_F_Y || f == LULESH_F_Z || f == LULESH_F_NODELIST) d->geo_valid = false;
  if (f < LULESH_F_NODELIST) {
    Kind k;
    double* p = f64_ptr(d, f, &k);
    if (!p) return LULESH_ERR_ARGUMENT;
    const double* h = (const double*)host;
    if ((rc = h2d(p, h, n, s))) return rc;
    // derived reciprocals follow the field
    if (f == LULESH_F_VOLO || f == LULESH_F_NODALMASS) {
      std::vector<double> inv(n);
      for (int64_t i = 0; i < n; ++i) inv[i] = 1.0 / h[i];
      if ((rc = h2d(f == LULESH_F_VOLO ? d->dd.inv_volo : d->dd.inv_nodalMass, inv.data(), n, s))) return rc;
      CK(cudaStreamSynchronize(s));
      return LULESH_OK;
    }
    CK(cudaStreamSynchronize(s));
    return LULESH_OK;
  }
  const int64_t* in = (const int64_t*)host;
  if (f == LULESH_F_ELEMBC) {
    if ((rc = h2d(d->dd.elemBC, (const unsigned int*)host, n, s))) return rc;
    CK(cudaStreamSynchronize(s));
    return LULESH_OK;
  }
  if (int* nb = neighbour_ptr(d, f)) {
    std::vector<int> t(n);
    for (int64_t i = 0; i < n; ++i) t[i] = (int)in[i];
    if ((rc = h2d(nb, t.data(), n, s))) return rc;
    CK(cudaStreamSynchronize(s));
    return LULESH_OK;
  }
  switch (f) {
    case LULESH_F_NODELIST: {
      std::vector<int> t(8 * E);
      for (int64_t i = 0; i < 8 * E; ++i)
        if (in[i] < 0 || in[i] >= N) return LULESH_ERR_ARGUMENT;
      for (int64_t e = 0; e < E; ++e)
        for (int c = 0; c < 8; ++c) t[c * E + e] = (int)in[8 * e + c];
      if ((rc = h2d(d->dd.nodelist, t.data(), 8 * E, s))) return rc;
      CK(cudaStreamSynchronize(s));
      return LULESH_OK;
    }
    case LULESH_F_SYMMX: case LULESH_F_SYMMY: case LULESH_F_SYMMZ: {
      std::vector<int>& dst = f == LULESH_F_SYMMX ? d->symmX : f == LULESH_F_SYMMY ? d->symmY : d->symmZ;
      for (int64_t i = 0; i < n; ++i) dst[i] = (int)in[i];
      return upload_node_bc(d);
    }
    default:
      return LULESH_ERR_ARGUMENT;  // connectivity lists and regions are fixed at creation
  }
}

int lulesh_verify(lulesh_domain* d, double out[4]) {
  if (!d || !out) return LULESH_ERR_ARGUMENT;
  CK(cudaSetDevice(d->params.device));
  const int64_t nx = d->params.nx;
  std::vector<double> e(nx * nx);
  int rc;
  if ((rc = d2h(e.data(), d->dd.e, nx * nx, d->stream))) return rc;
  CK(cudaStreamSynchronize(d->stream));
  // src/utils.jl:139-153
  double maxAbs = 0.0, maxRel = 0.0, total = 0.0;
  for (int64_t j = 1; j <= nx; ++j)
    for (int64_t k = j + 1; k <= nx; ++k) {
      const double a = e[(j - 1) * nx + k - 1], b = e[(k - 1) * nx + j - 1];
      const double ad = std::fabs(a - b);
      total += ad;
      if (maxAbs < ad) maxAbs = ad;
      const double rd = ad / b;
      if (maxRel < rd) maxRel = rd;
    }
  out[0] = e[0];
  out[1] = maxAbs;
  out[2] = total;
  out[3] = maxRel;
  return LULESH_OK;
}

int lulesh_get_tuning(const lulesh_domain* d, lulesh_tuning* out) {
  if (!d || !out) return LULESH_ERR_ARGUMENT;
  out->force_block = d->tuning.force;
  out->node_block = d->tuning.node;
  out->kin_block = d->tuning.kin;
  out->mat_block = d->tuning.mat;
  out->geometry = d->tuning.geo;
  return LULESH_OK;
}

int lulesh_set_tuning(lulesh_domain* d, const lulesh_tuning* t) {
  auto elem_ok = [](int b) { return b == 64 || b == 128 || b == 256; };
  if (!d || !t || !elem_ok(t->force_block) || !elem_ok(t->kin_block) || !elem_ok(t->mat_block) ||
      !(t->node_block == 128 || t->node_block == 256 || t->node_block == 512) ||
      !(t->geometry == 0 || t->geometry == 1))
    return LULESH_ERR_ARGUMENT;
  d->tuning.force = t->force_block;
  d->tuning.node = t->node_block;
  d->tuning.kin = t->kin_block;
  d->tuning.mat = t->mat_block;
  if (d->tuning.geo != t->geometry) d->geo_valid = false;
  d->tuning.geo = t->geometry;
  drop_graph(d);
  return LULESH_OK;
}

int lulesh_autotune(lulesh_domain* d, int32_t cycles, lulesh_tuning* chosen) {
  if (!d) return LULESH_ERR_ARGUMENT;
  TraceRange trace("lulesh_autotune");
  CK(cudaSetDevice(d->params.device));
  cudaStream_t s = d->stream;
  // save the fields the tuning cycles change, then restore them and the scalars
  DevDomain& dd = d->dd;
  double* node_f[6] = {dd.x, dd.y, dd.z, dd.xd, dd.yd, dd.zd};
  double* elem_f[5] = {dd.e, dd.p, dd.q, dd.v, dd.ss};
  const size_t nb = (size_t)d->N * sizeof(double), eb = (size_t)d->E * sizeof(double);
  char* save = nullptr;
  CK(cudaMalloc(&save, 6 * nb + 5 * eb));
  auto copy_all = [&](bool to_save) -> cudaError_t {
    char* p = save;
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < 6 && e == cudaSuccess; ++k, p += nb)
      e = cudaMemcpyAsync(to_save ? (void*)p : (void*)node_f[k], to_save ? (const void*)node_f[k] : (const void*)p,
                          nb, cudaMemcpyDeviceToDevice, s);
    for (int k = 0; k < 5 && e == cudaSuccess; ++k, p += eb)
      e = cudaMemcpyAsync(to_save ? (void*)p : (void*)elem_f[k], to_save ? (const void*)elem_f[k] : (const void*)p,
                          eb, cudaMemcpyDeviceToDevice, s);
    return e;
  };
  double sc_saved[LULESH_S_COUNT];
  std::memcpy(sc_saved, d->sc, sizeof(sc_saved));
  cudaError_t err = copy_all(true);
  if (err == cudaSuccess) {
    state_to_device_mirror(d);
    d->hst->first = 0;
    err = cudaMemcpyAsync(dd.st, d->hst, sizeof(DevState), cudaMemcpyHostToDevice, s);
  }
  if (err == cudaSuccess) {
    ensure_geometry(d);
    err = autotune_blocks(dd, make_params(d), d->params.keep_aux != 0, 1, s, cycles, d->tuning);
  }
  if (err == cudaSuccess) err = copy_all(false);
  if (err == cudaSuccess) err = cudaStreamSynchronize(s);
  cudaFree(save);
  std::memcpy(d->sc, sc_saved, sizeof(sc_saved));
  drop_graph(d);
  d->geo_valid = false;  // the tuning cycles moved the positions the geometry describes
  CK(err);
  return chosen ? lulesh_get_tuning(d, chosen) : LULESH_OK;
}

}  // extern "C"
