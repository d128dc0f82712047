// The single-problem handle (struct lulesh_domain) and the helpers other
// translation units (the adjoint) share with lulesh_capi.cu.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "../../include/lulesh_gb300.h"
#include "lulesh_internal.h"
#include "lulesh_kernels.h"

namespace lulesh {
constexpr int kNumKernels = 5;
}  // namespace lulesh

struct lulesh_domain {
  lulesh_params params;
  int64_t E = 0, N = 0;
  double sc[LULESH_S_COUNT];  // Domain scalars (LULESH_S_*), cycle stored as double
  int32_t status = 0, site = 0;
  lulesh::DevDomain dd{};
  void* arena = nullptr;
  void* region_buf = nullptr;  // regOrder + posReps when params.region_reps
  cudaStream_t stream = nullptr;
  lulesh::DevState* hst = nullptr;  // pinned mirror of the device state
  cudaGraphExec_t graph = nullptr;
  int64_t graph_key = -1;
  // dd.nextGeo holds the force kernel's geometry of the current positions
  // (cleared when the host changes positions or a step stops early)
  bool geo_valid = false;
  // host copies of what only the host uses
  std::vector<int> symmX, symmY, symmZ;
  // a block mesh (lulesh_create_blocks): blocks per edge, packed -> whole-mesh
  // element and node ids, and the corner slot each ghost corner copies
  int blocks_per_edge = 1;
  std::vector<int> elemGlobal, nodeGlobal, haloCornerSrc;
  std::vector<int64_t> regNumList, regElemlist, regCSR, regReps, regSorted, regElemSize;
  // timing: a ring of cycles x (kNumKernels+1) events, read back when full
  // or when the caller asks, so timed runs never stall per cycle
  bool timing = false;
  std::vector<cudaEvent_t> ring;
  int ring_used = 0;
  lulesh::Tuning tuning;
  double kernel_ms[lulesh::kNumKernels] = {};
  int64_t cycle_i() const { return (int64_t)sc[LULESH_S_CYCLE]; }
};

namespace lulesh {
// Kernel parameters from the handle's Domain scalars.
Params make_params(const lulesh_domain* d);
// Forms the force kernel's geometry on the handle's stream unless it is valid.
void ensure_geometry(lulesh_domain* d);
// Status bits of a step -> (lulesh_status, lulesh_site) in the reference's order.
void decode_status(unsigned bits, int32_t* status, int32_t* site);
// Host scalars -> pinned device-state mirror (fresh accumulators, first = 1).
void state_to_device_mirror(lulesh_domain* d);
// Pinned device-state mirror -> host scalars (folding the dt minima).
void state_from_device_mirror(lulesh_domain* d);
}  // namespace lulesh
