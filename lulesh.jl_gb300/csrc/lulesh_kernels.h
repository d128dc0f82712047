// Launchers of the step kernels (lulesh_kernels.cu).
#pragma once

#include <cuda_runtime.h>

#include "lulesh_internal.h"

namespace lulesh {

// Element kernels are compiled for blocks of up to kMaxElemBlock threads and
// the node kernel for up to kMaxNodeBlock (the register budget is the same
// 255 per thread either way), so the block size is a launch-time choice.
constexpr int kMaxElemBlock = 256;
constexpr int kMaxNodeBlock = 512;

// Launch configuration chosen by the autotuner (defaults are the block sizes
// that measured best for the 150^3 problem). `geo` is the fusion split of the
// force geometry: 0 formed by k_kinematics of the cycle before and stored in
// DevDomain::nextGeo (fewer FP64 instructions, 816 more bytes per element
// and cycle), 1 formed inside k_force from the positions. Both give bitwise
// the same results. The taping kernels of the adjoint always use 0.
struct Tuning {
  int force = 128;
  int node = 256;
  int kin = 128;
  int mat = 128;
  int geo = 0;
};

// k_geometry: the force kernel's geometry of the current positions (needed
// before a step whenever the positions did not come from the last step).
void launch_geometry(const DevDomain& d, cudaStream_t s);
void launch_force(const DevDomain& d, const Params& prm, const Tuning& t, cudaStream_t s);
void launch_node(const DevDomain& d, const Params& prm, bool aux, const Tuning& t, cudaStream_t s);
void launch_kinematics(const DevDomain& d, const Params& prm, bool aux, const Tuning& t, cudaStream_t s);
void launch_material(const DevDomain& d, const Params& prm, bool aux, const Tuning& t, cudaStream_t s);
void launch_time_increment(DevState* st, int n, const Params& prm, cudaStream_t s);

// Picks block sizes for the four step kernels by timing them on the live
// problem (lulesh_tune.cu); the state advances, so callers save and restore it.
cudaError_t autotune_blocks(const DevDomain& d, const Params& prm, bool aux, int ninst, cudaStream_t s,
                            int cycles, Tuning& t);

}  // namespace lulesh
