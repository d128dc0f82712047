// Launchers of the step kernels (lulesh_kernels.cu).
#pragma once

#include <cuda_runtime.h>

#include "lulesh_internal.h"

namespace lulesh {

constexpr int kForceBlock = 128;
constexpr int kNodeBlock = 256;
constexpr int kKinBlock = 128;
constexpr int kMatBlock = 128;

void launch_force(const DevDomain& d, const Params& prm, cudaStream_t s);
void launch_node(const DevDomain& d, const Params& prm, bool aux, cudaStream_t s);
void launch_kinematics(const DevDomain& d, const Params& prm, bool aux, cudaStream_t s);
void launch_material(const DevDomain& d, const Params& prm, bool aux, cudaStream_t s);
void launch_time_increment(DevState* st, const Params& prm, long long num_iters, cudaStream_t s);

}  // namespace lulesh
