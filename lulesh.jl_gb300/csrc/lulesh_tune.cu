// Block-size autotuner shared by the single-problem handle and the ensemble.
//
// Coordinate descent: for each of the four step kernels in turn, every
// candidate block size runs `cycles` full cycles on the live problem with
// CUDA events around that kernel only; the fastest candidate is kept before
// the next kernel is tuned. The caller saves and restores the state.
#include <climits>

#include "lulesh_kernels.h"

namespace lulesh {

namespace {
void launch_phase(int q, const DevDomain& d, const Params& prm, bool aux, const Tuning& t, cudaStream_t s) {
  switch (q) {
    case 0: launch_force(d, prm, t, s); break;
    case 1: launch_node(d, prm, aux, t, s); break;
    case 2: launch_kinematics(d, prm, aux, t, s); break;
    default: launch_material(d, prm, aux, t, s); break;
  }
}
}  // namespace

cudaError_t autotune_blocks(const DevDomain& d, const Params& prm, bool aux, int ninst, cudaStream_t s,
                            int cycles, Tuning& t) {
  static const int elem_cand[3] = {64, 128, 256};
  static const int node_cand[3] = {128, 256, 512};
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t err = cudaEventCreate(&e0);
  if (err == cudaSuccess) err = cudaEventCreate(&e1);
  if (cycles < 1) cycles = 1;
  for (int k = 0; k < 4 && err == cudaSuccess; ++k) {
    int* slot = k == 0 ? &t.force : k == 1 ? &t.node : k == 2 ? &t.kin : &t.mat;
    const int* cand = (k == 1) ? node_cand : elem_cand;
    float best = 3.0e38f;
    int best_bs = *slot;
    for (int j = 0; j < 3 && err == cudaSuccess; ++j) {
      *slot = cand[j];
      float total = 0.f;
      for (int c = 0; c <= cycles && err == cudaSuccess; ++c) {  // cycle 0 warms up
        launch_time_increment(d.st, ninst, prm, s);
        for (int q = 0; q < 4; ++q) {
          if (q == k) cudaEventRecord(e0, s);
          launch_phase(q, d, prm, aux, t, s);
          if (q == k) cudaEventRecord(e1, s);
        }
        err = cudaEventSynchronize(e1);
        if (err == cudaSuccess && c > 0) {
          float ms = 0.f;
          cudaEventElapsedTime(&ms, e0, e1);
          total += ms;
        }
      }
      if (total < best) { best = total; best_bs = cand[j]; }
    }
    *slot = best_bs;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (err == cudaSuccess) err = cudaGetLastError();
  return err;
}

}  // namespace lulesh
