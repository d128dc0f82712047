// Autotuner shared by the single-problem handle and the ensemble: block
// sizes of the four step kernels and the fusion split of the force geometry.
//
// Coordinate descent: for each step kernel in turn, every candidate block
// size runs `cycles` full cycles on the live problem with CUDA events around
// each kernel; the fastest candidate for that kernel is kept before the next
// kernel is tuned. This runs with the stored-geometry split (k_kinematics
// forms the next cycle's force geometry and stores it). Then the other split
// (k_force forms the geometry itself, k_kinematics stores none) gets its own
// force and kinematics block sizes the same way, and the split whose force +
// kinematics time is lower is kept. Every choice gives bitwise the same
// results. The caller saves and restores the state, and has the stored
// geometry of the current positions ready before the call.
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

// Runs 1 + cycles full cycles with tuning t (the first warms up) and adds each
// step kernel's time over the timed cycles to ms[0..3].
cudaError_t phase_times(const DevDomain& d, const Params& prm, bool aux, int ninst, cudaStream_t s, int cycles,
                        const Tuning& t, cudaEvent_t* ev, float ms[4]) {
  for (int q = 0; q < 4; ++q) ms[q] = 0.f;
  cudaError_t err = cudaSuccess;
  for (int c = 0; c <= cycles && err == cudaSuccess; ++c) {
    launch_time_increment(d.st, ninst, prm, s);
    for (int q = 0; q < 4; ++q) {
      cudaEventRecord(ev[q], s);
      launch_phase(q, d, prm, aux, t, s);
    }
    cudaEventRecord(ev[4], s);
    err = cudaEventSynchronize(ev[4]);
    if (err == cudaSuccess && c > 0) {
      for (int q = 0; q < 4; ++q) {
        float x = 0.f;
        cudaEventElapsedTime(&x, ev[q], ev[q + 1]);
        ms[q] += x;
      }
    }
  }
  return err;
}

// Coordinate descent over the block sizes of the kernels in `which` (bits
// 0..3: force, node, kinematics, material); returns the kernels' times with
// the chosen sizes in best_ms.
cudaError_t descend(const DevDomain& d, const Params& prm, bool aux, int ninst, cudaStream_t s, int cycles,
                    unsigned which, Tuning& t, cudaEvent_t* ev, float best_ms[4]) {
  static const int elem_cand[3] = {64, 128, 256};
  static const int node_cand[3] = {128, 256, 512};
  cudaError_t err = cudaSuccess;
  for (int q = 0; q < 4; ++q) best_ms[q] = 3.0e38f;
  for (int k = 0; k < 4 && err == cudaSuccess; ++k) {
    if (!(which & (1u << k))) continue;
    int* slot = k == 0 ? &t.force : k == 1 ? &t.node : k == 2 ? &t.kin : &t.mat;
    const int* cand = (k == 1) ? node_cand : elem_cand;
    float best = 3.0e38f;
    int best_bs = *slot;
    for (int j = 0; j < 3 && err == cudaSuccess; ++j) {
      *slot = cand[j];
      float ms[4];
      err = phase_times(d, prm, aux, ninst, s, cycles, t, ev, ms);
      if (err == cudaSuccess && ms[k] < best) {
        best = ms[k];
        best_bs = cand[j];
        for (int q = 0; q < 4; ++q) best_ms[q] = ms[q];
      }
    }
    *slot = best_bs;
  }
  return err;
}
}  // namespace

cudaError_t autotune_blocks(const DevDomain& d, const Params& prm, bool aux, int ninst, cudaStream_t s,
                            int cycles, Tuning& t) {
  cudaEvent_t ev[5] = {};
  cudaError_t err = cudaSuccess;
  for (int i = 0; i < 5 && err == cudaSuccess; ++i) err = cudaEventCreate(&ev[i]);
  if (cycles < 1) cycles = 1;
  // the stored split first: its force kernel reads the geometry the caller
  // formed, and each kinematics launch stores the next one
  Tuning stored = t, inline_geo;
  stored.geo = 0;
  float ms0[4] = {}, ms1[4] = {};
  if (err == cudaSuccess) err = descend(d, prm, aux, ninst, s, cycles, 0xFu, stored, ev, ms0);
  // then the inline split, which reads no stored geometry
  inline_geo = stored;
  inline_geo.geo = 1;
  if (err == cudaSuccess) err = descend(d, prm, aux, ninst, s, cycles, 0x5u, inline_geo, ev, ms1);
  if (err == cudaSuccess) {
    // force + kinematics under each split, each with its own best block sizes
    float t0 = 0.f, t1 = 0.f;
    err = phase_times(d, prm, aux, ninst, s, cycles, inline_geo, ev, ms1);
    t1 = ms1[0] + ms1[2];
    // measure the stored split last, after a geometry pass of the current
    // positions (the inline cycles left the stored geometry behind)
    if (err == cudaSuccess) {
      launch_geometry(d, s);
      err = phase_times(d, prm, aux, ninst, s, cycles, stored, ev, ms0);
      t0 = ms0[0] + ms0[2];
    }
    if (err == cudaSuccess) t = (t1 < t0) ? inline_geo : stored;
  }
  for (int i = 0; i < 5; ++i)
    if (ev[i]) cudaEventDestroy(ev[i]);
  if (err == cudaSuccess) err = cudaGetLastError();
  return err;
}

}  // namespace lulesh
