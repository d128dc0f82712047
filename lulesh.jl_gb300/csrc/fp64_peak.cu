// FP64 issue-rate probe: the denominator of the FP64 roofline this step is
// bound by. Independent FMA (or add) chains per thread, fixed trip counts,
// timed with CUDA events on a private stream.
#include <cuda_runtime.h>

#include "../../include/lulesh_gb300.h"

namespace {

template <bool FMA>
__global__ void k_fp64_chains(double* out, int iters, double a, double b) {
  double r[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) r[k] = threadIdx.x * 1e-9 + k;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) r[k] = FMA ? fma(r[k], a, b) : r[k] + b;
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += r[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

extern "C" int lulesh_measure_fp64_peak(int32_t device, double* fma_per_s, double* add_per_s) {
  if (!fma_per_s || !add_per_s) return LULESH_ERR_ARGUMENT;
  if (cudaSetDevice(device) != cudaSuccess) return LULESH_ERR_CUDA;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return LULESH_ERR_CUDA;
  const int threads = 256, blocks = sms * 8, iters = 4096;
  const size_t n = (size_t)threads * blocks;
  double* buf = nullptr;
  cudaStream_t s = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = LULESH_OK;
  if (cudaMalloc(&buf, n * sizeof(double)) != cudaSuccess) return LULESH_ERR_MEMORY;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
      cudaEventCreate(&e1) != cudaSuccess) {
    rc = LULESH_ERR_CUDA;
  }
  for (int which = 0; which < 2 && rc == LULESH_OK; ++which) {
    float best = 1e30f;
    for (int rep = 0; rep < 3; ++rep) {
      cudaEventRecord(e0, s);
      if (which == 0) k_fp64_chains<true><<<blocks, threads, 0, s>>>(buf, iters, 0.999, 1e-3);
      else k_fp64_chains<false><<<blocks, threads, 0, s>>>(buf, iters, 0.999, 1e-3);
      cudaEventRecord(e1, s);
      if (cudaEventSynchronize(e1) != cudaSuccess) { rc = LULESH_ERR_CUDA; break; }
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (ms < best) best = ms;
    }
    const double ops = (double)n * iters * 8.0;
    (which == 0 ? *fma_per_s : *add_per_s) = ops / (best * 1e-3);
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (s) cudaStreamDestroy(s);
  cudaFree(buf);
  return rc;
}
