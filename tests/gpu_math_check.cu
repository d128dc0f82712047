// Accuracy of the step kernels' math helpers against CUDA's own functions:
// inv_cbrt against rcbrt, recip3 against three divisions, x*rsqrt(x) against
// sqrt. Prints the largest error of each in units in the last place of the
// CUDA result, as one JSON line. Built and run by tests/test_gpu_math.py.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "lulesh_device.cuh"

using lulesh::inv_cbrt;
using lulesh::recip3;

__global__ void k_check(int n, const double* x, const double* a, const double* b, const double* c, double* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[8 * i + 0] = inv_cbrt(x[i]);
  out[8 * i + 1] = rcbrt(x[i]);
  double ia, ib, ic;
  recip3(a[i], b[i], c[i], ia, ib, ic);
  out[8 * i + 2] = ia - 1.0 / a[i];
  out[8 * i + 3] = ib - 1.0 / b[i];
  out[8 * i + 4] = ic - 1.0 / c[i];
  out[8 * i + 5] = x[i] * rsqrt(x[i]);
  out[8 * i + 6] = sqrt(x[i]);
  out[8 * i + 7] = 0.0;
}

static double ulp(double v) {
  v = std::fabs(v);
  return std::nextafter(v, INFINITY) - v;
}

int main() {
  const int n = 1 << 20;
  std::vector<double> x(n), a(n), b(n), c(n), out(8 * (size_t)n);
  uint64_t s = 0x9E3779B97F4A7C15ull;
  auto u01 = [&]() {
    s ^= s << 13; s ^= s >> 7; s ^= s << 17;
    return (double)(s >> 11) * (1.0 / 9007199254740992.0);
  };
  for (int i = 0; i < n; ++i) {
    x[i] = std::pow(10.0, -36.0 + 66.0 * u01());  // 1e-36 .. 1e30 (both branches of inv_cbrt)
    a[i] = std::pow(10.0, -9.0 + 18.0 * u01());   // relative volumes within eosvmin..eosvmax
    b[i] = std::pow(10.0, -9.0 + 18.0 * u01());
    c[i] = std::pow(10.0, -20.0 + 23.0 * u01());  // |vdov| + 1e-20
    if (i % 64 == 0) {
      // operands whose products leave the normal range (the division fallback)
      a[i] = std::pow(10.0, -300.0 + 600.0 * u01());
      b[i] = std::pow(10.0, -300.0 + 600.0 * u01());
      c[i] = std::pow(10.0, -300.0 + 600.0 * u01());
    }
  }
  double *dx, *da, *db, *dc, *dout;
  const size_t bytes = (size_t)n * sizeof(double);
  if (cudaMalloc(&dx, bytes) || cudaMalloc(&da, bytes) || cudaMalloc(&db, bytes) || cudaMalloc(&dc, bytes) ||
      cudaMalloc(&dout, 8 * bytes)) {
    std::printf("{\"error\": \"cudaMalloc\"}\n");
    return 1;
  }
  cudaMemcpy(dx, x.data(), bytes, cudaMemcpyHostToDevice);
  cudaMemcpy(da, a.data(), bytes, cudaMemcpyHostToDevice);
  cudaMemcpy(db, b.data(), bytes, cudaMemcpyHostToDevice);
  cudaMemcpy(dc, c.data(), bytes, cudaMemcpyHostToDevice);
  k_check<<<(n + 255) / 256, 256>>>(n, dx, da, db, dc, dout);
  if (cudaMemcpy(out.data(), dout, 8 * bytes, cudaMemcpyDeviceToHost) != cudaSuccess) {
    std::printf("{\"error\": \"%s\"}\n", cudaGetErrorString(cudaGetLastError()));
    return 1;
  }
  double e_cbrt = 0.0, e_rec = 0.0, e_sqrt = 0.0;
  for (int i = 0; i < n; ++i) {
    const double* o = &out[8 * (size_t)i];
    e_cbrt = std::fmax(e_cbrt, std::fabs(o[0] - o[1]) / ulp(o[1]));
    e_rec = std::fmax(e_rec, std::fabs(o[2]) / ulp(1.0 / a[i]));
    e_rec = std::fmax(e_rec, std::fabs(o[3]) / ulp(1.0 / b[i]));
    e_rec = std::fmax(e_rec, std::fabs(o[4]) / ulp(1.0 / c[i]));
    e_sqrt = std::fmax(e_sqrt, std::fabs(o[5] - o[6]) / ulp(o[6]));
  }
  std::printf("{\"n\": %d, \"inv_cbrt_ulps\": %.3f, \"recip3_ulps\": %.3f, \"sqrt_ulps\": %.3f}\n", n, e_cbrt, e_rec,
              e_sqrt);
  cudaFree(dx); cudaFree(da); cudaFree(db); cudaFree(dc); cudaFree(dout);
  return 0;
}
