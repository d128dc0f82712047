// Nodal forces without any device allocation.
//
// Who needs this: callers that keep the Domain's arrays in device memory they
// manage themselves and must not have a library allocate behind their back,
// for example a Julia program whose CuArrays come from its own memory pool,
// or a host application that budgets every byte of device memory up front.
// Such callers pass device pointers to their own inputs and outputs; the
// per-corner force scratch this computation needs lives in a fixed array
// compiled into the library (g_corner_scratch below), so nothing here calls
// cudaMalloc, cudaFree or any allocating routine.
//
// Costs and limits:
//  * the array holds kStaticMaxElems elements' corner forces (6 MiB plus a
//    status word); CUDA loads the library's device code lazily, so a device
//    commits the array at the first call made there and keeps it until the
//    process exits;
//  * all calls share it: two calls that overlap on the GPU (different
//    streams, or different host threads) race on it and give wrong forces;
//  * the first call on a device looks up the array's device address (once
//    per device); make that first call before any stream capture.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/lulesh_gb300.h"
#include "lulesh_device.cuh"

namespace lulesh {
namespace {

constexpr int64_t kStaticMaxElems = LULESH_STATIC_MAX_ELEMS;

// [0, 24*max): corner forces, component-major then element-major
// (x: [0, 8*max), y: [8*max, 16*max), z: [16*max, 24*max)), index 8*e + c
// as the reference's fx_elem; [24*max]: status bits of the last call.
static __device__ __align__(256) double g_corner_scratch[24 * kStaticMaxElems + 32];

constexpr int kMaxDevices = 64;
void* g_scratch_addr[kMaxDevices] = {};
std::mutex g_scratch_mutex;

// Address of g_corner_scratch on the current device (looked up once).
int scratch_address(double** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return LULESH_ERR_CUDA;
  if (dev < 0 || dev >= kMaxDevices) return LULESH_ERR_ARGUMENT;
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_corner_scratch) != cudaSuccess || !p) return LULESH_ERR_CUDA;
    g_scratch_addr[dev] = p;
  }
  *out = static_cast<double*>(g_scratch_addr[dev]);
  return LULESH_OK;
}

// Corner forces of one element: stress integration (src/domain.jl:1087-1110)
// plus the FB hourglass force (src/domain.jl:1462-1694), written to the
// scratch in the reference's fx_elem layout (8*e + c). The formulation is its
// own (Walsh coefficients, each voluDer call as one FMA chain) rather than the
// step kernels' shared face-diagonal functions; the tests hold it to the
// step's forces and to the CPU oracle's calcForceForNodes at 1e-8.
template <int MODE>
__global__ void __launch_bounds__(128) k_static_corner_forces(lulesh_force_args a, double* scratch,
                                                               int64_t max_elems) {
  const int64_t E = a.num_elem;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= E) return;
  unsigned* status = reinterpret_cast<unsigned*>(scratch + 24 * max_elems);
  int64_t nd[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) nd[c] = a.nodelist[8 * e + c];
  double x[8], y[8], z[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) { x[c] = a.x[nd[c]]; y[c] = a.y[nd[c]]; z[c] = a.z[nd[c]]; }
  double wx[3], wy[3], wz[3], hmx[4], hmy[4], hmz[4];
  walsh7(x, wx, hmx);
  walsh7(y, wy, hmy);
  walsh7(z, wz, hmz);
  {
    const double cxet = fma(wz[0], wy[2], -(wy[0] * wz[2]));
    const double cyet = fma(wx[0], wz[2], -(wz[0] * wx[2]));
    const double czet = fma(wy[0], wx[2], -(wx[0] * wy[2]));
    const double det = fma(wx[1], cxet, fma(wy[1], cyet, wz[1] * czet));
    if (le_zero(det)) atomicOr(status, ST_EARLY);
  }
  double Bx[8], By[8], Bz[8];
  {
    constexpr int fd[6][4] = {{2, 0, 3, 1}, {5, 0, 1, 4}, {6, 1, 2, 5},
                              {7, 2, 3, 6}, {4, 3, 0, 7}, {6, 4, 5, 7}};
    double nx[6], ny[6], nz[6];
#pragma unroll
    for (int f = 0; f < 6; ++f)
      cross(x[fd[f][0]] - x[fd[f][1]], y[fd[f][0]] - y[fd[f][1]], z[fd[f][0]] - z[fd[f][1]],
            x[fd[f][2]] - x[fd[f][3]], y[fd[f][2]] - y[fd[f][3]], z[fd[f][2]] - z[fd[f][3]],
            nx[f], ny[f], nz[f]);
    constexpr int nf[8][3] = {{0, 1, 4}, {0, 1, 2}, {0, 2, 3}, {0, 3, 4},
                              {1, 4, 5}, {1, 2, 5}, {2, 3, 5}, {3, 4, 5}};
#pragma unroll
    for (int n = 0; n < 8; ++n) {
      Bx[n] = (nx[nf[n][0]] + nx[nf[n][1]]) + nx[nf[n][2]];
      By[n] = (ny[nf[n][0]] + ny[nf[n][1]]) + ny[nf[n][2]];
      Bz[n] = (nz[nf[n][0]] + nz[nf[n][1]]) + nz[nf[n][2]];
    }
    if (!(MODE & 1)) {  // src/domain.jl:1050-1055
      By[0] = By[0] + ny[4];
      Bz[0] = nz[0] + nz[1];
    }
  }
  double dvx[8], dvy[8], dvz[8];
  {
    double ex[12], ey[12], ez[12];
    constexpr int ea[12] = {0, 0, 0, 1, 1, 2, 2, 3, 4, 4, 5, 6};
    constexpr int eb[12] = {1, 3, 4, 2, 5, 3, 6, 7, 5, 7, 6, 7};
#pragma unroll
    for (int k = 0; k < 12; ++k) {
      ex[k] = x[ea[k]] + x[eb[k]];
      ey[k] = y[ea[k]] + y[eb[k]];
      ez[k] = z[ea[k]] + z[eb[k]];
    }
    // edge ids of (q1q2, q0q1, q0q4, q3q4, q2q5, q3q5) for each voluDer call
    constexpr int pe[8][6] = {{5, 3, 4, 8, 7, 9}, {3, 0, 2, 9, 6, 11}, {0, 1, 7, 11, 4, 10},
                              {1, 5, 6, 10, 2, 8}, {10, 11, 7, 1, 4, 0}, {11, 9, 2, 0, 6, 3},
                              {9, 8, 4, 3, 7, 5}, {8, 10, 6, 5, 2, 1}};
    constexpr int owner[8] = {0, 3, 2, 1, 4, 5, 6, 7};
#pragma unroll
    for (int n = 0; n < 8; ++n) {
      const int p12 = pe[n][0], p01 = pe[n][1], p04 = pe[n][2], p34 = pe[n][3], p25 = pe[n][4],
                p35 = pe[n][5];
      const double vx = fma(ey[p12], ez[p01], fma(-ey[p01], ez[p12], fma(ey[p04], ez[p34],
                        fma(-ey[p34], ez[p04], fma(-ey[p25], ez[p35], ey[p35] * ez[p25])))));
      const double vy = fma(-ex[p12], ez[p01], fma(ex[p01], ez[p12], fma(-ex[p04], ez[p34],
                        fma(ex[p34], ez[p04], fma(ex[p25], ez[p35], -(ex[p35] * ez[p25]))))));
      const double vz = fma(-ey[p12], ex[p01], fma(ey[p01], ex[p12], fma(-ey[p04], ex[p34],
                        fma(ey[p34], ex[p04], fma(ey[p25], ex[p35], -(ey[p35] * ex[p25]))))));
      const int slot = (MODE & 2) ? owner[n] : n;
      dvx[slot] = vx; dvy[slot] = vy; dvz[slot] = vz;
    }
  }
  const double v = a.v[e];
  const double determ = a.volo[e] * v;
  if (le_zero(v)) atomicOr(status, ST_HOURGLASS);
  const double s8 = ((-a.p[e]) - a.q[e]) * 0.125;
  double* out[3] = {scratch, scratch + 8 * max_elems, scratch + 16 * max_elems};
  const double* Bc[3] = {Bx, By, Bz};
  if (a.hgcoef > 0.0) {
    const double vi12 = 1.0 / (12.0 * determ);
#pragma unroll
    for (int m = 0; m < 4; ++m) { hmx[m] *= vi12; hmy[m] *= vi12; hmz[m] *= vi12; }
    double hg[8][4];
#pragma unroll
    for (int n = 0; n < 8; ++n)
#pragma unroll
      for (int m = 0; m < 4; ++m)
        hg[n][m] = fma(-dvz[n], hmz[m], fma(-dvy[n], hmy[m], fma(-dvx[n], hmx[m], gamma_nm(n, m))));
    const double coef = ((-a.hgcoef * 0.01) * a.ss[e]) * a.elemMass[e] * rcbrt(determ);
    const double* vel[3] = {a.xd, a.yd, a.zd};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      double vv[8];
#pragma unroll
      for (int c = 0; c < 8; ++c) vv[c] = vel[k][nd[c]];
      double h[4];
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        double s = hg[0][m] * vv[0];
#pragma unroll
        for (int n = 1; n < 8; ++n) s = fma(hg[n][m], vv[n], s);
        h[m] = coef * s;
      }
#pragma unroll
      for (int n = 0; n < 8; ++n) {
        const double hgf = fma(hg[n][0], h[0], fma(hg[n][1], h[1], fma(hg[n][2], h[2], hg[n][3] * h[3])));
        out[k][8 * e + n] = fma(s8, Bc[k][n], hgf);
      }
    }
  } else {
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
      for (int n = 0; n < 8; ++n) out[k][8 * e + n] = s8 * Bc[k][n];
  }
}

// fx = sum of the node's corner forces in nodeElemCornerList order
// (src/domain.jl:1112-1127).
__global__ void __launch_bounds__(256) k_static_gather(lulesh_force_args a, const double* scratch,
                                                        int64_t max_elems) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= a.num_node) return;
  const int64_t s = a.nodeElemStart[n], cnt = a.nodeElemCount[n];
  double fx = 0.0, fy = 0.0, fz = 0.0;
  for (int64_t i = 0; i < cnt; ++i) {
    const int64_t k = a.nodeElemCornerList[s + i] - 1;
    if (i == 0) {
      fx = scratch[k]; fy = scratch[8 * max_elems + k]; fz = scratch[16 * max_elems + k];
    } else {
      fx += scratch[k]; fy += scratch[8 * max_elems + k]; fz += scratch[16 * max_elems + k];
    }
  }
  a.fx[n] = fx;
  a.fy[n] = fy;
  a.fz[n] = fz;
}

}  // namespace
}  // namespace lulesh

extern "C" int lulesh_calc_force_for_nodes_static(const lulesh_force_args* args, void* stream,
                                                  int32_t* site) {
  using namespace lulesh;
  if (site) *site = LULESH_SITE_NONE;
  if (!args) return LULESH_ERR_ARGUMENT;
  const lulesh_force_args& a = *args;
  if (a.num_elem < 1 || a.num_node < 1 || a.mode < 0 || a.mode > 7 || !a.nodelist || !a.nodeElemStart ||
      !a.nodeElemCount || !a.nodeElemCornerList || !a.x || !a.y || !a.z || !a.xd || !a.yd || !a.zd ||
      !a.p || !a.q || !a.ss || !a.v || !a.volo || !a.elemMass || !a.fx || !a.fy || !a.fz)
    return LULESH_ERR_ARGUMENT;
  if (a.num_elem > kStaticMaxElems) return LULESH_ERR_ARGUMENT;  // beyond the fixed scratch
  double* scratch = nullptr;
  int rc = scratch_address(&scratch);
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  unsigned* status = reinterpret_cast<unsigned*>(scratch + 24 * kStaticMaxElems);
  if (cudaMemsetAsync(status, 0, sizeof(unsigned), s) != cudaSuccess) return LULESH_ERR_CUDA;
  const int eg = (int)((a.num_elem + 127) / 128);
  switch (a.mode & 3) {
    case 0: k_static_corner_forces<0><<<eg, 128, 0, s>>>(a, scratch, kStaticMaxElems); break;
    case 1: k_static_corner_forces<1><<<eg, 128, 0, s>>>(a, scratch, kStaticMaxElems); break;
    case 2: k_static_corner_forces<2><<<eg, 128, 0, s>>>(a, scratch, kStaticMaxElems); break;
    default: k_static_corner_forces<3><<<eg, 128, 0, s>>>(a, scratch, kStaticMaxElems); break;
  }
  k_static_gather<<<(int)((a.num_node + 255) / 256), 256, 0, s>>>(a, scratch, kStaticMaxElems);
  if (cudaGetLastError() != cudaSuccess) return LULESH_ERR_CUDA;
  unsigned bits = 0;
  if (cudaMemcpyAsync(&bits, status, sizeof(unsigned), cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return LULESH_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return LULESH_ERR_CUDA;
  if (bits & ST_EARLY) { if (site) *site = LULESH_SITE_EARLY; return LULESH_ERR_VOLUME; }
  if (bits & ST_HOURGLASS) { if (site) *site = LULESH_SITE_HOURGLASS; return LULESH_ERR_VOLUME; }
  return LULESH_OK;
}
