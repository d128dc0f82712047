// Host construction of the single-rank Sedov problem: Domain(prob),
// src/domain.jl:467-771, and createRegionIndexSets!, src/domain.jl:338-465.
// Compiled with -ffp-contract=off so coordinates, volumes, masses and the
// initial dt are the same bits the reference computes.
#include "lulesh_setup.h"

#include <cmath>
#include <random>

namespace lulesh {

static double elem_volume(const double x[8], const double y[8], const double z[8]) {
  // calcElemVolume, src/utils.jl:36-116, in the reference's evaluation order
  auto tp = [](double x1, double y1, double z1, double x2, double y2, double z2, double x3,
               double y3, double z3) {
    return ((x1 * ((y2 * z3) - (z2 * y3)) + x2 * ((z1 * y3) - (y1 * z3))) + x3 * ((y1 * z2) - (z1 * y2)));
  };
  const double dx61 = x[6] - x[1], dy61 = y[6] - y[1], dz61 = z[6] - z[1];
  const double dx70 = x[7] - x[0], dy70 = y[7] - y[0], dz70 = z[7] - z[0];
  const double dx63 = x[6] - x[3], dy63 = y[6] - y[3], dz63 = z[6] - z[3];
  const double dx20 = x[2] - x[0], dy20 = y[2] - y[0], dz20 = z[2] - z[0];
  const double dx50 = x[5] - x[0], dy50 = y[5] - y[0], dz50 = z[5] - z[0];
  const double dx64 = x[6] - x[4], dy64 = y[6] - y[4], dz64 = z[6] - z[4];
  const double dx31 = x[3] - x[1], dy31 = y[3] - y[1], dz31 = z[3] - z[1];
  const double dx72 = x[7] - x[2], dy72 = y[7] - y[2], dz72 = z[7] - z[2];
  const double dx43 = x[4] - x[3], dy43 = y[4] - y[3], dz43 = z[4] - z[3];
  const double dx57 = x[5] - x[7], dy57 = y[5] - y[7], dz57 = z[5] - z[7];
  const double dx14 = x[1] - x[4], dy14 = y[1] - y[4], dz14 = z[1] - z[4];
  const double dx25 = x[2] - x[5], dy25 = y[2] - y[5], dz25 = z[2] - z[5];
  double v = (tp(dx31 + dx72, dx63, dx20, dy31 + dy72, dy63, dy20, dz31 + dz72, dz63, dz20) +
              tp(dx43 + dx57, dx64, dx70, dy43 + dy57, dy64, dy70, dz43 + dz57, dz64, dz70)) +
             tp(dx14 + dx25, dx61, dx50, dy14 + dy25, dy61, dy50, dz14 + dz25, dz61, dz50);
  return v * (1.0 / 12.0);
}

void build_regions(HostMesh& m, int nr, int balance, int cost, uint64_t seed, int rank) {
  const int64_t E = m.E;
  std::mt19937_64 rng(seed);
  // Julia's rand(Int) is a signed 64-bit draw; its % keeps the dividend's sign.
  auto draw = [&]() -> int64_t { return (int64_t)rng(); };
  std::vector<int64_t> size(nr, 0);
  m.regNumList.assign(E, 0);
  if (nr == 1) {
    for (int64_t i = 0; i < E; ++i) m.regNumList[i] = 1;
  } else {
    std::vector<int64_t> binEnd(nr);
    int64_t denom = 0;
    for (int i = 1; i <= nr; ++i) {
      int64_t w = 1;
      for (int k = 0; k < balance; ++k) w *= i;
      denom += w;
      binEnd[i - 1] = denom;
    }
    int64_t next = 0, last = -1;
    auto pick = [&]() -> int64_t {
      const int64_t r = draw() % denom;
      int64_t i = 0;
      while (r >= binEnd[i]) ++i;
      return ((i + rank) % nr) + 1;  // region numbers rotate by the rank
    };
    while (next < E) {
      int64_t region = pick();
      while (region == last) region = pick();
      const int64_t bin = draw() % 1000;
      int64_t count;
      if (bin < 773) count = draw() % 15 + 1;
      else if (bin < 937) count = draw() % 16 + 16;
      else if (bin < 970) count = draw() % 32 + 32;
      else if (bin < 974) count = draw() % 64 + 64;
      else if (bin < 978) count = draw() % 128 + 128;
      else if (bin < 981) count = draw() % 256 + 256;
      else count = draw() % 1537 + 512;
      const int64_t end = count + next;
      while (next < end && next < E) m.regNumList[next++] = region;
      last = region;
    }
  }
  for (int64_t i = 0; i < E; ++i) size[m.regNumList[i] - 1] += 1;
  m.regReps.assign(nr, 0);
  for (int r = 1; r <= nr; ++r) {
    int64_t rep;
    if (r < nr / 2) rep = 1;
    else if (r < nr - (nr + 15) / 20) rep = 1 + cost;
    else rep = 10 * (1 + cost);
    m.regReps[r - 1] = rep;
  }
  // sortRegions, src/domain.jl:313-336: a bubble pass whose inner bound is
  // numReg-i-1 (one comparison short of a full sort), ordering by reps.
  std::vector<int64_t> index(nr);
  for (int v = 0; v < nr; ++v) index[v] = v + 1;
  for (int i = 1; i <= nr - 1; ++i)
    for (int j = 1; j <= nr - i - 1; ++j)
      if (m.regReps[j - 1] < m.regReps[j]) {
        std::swap(m.regReps[j - 1], m.regReps[j]);
        std::swap(size[j - 1], size[j]);
        std::swap(index[j - 1], index[j]);
      }
  m.regSorted.assign(nr, 0);
  for (int i = 1; i <= nr; ++i) m.regSorted[index[i - 1] - 1] = i;
  m.regCSR.assign(nr, 0);
  for (int i = 2; i <= nr; ++i) m.regCSR[i - 1] = m.regCSR[i - 2] + size[i - 2];
  m.regElemlist.assign(E, 0);
  for (int64_t i = 1; i <= E; ++i) {
    const int64_t r = m.regSorted[m.regNumList[i - 1] - 1];
    m.regElemlist[m.regCSR[r - 1]] = i;
    m.regCSR[r - 1] += 1;
  }
  m.regElemSize = size;
}

void build_mesh(HostMesh& m, int nx, int nr, int balance, int cost, uint64_t seed, double einit) {
  const int64_t en = nx + 1;
  m.nx = nx;
  m.E = (int64_t)nx * nx * nx;
  m.N = en * en * en;
  const int64_t E = m.E, N = m.N;

  // buildMesh!, src/domain.jl:117-174: coordinate = 1.125*index/nx
  m.x.resize(N); m.y.resize(N); m.z.resize(N);
  int64_t n = 0;
  for (int64_t pl = 0; pl < en; ++pl) {
    const double tz = 1.125 * (double)pl / (double)nx;
    for (int64_t r = 0; r < en; ++r) {
      const double ty = 1.125 * (double)r / (double)nx;
      for (int64_t c = 0; c < en; ++c) {
        m.x[n] = 1.125 * (double)c / (double)nx;
        m.y[n] = ty;
        m.z[n] = tz;
        ++n;
      }
    }
  }
  m.nodelist.resize(8 * E);
  int64_t z = 0;
  n = 0;
  for (int64_t pl = 0; pl < nx; ++pl) {
    for (int64_t r = 0; r < nx; ++r) {
      for (int64_t c = 0; c < nx; ++c) {
        int* nl = &m.nodelist[8 * z];
        nl[0] = (int)n;
        nl[1] = (int)(n + 1);
        nl[2] = (int)(n + en + 1);
        nl[3] = (int)(n + en);
        nl[4] = (int)(n + en * en);
        nl[5] = (int)(n + en * en + 1);
        nl[6] = (int)(n + en * en + en + 1);
        nl[7] = (int)(n + en * en + en);
        ++z;
        ++n;
      }
      ++n;
    }
    n += en;
  }

  // symmetry plane node sets (setupSymmetryPlanes, src/domain.jl:773-791)
  const int64_t nb = en * en;
  m.symmX.resize(nb); m.symmY.resize(nb); m.symmZ.resize(nb);
  n = 0;
  for (int64_t i = 0; i < en; ++i)
    for (int64_t j = 0; j < en; ++j) {
      m.symmZ[n] = (int)(i * en + j);
      m.symmY[n] = (int)(i * en * en + j);
      m.symmX[n] = (int)(i * en * en + j * en);
      ++n;
    }

  // node -> element-corner lists (src/domain.jl:614-654), element order
  m.nodeElemCount.assign(N, 0);
  for (int64_t i = 0; i < 8 * E; ++i) m.nodeElemCount[m.nodelist[i]] += 1;
  m.nodeElemStart.assign(N + 1, 0);
  for (int64_t i = 0; i < N; ++i) m.nodeElemStart[i + 1] = m.nodeElemStart[i] + m.nodeElemCount[i];
  m.cornerList.resize(8 * E);  // value c*E + e
  {
    std::vector<int> fill(N, 0);
    for (int64_t e = 0; e < E; ++e)
      for (int c = 0; c < 8; ++c) {
        const int g = m.nodelist[8 * e + c];
        m.cornerList[m.nodeElemStart[g] + fill[g]] = (int)(c * E + e);
        fill[g] += 1;
      }
  }

  // volumes and masses (src/domain.jl:709-731)
  m.volo.resize(E); m.elemMass.resize(E);
  m.nodalMass.assign(N, 0.0);
  for (int64_t e = 0; e < E; ++e) {
    double xl[8], yl[8], zl[8];
    for (int c = 0; c < 8; ++c) {
      const int g = m.nodelist[8 * e + c];
      xl[c] = m.x[g]; yl[c] = m.y[g]; zl[c] = m.z[g];
    }
    const double v = elem_volume(xl, yl, zl);
    m.volo[e] = v;
    m.elemMass[e] = v;
    for (int c = 0; c < 8; ++c) {
      const int g = m.nodelist[8 * e + c];
      m.nodalMass[g] = m.nodalMass[g] + v / 8.0;
    }
  }

  // energy deposit and initial dt (src/domain.jl:738-749)
  const double scale = (double)nx / 45.0;
  m.einit = einit > 0.0 ? einit : 3.948746e+7 * scale * scale * scale;
  m.deltatime = (0.5 * std::cbrt(m.volo[0])) / std::sqrt(2.0 * m.einit);

  // element neighbours (setupElementConnectivities, src/domain.jl:793-820),
  // raw Julia values (0-based ids, lxim of element 0 is 1 as written)
  m.lxim.assign(E, 0); m.lxip.assign(E, 0); m.letam.assign(E, 0); m.letap.assign(E, 0);
  m.lzetam.assign(E, 0); m.lzetap.assign(E, 0);
  m.lxim[0] = 1;
  for (int64_t i = 1; i <= E - 1; ++i) { m.lxim[i] = (int)(i - 1); m.lxip[i - 1] = (int)i; }
  m.lxip[E - 1] = (int)(E - 1);
  for (int64_t i = 0; i < nx; ++i) { m.letam[i] = (int)i; m.letap[E - nx + i] = (int)i; }
  for (int64_t i = nx; i <= E - 1; ++i) { m.letam[i] = (int)(i - nx); m.letap[i - nx] = (int)i; }
  const int64_t e2 = (int64_t)nx * nx;
  for (int64_t i = 0; i < e2; ++i) { m.lzetam[i] = (int)i; m.lzetap[E - e2 + i] = (int)(E - e2 + i); }
  for (int64_t i = e2; i <= E - 1; ++i) { m.lzetam[i] = (int)(i - e2); m.lzetap[i - e2] = (int)i; }

  // boundary conditions (setupBoundaryConditions, src/domain.jl:822-916)
  m.elemBC.assign(E, 0u);
  for (int64_t i = 0; i < nx; ++i) {
    const int64_t planeInc = i * e2, rowInc = i * nx;
    for (int64_t j = 0; j < nx; ++j) {
      m.elemBC[rowInc + j] |= 0x01000u;                     // ZETA_M_SYMM
      m.elemBC[rowInc + j + E - e2] |= 0x10000u;            // ZETA_P_FREE
      m.elemBC[planeInc + j] |= 0x00040u;                   // ETA_M_SYMM
      m.elemBC[planeInc + j + e2 - nx] |= 0x00400u;         // ETA_P_FREE
      m.elemBC[planeInc + j * nx] |= 0x00001u;              // XI_M_SYMM
      m.elemBC[planeInc + j * nx + nx - 1] |= 0x00010u;     // XI_P_FREE
    }
  }

  build_regions(m, nr, balance, cost, seed);
}

}  // namespace lulesh
