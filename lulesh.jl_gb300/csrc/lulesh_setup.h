// Host-side construction of the Sedov problem (lulesh_setup.cpp).
#pragma once

#include <cstdint>
#include <vector>

namespace lulesh {

struct HostMesh {
  int nx = 0;
  int64_t E = 0, N = 0;
  std::vector<double> x, y, z, volo, elemMass, nodalMass;
  std::vector<int> nodelist;                 // 8E, element-major, 0-based node ids
  std::vector<int> lxim, lxip, letam, letap, lzetam, lzetap;  // raw Julia values
  std::vector<unsigned int> elemBC;
  std::vector<int> symmX, symmY, symmZ;
  std::vector<int> nodeElemCount;            // N
  std::vector<int> nodeElemStart;            // N+1
  std::vector<int> cornerList;               // 8E, values c*E + e
  std::vector<int64_t> regNumList, regElemlist, regCSR, regReps, regSorted, regElemSize;
  double einit = 0.0, deltatime = 0.0;
};

// Builds the nx^3 single-rank Sedov mesh exactly as Domain(prob) does. A
// positive einit replaces the energy deposited in the origin element (and
// the initial dt computed from it); 0 keeps 3.948746e7*(nx/45)^3.
void build_mesh(HostMesh& m, int nx, int nr, int balance, int cost, uint64_t seed, double einit = 0.0);

// createRegionIndexSets! (results-neutral region layout).
void build_regions(HostMesh& m, int nr, int balance, int cost, uint64_t seed);

}  // namespace lulesh
