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
  // A block-partitioned mesh (build_block_mesh) packs tp^3 blocks; its
  // limiter reads and node gathers that cross a block face go through ghost
  // slots filled by halo copies. Zero sizes mean a single block (Eg = E,
  // corner slots = corner list entries = 8E).
  int blocks_per_edge = 1;
  int64_t Eg = 0, nCornerSlot = 0, nCornerList = 0;
  std::vector<int> haloDelvSrc, haloDelvDst;      // per ghost delv slot: source element, receiving block
  std::vector<int> haloCornerSrc, haloCornerDst;  // per ghost corner slot: source slot c*E + e, receiving block
  std::vector<int> elemGlobal, nodeGlobal;        // packed -> global element / node of the whole mesh
  std::vector<int> regionOrder, regionReps;       // region cost model of a block mesh (build_block_regions)
};

// Builds the nx^3 single-rank Sedov mesh exactly as Domain(prob) does. A
// positive einit replaces the energy deposited in the origin element (and
// the initial dt computed from it); 0 keeps 3.948746e7*(nx/45)^3.
void build_mesh(HostMesh& m, int nx, int nr, int balance, int cost, uint64_t seed, double einit = 0.0);

// createRegionIndexSets! (results-neutral region layout) of rank `rank`: the
// reference seeds each rank's draws with its rank and rotates the region
// numbers by it (src/domain.jl:338-465); a single rank is rank 0.
void build_regions(HostMesh& m, int nr, int balance, int cost, uint64_t seed, int rank = 0);

// The region sets of a block mesh: block b gets rank b's (draws seeded with
// seed + b, numbers rotated by b) over its own elements. regNumList and
// regElemlist hold every block's entries in packed order (regElemlist's
// 1-based ids are packed ids); regCSR, regReps, regSorted and regElemSize are
// block 0's; regionOrder / regionReps give the cost model's packed element
// of every position and its rep count, block after block.
void build_block_regions(HostMesh& m, int nx, int tp, int nr, int balance, int cost, uint64_t seed);

// The reference's multi-rank decomposition (initMeshDecomp, src/LULESH.jl:62-97:
// tp^3 ranks, rank r the block col = r % tp, row = (r / tp) % tp,
// plane = r / tp^2 of edge nx) of the (tp*nx)^3 mesh `g` (built by
// build_mesh), packed block after block into `m`: each block's elements and
// (nx+1)^3 nodes in the reference's per-rank order, nodes on block faces
// duplicated in every block that touches them, COMM masks on block faces
// (src/domain.jl:822-916). Values come from `g`, so the blocks hold the whole
// mesh's bits. The limiter's neighbour reads and each node's corner gather
// keep the whole mesh's order; where they cross a block face they read ghost
// slots that the halo copies fill from the neighbouring block (the reads of
// commMonoQ and commSBN, src/comm.jl:1127, 776). `mode` selects the xi-plus
// read of the limiter (the reference's defect unless bit 4 is set).
void build_block_mesh(HostMesh& m, const HostMesh& g, int nx, int tp, int mode);

}  // namespace lulesh
