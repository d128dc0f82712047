// The multi-rank decomposition as blocks of one mesh (build_block_mesh).
//
// The reference runs a cube of tp^3 MPI ranks, each an nx^3 block of the
// (tp*nx)^3 mesh (initMeshDecomp, src/LULESH.jl:62-97), and exchanges three
// things per cycle: the nodal forces of nodes on block faces (commSBN,
// src/comm.jl:776), the positions and velocities of those nodes
// (commSyncPosVel, :1251) and the monotonic-Q gradients of the elements
// beside a block face (commMonoQ, :1127), plus a min-allreduce of the time
// step (comm_min, src/mpi.jl:81).
//
// Here the blocks are packed into one index space, block after block, each in
// the reference's per-rank element and node order, nodes on block faces
// duplicated. Every value that crosses a block face goes through a ghost
// slot a halo copy fills from the block that owns it:
//  * a node's force is the sum of its corner forces in the whole mesh's
//    nodeElemCornerList order; the corners that belong to another block are
//    ghost corner slots (what commSBN sums, at corner granularity). Every copy
//    of a shared node therefore sums the same values in the same order and
//    gets the same bits, so positions and velocities agree without the
//    overwrite commSyncPosVel does;
//  * the limiter's reads of a neighbour across a block face are ghost delv
//    slots (the values commMonoQ sends);
//  * all blocks reduce their Courant and hydro minima into one step state
//    (the min-allreduce).
// The result is bitwise the single-block run of the whole mesh, which the
// tests check. The reference's own multi-rank setup differs in ways that are
// defects, not method: its ghost offsets test the functions m_planeMax,
// m_rowMin, m_rowMax, m_colMin, m_colMax instead of calling them, and its
// eta-face ghost indices add rowInc where the plane offset belongs
// (src/domain.jl:838-905); nodal masses are summed per rank before the first
// commSBN. Those are not reproduced.
#include <algorithm>
#include <cstdint>
#include <unordered_map>

#include "lulesh_setup.h"

namespace lulesh {

namespace {
// BC mask bits, src/bc.jl:3-30
constexpr unsigned kXiM = 0x00007, kXiMComm = 0x00004, kXiP = 0x00038, kXiPComm = 0x00020;
constexpr unsigned kEtaM = 0x001c0, kEtaMComm = 0x00100, kEtaP = 0x00e00, kEtaPComm = 0x00800;
constexpr unsigned kZetaM = 0x07000, kZetaMComm = 0x04000, kZetaP = 0x38000, kZetaPComm = 0x20000;
}  // namespace

void build_block_mesh(HostMesh& m, const HostMesh& g, int nx, int tp, int mode) {
  const int64_t nxg = (int64_t)nx * tp, eng = nxg + 1, en = nx + 1;
  const int64_t nb = (int64_t)tp * tp * tp, Eb = (int64_t)nx * nx * nx, Nb = en * en * en;
  const int64_t E = nb * Eb, N = nb * Nb, Eglob = g.E;
  m = HostMesh();
  m.nx = nx;
  m.blocks_per_edge = tp;
  m.E = E;
  m.N = N;
  m.einit = g.einit;
  m.deltatime = g.deltatime;

  // packed index of a global element (its owning block) and of a global node
  // within a given block
  auto elem_packed = [&](int64_t ge) -> int64_t {
    const int64_t gi = ge % nxg, gj = (ge / nxg) % nxg, gk = ge / (nxg * nxg);
    const int64_t b = ((gk / nx) * tp + gj / nx) * tp + gi / nx;
    return b * Eb + ((gk % nx) * nx + gj % nx) * nx + gi % nx;
  };
  auto block_of_packed_elem = [&](int64_t pe) { return pe / Eb; };

  m.elemGlobal.resize(E);
  m.nodeGlobal.resize(N);
  m.x.resize(N); m.y.resize(N); m.z.resize(N); m.nodalMass.resize(N);
  m.volo.resize(E); m.elemMass.resize(E);
  m.nodelist.resize(8 * E);
  m.elemBC.resize(E);
  m.lxim.resize(E); m.lxip.resize(E); m.letam.resize(E); m.letap.resize(E); m.lzetam.resize(E); m.lzetap.resize(E);

  // global symmetry-plane membership of every node
  std::vector<unsigned char> gsym(g.N, 0);
  for (int v : g.symmX) gsym[v] |= 1u;
  for (int v : g.symmY) gsym[v] |= 2u;
  for (int v : g.symmZ) gsym[v] |= 4u;

  for (int64_t b = 0; b < nb; ++b) {
    const int64_t col = b % tp, row = (b / tp) % tp, plane = b / (tp * tp);
    // nodes
    for (int64_t k = 0; k < en; ++k)
      for (int64_t j = 0; j < en; ++j)
        for (int64_t i = 0; i < en; ++i) {
          const int64_t pn = b * Nb + (k * en + j) * en + i;
          const int64_t gn = ((plane * nx + k) * eng + (row * nx + j)) * eng + (col * nx + i);
          m.nodeGlobal[pn] = (int)gn;
          m.x[pn] = g.x[gn]; m.y[pn] = g.y[gn]; m.z[pn] = g.z[gn];
          m.nodalMass[pn] = g.nodalMass[gn];
          if (gsym[gn] & 1u) m.symmX.push_back((int)pn);
          if (gsym[gn] & 2u) m.symmY.push_back((int)pn);
          if (gsym[gn] & 4u) m.symmZ.push_back((int)pn);
        }
    auto node_packed = [&](int64_t gn) -> int64_t {
      const int64_t gi = gn % eng, gj = (gn / eng) % eng, gk = gn / (eng * eng);
      return b * Nb + ((gk - plane * nx) * en + (gj - row * nx)) * en + (gi - col * nx);
    };
    // ghost delv slots of this block, one per remote element it reads
    std::unordered_map<int64_t, int64_t> ghost_of;
    auto target = [&](int64_t ge_t) -> int64_t {
      const int64_t pt = elem_packed(ge_t);
      if (block_of_packed_elem(pt) == b) return pt;
      auto it = ghost_of.find(ge_t);
      if (it != ghost_of.end()) return it->second;
      const int64_t slot = E + (int64_t)m.haloDelvSrc.size();
      m.haloDelvSrc.push_back((int)pt);
      m.haloDelvDst.push_back((int)b);
      ghost_of.emplace(ge_t, slot);
      return slot;
    };
    for (int64_t k = 0; k < nx; ++k)
      for (int64_t j = 0; j < nx; ++j)
        for (int64_t i = 0; i < nx; ++i) {
          const int64_t pe = b * Eb + (k * nx + j) * nx + i;
          const int64_t ge = ((plane * nx + k) * nxg + (row * nx + j)) * nxg + (col * nx + i);
          m.elemGlobal[pe] = (int)ge;
          m.volo[pe] = g.volo[ge];
          m.elemMass[pe] = g.elemMass[ge];
          for (int c = 0; c < 8; ++c) m.nodelist[8 * pe + c] = (int)node_packed(g.nodelist[8 * ge + c]);
          const unsigned gm = g.elemBC[ge];
          unsigned mask = gm;
          if (i == 0 && col > 0) mask |= kXiMComm;
          if (i == nx - 1 && col < tp - 1) mask |= kXiPComm;
          if (j == 0 && row > 0) mask |= kEtaMComm;
          if (j == nx - 1 && row < tp - 1) mask |= kEtaPComm;
          if (k == 0 && plane > 0) mask |= kZetaMComm;
          if (k == nx - 1 && plane < tp - 1) mask |= kZetaPComm;
          m.elemBC[pe] = mask;
          // the element the whole-mesh limiter reads in each direction: where
          // its face is interior (no bits in the whole mesh's mask), the
          // neighbour index; otherwise it reads itself, a constant or nothing
          auto nb_of = [&](const std::vector<int>& raw, unsigned bits, int shift) -> int64_t {
            if ((gm & bits) != 0u) return pe + shift;
            return target((int64_t)raw[ge] - shift) + shift;
          };
          const int xpshift = (mode & 4) ? 0 : 1;  // the reference's xi-plus read is delv_xi[lxip - 1]
          m.lxim[pe] = (int)nb_of(g.lxim, kXiM, 0);
          m.lxip[pe] = (int)nb_of(g.lxip, kXiP, xpshift);
          m.letam[pe] = (int)nb_of(g.letam, kEtaM, 0);
          m.letap[pe] = (int)nb_of(g.letap, kEtaP, 0);
          m.lzetam[pe] = (int)nb_of(g.lzetam, kZetaM, 0);
          m.lzetap[pe] = (int)nb_of(g.lzetap, kZetaP, 0);
        }
  }
  m.Eg = E + (int64_t)m.haloDelvSrc.size();

  // each node's corners in the whole mesh's order; a corner of another
  // block's element is a ghost corner slot of this block
  m.nodeElemCount.assign(N, 0);
  m.nodeElemStart.assign(N + 1, 0);
  m.cornerList.clear();
  m.cornerList.reserve(8 * E + 6 * Eb);
  for (int64_t b = 0; b < nb; ++b) {
    std::unordered_map<int64_t, int64_t> ghost_of;  // global corner value -> slot
    for (int64_t ln = 0; ln < Nb; ++ln) {
      const int64_t pn = b * Nb + ln;
      const int64_t gn = m.nodeGlobal[pn];
      const int64_t s = g.nodeElemStart[gn], t = g.nodeElemStart[gn + 1];
      m.nodeElemStart[pn] = (int)m.cornerList.size();
      for (int64_t q = s; q < t; ++q) {
        const int64_t v = g.cornerList[q];
        const int64_t c = v / Eglob, ge = v % Eglob;
        const int64_t pe = elem_packed(ge);
        int64_t slot;
        if (block_of_packed_elem(pe) == b) {
          slot = c * E + pe;
        } else {
          auto it = ghost_of.find(v);
          if (it != ghost_of.end()) {
            slot = it->second;
          } else {
            slot = 8 * E + (int64_t)m.haloCornerSrc.size();
            m.haloCornerSrc.push_back((int)(c * E + pe));
            m.haloCornerDst.push_back((int)b);
            ghost_of.emplace(v, slot);
          }
        }
        m.cornerList.push_back((int)slot);
      }
      m.nodeElemCount[pn] = (int)(t - s);
    }
  }
  m.nodeElemStart[N] = (int)m.cornerList.size();
  m.nCornerList = (int64_t)m.cornerList.size();
  m.nCornerSlot = 8 * E + (int64_t)m.haloCornerSrc.size();
}

void build_block_regions(HostMesh& m, int nx, int tp, int nr, int balance, int cost, uint64_t seed) {
  const int64_t Eb = (int64_t)nx * nx * nx, nb = (int64_t)tp * tp * tp, E = nb * Eb;
  m.regNumList.assign(E, 0);
  m.regElemlist.assign(E, 0);
  m.regionOrder.assign(E, 0);
  m.regionReps.assign(E, 0);
  for (int64_t b = 0; b < nb; ++b) {
    HostMesh r;
    r.E = Eb;
    build_regions(r, nr, balance, cost, seed + (uint64_t)b, (int)b);
    const int64_t off = b * Eb;
    int64_t pos = 0;
    for (size_t q = 0; q < r.regElemSize.size(); ++q)
      for (int64_t k = 0; k < r.regElemSize[q]; ++k, ++pos) {
        m.regionOrder[off + pos] = (int)(off + r.regElemlist[pos] - 1);
        m.regionReps[off + pos] = (int)r.regReps[q];
      }
    for (int64_t k = 0; k < Eb; ++k) {
      m.regNumList[off + k] = r.regNumList[k];
      m.regElemlist[off + k] = off + r.regElemlist[k];
    }
    if (b == 0) {
      m.regCSR = r.regCSR;
      m.regReps = r.regReps;
      m.regSorted = r.regSorted;
      m.regElemSize = r.regElemSize;
    }
  }
}

}  // namespace lulesh
