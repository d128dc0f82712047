// Device memory layout of one problem or one packed ensemble: every array
// of a DevDomain carved from a single allocation, 256-byte aligned.
#pragma once

#include <cstddef>
#include <cstdint>

#include "lulesh_internal.h"

namespace lulesh {

struct Carver {
  char* base;
  size_t off = 0;
  template <class T> T* take(size_t n) {
    off = (off + 255) & ~size_t(255);
    T* p = reinterpret_cast<T*>(base ? base + off : nullptr);
    off += n * sizeof(T);
    return p;
  }
};

// Points dd's arrays into `base` (or only measures when base is null) and
// returns the bytes needed. ninst > 0 adds the ensemble's per-element and
// per-node instance ids, per-instance hgcoef and ninst step states;
// ninst == 0 is a single problem with one step state.
// Eg, nCornerSlot and nCornerList (0 = E, 8E, 8E) size the ghost-extended
// arrays of a block-partitioned mesh.
inline size_t layout(DevDomain& dd, char* base, int64_t E, int64_t N, bool aux, int ninst, int64_t Eg = 0,
                     int64_t nCornerSlot = 0, int64_t nCornerList = 0) {
  if (Eg <= 0) Eg = E;
  if (nCornerSlot <= 0) nCornerSlot = 8 * E;
  if (nCornerList <= 0) nCornerList = 8 * E;
  dd.Eg = (int)Eg;
  dd.nCornerSlot = (int)nCornerSlot;
  dd.nCornerList = (int)nCornerList;
  dd.haloDelvSrc = nullptr;
  dd.haloCornerSrc = nullptr;
  Carver c{base};
  dd.x = c.take<double>(N); dd.y = c.take<double>(N); dd.z = c.take<double>(N);
  dd.xd = c.take<double>(N); dd.yd = c.take<double>(N); dd.zd = c.take<double>(N);
  dd.nodalMass = c.take<double>(N); dd.inv_nodalMass = c.take<double>(N);
  if (aux) {
    dd.xdd = c.take<double>(N); dd.ydd = c.take<double>(N); dd.zdd = c.take<double>(N);
    dd.fx = c.take<double>(N); dd.fy = c.take<double>(N); dd.fz = c.take<double>(N);
  } else {
    dd.xdd = dd.ydd = dd.zdd = dd.fx = dd.fy = dd.fz = nullptr;
  }
  dd.nodeBC = c.take<unsigned char>(N);
  dd.nodeElemStart = c.take<int>(N + 1);
  dd.cornerList = c.take<int>(nCornerList);
  dd.nodelist = c.take<int>(8 * E);
  dd.e = c.take<double>(E); dd.p = c.take<double>(E); dd.q = c.take<double>(E); dd.v = c.take<double>(E);
  dd.volo = c.take<double>(E); dd.inv_volo = c.take<double>(E); dd.elemMass = c.take<double>(E);
  dd.ss = c.take<double>(E); dd.ql = c.take<double>(E); dd.qq = c.take<double>(E);
  dd.vnew = c.take<double>(E); dd.delv = c.take<double>(E); dd.arealg = c.take<double>(E);
  dd.vdov = c.take<double>(E);
  dd.delv_xi = c.take<double>(Eg); dd.delv_eta = c.take<double>(Eg); dd.delv_zeta = c.take<double>(Eg);
  dd.delx_xi = c.take<double>(E); dd.delx_eta = c.take<double>(E); dd.delx_zeta = c.take<double>(E);
  if (aux) {
    dd.dxx = c.take<double>(E); dd.dyy = c.take<double>(E); dd.dzz = c.take<double>(E);
  } else {
    dd.dxx = dd.dyy = dd.dzz = nullptr;
  }
  dd.elemBC = c.take<unsigned int>(E);
  dd.lxim = c.take<int>(E); dd.lxip = c.take<int>(E); dd.letam = c.take<int>(E);
  dd.letap = c.take<int>(E); dd.lzetam = c.take<int>(E); dd.lzetap = c.take<int>(E);
  dd.regElemlist0 = nullptr;
  dd.regOfSlot = nullptr;
  dd.fcx = c.take<double>(nCornerSlot); dd.fcy = c.take<double>(nCornerSlot); dd.fcz = c.take<double>(nCornerSlot);
  dd.nextGeo = c.take<double>((size_t)kGeoSlots * E);
  dd.tapeGeoNext = nullptr;
  dd.tapeDiag = nullptr;
  dd.st = c.take<DevState>(ninst > 0 ? ninst : 1);
  if (ninst > 0) {
    dd.elemInst = c.take<int>(E);
    dd.nodeInst = c.take<int>(N);
    dd.instHg = c.take<double>(ninst);
  } else {
    dd.elemInst = nullptr;
    dd.nodeInst = nullptr;
    dd.instHg = nullptr;
  }
  dd.ninst = ninst > 0 ? ninst : 1;
  // the halo sources of a block-partitioned mesh
  if (Eg > E) dd.haloDelvSrc = c.take<int>(Eg - E);
  if (nCornerSlot > 8 * E) dd.haloCornerSrc = c.take<int>(nCornerSlot - 8 * E);
  return c.off + 256;
}

}  // namespace lulesh
