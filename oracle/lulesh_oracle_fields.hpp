// Name -> member tables of the oracle's Domain<T>, shared by the double and
// the dual-number C entry points (test infrastructure only).
#pragma once

#include <cstring>
#include <vector>

#include "lulesh_oracle.hpp"

namespace lulesh_oracle {

template <class T>
std::vector<T>* field_by_name(Domain<T>* d, const char* name) {
  using D = Domain<T>;
  struct E { const char* n; std::vector<T> D::*m; };
  static const E tab[] = {
      {"e", &D::e}, {"p", &D::p}, {"q", &D::q}, {"ql", &D::ql}, {"qq", &D::qq}, {"v", &D::v},
      {"volo", &D::volo}, {"delv", &D::delv}, {"vdov", &D::vdov}, {"arealg", &D::arealg},
      {"ss", &D::ss}, {"elemMass", &D::elemMass}, {"vnew", &D::vnew}, {"delv_xi", &D::delv_xi},
      {"delv_eta", &D::delv_eta}, {"delv_zeta", &D::delv_zeta}, {"delx_xi", &D::delx_xi},
      {"delx_eta", &D::delx_eta}, {"delx_zeta", &D::delx_zeta}, {"dxx", &D::dxx}, {"dyy", &D::dyy},
      {"dzz", &D::dzz}, {"x", &D::x}, {"y", &D::y}, {"z", &D::z}, {"xd", &D::xd}, {"yd", &D::yd},
      {"zd", &D::zd}, {"xdd", &D::xdd}, {"ydd", &D::ydd}, {"zdd", &D::zdd}, {"fx", &D::fx},
      {"fy", &D::fy}, {"fz", &D::fz}, {"nodalMass", &D::nodalMass}, {"determ", &D::determ},
      {"fx_elem", &D::fx_elem}, {"fy_elem", &D::fy_elem}, {"fz_elem", &D::fz_elem},
      {"dvdx", &D::dvdx}, {"dvdy", &D::dvdy}, {"dvdz", &D::dvdz},
  };
  for (const auto& t : tab)
    if (!std::strcmp(t.n, name)) return &(d->*(t.m));
  return nullptr;
}

template <class T>
std::vector<int64_t>* index_field_by_name(Domain<T>* d, const char* name) {
  using D = Domain<T>;
  struct E { const char* n; std::vector<int64_t> D::*m; };
  static const E tab[] = {
      {"matElemlist", &D::matElemlist}, {"nodelist", &D::nodelist}, {"lxim", &D::lxim},
      {"lxip", &D::lxip}, {"letam", &D::letam}, {"letap", &D::letap}, {"lzetam", &D::lzetam},
      {"lzetap", &D::lzetap}, {"symmX", &D::symmX}, {"symmY", &D::symmY}, {"symmZ", &D::symmZ},
      {"nodeElemCount", &D::nodeElemCount}, {"nodeElemStart", &D::nodeElemStart},
      {"nodeElemCornerList", &D::nodeElemCornerList}, {"regElemSize", &D::regElemSize},
      {"regCSR", &D::regCSR}, {"regReps", &D::regReps}, {"regNumList", &D::regNumList},
      {"regElemlist", &D::regElemlist}, {"regSorted", &D::regSorted},
  };
  for (const auto& t : tab)
    if (!std::strcmp(t.n, name)) return &(d->*(t.m));
  return nullptr;
}

template <class T>
T* scalar_by_name(Domain<T>* d, const char* name) {
  using D = Domain<T>;
  struct E { const char* n; T D::*m; };
  static const E tab[] = {
      {"dtfixed", &D::dtfixed}, {"deltatimemultlb", &D::deltatimemultlb},
      {"deltatimemultub", &D::deltatimemultub}, {"stoptime", &D::stoptime}, {"dtmax", &D::dtmax},
      {"dthydro", &D::dthydro}, {"dtcourant", &D::dtcourant}, {"time", &D::time},
      {"deltatime", &D::deltatime}, {"u_cut", &D::u_cut}, {"hgcoef", &D::hgcoef},
      {"qstop", &D::qstop}, {"monoq_max_slope", &D::monoq_max_slope},
      {"monoq_limiter_mult", &D::monoq_limiter_mult}, {"e_cut", &D::e_cut}, {"p_cut", &D::p_cut},
      {"ss4o3", &D::ss4o3}, {"q_cut", &D::q_cut}, {"v_cut", &D::v_cut},
      {"qlc_monoq", &D::qlc_monoq}, {"qqc_monoq", &D::qqc_monoq}, {"qqc", &D::qqc},
      {"eosvmax", &D::eosvmax}, {"eosvmin", &D::eosvmin}, {"pmin", &D::pmin}, {"emin", &D::emin},
      {"dvovmax", &D::dvovmax}, {"refdens", &D::refdens},
  };
  for (const auto& t : tab)
    if (!std::strcmp(t.n, name)) return &(d->*(t.m));
  return nullptr;
}

}  // namespace lulesh_oracle
