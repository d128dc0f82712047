// Forward-mode (dual-number) instance of the oracle: Domain<Dual> carries one
// tangent beside every value through the same restated arithmetic, so a run
// gives the exact Jacobian-vector product J v of the LagrangeLeapFrog cycles
// along the branches the run takes (clamps, limiter cases, dt minima). Test
// infrastructure only: it checks the product's reverse-mode adjoint (a
// vector-Jacobian product) through <w, J v> = <J^T w, v>.
//
// The value parts are computed with exactly the double oracle's operations in
// the same order (build with -ffp-contract=off), so a Domain<Dual> run has the
// double oracle's values bit for bit.
#include <cmath>
#include <cstdint>
#include <cstring>

namespace lulesh_oracle {

struct Dual {
  double v = 0.0, d = 0.0;
  Dual() = default;
  Dual(double a) : v(a), d(0.0) {}  // NOLINT: constants enter as plain doubles
  Dual(double a, double b) : v(a), d(b) {}
  explicit operator double() const { return v; }
  Dual& operator+=(const Dual& b) { d = d + b.d; v = v + b.v; return *this; }
  Dual& operator-=(const Dual& b) { d = d - b.d; v = v - b.v; return *this; }
  Dual& operator*=(const Dual& b) { d = d * b.v + v * b.d; v = v * b.v; return *this; }
  Dual& operator/=(const Dual& b) { const double q = v / b.v; d = (d - q * b.d) / b.v; v = q; return *this; }
};
inline Dual operator-(const Dual& a) { return Dual(-a.v, -a.d); }
inline Dual operator+(Dual a, const Dual& b) { return a += b; }
inline Dual operator-(Dual a, const Dual& b) { return a -= b; }
inline Dual operator*(Dual a, const Dual& b) { return a *= b; }
inline Dual operator/(Dual a, const Dual& b) { return a /= b; }
inline bool operator<(const Dual& a, const Dual& b) { return a.v < b.v; }
inline bool operator>(const Dual& a, const Dual& b) { return a.v > b.v; }
inline bool operator<=(const Dual& a, const Dual& b) { return a.v <= b.v; }
inline bool operator>=(const Dual& a, const Dual& b) { return a.v >= b.v; }
inline bool operator==(const Dual& a, const Dual& b) { return a.v == b.v; }
inline bool operator!=(const Dual& a, const Dual& b) { return a.v != b.v; }
// d sqrt(a) = da / (2 sqrt(a)); d cbrt(a) = da / (3 cbrt(a)^2); a zero
// tangent stays zero where the value is zero.
inline Dual sqrt(const Dual& a) {
  const double r = std::sqrt(a.v);
  return Dual(r, a.d == 0.0 ? 0.0 : a.d / (2.0 * r));
}
inline Dual cbrt(const Dual& a) {
  const double r = std::cbrt(a.v);
  return Dual(r, a.d == 0.0 ? 0.0 : a.d / (3.0 * r * r));
}
inline Dual fabs(const Dual& a) { return a.v < 0.0 ? -a : a; }

}  // namespace lulesh_oracle

#include "lulesh_oracle.hpp"
#include "lulesh_oracle_fields.hpp"

using namespace lulesh_oracle;
using DD = Domain<Dual>;

extern "C" {

void* ord_create(int nx, int nr, int balance, int cost, int mode, unsigned long long seed) {
  if (nx < 1 || nr < 1) return nullptr;
  Problem prob;
  prob.nx = nx; prob.nr = nr; prob.balance = balance; prob.cost = cost; prob.mode = mode;
  prob.region_seed = seed;
  DD* d = new DD();
  buildDomain(*d, prob);
  return d;
}

void ord_destroy(void* h) { delete static_cast<DD*>(h); }
long long ord_num_elem(void* h) { return static_cast<DD*>(h)->numElem; }
long long ord_num_node(void* h) { return static_cast<DD*>(h)->numNode; }
long long ord_cycle(void* h) { return static_cast<DD*>(h)->cycle; }
void ord_set_cycle(void* h, long long c) { static_cast<DD*>(h)->cycle = c; }

// Values and/or tangents of a field (either pointer may be null).
int ord_set_field(void* h, const char* name, const double* val, const double* tan, long long n) {
  auto* f = field_by_name(static_cast<DD*>(h), name);
  if (!f || (long long)f->size() != n) return -1;
  for (long long i = 0; i < n; ++i) {
    if (val) (*f)[i].v = val[i];
    if (tan) (*f)[i].d = tan[i];
  }
  return 0;
}

int ord_get_field(void* h, const char* name, double* val, double* tan, long long n) {
  auto* f = field_by_name(static_cast<DD*>(h), name);
  if (!f || (long long)f->size() != n) return -1;
  for (long long i = 0; i < n; ++i) {
    if (val) val[i] = (*f)[i].v;
    if (tan) tan[i] = (*f)[i].d;
  }
  return 0;
}

int ord_set_scalar(void* h, const char* name, double val, double tan) {
  Dual* s = scalar_by_name(static_cast<DD*>(h), name);
  if (!s) return -1;
  *s = Dual(val, tan);
  return 0;
}

int ord_get_scalar(void* h, const char* name, double* val, double* tan) {
  Dual* s = scalar_by_name(static_cast<DD*>(h), name);
  if (!s) return -1;
  if (val) *val = s->v;
  if (tan) *tan = s->d;
  return 0;
}

int ord_time_increment(void* h) { timeIncrement(*static_cast<DD*>(h)); return 0; }
int ord_lagrange_leapfrog(void* h) { return lagrangeLeapFrog(*static_cast<DD*>(h)); }

// n cycles of timeIncrement! + lagrangeLeapFrog, stopping early once time
// reaches stoptime (the examples/benchmark.jl loop condition).
int ord_cycles(void* h, long long n) {
  DD* d = static_cast<DD*>(h);
  for (long long k = 0; k < n && d->time.v < d->stoptime.v; ++k) {
    timeIncrement(*d);
    int st = lagrangeLeapFrog(*d);
    if (st) return st;
  }
  return 0;
}

}  // extern "C"
