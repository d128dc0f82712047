// C entry points over the oracle (test infrastructure only; see the header of
// lulesh_oracle.hpp). Fields are exposed by name as pointers into the
// oracle's own storage so tests can read and overwrite state in place.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "lulesh_oracle.hpp"
#include "lulesh_oracle_fields.hpp"

#ifdef _OPENMP
#include <omp.h>
#endif

using namespace lulesh_oracle;
using D = Domain<double>;

static std::vector<double>* f64_field(D* d, const char* name) { return field_by_name(d, name); }
static std::vector<int64_t>* i64_field(D* d, const char* name) { return index_field_by_name(d, name); }
static double* f64_scalar(D* d, const char* name) { return scalar_by_name(d, name); }

extern "C" {

void* ora_create(int nx, int nr, int balance, int cost, int mode, unsigned long long seed) {
  if (nx < 1 || nr < 1) return nullptr;
  Problem prob;
  prob.nx = nx; prob.nr = nr; prob.balance = balance; prob.cost = cost; prob.mode = mode;
  prob.region_seed = seed;
  D* d = new D();
  buildDomain(*d, prob);
  return d;
}

void ora_destroy(void* h) { delete static_cast<D*>(h); }

long long ora_num_elem(void* h) { return static_cast<D*>(h)->numElem; }
long long ora_num_node(void* h) { return static_cast<D*>(h)->numNode; }
long long ora_cycle(void* h) { return static_cast<D*>(h)->cycle; }
void ora_set_cycle(void* h, long long c) { static_cast<D*>(h)->cycle = c; }
int ora_error_site(void* h) { return static_cast<D*>(h)->error_site; }
long long ora_error_index(void* h) { return static_cast<D*>(h)->error_index; }

double* ora_field_f64(void* h, const char* name, long long* n) {
  auto* f = f64_field(static_cast<D*>(h), name);
  if (!f) return nullptr;
  *n = (long long)f->size();
  return f->data();
}

long long* ora_field_i64(void* h, const char* name, long long* n) {
  auto* f = i64_field(static_cast<D*>(h), name);
  if (!f) return nullptr;
  *n = (long long)f->size();
  return reinterpret_cast<long long*>(f->data());
}

unsigned int* ora_elem_bc(void* h, long long* n) {
  D* d = static_cast<D*>(h);
  *n = (long long)d->elemBC.size();
  return d->elemBC.data();
}

int ora_get_scalar(void* h, const char* name, double* out) {
  double* s = f64_scalar(static_cast<D*>(h), name);
  if (!s) return -1;
  *out = *s;
  return 0;
}

int ora_set_scalar(void* h, const char* name, double v) {
  double* s = f64_scalar(static_cast<D*>(h), name);
  if (!s) return -1;
  *s = v;
  return 0;
}

// Replaces the deposited origin energy and the initial dt computed from it,
// as src/domain.jl:738-749 does for the default energy.
void ora_set_einit(void* h, double einit) {
  D* d = static_cast<D*>(h);
  d->e[0] = einit;
  d->deltatime = (0.5 * std::cbrt(d->volo[0])) / std::sqrt(2.0 * einit);
}

int ora_time_increment(void* h) { timeIncrement(*static_cast<D*>(h)); return 0; }
int ora_lagrange_leapfrog(void* h) { return lagrangeLeapFrog(*static_cast<D*>(h)); }
int ora_lagrange_nodal(void* h) { return lagrangeNodal(*static_cast<D*>(h)); }
int ora_lagrange_elements(void* h) { return lagrangeElements(*static_cast<D*>(h)); }
int ora_force_for_nodes(void* h) { return calcForceForNodes(*static_cast<D*>(h)); }
int ora_time_constraints(void* h) { calcTimeConstraintsForElems(*static_cast<D*>(h)); return 0; }

// The examples/benchmark.jl:82-98 loop: timeIncrement!, lagrangeLeapFrog,
// stop at stoptime or once cycle >= num_iters. Returns the step status.
int ora_run(void* h, long long num_iters) {
  D* d = static_cast<D*>(h);
  while (d->time < d->stoptime) {
    timeIncrement(*d);
    int st = lagrangeLeapFrog(*d);
    if (st) return st;
    if (d->cycle >= num_iters) break;
  }
  return 0;
}

void ora_symmetry(void* h, double* out3) { symmetryCheck(*static_cast<D*>(h), out3); }

int ora_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void ora_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

}  // extern "C"

#ifdef ORACLE_MAIN
// Command line: lulesh_oracle -s N [-i iters] [-r nr] [-b balance] [-c cost]
// [--lulesh2] [-t threads]. Prints the reference's verifyAndWriteFinalOutput
// report (src/utils.jl:124-164) for the run.
int main(int argc, char** argv) {
  int nx = 30, nr = 11, balance = 1, cost = 1, mode = FAITHFUL, threads = 0;
  long long iters = (1LL << 62);
  for (int i = 1; i < argc; ++i) {
    std::string a = argv[i];
    auto next = [&]() { return (i + 1 < argc) ? argv[++i] : (char*)"0"; };
    if (a == "-s") nx = std::atoi(next());
    else if (a == "-i") iters = std::atoll(next());
    else if (a == "-r") nr = std::atoi(next());
    else if (a == "-b") balance = std::atoi(next());
    else if (a == "-c") cost = std::atoi(next());
    else if (a == "-t") threads = std::atoi(next());
    else if (a == "--lulesh2") mode = LULESH2;
    else if (a == "-m") mode = std::atoi(next());
    else { std::fprintf(stderr, "unknown argument %s\n", a.c_str()); return 2; }
  }
  ora_set_threads(threads);
  void* h = ora_create(nx, nr, balance, cost, mode, 0);
  D* d = static_cast<D*>(h);
  auto t0 = std::chrono::steady_clock::now();
  int st = ora_run(h, iters);
  auto t1 = std::chrono::steady_clock::now();
  double elapsed = std::chrono::duration<double>(t1 - t0).count();
  if (st) { std::printf("step status %d (site %d, index %lld)\n", st, d->error_site, (long long)d->error_index); return 1; }
  double sym[3];
  symmetryCheck(*d, sym);
  double grind = ((elapsed * 1e6) / (double)d->cycle) / (double)((long long)nx * nx * nx);
  std::printf("Run completed:\n");
  std::printf("   Problem size        =  %d\n", nx);
  std::printf("   MPI tasks           =  1\n");
  std::printf("   Iteration count     =  %lld\n", (long long)d->cycle);
  std::printf("   Final Origin Energy =  %.6e\n", d->e[0]);
  std::printf("   Testing Plane 0 of Energy Array on rank 0:\n");
  std::printf("        MaxAbsDiff   = %.6e\n", sym[0]);
  std::printf("        TotalAbsDiff = %.6e\n", sym[1]);
  std::printf("        MaxRelDiff   = %.6e\n", sym[2]);
  std::printf("\nElapsed time         = %.2f (s)\n", elapsed);
  std::printf("Grind time (us/z/c)  =  %.8f  (per dom)\n", grind);
  std::printf("FOM                  = %.8f (z/s)\n", 1000.0 / grind);
  std::printf("final time           = %.17g\n", d->time);
  std::printf("threads              = %d\n", ora_max_threads());
  ora_destroy(h);
  return 0;
}
#endif
