// Full-state files: save a handle's step state (the 11 state fields and all
// Domain scalars) to a binary file and load it back into a handle of the same
// problem. The reference has no checkpoint format; this one exists so runs can
// be resumed, compared offline, or restarted from a dump.
//
// Layout (little-endian):
//   "LULESHS1"                                   8 bytes
//   int32 version (1), nx, nr, balance, cost, mode
//   int64 numElem, numNode
//   int32 scalar count (LULESH_S_COUNT), field count (11)
//   double scalars[LULESH_S_COUNT]               (cycle stored as a double)
//   per field: int32 id, int64 count, double values[count]
//   uint64 FNV-1a hash of every byte after the magic up to here
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/lulesh_gb300.h"
#include "lulesh_handle.h"

namespace {

const char kMagic[8] = {'L', 'U', 'L', 'E', 'S', 'H', 'S', '1'};
const int32_t kVersion = 1;
const int32_t kStateFields[11] = {LULESH_F_X, LULESH_F_Y, LULESH_F_Z, LULESH_F_XD, LULESH_F_YD, LULESH_F_ZD,
                                  LULESH_F_E, LULESH_F_P, LULESH_F_Q, LULESH_F_V, LULESH_F_SS};

struct Hash {
  uint64_t h = 1469598103934665603ull;  // FNV-1a offset basis
  void add(const void* p, size_t n) {
    const unsigned char* b = static_cast<const unsigned char*>(p);
    for (size_t i = 0; i < n; ++i) { h ^= b[i]; h *= 1099511628211ull; }
  }
};

struct Writer {
  FILE* f;
  Hash hash;
  bool ok = true;
  void put(const void* p, size_t n) {
    if (ok && std::fwrite(p, 1, n, f) != n) ok = false;
    hash.add(p, n);
  }
};

struct Reader {
  FILE* f;
  Hash hash;
  bool ok = true;
  void get(void* p, size_t n) {
    if (ok && std::fread(p, 1, n, f) != n) ok = false;
    if (ok) hash.add(p, n);
  }
};

}  // namespace

extern "C" {

int lulesh_save_state(lulesh_domain* d, const char* path) {
  if (!d || !path) return LULESH_ERR_ARGUMENT;
  std::vector<std::vector<double>> fields(11);
  for (int k = 0; k < 11; ++k) {
    int64_t n = 0;
    int rc = lulesh_field_length(d, kStateFields[k], &n);
    if (rc) return rc;
    fields[k].resize(n);
    if ((rc = lulesh_download_field(d, kStateFields[k], fields[k].data(), n))) return rc;
  }
  FILE* f = std::fopen(path, "wb");
  if (!f) return LULESH_ERR_ARGUMENT;
  Writer w{f, Hash{}, true};
  if (std::fwrite(kMagic, 1, 8, f) != 8) w.ok = false;
  const lulesh_params& p = d->params;
  const int32_t head[6] = {kVersion, p.nx, p.nr, p.balance, p.cost, p.mode};
  w.put(head, sizeof(head));
  const int64_t sizes[2] = {d->E, d->N};
  w.put(sizes, sizeof(sizes));
  const int32_t counts[2] = {LULESH_S_COUNT, 11};
  w.put(counts, sizeof(counts));
  w.put(d->sc, sizeof(double) * LULESH_S_COUNT);
  for (int k = 0; k < 11; ++k) {
    const int64_t n = (int64_t)fields[k].size();
    w.put(&kStateFields[k], sizeof(int32_t));
    w.put(&n, sizeof(n));
    w.put(fields[k].data(), sizeof(double) * n);
  }
  const uint64_t h = w.hash.h;
  if (w.ok && std::fwrite(&h, 1, sizeof(h), f) != sizeof(h)) w.ok = false;
  if (std::fclose(f) != 0) w.ok = false;
  return w.ok ? LULESH_OK : LULESH_ERR_ARGUMENT;
}

int lulesh_load_state(lulesh_domain* d, const char* path) {
  if (!d || !path) return LULESH_ERR_ARGUMENT;
  FILE* f = std::fopen(path, "rb");
  if (!f) return LULESH_ERR_ARGUMENT;
  Reader r{f, Hash{}, true};
  char magic[8];
  if (std::fread(magic, 1, 8, f) != 8 || std::memcmp(magic, kMagic, 8) != 0) { std::fclose(f); return LULESH_ERR_ARGUMENT; }
  int32_t head[6];
  int64_t sizes[2];
  int32_t counts[2];
  r.get(head, sizeof(head));
  r.get(sizes, sizeof(sizes));
  r.get(counts, sizeof(counts));
  const lulesh_params& p = d->params;
  // the file must describe this handle's problem
  if (!r.ok || head[0] != kVersion || head[1] != p.nx || head[2] != p.nr || head[3] != p.balance ||
      head[4] != p.cost || head[5] != p.mode || sizes[0] != d->E || sizes[1] != d->N ||
      counts[0] != LULESH_S_COUNT || counts[1] != 11) {
    std::fclose(f);
    return LULESH_ERR_ARGUMENT;
  }
  double sc[LULESH_S_COUNT];
  r.get(sc, sizeof(sc));
  std::vector<std::vector<double>> fields(11);
  for (int k = 0; k < 11 && r.ok; ++k) {
    int32_t id = -1;
    int64_t n = -1;
    r.get(&id, sizeof(id));
    r.get(&n, sizeof(n));
    int64_t want = -1;
    if (!r.ok || id != kStateFields[k] || lulesh_field_length(d, id, &want) != LULESH_OK || n != want) {
      r.ok = false;
      break;
    }
    fields[k].resize(n);
    r.get(fields[k].data(), sizeof(double) * n);
  }
  uint64_t h = 0;
  const uint64_t expect = r.hash.h;
  if (!r.ok || std::fread(&h, 1, sizeof(h), f) != sizeof(h) || h != expect) {
    std::fclose(f);
    return LULESH_ERR_ARGUMENT;
  }
  std::fclose(f);
  // only a complete, verified file touches the handle
  for (int k = 0; k < 11; ++k) {
    const int rc = lulesh_upload_field(d, kStateFields[k], fields[k].data(), (int64_t)fields[k].size());
    if (rc) return rc;
  }
  for (int id = 0; id < LULESH_S_COUNT; ++id) {
    const int rc = lulesh_set_scalar(d, id, sc[id]);
    if (rc) return rc;
  }
  return LULESH_OK;
}

}  // extern "C"
