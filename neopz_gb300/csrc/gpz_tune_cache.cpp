// On-disk cache of the autotuners' choices (gpz_tuning_cache): the FP32
// operator layout of the mixed solves and the block size of the hp element
// kernels.  Both are measured on the device the first time a pattern is
// assembled; with a cache file set, a later context (another process, another
// run) with the same device and the same mesh structure takes the stored choice
// instead of timing every candidate again.  The key holds the tuner, the
// device (name, SM count, compute capability), the sizes and a 64-bit FNV-1a
// hash of the mesh's connectivity (element types, materials, side connects,
// block positions and sizes) -- not the coefficients, which do not change a
// kernel's time -- and the tuner version below, raised whenever a candidate
// kernel changes.  The file is JSON lines, one choice per line, appended; the
// last line with a key wins.
#include <cstdio>
#include <cstring>
#include <string>

#include "gpz_internal.h"

namespace gpz {
namespace {

constexpr int kTuneVersion = 3;

uint64_t fnv(uint64_t h, const void *p, size_t n) {
  const unsigned char *b = (const unsigned char *)p;
  for (size_t i = 0; i < n; i++) {
    h ^= b[i];
    h *= 1099511628211ull;
  }
  return h;
}

std::string json_safe(const char *s) {
  std::string r(s);
  for (char &ch : r)
    if (ch == '"' || ch == '\\' || (unsigned char)ch < 32) ch = '_';
  return r;
}

}  // namespace

std::string tune_key(Ctx &c, const char *tuner) {
  int dev = 0;
  cudaDeviceProp prop;
  std::memset(&prop, 0, sizeof(prop));
  if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&prop, dev) != cudaSuccess)
    std::snprintf(prop.name, sizeof(prop.name), "unknown");
  uint64_t h = 1469598103934665603ull;
  h = fnv(h, c.h_el_type.data(), c.h_el_type.size() * sizeof(int32_t));
  h = fnv(h, c.h_el_mat.data(), c.h_el_mat.size() * sizeof(int32_t));
  h = fnv(h, c.h_el_conn.data(), c.h_el_conn.size() * sizeof(int64_t));
  h = fnv(h, c.h_block_pos.data(), c.h_block_pos.size() * sizeof(int64_t));
  h = fnv(h, c.h_block_size.data(), c.h_block_size.size() * sizeof(int32_t));
  char buf[512];
  std::snprintf(buf, sizeof(buf), "%s|%s|sm%d|cc%d.%d|neq%lld|nnz%lld|nel%lld|nstate%d|filter%d|mesh%016llx|v%d",
                tuner, json_safe(prop.name).c_str(), prop.multiProcessorCount, prop.major, prop.minor,
                (long long)c.neq, (long long)c.nnz, (long long)c.nel, c.nstate, c.flt.active ? 1 : 0,
                (unsigned long long)h, kTuneVersion);
  return buf;
}

int tune_cache_lookup(const Ctx &c, const std::string &key) {
  if (c.tune_cache.empty()) return -1;
  FILE *f = std::fopen(c.tune_cache.c_str(), "r");
  if (!f) return -1;
  const std::string needle = "\"key\": \"" + key + "\"";
  int found = -1;
  std::string line;
  char chunk[4096];
  while (std::fgets(chunk, sizeof(chunk), f)) {
    line += chunk;
    if (line.empty() || line.back() != '\n') continue;  // a line longer than the chunk
    if (line.find(needle) != std::string::npos) {
      const size_t at = line.find("\"choice\": ");
      if (at != std::string::npos) found = std::atoi(line.c_str() + at + 10);
    }
    line.clear();
  }
  std::fclose(f);
  return found;
}

void tune_cache_store(const Ctx &c, const std::string &key, int choice, const std::string &report) {
  if (c.tune_cache.empty()) return;
  FILE *f = std::fopen(c.tune_cache.c_str(), "a");
  if (!f) return;  // an unwritable cache only costs the next run its tuning
  std::fprintf(f, "{\"key\": \"%s\", \"choice\": %d, \"report\": %s}\n", key.c_str(), choice,
               report.empty() ? "{}" : report.c_str());
  std::fclose(f);
}

}  // namespace gpz
