// Autotuner table: per device, the smallest contribution block formed on
// the tensor cores (the SIMT / tensor-core crossover) and the tile width of
// the tensor-core Schur update for each size class of launch.  The numbers
// are measured by the autotuner in numeric.cu; this file keeps them per
// device, formats and parses them as one text line, and reads and writes
// the optional tune cache named by SPRAL_GB300_TUNE_CACHE, so that a process
// can reuse another's measurements on the same kind of GPU.
//
// Line format (one device per line, fields separated by single spaces):
//   spral_gb300-tune v1 <device key> tc_min_cm=<int> bn=<m>:<bn>,<m>:<bn>,...
// where the pairs give, in increasing m, the tile width for launches whose
// largest contribution block has at most m rows (the last pair covers every
// larger launch).  The device key is the device name with spaces replaced by
// '_', then "-sm<multiprocessors>-cc<major><minor>".
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "tune.h"

namespace ssids300 {

static std::mutex g_tab_mutex;
static TuneTable g_tab[kTuneMaxDevices];

bool tune_get(int dev, TuneTable& out) {
  if (dev < 0 || dev >= kTuneMaxDevices) return false;
  std::lock_guard<std::mutex> lock(g_tab_mutex);
  if (g_tab[dev].tc_min_cm <= 0) return false;
  out = g_tab[dev];
  return true;
}

void tune_set(int dev, const TuneTable& t) {
  if (dev < 0 || dev >= kTuneMaxDevices) return;
  std::lock_guard<std::mutex> lock(g_tab_mutex);
  g_tab[dev] = t;
}

int tune_bn_for(const TuneTable& t, int max_m) {
  if (t.nb <= 0) return kTuneDefaultBn;
  for (int i = 0; i < t.nb; ++i)
    if (max_m <= t.bucket_m[i]) return t.bn[i];
  return t.bn[t.nb - 1];
}

std::string tune_format(const std::string& key, const TuneTable& t) {
  std::ostringstream o;
  o << kTuneMagic << " v1 " << key << " tc_min_cm=" << t.tc_min_cm << " bn=";
  for (int i = 0; i < t.nb; ++i) o << (i ? "," : "") << t.bucket_m[i] << ":" << t.bn[i];
  return o.str();
}

static bool valid_bn(int bn) { return bn == 64 || bn == 128 || bn == 256; }

bool tune_parse(const std::string& line, std::string& key, TuneTable& t) {
  std::istringstream in(line);
  std::string magic, ver, k, f1, f2, extra;
  if (!(in >> magic >> ver >> k >> f1 >> f2) || (in >> extra)) return false;
  if (magic != kTuneMagic || ver != "v1") return false;
  if (f1.compare(0, 10, "tc_min_cm=") != 0 || f2.compare(0, 3, "bn=") != 0) return false;
  TuneTable r;
  char* end = nullptr;
  const long cm = std::strtol(f1.c_str() + 10, &end, 10);
  if (*end != '\0' || cm <= 0 || cm > (1L << 30)) return false;
  r.tc_min_cm = (int)cm;
  const char* p = f2.c_str() + 3;
  int prev = 0;
  while (*p) {
    if (r.nb >= kTuneMaxBuckets) return false;
    const long m = std::strtol(p, &end, 10);
    if (end == p || *end != ':' || m <= prev || m > (1L << 30)) return false;
    p = end + 1;
    const long bn = std::strtol(p, &end, 10);
    if (end == p || !valid_bn((int)bn)) return false;
    r.bucket_m[r.nb] = (int)m;
    r.bn[r.nb] = (int)bn;
    ++r.nb;
    prev = (int)m;
    p = end;
    if (*p == ',') {
      ++p;
      if (!*p) return false;
    } else if (*p) {
      return false;
    }
  }
  if (r.nb == 0) return false;
  key = k;
  t = r;
  return true;
}

bool tune_cache_lookup(const char* path, const std::string& key, TuneTable& t) {
  if (!path || !*path) return false;
  std::ifstream f(path);
  if (!f) return false;
  std::string line, k;
  bool found = false;
  while (std::getline(f, line)) {
    TuneTable r;
    if (tune_parse(line, k, r) && k == key) {
      t = r;
      found = true;  // the last line for a key wins
    }
  }
  return found;
}

bool tune_cache_store(const char* path, const std::string& key, const TuneTable& t) {
  if (!path || !*path) return false;
  std::vector<std::string> keep;
  {
    std::ifstream f(path);
    std::string line, k;
    TuneTable r;
    while (f && std::getline(f, line))
      if (tune_parse(line, k, r) && k != key) keep.push_back(line);
  }
  keep.push_back(tune_format(key, t));
  // write a sibling file, then rename it over the cache: readers see the
  // old or the new file, never a partial one
  const std::string tmp = std::string(path) + ".tmp" + std::to_string((long)std::rand());
  {
    std::ofstream o(tmp, std::ios::trunc);
    if (!o) return false;
    for (auto& l : keep) o << l << "\n";
    if (!o) return false;
  }
  if (std::rename(tmp.c_str(), path) != 0) {
    std::remove(tmp.c_str());
    return false;
  }
  return true;
}

}  // namespace ssids300

// ---------------------------------------------------------------------------
// C-ABI helpers of the tune line and cache (host only; no GPU needed).
// A table is passed as ints: [tc_min_cm, nb, m_0, bn_0, ..., m_{nb-1}, bn_{nb-1}].
// ---------------------------------------------------------------------------
namespace {
int table_to_ints(const ssids300::TuneTable& t, int* out, int nout) {
  const int need = 2 + 2 * t.nb;
  if (!out || nout < need) return -1;
  out[0] = t.tc_min_cm;
  out[1] = t.nb;
  for (int i = 0; i < t.nb; ++i) { out[2 + 2 * i] = t.bucket_m[i]; out[3 + 2 * i] = t.bn[i]; }
  return need;
}
bool ints_to_table(const int* in, int nin, ssids300::TuneTable& t) {
  if (!in || nin < 2 || in[1] < 1 || in[1] > ssids300::kTuneMaxBuckets || nin < 2 + 2 * in[1])
    return false;
  t = ssids300::TuneTable{};
  t.tc_min_cm = in[0];
  t.nb = in[1];
  for (int i = 0; i < t.nb; ++i) { t.bucket_m[i] = in[2 + 2 * i]; t.bn[i] = in[3 + 2 * i]; }
  // validate through the parser: one source of truth for what a table may hold
  std::string key;
  ssids300::TuneTable r;
  return ssids300::tune_parse(ssids300::tune_format("k", t), key, r);
}
}  // namespace

extern "C" int spral_ssids_gpu_tune_parse(const char* line, char* key, int key_cap, int* out,
                                          int nout) {
  if (!line) return -1;
  std::string k;
  ssids300::TuneTable t;
  if (!ssids300::tune_parse(line, k, t)) return -1;
  if (key && key_cap > 0) {
    std::snprintf(key, (size_t)key_cap, "%s", k.c_str());
    if ((int)k.size() >= key_cap) return -1;
  }
  return table_to_ints(t, out, nout);
}

extern "C" int spral_ssids_gpu_tune_format(const char* key, const int* in, int nin, char* buf,
                                           int cap) {
  ssids300::TuneTable t;
  if (!key || !*key || std::strchr(key, ' ') || !ints_to_table(in, nin, t)) return -1;
  const std::string s = ssids300::tune_format(key, t);
  if (!buf || cap <= (int)s.size()) return -1;
  std::snprintf(buf, (size_t)cap, "%s", s.c_str());
  return (int)s.size();
}

extern "C" int spral_ssids_gpu_tune_cache_lookup(const char* path, const char* key, int* out,
                                                 int nout) {
  ssids300::TuneTable t;
  if (!key || !ssids300::tune_cache_lookup(path, key, t)) return 0;
  return table_to_ints(t, out, nout);
}

extern "C" int spral_ssids_gpu_tune_cache_store(const char* path, const char* key, const int* in,
                                                int nin) {
  ssids300::TuneTable t;
  if (!key || !*key || std::strchr(key, ' ') || !ints_to_table(in, nin, t)) return -1;
  return ssids300::tune_cache_store(path, key, t) ? 0 : -1;
}
