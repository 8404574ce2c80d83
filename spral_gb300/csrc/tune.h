// Autotuner table of the numeric factorization (host side; see tune.cpp).
#pragma once
#include <string>

namespace ssids300 {

constexpr int kTuneMaxDevices = 64;
constexpr int kTuneMaxBuckets = 8;
constexpr int kTuneDefaultBn = 256;  // tile width before (or without) a measurement
constexpr const char* kTuneMagic = "spral_gb300-tune";

struct TuneTable {
  int tc_min_cm = 0;  // smallest contribution block on the tensor cores; 0: none yet
  int nb = 0;         // size classes of a launch's largest contribution block
  int bucket_m[kTuneMaxBuckets] = {};
  int bn[kTuneMaxBuckets] = {};
};

bool tune_get(int dev, TuneTable& out);
void tune_set(int dev, const TuneTable& t);
// tile width for a launch whose largest contribution block has max_m rows
int tune_bn_for(const TuneTable& t, int max_m);
std::string tune_format(const std::string& key, const TuneTable& t);
bool tune_parse(const std::string& line, std::string& key, TuneTable& t);
bool tune_cache_lookup(const char* path, const std::string& key, TuneTable& t);
bool tune_cache_store(const char* path, const std::string& key, const TuneTable& t);

}  // namespace ssids300
