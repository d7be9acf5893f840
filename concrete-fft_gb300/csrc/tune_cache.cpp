// tune_cache.cpp -- persisted results of Method::Measure.
//
// Every *_create_measure entry point first looks up (GPU model, plan kind,
// size) here and only times candidates on a miss; its choice is then stored.
// cfft_tune_save / cfft_tune_load write and read the table as text, one entry
// per line: <gpu name>\t<kind>\t<n>\t<algo>\t<base_n>\t<threads>\t<tpc>\t<int_adds>.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <tuple>

#include "cfft_internal.h"
#include "tune_cache.h"

namespace cfft {
namespace {
std::mutex g_mu;
std::map<std::tuple<std::string, int, uint64_t>, TuneVal> g_table;

std::string device_name() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return "unknown";
  cudaDeviceProp p;
  if (cudaGetDeviceProperties(&p, dev) != cudaSuccess) return "unknown";
  std::string s = p.name;
  for (char& c : s)
    if (c == '\t' || c == '\n') c = ' ';
  return s;
}
}  // namespace

bool tune_lookup(int kind, uint64_t n, TuneVal* v) {
  const auto key = std::make_tuple(device_name(), kind, n);
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_table.find(key);
  if (it == g_table.end()) return false;
  *v = it->second;
  return true;
}

void tune_store(int kind, uint64_t n, const TuneVal& v) {
  const auto key = std::make_tuple(device_name(), kind, n);
  std::lock_guard<std::mutex> lk(g_mu);
  g_table[key] = v;
}

}  // namespace cfft

extern "C" {

cfft_status cfft_tune_save(const char* path) {
  if (!path) return cfft::fail_status(CFFT_ERR_INVALID_ARGUMENT, "null path");
  std::ofstream f(path);
  if (!f) return cfft::fail_status(CFFT_ERR_INVALID_ARGUMENT, std::string("cannot write ") + path);
  std::lock_guard<std::mutex> lk(cfft::g_mu);
  for (const auto& kv : cfft::g_table) {
    const auto& v = kv.second;
    f << std::get<0>(kv.first) << '\t' << std::get<1>(kv.first) << '\t' << std::get<2>(kv.first) << '\t' << v.algo
      << '\t' << v.base_n << '\t' << v.threads << '\t' << v.tpc << '\t' << v.emu << '\n';
  }
  return f ? CFFT_OK : cfft::fail_status(CFFT_ERR_INVALID_ARGUMENT, "write failed");
}

cfft_status cfft_tune_load(const char* path) {
  if (!path) return cfft::fail_status(CFFT_ERR_INVALID_ARGUMENT, "null path");
  std::ifstream f(path);
  if (!f) return cfft::fail_status(CFFT_ERR_INVALID_ARGUMENT, std::string("cannot read ") + path);
  std::string line;
  size_t lineno = 0;
  std::map<std::tuple<std::string, int, uint64_t>, cfft::TuneVal> add;
  while (std::getline(f, line)) {
    ++lineno;
    if (line.empty()) continue;
    std::istringstream ss(line);
    std::string gpu, field;
    std::getline(ss, gpu, '\t');
    long long vals[7];
    for (int i = 0; i < 7; ++i) {
      if (!std::getline(ss, field, '\t'))
        return cfft::fail_status(CFFT_ERR_INVALID_ARGUMENT, "tune cache line " + std::to_string(lineno) +
                                                                ": expected 8 tab-separated fields");
      char* end = nullptr;
      vals[i] = std::strtoll(field.c_str(), &end, 10);
      if (end == field.c_str() || *end != '\0')
        return cfft::fail_status(CFFT_ERR_INVALID_ARGUMENT, "tune cache line " + std::to_string(lineno) +
                                                                ": bad number '" + field + "'");
    }
    if (vals[0] < 0 || vals[0] > 2 || vals[2] < 0 || vals[2] > 7 || vals[6] < 0 || vals[6] > 8)
      return cfft::fail_status(CFFT_ERR_INVALID_ARGUMENT, "tune cache line " + std::to_string(lineno) +
                                                              ": value out of range");
    add[std::make_tuple(gpu, (int)vals[0], (uint64_t)vals[1])] =
        cfft::TuneVal{(int)vals[2], (uint64_t)vals[3], (int)vals[4], (int)vals[5], (int)vals[6]};
  }
  std::lock_guard<std::mutex> lk(cfft::g_mu);
  for (auto& kv : add) cfft::g_table[kv.first] = kv.second;
  return CFFT_OK;
}

void cfft_tune_clear(void) {
  std::lock_guard<std::mutex> lk(cfft::g_mu);
  cfft::g_table.clear();
}

size_t cfft_tune_entries(void) {
  std::lock_guard<std::mutex> lk(cfft::g_mu);
  return cfft::g_table.size();
}

}  // extern "C"
