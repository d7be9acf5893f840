// tune_cache.h -- the Method::Measure result table (tune_cache.cpp).
#pragma once
#include <cstdint>
#include <string>

#include "../../include/cfft.h"

namespace cfft {

// kind: 0 ordered plan, 1 unordered plan, 2 u64 product plan
struct TuneVal {
  int algo;
  uint64_t base_n;
  int threads;
  int tpc;
  int emu;
};

bool tune_lookup(int kind, uint64_t n, TuneVal* v);
void tune_store(int kind, uint64_t n, const TuneVal& v);
cfft_status fail_status(cfft_status s, const std::string& msg);

}  // namespace cfft
