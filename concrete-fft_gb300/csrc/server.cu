// server.cu -- continuous-batching request loop for negacyclic u64 products.
//
// Requests arrive as a seeded Poisson stream.  Each carries (k+1)*l products of
// one size N: digit polynomials (signed, b-bit) times Fourier-domain operands
// that stay resident on the device (the shape of a TFHE external product).
// The digit sources and the operands are device-resident pools built at
// creation; a request picks rows of them, so its content is a pure function of
// (seed, request id) and can be recomputed alone for checking.
//
// Batched mode: every loop iteration admits the requests that have arrived
// while the device memory gate (the output bytes in flight against the
// device's free memory, read live) and the output ring allow, and as soon as one
// of `max_inflight` launch slots is free, launches everything admitted since
// the previous launch as one product-engine run on that slot's stream,
// followed by the copy of the results into a pinned host ring.  Products of
// N >= 8192 (cluster_log2N) leave the engine launch: a second stream of the
// slot runs them one per thread-block cluster (split_product.cuh), beside the
// engine, so a large product takes 1/4-1/8 of its one-CTA time.  Launch slots
// run concurrently, so requests that arrive while others are on the GPU are
// admitted and overlap with them.  A request is done when its launch's event
// has completed; its latency is measured on the host clock from its arrival.
//
// Plain mode (the comparator): requests in arrival order, one at a time, each
// product through the unfused pipeline with one launch per step, and the
// results copied back before the next request starts.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <map>
#include <thread>
#include <vector>

#include "../../include/cfft.h"
#include "cfft_internal.h"
#include "runtime.h"

using namespace cfft;

namespace {

inline uint64_t splitmix(uint64_t& s) {
  uint64_t z = (s += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
inline double u01(uint64_t& s) { return (double)(splitmix(s) >> 11) * (1.0 / 9007199254740992.0); }

constexpr int kPoolRows = 64;   // digit polynomials per size
constexpr int kSlots = 3;       // launch slots (concurrent runs)
// Item records per launch slot, allocated at creation: growing them inside the
// loop (cudaFree synchronises the device, cudaMallocHost is slow) showed up as
// millisecond latency spikes the first time a larger batch formed.
constexpr size_t kSlotItems = 65536;

struct ReqDesc {
  uint64_t id;
  double arrival;  // seconds from the start
  uint32_t log2N, nprod;
  uint32_t rows[16], ops[16];
};

struct SizePool {
  uint32_t log2N = 0;
  int64_t* digits = nullptr;  // kPoolRows x N, device
  double* bhat = nullptr;     // nops x N/2 c64, device
  uint32_t nops = 0;
};

struct Slot {
  cudaStream_t stream = nullptr;
  cudaStream_t stream2 = nullptr;  // cluster launches of the slot's large products
  cudaEvent_t done = nullptr;
  cudaEvent_t items_ready = nullptr, big_done = nullptr;
  unsigned int* counter = nullptr;
  double* ws = nullptr;
  cfft_product_item* d_items = nullptr;
  cfft_product_item* h_items = nullptr;      // page-locked
  cfft_product_item* h_items_dev = nullptr;  // the device address of h_items
  size_t item_cap = 0;
  bool busy = false;
  std::vector<size_t> reqs;  // indices into the request table
};

struct Live {
  ReqDesc d;
  uint64_t ring_off = 0, ring_bytes = 0, ring_end = 0;  // offset in the ring; end in the monotonic byte count
  double t_done = -1;
  uint64_t ticket = 0;  // via the work queue
};

}  // namespace

struct cfft_server {
  const cfft_product_engine* engine = nullptr;
  uint64_t seed = 0;
  std::vector<SizePool> pools;
  Slot slots[kSlots];
  // output ring (device) and its pinned host mirror
  uint8_t* d_ring = nullptr;
  uint8_t* h_ring = nullptr;
  uint8_t* h_ring_dev = nullptr;  // the device address of h_ring (page-locked)
  uint64_t ring_cap = 0;
  std::map<uint64_t, std::vector<uint64_t>> recorded;
  std::vector<double> last_latency;
};

namespace {

double now_s(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

const SizePool* pool_of(const cfft_server* s, uint32_t log2N) {
  for (const auto& p : s->pools)
    if (p.log2N == log2N) return &p;
  return nullptr;
}

// Request content as a function of (seed, id).
ReqDesc make_request(const cfft_server* s, const cfft_serve_config& c, uint64_t id, double arrival) {
  uint64_t st = s->seed * 0x2545f4914f6cdd1dull ^ (id + 1) * 0x9e3779b97f4a7c15ull;
  ReqDesc r;
  r.id = id;
  r.arrival = arrival;
  r.log2N = c.log2N_min + (uint32_t)(splitmix(st) % (c.log2N_max - c.log2N_min + 1));
  const uint32_t k = 1 + (uint32_t)(splitmix(st) % c.k_max);
  const uint32_t l = 1 + (uint32_t)(splitmix(st) % c.l_max);
  r.nprod = std::min<uint32_t>((k + 1) * l, 16);
  const SizePool* p = pool_of(s, r.log2N);
  for (uint32_t i = 0; i < r.nprod; ++i) {
    r.rows[i] = (uint32_t)(splitmix(st) % kPoolRows);
    r.ops[i] = (uint32_t)(splitmix(st) % (p ? p->nops : 1));
  }
  return r;
}

void fill_items(const cfft_server* s, const ReqDesc& r, uint8_t* out_dev, cfft_product_item* items) {
  const SizePool* p = pool_of(s, r.log2N);
  const size_t N = size_t(1) << r.log2N;
  for (uint32_t i = 0; i < r.nprod; ++i) {
    items[i].a = (const uint64_t*)(p->digits + (size_t)r.rows[i] * N);
    items[i].bhat = p->bhat + (size_t)r.ops[i] * N;  // N/2 c64 = N doubles
    items[i].out = (uint64_t*)out_dev + (size_t)i * N;
    items[i].log2N = r.log2N;
    items[i].reserved = 0;
  }
}

cfft_status ensure_items(Slot& sl, size_t n) {
  if (n <= sl.item_cap) return CFFT_OK;
  const size_t cap = std::max<size_t>(n, 2 * sl.item_cap);
  if (sl.d_items) cudaFree(sl.d_items);
  if (sl.h_items) cudaFreeHost(sl.h_items);
  sl.d_items = nullptr;
  sl.h_items = nullptr;
  CFFT_CUDA_TRY(cudaMalloc(&sl.d_items, cap * sizeof(cfft_product_item)));
  CFFT_CUDA_TRY(cudaMallocHost(&sl.h_items, cap * sizeof(cfft_product_item)));
  CFFT_CUDA_TRY(cudaHostGetDevicePointer((void**)&sl.h_items_dev, sl.h_items, 0));
  sl.item_cap = cap;
  return CFFT_OK;
}

// Byte ring: allocations in admission order, never split across the wrap;
// `tail` advances to the end of the oldest allocation once it is released.
struct RingAlloc {
  uint64_t cap, head = 0, tail = 0;  // monotonic byte counts
  explicit RingAlloc(uint64_t c) : cap(c) {}
  bool alloc(uint64_t n, uint64_t* off, uint64_t* end) {
    n = (n + 255) & ~uint64_t(255);
    const uint64_t pos = head % cap;
    const uint64_t pad = pos + n > cap ? cap - pos : 0;
    if (head + pad + n - tail > cap) return false;
    *off = (head + pad) % cap;
    head += pad + n;
    *end = head;
    return true;
  }
};

// Device memory gate: admitted, unfinished requests hold their output bytes,
// and their sum stays within the device's free memory less a reserve.  A
// reader thread refreshes the budget from cudaMemGetInfo every 20 ms while the
// run lasts, so memory that other users of the device take or release during
// the run moves the gate.  The reading stays off the request loop, where a
// driver query can take up to a millisecond; from this thread, a run at 20 k
// requests/s measures the same p99 as one on a fixed stand-in budget
// (0.103-0.110 against 0.103-0.121 ms).  mem_free_override
// replaces the reading (tests fake a small device).  When nothing is in flight
// a request is admitted whatever the budget, so a budget smaller than one
// request slows the stream but cannot stall it.
struct MemGate {
  uint64_t reserve, override_free;
  std::atomic<uint64_t> budget{0};
  std::atomic<uint64_t> min_budget{~uint64_t(0)};
  std::atomic<bool> stop{false};
  std::thread reader;
  uint64_t inflight = 0;  // request loop only
  MemGate(uint64_t r, uint64_t o) : reserve(r), override_free(o) {}
  ~MemGate() { finish(); }
  void record(size_t free_b) {
    const uint64_t v = free_b > reserve ? free_b - reserve : 0;
    budget.store(v, std::memory_order_relaxed);
    uint64_t m = min_budget.load(std::memory_order_relaxed);
    while (v < m && !min_budget.compare_exchange_weak(m, v, std::memory_order_relaxed)) {
    }
  }
  // first reading now (the loop admits against it from the start), then the reader thread
  void start() {
    if (override_free) {
      record(override_free);
      return;
    }
    int dev = 0;
    cudaGetDevice(&dev);
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess) record(free_b);
    reader = std::thread([this, dev] {
      cudaSetDevice(dev);
      while (!stop.load(std::memory_order_relaxed)) {
        std::this_thread::sleep_for(std::chrono::milliseconds(20));
        size_t f = 0, t = 0;
        if (cudaMemGetInfo(&f, &t) == cudaSuccess) record(f);  // else keep the previous budget
      }
    });
  }
  void finish() {
    stop.store(true, std::memory_order_relaxed);
    if (reader.joinable()) reader.join();
  }
  bool admits(uint64_t bytes) const {
    return inflight == 0 || inflight + bytes <= budget.load(std::memory_order_relaxed);
  }
};

void free_server(cfft_server* s) {
  for (auto& p : s->pools) {
    if (p.digits) cudaFree(p.digits);
    if (p.bhat) cudaFree(p.bhat);
  }
  for (auto& sl : s->slots) {
    if (sl.stream) cudaStreamDestroy(sl.stream);
    if (sl.stream2) cudaStreamDestroy(sl.stream2);
    if (sl.done) cudaEventDestroy(sl.done);
    if (sl.items_ready) cudaEventDestroy(sl.items_ready);
    if (sl.big_done) cudaEventDestroy(sl.big_done);
    if (sl.counter) cudaFree(sl.counter);
    if (sl.ws) cudaFree(sl.ws);
    if (sl.d_items) cudaFree(sl.d_items);
    if (sl.h_items) cudaFreeHost(sl.h_items);
  }
  if (s->d_ring) cudaFree(s->d_ring);
  if (s->h_ring) cudaFreeHost(s->h_ring);
}

cfft_status run_alone(cfft_server* s, const ReqDesc& r, uint64_t* out_host) {
  Slot& sl = s->slots[0];
  cfft_status st = ensure_items(sl, r.nprod);
  if (st != CFFT_OK) return st;
  const size_t N = size_t(1) << r.log2N;
  uint64_t* d_out = nullptr;
  CFFT_CUDA_TRY(cudaMalloc(&d_out, r.nprod * N * 8));
  fill_items(s, r, (uint8_t*)d_out, sl.h_items);
  CFFT_CUDA_TRY(cudaMemcpyAsync(sl.d_items, sl.h_items, r.nprod * sizeof(cfft_product_item), cudaMemcpyHostToDevice,
                                sl.stream));
  st = cfft_product_engine_run(s->engine, sl.d_items, r.nprod, sl.counter, sl.ws, sl.stream);
  if (st == CFFT_OK) {
    CFFT_CUDA_TRY(cudaMemcpyAsync(out_host, d_out, r.nprod * N * 8, cudaMemcpyDeviceToHost, sl.stream));
    CFFT_CUDA_TRY(cudaStreamSynchronize(sl.stream));
  }
  cudaFree(d_out);
  return st;
}

}  // namespace

extern "C" {

cfft_status cfft_server_create(const cfft_product_engine* engine, const uint32_t* log2N, size_t nsizes,
                               uint64_t operand_bytes, uint64_t ring_bytes, uint64_t seed, cfft_server** out) {
  if (!engine || !out || !log2N || nsizes == 0) return fail(CFFT_ERR_INVALID_ARGUMENT, "null argument");
  *out = nullptr;
  auto* s = new cfft_server();
  s->engine = engine;
  s->seed = seed;
  cfft_status st = CFFT_OK;
  cudaStream_t prep;
  if (cudaStreamCreateWithFlags(&prep, cudaStreamNonBlocking) != cudaSuccess) st = CFFT_ERR_CUDA;
  uint64_t rs = seed ^ 0x5bd1e995ull;
  for (size_t i = 0; i < nsizes && st == CFFT_OK; ++i) {
    const cfft_u64_product_plan* plan = cfft_product_engine_plan(engine, log2N[i]);
    if (!plan) {
      st = fail(CFFT_ERR_INVALID_ARGUMENT, "server size not configured in the engine");
      break;
    }
    SizePool p;
    p.log2N = log2N[i];
    const size_t N = size_t(1) << log2N[i];
    p.nops = (uint32_t)std::max<uint64_t>(1, operand_bytes / nsizes / (N / 2 * 16));
    // digit rows: b = 4 + row % 7 bits, uniform in [-2^(b-1), 2^(b-1))
    std::vector<int64_t> dig((size_t)kPoolRows * N);
    for (int r = 0; r < kPoolRows; ++r) {
      const int b = 4 + r % 7;
      for (size_t j = 0; j < N; ++j) dig[(size_t)r * N + j] = (int64_t)(splitmix(rs) % (1ull << b)) - (1ll << (b - 1));
    }
    st = upload(dig.data(), dig.size(), &p.digits);
    if (st != CFFT_OK) break;
    if (cudaMalloc(&p.bhat, (size_t)p.nops * N * sizeof(double)) != cudaSuccess) {
      st = fail(CFFT_ERR_OUT_OF_MEMORY, "resident operands do not fit");
      s->pools.push_back(p);
      break;
    }
    // operands: Fourier transforms of uniform u64 polynomials, prepared in chunks
    const size_t chunk = std::max<size_t>(1, (size_t(1) << 24) / N);
    std::vector<uint64_t> src(chunk * N);
    int64_t* d_src = nullptr;
    if (cudaMalloc(&d_src, chunk * N * 8) != cudaSuccess) st = CFFT_ERR_OUT_OF_MEMORY;
    for (size_t c0 = 0; c0 < p.nops && st == CFFT_OK; c0 += chunk) {
      const size_t c = std::min<size_t>(chunk, p.nops - c0);
      for (size_t j = 0; j < c * N; ++j) src[j] = splitmix(rs);
      if (cudaMemcpyAsync(d_src, src.data(), c * N * 8, cudaMemcpyHostToDevice, prep) != cudaSuccess) {
        st = CFFT_ERR_CUDA;
        break;
      }
      st = cfft_u64_prepare_operand(plan, d_src, p.bhat + c0 * N, c, prep);
      if (st == CFFT_OK && cudaStreamSynchronize(prep) != cudaSuccess) st = CFFT_ERR_CUDA;
    }
    if (d_src) cudaFree(d_src);
    s->pools.push_back(p);
  }
  if (st == CFFT_OK) {
    const size_t ws = cfft_product_engine_workspace_bytes(engine);
    for (auto& sl : s->slots) {
      if (cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking) != cudaSuccess ||
          cudaStreamCreateWithFlags(&sl.stream2, cudaStreamNonBlocking) != cudaSuccess ||
          cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming) != cudaSuccess ||
          cudaEventCreateWithFlags(&sl.items_ready, cudaEventDisableTiming) != cudaSuccess ||
          cudaEventCreateWithFlags(&sl.big_done, cudaEventDisableTiming) != cudaSuccess ||
          cudaMalloc(&sl.counter, 64) != cudaSuccess || (ws && cudaMalloc(&sl.ws, ws) != cudaSuccess)) {
        st = fail(CFFT_ERR_OUT_OF_MEMORY, "server launch slots");
        break;
      }
      st = ensure_items(sl, kSlotItems);
      if (st != CFFT_OK) break;
    }
  }
  if (st == CFFT_OK) {
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    s->ring_cap = ring_bytes ? ring_bytes : std::min<uint64_t>(free_b / 4, uint64_t(4) << 30);
    if (cudaMalloc(&s->d_ring, s->ring_cap) != cudaSuccess || cudaMallocHost(&s->h_ring, s->ring_cap) != cudaSuccess ||
        cudaHostGetDevicePointer((void**)&s->h_ring_dev, s->h_ring, 0) != cudaSuccess)
      st = fail(CFFT_ERR_OUT_OF_MEMORY, "server output ring");
  }
  cudaStreamDestroy(prep);
  if (st != CFFT_OK) {
    free_server(s);
    delete s;
    return st;
  }
  *out = s;
  return CFFT_OK;
}

void cfft_server_destroy(cfft_server* s) {
  if (!s) return;
  free_server(s);
  delete s;
}

cfft_status cfft_server_run(cfft_server* s, const cfft_serve_config* cfg, cfft_serve_stats* stats) {
  if (!s || !cfg || !stats) return fail(CFFT_ERR_INVALID_ARGUMENT, "null argument");
  const cfft_serve_config c = *cfg;
  if (c.rate <= 0 || c.duration_s <= 0 || c.k_max < 1 || c.l_max < 1 || c.log2N_max < c.log2N_min)
    return fail(CFFT_ERR_INVALID_ARGUMENT, "bad serving configuration");
  for (uint32_t lN = c.log2N_min; lN <= c.log2N_max; ++lN)
    if (!pool_of(s, lN)) return fail(CFFT_ERR_INVALID_ARGUMENT, "request size not in the server's pools");
  if (s->ring_cap < ((uint64_t)16 << (c.log2N_max + 3)) + 256)
    return fail(CFFT_ERR_INVALID_ARGUMENT, "output ring smaller than the largest request");
  std::memset(stats, 0, sizeof(*stats));
  s->recorded.clear();
  // arrivals (seeded exponential inter-arrival times)
  std::vector<Live> reqs;
  {
    uint64_t ast = s->seed * 0x632be59bd9b4e019ull + 7;
    double t = 0;
    for (uint64_t id = 0;; ++id) {
      t += -std::log(1.0 - u01(ast)) / c.rate;
      if (t > c.duration_s) break;
      Live lv;
      lv.d = make_request(s, c, id, t);
      reqs.push_back(lv);
    }
  }
  RingAlloc ring(s->ring_cap);
  std::deque<size_t> ring_order;  // requests holding ring space, in allocation order
  size_t next = 0;                // next request to arrive
  std::deque<size_t> waiting;
  std::vector<size_t> batch;
  std::vector<cfft_product_item> items;
  uint64_t deferred = 0, launches = 0, mem_deferred = 0;
  MemGate gate(c.mem_reserve_bytes, c.mem_free_override);
  if (!c.plain) gate.start();
  const auto t0 = std::chrono::steady_clock::now();
  const uint32_t nslots = std::max<uint32_t>(1, std::min<uint32_t>(c.max_inflight ? c.max_inflight : kSlots, kSlots));
  // products of at least this size run one per thread-block cluster (sizes whose plan
  // has a cluster kernel); automatic (cluster_log2N = 0): N >= 8192, and every size in
  // a launch of at most kClusterAllItems products, whose products would otherwise each
  // take one SM of a mostly idle GPU
  const uint32_t big_log2N = c.cluster_log2N ? c.cluster_log2N : 13;
  bool on_cluster_big[18] = {}, on_cluster_all[18] = {};
  for (uint32_t lN = 0; lN <= 17; ++lN) {
    const cfft_u64_product_plan* p = cfft_product_engine_plan(s->engine, lN);
    const bool split = p && u64_product_splittable(p);
    on_cluster_big[lN] = split && lN >= big_log2N;
    on_cluster_all[lN] = c.cluster_log2N ? on_cluster_big[lN] : split;
  }
  size_t done_count = 0;

  auto record = [&](size_t ri) {
    Live& r = reqs[ri];
    if (c.record_every && r.d.id % c.record_every == 0) {
      const size_t words = (size_t)r.d.nprod << r.d.log2N;
      s->recorded[r.d.id].assign((uint64_t*)(s->h_ring + r.ring_off), (uint64_t*)(s->h_ring + r.ring_off) + words);
    }
  };

  if (c.plain) {
    // one request at a time; each product through the unfused pipeline, one launch per step
    Slot& sl = s->slots[0];
    double* z = nullptr;
    size_t zcap = 0;
    for (size_t ri = 0; ri < reqs.size(); ++ri) {
      Live& r = reqs[ri];
      while (now_s(t0) < r.d.arrival) {
      }
      const size_t N = size_t(1) << r.d.log2N;
      const cfft_u64_product_plan* plan = cfft_product_engine_plan(s->engine, r.d.log2N);
      cfft_unordered_plan* fft = cfft_u64_product_fft(plan);
      if (zcap < N) {
        if (z) cudaFree(z);
        CFFT_CUDA_TRY(cudaMalloc(&z, N * 8));
        zcap = N;
      }
      const SizePool* p = pool_of(s, r.d.log2N);
      r.ring_off = 0;
      for (uint32_t i = 0; i < r.d.nprod; ++i) {
        const uint64_t* a = (const uint64_t*)(p->digits + (size_t)r.d.rows[i] * N);
        const double* bh = p->bhat + (size_t)r.d.ops[i] * N;
        uint64_t* o = (uint64_t*)s->d_ring + (size_t)i * N;
        cfft_status st = cfft_u64_fold_twist(plan, a, z, 1, sl.stream);
        if (st == CFFT_OK) st = cfft_unordered_fwd(fft, z, 1, sl.stream);
        if (st == CFFT_OK) st = cfft_c64_pointwise(bh, 0, z, N / 2, 1, sl.stream);
        if (st == CFFT_OK) st = cfft_unordered_inv(fft, z, 1, sl.stream);
        if (st == CFFT_OK) st = cfft_u64_untwist_round(plan, z, o, 1, sl.stream);
        if (st != CFFT_OK) return st;
        launches += 5;
      }
      CFFT_CUDA_TRY(cudaMemcpyAsync(s->h_ring, s->d_ring, (size_t)r.d.nprod * N * 8, cudaMemcpyDeviceToHost, sl.stream));
      CFFT_CUDA_TRY(cudaStreamSynchronize(sl.stream));
      r.t_done = now_s(t0);
      record(ri);
      ++done_count;
    }
    if (z) cudaFree(z);
  } else if (c.via_queue) {
    // the same stream through the public work queue: each admitted request is
    // submitted on arrival; its ticket is polled until done
    cfft_product_queue_config qc{std::min<uint32_t>(nslots, 4), c.cluster_log2N};
    cfft_product_queue* q = nullptr;
    cfft_status st = cfft_product_queue_create(s->engine, &qc, &q);
    if (st != CFFT_OK) return st;
    std::vector<size_t> inflight;
    std::vector<cfft_product_item> its;
    for (;;) {
      const double now = now_s(t0);
      while (next < reqs.size() && reqs[next].d.arrival <= now) waiting.push_back(next++);
      while (!waiting.empty()) {
        Live& r = reqs[waiting.front()];
        r.ring_bytes = (uint64_t)r.d.nprod << (r.d.log2N + 3);
        if (!gate.admits(r.ring_bytes)) {
          ++mem_deferred;
          break;
        }
        if (!ring.alloc(r.ring_bytes, &r.ring_off, &r.ring_end)) {
          ++deferred;
          break;
        }
        gate.inflight += r.ring_bytes;
        its.resize(r.d.nprod);
        fill_items(s, r.d, s->h_ring_dev + r.ring_off, its.data());
        st = cfft_product_queue_submit(q, its.data(), its.size(), &r.ticket);
        if (st != CFFT_OK) break;
        ring_order.push_back(waiting.front());
        inflight.push_back(waiting.front());
        waiting.pop_front();
      }
      if (st != CFFT_OK) break;
      for (size_t k = 0; k < inflight.size();) {
        const int pr = cfft_product_queue_poll(q, reqs[inflight[k]].ticket);
        if (pr < 0) {
          st = (cfft_status)pr;
          break;
        }
        if (pr == 0) {
          ++k;
          continue;
        }
        reqs[inflight[k]].t_done = now_s(t0);
        gate.inflight -= reqs[inflight[k]].ring_bytes;
        record(inflight[k]);
        ++done_count;
        inflight[k] = inflight.back();
        inflight.pop_back();
      }
      if (st != CFFT_OK) break;
      while (!ring_order.empty() && reqs[ring_order.front()].t_done >= 0) {
        ring.tail = reqs[ring_order.front()].ring_end;
        ring_order.pop_front();
      }
      if (done_count == reqs.size()) break;
    }
    cfft_product_queue_destroy(q);
    if (st != CFFT_OK) return st;
    launches = 0;  // counted by the queue, not here
  } else {
    // direct mode: the kernels read the item records from the slot's page-locked
    // array and store the results into the page-locked host ring (across
    // NVLink-C2C on a Grace host); no copy in either direction
    const bool direct = c.staged_io == 0;
    uint8_t* out_ring = direct ? s->h_ring_dev : s->d_ring;
    for (;;) {
      const double now = now_s(t0);
      while (next < reqs.size() && reqs[next].d.arrival <= now) waiting.push_back(next++);
      // admission: the device memory gate, then output ring space
      while (!waiting.empty()) {
        Live& r = reqs[waiting.front()];
        r.ring_bytes = (uint64_t)r.d.nprod << (r.d.log2N + 3);
        if (!gate.admits(r.ring_bytes)) {
          ++mem_deferred;
          break;
        }
        if (!ring.alloc(r.ring_bytes, &r.ring_off, &r.ring_end)) {
          ++deferred;
          break;
        }
        gate.inflight += r.ring_bytes;
        ring_order.push_back(waiting.front());
        batch.push_back(waiting.front());
        waiting.pop_front();
      }
      // launch the admitted batch on a free slot
      if (!batch.empty()) {
        for (uint32_t k = 0; k < nslots; ++k) {
          Slot& sl = s->slots[k];
          if (sl.busy) continue;
          size_t nitems = 0;
          for (size_t ri : batch) nitems += reqs[ri].d.nprod;
          const bool* on_cluster = nitems <= kClusterAllItems ? on_cluster_all : on_cluster_big;
          cfft_status st = ensure_items(sl, nitems);
          if (st != CFFT_OK) return st;
          // item records: the engine's products first, then the large ones grouped by N
          size_t at = 0;
          for (size_t ri : batch)
            if (!on_cluster[reqs[ri].d.log2N]) {
              fill_items(s, reqs[ri].d, out_ring + reqs[ri].ring_off, sl.h_items + at);
              at += reqs[ri].d.nprod;
            }
          const size_t nsmall = at;
          size_t group_first[18] = {}, group_count[18] = {};
          for (uint32_t lN = 0; lN <= 17; ++lN) {
            if (!on_cluster[lN]) continue;
            group_first[lN] = at;
            for (size_t ri : batch)
              if (reqs[ri].d.log2N == lN) {
                fill_items(s, reqs[ri].d, out_ring + reqs[ri].ring_off, sl.h_items + at);
                at += reqs[ri].d.nprod;
              }
            group_count[lN] = at - group_first[lN];
          }
          const cfft_product_item* items = direct ? sl.h_items_dev : sl.d_items;
          if (!direct)
            CFFT_CUDA_TRY(cudaMemcpyAsync(sl.d_items, sl.h_items, nitems * sizeof(cfft_product_item),
                                          cudaMemcpyHostToDevice, sl.stream));
          if (nsmall < nitems) {
            if (!direct) {
              CFFT_CUDA_TRY(cudaEventRecord(sl.items_ready, sl.stream));
              CFFT_CUDA_TRY(cudaStreamWaitEvent(sl.stream2, sl.items_ready, 0));
            }
            for (uint32_t lN = 0; lN <= 17; ++lN) {
              if (!group_count[lN]) continue;
              st = u64_product_split_items(cfft_product_engine_plan(s->engine, lN), items + group_first[lN],
                                           group_count[lN], sl.stream2);
              if (st != CFFT_OK) return st;
            }
            CFFT_CUDA_TRY(cudaEventRecord(sl.big_done, sl.stream2));
          }
          if (nsmall) {
            st = cfft_product_engine_run(s->engine, items, nsmall, sl.counter, sl.ws, sl.stream);
            if (st != CFFT_OK) return st;
          }
          if (nsmall < nitems) CFFT_CUDA_TRY(cudaStreamWaitEvent(sl.stream, sl.big_done, 0));
          // staged mode: results back to the pinned host ring (in direct mode the kernels
          // stored them there).  The batch's requests were allocated in admission order,
          // so they are contiguous (256-byte aligned) except across the wrap; one copy
          // per contiguous run
          if (!direct) {
            uint64_t run_off = 0, run_end = 0;
            bool have_run = false;
            for (size_t ri : batch) {
              const uint64_t off = reqs[ri].ring_off, end = off + reqs[ri].ring_bytes;
              if (have_run && off == ((run_end + 255) & ~uint64_t(255))) {
                run_end = end;
                continue;
              }
              if (have_run)
                CFFT_CUDA_TRY(cudaMemcpyAsync(s->h_ring + run_off, s->d_ring + run_off, run_end - run_off,
                                              cudaMemcpyDeviceToHost, sl.stream));
              run_off = off;
              run_end = end;
              have_run = true;
            }
            if (have_run)
              CFFT_CUDA_TRY(cudaMemcpyAsync(s->h_ring + run_off, s->d_ring + run_off, run_end - run_off,
                                            cudaMemcpyDeviceToHost, sl.stream));
          }
          CFFT_CUDA_TRY(cudaEventRecord(sl.done, sl.stream));
          sl.busy = true;
          sl.reqs = batch;
          batch.clear();
          ++launches;
          stats->mean_batch += (double)nitems;
          break;
        }
      }
      // completions
      for (uint32_t k = 0; k < nslots; ++k) {
        Slot& sl = s->slots[k];
        if (!sl.busy) continue;
        const cudaError_t q = cudaEventQuery(sl.done);
        if (q == cudaErrorNotReady) continue;
        if (q != cudaSuccess) return fail(CFFT_ERR_CUDA, std::string("server launch: ") + cudaGetErrorString(q));
        const double t = now_s(t0);
        for (size_t ri : sl.reqs) {
          reqs[ri].t_done = t;
          gate.inflight -= reqs[ri].ring_bytes;
          record(ri);
          ++done_count;
        }
        sl.reqs.clear();
        sl.busy = false;
      }
      // release ring space in allocation order
      while (!ring_order.empty() && reqs[ring_order.front()].t_done >= 0) {
        ring.tail = reqs[ring_order.front()].ring_end;
        ring_order.pop_front();
      }
      if (done_count == reqs.size()) break;
    }
  }
  // statistics
  std::vector<double> lat;
  double first = 1e30, last = 0;
  uint64_t prods = 0, out_bytes = 0;
  for (const auto& r : reqs) {
    lat.push_back(r.t_done - r.d.arrival);
    first = std::min(first, r.d.arrival);
    last = std::max(last, r.t_done);
    prods += r.d.nprod;
    out_bytes += (uint64_t)r.d.nprod << (r.d.log2N + 3);
  }
  std::sort(lat.begin(), lat.end());
  auto pct = [&](double q) { return lat.empty() ? 0.0 : lat[std::min(lat.size() - 1, (size_t)(q * lat.size()))]; };
  stats->requests = reqs.size();
  stats->products = prods;
  stats->launches = launches;
  stats->span_s = last - first;
  stats->products_per_s = stats->span_s > 0 ? prods / stats->span_s : 0;
  stats->p50_ms = pct(0.50) * 1e3;
  stats->p99_ms = pct(0.99) * 1e3;
  stats->max_ms = lat.empty() ? 0 : lat.back() * 1e3;
  stats->mean_batch = launches && !c.plain ? stats->mean_batch / launches : 1.0;
  stats->deferred_admissions = deferred + mem_deferred;
  stats->memory_deferrals = mem_deferred;
  stats->input_bytes = prods * sizeof(cfft_product_item);
  stats->output_bytes = out_bytes;
  gate.finish();
  const uint64_t mb = gate.min_budget.load();
  stats->min_memory_budget_mib = mb == ~uint64_t(0) ? -1.0 : mb / 1048576.0;
  (void)ring;
  s->last_latency = lat;
  return CFFT_OK;
}

size_t cfft_server_recorded(const cfft_server* s) { return s ? s->recorded.size() : 0; }

cfft_status cfft_server_recorded_ids(const cfft_server* s, uint64_t* ids, size_t cap) {
  if (!s || !ids) return fail(CFFT_ERR_INVALID_ARGUMENT, "null argument");
  size_t i = 0;
  for (const auto& kv : s->recorded) {
    if (i == cap) break;
    ids[i++] = kv.first;
  }
  return CFFT_OK;
}

cfft_status cfft_server_request_shape(const cfft_server* s, const cfft_serve_config* cfg, uint64_t id,
                                      uint32_t* log2N, uint32_t* nprod) {
  if (!s || !cfg) return fail(CFFT_ERR_INVALID_ARGUMENT, "null argument");
  const ReqDesc r = make_request(s, *cfg, id, 0.0);
  if (log2N) *log2N = r.log2N;
  if (nprod) *nprod = r.nprod;
  return CFFT_OK;
}

cfft_status cfft_server_recorded_output(const cfft_server* s, uint64_t id, uint64_t* out, size_t words) {
  if (!s || !out) return fail(CFFT_ERR_INVALID_ARGUMENT, "null argument");
  auto it = s->recorded.find(id);
  if (it == s->recorded.end()) return fail(CFFT_ERR_INVALID_ARGUMENT, "request not recorded");
  if (words != it->second.size()) return fail(CFFT_ERR_LENGTH_MISMATCH, "output size differs");
  std::memcpy(out, it->second.data(), words * 8);
  return CFFT_OK;
}

cfft_status cfft_server_run_alone(cfft_server* s, const cfft_serve_config* cfg, uint64_t id, uint64_t* out,
                                  size_t words) {
  if (!s || !cfg || !out) return fail(CFFT_ERR_INVALID_ARGUMENT, "null argument");
  const ReqDesc r = make_request(s, *cfg, id, 0.0);
  if (words != ((size_t)r.nprod << r.log2N)) return fail(CFFT_ERR_LENGTH_MISMATCH, "output size differs");
  return run_alone(s, r, out);
}

cfft_status cfft_server_request_inputs(const cfft_server* s, const cfft_serve_config* cfg, uint64_t id,
                                       int64_t* digits, double* bhat) {
  if (!s || !cfg) return fail(CFFT_ERR_INVALID_ARGUMENT, "null argument");
  const ReqDesc r = make_request(s, *cfg, id, 0.0);
  const SizePool* p = pool_of(s, r.log2N);
  const size_t N = size_t(1) << r.log2N;
  for (uint32_t i = 0; i < r.nprod; ++i) {
    if (digits)
      CFFT_CUDA_TRY(cudaMemcpy(digits + i * N, p->digits + (size_t)r.rows[i] * N, N * 8, cudaMemcpyDeviceToHost));
    if (bhat) CFFT_CUDA_TRY(cudaMemcpy(bhat + i * N, p->bhat + (size_t)r.ops[i] * N, N * 8, cudaMemcpyDeviceToHost));
  }
  return CFFT_OK;
}

}  // extern "C"
