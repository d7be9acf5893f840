// queue.cu -- the product engine behind a work queue: submit / poll / wait.
//
// Callers on any thread submit groups of product items (cfft_product_item) and
// get a ticket.  One worker thread per queue gathers everything pending into
// the next launch on a free slot: the engine's persistent kernel over the
// small products and, beside it on a second stream, one thread-block cluster
// per product of N >= 2^cluster_log2N (the continuous batching of the serving
// loop, behind a public API).  A slot's item records sit in page-locked host
// memory that the kernels read through its device address, so a launch is the
// kernels and one event.  The worker polls the slots' events and marks their
// tickets done; callers poll a ticket or block on it.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "cfft_internal.h"
#include "runtime.h"

using namespace cfft;

namespace {

constexpr int kMaxQueueSlots = 4;
constexpr size_t kQueueSlotItems = 4096;

struct QSlot {
  cudaStream_t stream = nullptr, stream2 = nullptr;
  cudaEvent_t done = nullptr, big_done = nullptr;
  unsigned int* counter = nullptr;
  double* ws = nullptr;
  cfft_product_item* h_items = nullptr;      // page-locked
  cfft_product_item* h_items_dev = nullptr;  // its device address
  size_t cap = 0;
  bool busy = false;
  std::vector<uint64_t> tickets;
};

struct Pending {
  uint64_t ticket;
  std::vector<cfft_product_item> items;
};

}  // namespace

struct cfft_product_queue {
  const cfft_product_engine* engine = nullptr;
  int device = 0;
  int nslots = 3;
  bool on_cluster[32] = {};      // launches of more than kClusterAllItems products
  bool on_cluster_all[32] = {};  // smaller launches
  QSlot slots[kMaxQueueSlots];
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Pending> pending;
  std::unordered_map<uint64_t, int> state;  // ticket -> 0 queued or running, 1 done, < 0 failed
  uint64_t next_ticket = 1;
  bool stop = false;
  std::thread worker;
};

namespace {

cfft_status grow_items(QSlot& sl, size_t n) {
  if (n <= sl.cap) return CFFT_OK;
  const size_t cap = std::max(n, 2 * sl.cap);
  if (sl.h_items) cudaFreeHost(sl.h_items);
  sl.h_items = sl.h_items_dev = nullptr;
  sl.cap = 0;
  CFFT_CUDA_TRY(cudaMallocHost(&sl.h_items, cap * sizeof(cfft_product_item)));
  CFFT_CUDA_TRY(cudaHostGetDevicePointer((void**)&sl.h_items_dev, sl.h_items, 0));
  sl.cap = cap;
  return CFFT_OK;
}

// One launch on a free slot: the engine's items first, then the cluster items grouped by N.
cfft_status launch_slot(cfft_product_queue* q, QSlot& sl, const std::vector<Pending>& batch) {
  size_t nitems = 0;
  for (const auto& p : batch) nitems += p.items.size();
  const bool* on_cluster = nitems <= kClusterAllItems ? q->on_cluster_all : q->on_cluster;
  cfft_status st = grow_items(sl, nitems);
  if (st != CFFT_OK) return st;
  size_t at = 0;
  for (const auto& p : batch)
    for (const auto& it : p.items)
      if (!on_cluster[it.log2N]) sl.h_items[at++] = it;
  const size_t nsmall = at;
  size_t first[32] = {}, count[32] = {};
  for (uint32_t lN = 0; lN < 32; ++lN) {
    if (!on_cluster[lN]) continue;
    first[lN] = at;
    for (const auto& p : batch)
      for (const auto& it : p.items)
        if (it.log2N == lN) sl.h_items[at++] = it;
    count[lN] = at - first[lN];
  }
  if (nsmall < nitems) {
    for (uint32_t lN = 0; lN < 32; ++lN) {
      if (!count[lN]) continue;
      st = u64_product_split_items(cfft_product_engine_plan(q->engine, lN), sl.h_items_dev + first[lN], count[lN],
                                   sl.stream2);
      if (st != CFFT_OK) return st;
    }
    CFFT_CUDA_TRY(cudaEventRecord(sl.big_done, sl.stream2));
  }
  if (nsmall) {
    st = cfft_product_engine_run(q->engine, sl.h_items_dev, nsmall, sl.counter, sl.ws, sl.stream);
    if (st != CFFT_OK) return st;
  }
  if (nsmall < nitems) CFFT_CUDA_TRY(cudaStreamWaitEvent(sl.stream, sl.big_done, 0));
  CFFT_CUDA_TRY(cudaEventRecord(sl.done, sl.stream));
  return CFFT_OK;
}

void finish(cfft_product_queue* q, const std::vector<uint64_t>& tickets, int result) {
  for (uint64_t t : tickets) q->state[t] = result;
}

// After its last launch completes the worker keeps polling for this long before it
// blocks on the condition variable: a request that arrives meanwhile is launched
// without the scheduler's wake-up latency (tens of microseconds).
constexpr auto kQueueSpin = std::chrono::microseconds(200);

void worker_main(cfft_product_queue* q) {
  cudaSetDevice(q->device);
  std::unique_lock<std::mutex> lk(q->mu);
  auto idle_since = std::chrono::steady_clock::now();
  for (;;) {
    int free_slot = -1;
    bool any_busy = false;
    for (int k = 0; k < q->nslots; ++k) {
      if (q->slots[k].busy) any_busy = true;
      else if (free_slot < 0) free_slot = k;
    }
    if (!q->pending.empty() && free_slot >= 0) {
      // everything pending goes into this launch (the slot's records grow to fit)
      std::vector<Pending> batch(std::make_move_iterator(q->pending.begin()),
                                 std::make_move_iterator(q->pending.end()));
      q->pending.clear();
      QSlot& sl = q->slots[free_slot];
      sl.tickets.clear();
      for (const auto& p : batch) sl.tickets.push_back(p.ticket);
      lk.unlock();
      const cfft_status st = launch_slot(q, sl, batch);
      if (st != CFFT_OK) {
        // part of the launch may be running (the clusters on the second stream):
        // let it end before the slot's records can be rewritten
        cudaStreamSynchronize(sl.stream2);
        cudaStreamSynchronize(sl.stream);
      }
      lk.lock();
      if (st == CFFT_OK) {
        sl.busy = true;
      } else {
        finish(q, sl.tickets, (int)st);
        q->cv_done.notify_all();
      }
      continue;
    }
    if (!any_busy) {
      if (q->stop && q->pending.empty()) break;
      if (std::chrono::steady_clock::now() - idle_since < kQueueSpin) {
        lk.unlock();
        std::this_thread::yield();
        lk.lock();
        continue;
      }
      q->cv_work.wait(lk);
      idle_since = std::chrono::steady_clock::now();
      continue;
    }
    // launches in flight: look at their events without holding the lock
    lk.unlock();
    int done_slot = -1;
    cudaError_t err = cudaSuccess;
    for (int k = 0; k < q->nslots && done_slot < 0; ++k) {
      if (!q->slots[k].busy) continue;
      const cudaError_t e = cudaEventQuery(q->slots[k].done);
      if (e == cudaErrorNotReady) continue;
      done_slot = k;
      err = e;
    }
    lk.lock();
    if (done_slot < 0) {
      // nothing finished: yield the CPU once and look again (a timed wait would
      // add the scheduler's wake-up latency, tens of microseconds, to every request)
      lk.unlock();
      std::this_thread::yield();
      lk.lock();
      continue;
    }
    QSlot& sl = q->slots[done_slot];
    if (err != cudaSuccess) set_error(std::string("product queue launch: ") + cudaGetErrorString(err));
    finish(q, sl.tickets, err == cudaSuccess ? 1 : (int)CFFT_ERR_CUDA);
    sl.tickets.clear();
    sl.busy = false;
    idle_since = std::chrono::steady_clock::now();
    q->cv_done.notify_all();
  }
}

void free_queue(cfft_product_queue* q) {
  for (auto& sl : q->slots) {
    if (sl.stream) cudaStreamDestroy(sl.stream);
    if (sl.stream2) cudaStreamDestroy(sl.stream2);
    if (sl.done) cudaEventDestroy(sl.done);
    if (sl.big_done) cudaEventDestroy(sl.big_done);
    if (sl.counter) cudaFree(sl.counter);
    if (sl.ws) cudaFree(sl.ws);
    if (sl.h_items) cudaFreeHost(sl.h_items);
  }
}

// The device address of an item's buffer: device and managed memory as given,
// page-locked host memory through its mapping; pageable host memory is refused.
bool device_address(const void* p, const void** dev) {
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) {
    *dev = p;
    return true;
  }
  if (at.type == cudaMemoryTypeHost && at.devicePointer) {
    *dev = at.devicePointer;
    return true;
  }
  return false;
}

int ticket_result(cfft_product_queue* q, uint64_t ticket) {
  auto it = q->state.find(ticket);
  if (it == q->state.end()) return 1;  // done and already collected
  const int r = it->second;
  if (r != 0) q->state.erase(it);
  return r;
}

}  // namespace

extern "C" {

cfft_status cfft_product_queue_create(const cfft_product_engine* engine, const cfft_product_queue_config* config,
                                      cfft_product_queue** out) {
  if (!out) return fail(CFFT_ERR_INVALID_ARGUMENT, "null output pointer");
  *out = nullptr;
  if (!engine) return fail(CFFT_ERR_INVALID_ARGUMENT, "null engine");
  const uint32_t inflight = config && config->max_inflight ? config->max_inflight : 3;
  if (inflight > (uint32_t)kMaxQueueSlots) return fail(CFFT_ERR_INVALID_ARGUMENT, "max_inflight must be 0..4");
  const uint32_t big = config && config->cluster_log2N ? config->cluster_log2N : 13;
  auto* q = new cfft_product_queue();
  q->engine = engine;
  q->nslots = (int)inflight;
  cfft_status st = CFFT_OK;
  if (cudaGetDevice(&q->device) != cudaSuccess) st = fail(CFFT_ERR_CUDA, "no CUDA device");
  for (uint32_t lN = 0; lN < 32 && st == CFFT_OK; ++lN) {
    const cfft_u64_product_plan* p = lN <= 17 ? cfft_product_engine_plan(engine, lN) : nullptr;
    const bool split = p && u64_product_splittable(p);
    q->on_cluster[lN] = split && lN >= big;
    q->on_cluster_all[lN] = config && config->cluster_log2N ? q->on_cluster[lN] : split;
  }
  const size_t ws = cfft_product_engine_workspace_bytes(engine);
  for (int k = 0; k < q->nslots && st == CFFT_OK; ++k) {
    QSlot& sl = q->slots[k];
    if (cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&sl.stream2, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&sl.big_done, cudaEventDisableTiming) != cudaSuccess ||
        cudaMalloc(&sl.counter, 64) != cudaSuccess || (ws && cudaMalloc(&sl.ws, ws) != cudaSuccess)) {
      st = fail(CFFT_ERR_OUT_OF_MEMORY, "product queue slots");
      break;
    }
    st = grow_items(sl, kQueueSlotItems);
  }
  if (st != CFFT_OK) {
    free_queue(q);
    delete q;
    return st;
  }
  q->worker = std::thread(worker_main, q);
  *out = q;
  return CFFT_OK;
}

void cfft_product_queue_destroy(cfft_product_queue* queue) {
  if (!queue) return;
  {
    std::lock_guard<std::mutex> lk(queue->mu);
    queue->stop = true;
  }
  queue->cv_work.notify_all();
  if (queue->worker.joinable()) queue->worker.join();  // after every submitted group has run
  free_queue(queue);
  delete queue;
}

cfft_status cfft_product_queue_submit(cfft_product_queue* queue, const cfft_product_item* items, size_t count,
                                      uint64_t* ticket) {
  if (!queue || !ticket || (count && !items)) return fail(CFFT_ERR_INVALID_ARGUMENT, "null argument");
  *ticket = 0;
  // this thread's pointer queries need the queue's device context; the caller's
  // current device is put back on return
  int caller_dev = -1;
  cudaGetDevice(&caller_dev);
  cudaSetDevice(queue->device);
  struct Restore {
    int dev, mine;
    ~Restore() {
      if (dev >= 0 && dev != mine) cudaSetDevice(dev);
    }
  } restore{caller_dev, queue->device};
  Pending p;
  p.items.reserve(count);
  for (size_t i = 0; i < count; ++i) {
    cfft_product_item it = items[i];
    if (it.log2N > 17 || it.reserved != 0 || !cfft_product_engine_plan(queue->engine, it.log2N))
      return fail(CFFT_ERR_INVALID_SIZE, "item size not configured in the engine");
    const void *a = nullptr, *b = nullptr, *o = nullptr;
    if (!it.a || !it.bhat || !it.out || !device_address(it.a, &a) || !device_address(it.bhat, &b) ||
        !device_address(it.out, &o))
      return fail(CFFT_ERR_INVALID_ARGUMENT, "item buffers must be device or page-locked host memory");
    it.a = (const uint64_t*)a;
    it.bhat = (const double*)b;
    it.out = (uint64_t*)o;
    p.items.push_back(it);
  }
  {
    std::lock_guard<std::mutex> lk(queue->mu);
    if (queue->stop) return fail(CFFT_ERR_INVALID_ARGUMENT, "queue is shutting down");
    p.ticket = queue->next_ticket++;
    *ticket = p.ticket;
    if (count == 0) {
      queue->state[p.ticket] = 1;
      return CFFT_OK;
    }
    queue->state[p.ticket] = 0;
    queue->pending.push_back(std::move(p));
  }
  queue->cv_work.notify_one();
  return CFFT_OK;
}

int cfft_product_queue_poll(cfft_product_queue* queue, uint64_t ticket) {
  if (!queue) return (int)fail(CFFT_ERR_INVALID_ARGUMENT, "null queue");
  std::lock_guard<std::mutex> lk(queue->mu);
  if (ticket == 0 || ticket >= queue->next_ticket) return (int)fail(CFFT_ERR_INVALID_ARGUMENT, "unknown ticket");
  return ticket_result(queue, ticket);
}

cfft_status cfft_product_queue_wait(cfft_product_queue* queue, uint64_t ticket) {
  if (!queue) return fail(CFFT_ERR_INVALID_ARGUMENT, "null queue");
  std::unique_lock<std::mutex> lk(queue->mu);
  if (ticket == 0 || ticket >= queue->next_ticket) return fail(CFFT_ERR_INVALID_ARGUMENT, "unknown ticket");
  queue->cv_done.wait(lk, [&] {
    auto it = queue->state.find(ticket);
    return it == queue->state.end() || it->second != 0;
  });
  const int r = ticket_result(queue, ticket);
  return r == 1 ? CFFT_OK : (cfft_status)r;
}

}  // extern "C"
