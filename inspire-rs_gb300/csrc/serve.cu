// serve.cu -- the serving loop: continuous batching of seeded InspiRING
// queries over several CUDA streams.
//
// Submitted queries are copied into records of a pinned, device-mapped pool
// (rows ELL..2ELL-1 only: seeds and b-polys), or borrowed in place.  A
// dispatcher thread takes up to max_batch pending queries whenever one of its
// streams is free, writes one QueryDesc per query into that stream's pinned
// descriptor array, and issues descriptor copy -> respond -> event on the
// stream.  The Respond kernel reads each query's rows from, and writes its
// response to, pinned host memory over the host link (NVLink-C2C on a
// Grace-Blackwell node), so no host thread copies a batch and no extra
// kernel runs.  Batches on different streams overlap on the device, which
// also fills the SMs a single batch leaves idle.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <climits>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <thread>

#include <cuda.h>

#include "host.h"
#include "serve_policy.h"

using namespace ig;
using namespace ighost;

namespace {

int64_t now_ns() {
  return std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

// Pool record: [seeds ELL*32 (padded to 128)][b rows ELL*2N u64][out 4N u64][status]
constexpr size_t REC_SEEDS = 0;
constexpr size_t REC_BROWS = 128;
constexpr size_t REC_OUT = REC_BROWS + sizeof(uint64_t) * ELL * 2 * N;
constexpr size_t REC_STATUS = REC_OUT + sizeof(uint64_t) * 4 * N;
constexpr size_t REC_BYTES = (REC_STATUS + 16 + 255) & ~(size_t)255;
constexpr int TICKET_IDX_BITS = 24;

// Device bytes one query of a batch holds (its descriptor).
constexpr size_t SLOT_BYTES_PER_QUERY = sizeof(QueryDesc);

enum RecState { FREE = 0, PENDING = 1, INFLIGHT = 2, DONE = 3, COLLECTING = 4 };

struct Rec {
  uint64_t gen = 1;
  RecState state = FREE;
  const uint8_t* seeds = nullptr;   // host rows: the pool record's or borrowed
  const uint64_t* brows = nullptr;
  const inspire_db* db = nullptr;
  uint32_t shard = 0;
  int32_t client = 0;
  int64_t t_arrival = 0, t_done = 0;
  int64_t t_enqueue = 0;  // when the query became pending
  int cuda_error = 0;  // nonzero: the batch failed on the host side
  bool batch_lost = false;  // a CTA of the query's batch exited with copies in flight
};

struct Slot {
  cudaStream_t st = nullptr;
  cudaEvent_t ev = nullptr;
  QueryDesc* desc = nullptr;  // pinned (host)
  DevMem ddesc;               // the batch's descriptors in device memory
  std::vector<int> recs;
  bool busy = false;
  bool pair = false;  // the batch runs on the two-CTA cluster kernel (two SMs per query)
};

}  // namespace

struct inspire_server {
  inspire_ctx* ctx = nullptr;
  inspire_server_config cfg{};
  uint8_t* pool = nullptr;  // pinned, mapped; capacity records
  uint8_t* dpool = nullptr;  // the pool's device address
  std::vector<Rec> recs;
  std::deque<int> free_list, pending;
  std::vector<std::unique_ptr<Slot>> slots;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  bool stop = false;
  std::thread worker;
  uint64_t n_submitted = 0, n_completed = 0, n_batches = 0;
  int sm_count = 0;
  std::string worker_error;

  uint8_t* rec_ptr(int i) const { return pool + (size_t)i * REC_BYTES; }
  uint8_t* dev_rec_ptr(int i) const { return dpool + (size_t)i * REC_BYTES; }
  uint64_t ticket(int i) const { return (recs[i].gen << TICKET_IDX_BITS) | (uint64_t)i; }
  void run();
  int launch(Slot& s, const std::vector<int>& batch);
};

// Issue descriptor copy -> respond -> event for `batch` on slot `s`.
int inspire_server::launch(Slot& s, const std::vector<int>& batch) {
  const int n = (int)batch.size();
  for (int k = 0; k < n; k++) {
    const Rec& r = recs[batch[k]];
    uint8_t* p = dev_rec_ptr(batch[k]);
    QueryDesc& d = s.desc[k];
    memcpy(d.seeds, r.seeds, sizeof(d.seeds));
    d.brows = r.brows;
    d.out = reinterpret_cast<uint64_t*>(p + REC_OUT);
    d.status = reinterpret_cast<int32_t*>(p + REC_STATUS);
    d.db = DbView{r.db->E.as<uint32_t>(), r.db->H.as<uint16_t>(), r.db->nshards, 0};
    d.shard = r.shard;
    d.client = r.client;
  }
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (int rc = sync_client_table(ctx)) return rc;
  CUDA_TRY(cudaMemcpyAsync(s.ddesc.p, s.desc, sizeof(QueryDesc) * n, cudaMemcpyHostToDevice, s.st));
  RespondArgs a{};
  a.P = ctx->P;
  a.nq = n;
  a.yhat_table = ctx->client_table.as<const uint32_t*>();
  a.nclients = (int)ctx->client_ptrs.size();
  a.what = ctx->what3.as<uint32_t>();
  a.qdesc = s.ddesc.as<QueryDesc>();
  a.stage_wait_iters = cfg.stage_wait_iters;
  CUDA_TRY(launch_respond(a, true, s.st, 0, s.pair ? n : 0));
  CUDA_TRY(cudaEventRecord(s.ev, s.st));
  return INSPIRE_OK;
}

// The dispatcher.  Events are queried and batches launched without holding
// `mu` (only this thread changes a slot's batch), so submitters and pollers
// only ever wait for the short bookkeeping sections.
void inspire_server::run() {
  cudaSetDevice(ctx->device);
  std::vector<Slot*> finished, to_launch;
  std::vector<cudaError_t> fin_err;
  for (;;) {
    finished.clear();
    fin_err.clear();
    for (auto& sp : slots) {
      if (!sp->busy) continue;
      const cudaError_t e = cudaEventQuery(sp->ev);
      if (e == cudaErrorNotReady) continue;
      finished.push_back(sp.get());
      fin_err.push_back(e);
    }
    to_launch.clear();
    {
      std::unique_lock<std::mutex> lk(mu);
      const int64_t t = now_ns();
      for (size_t k = 0; k < finished.size(); k++) {
        Slot& s = *finished[k];
        const cudaError_t e = fin_err[k];
        // one query whose staged rows were still in flight when its CTA
        // exited makes every result of the launch unreliable
        bool lost = false;
        if (e == cudaSuccess)
          for (int i : s.recs)
            lost |= *reinterpret_cast<const volatile int32_t*>(rec_ptr(i) + REC_STATUS) == ERR_STAGE_LOST;
        for (int i : s.recs) recs[i].batch_lost = lost;
        for (int i : s.recs) {
          recs[i].state = DONE;
          recs[i].t_done = t;
          recs[i].cuda_error = e == cudaSuccess ? 0 : (int)e;
        }
        if (e != cudaSuccess) worker_error = std::string("serving batch: ") + cudaGetErrorString(e);
        n_completed += s.recs.size();
        s.recs.clear();
        s.busy = false;
      }
      // SMs the batches in flight occupy, then each free stream takes the
      // next batch (launch_batch_now) on the kernel use_pair_kernel picks
      // (serve_policy.h)
      const size_t pair_max = (size_t)std::max(0, ctx->pair_max.load(std::memory_order_relaxed));
      size_t inflight_sm = 0;
      for (const auto& sp : slots) inflight_sm += sp->busy ? batch_sms(sp->pair, sp->recs.size()) : 0;
      for (auto& sp : slots) {
        if (sp->busy || pending.empty()) continue;
        if (!launch_batch_now(pending.size(), cfg.max_batch, inflight_sm, (size_t)sm_count,
                              now_ns() - recs[pending.front()].t_enqueue, (int64_t)cfg.batch_wait_us * 1000))
          break;
        Slot& s = *sp;
        s.recs.clear();
        while (!pending.empty() && s.recs.size() < cfg.max_batch) {
          const int i = pending.front();
          pending.pop_front();
          recs[i].state = INFLIGHT;
          s.recs.push_back(i);
        }
        s.busy = true;
        n_batches++;
        const size_t nb = s.recs.size();
        s.pair = use_pair_kernel(nb, pair_max, inflight_sm, (size_t)sm_count);
        inflight_sm += batch_sms(s.pair, nb);
        to_launch.push_back(&s);
      }
      bool any_busy = false;
      for (const auto& sp : slots) any_busy |= sp->busy;
      if (stop && !any_busy && pending.empty()) break;
      // nothing in flight: pending queries (if any) were launched above
      if (finished.empty() && to_launch.empty() && !any_busy) {
        cv_work.wait(lk, [&] { return stop || !pending.empty(); });
        continue;
      }
    }
    if (!finished.empty()) cv_done.notify_all();
    for (Slot* sp : to_launch) {
      Slot& s = *sp;
      const int rc = launch(s, s.recs);
      if (rc != INSPIRE_OK) {  // fail the batch's queries; the loop keeps serving
        cudaStreamSynchronize(s.st);
        std::lock_guard<std::mutex> lk(mu);
        worker_error = g_last_error;
        const int64_t t = now_ns();
        for (int i : s.recs) {
          recs[i].state = DONE;
          recs[i].t_done = t;
          recs[i].cuda_error = rc;
        }
        n_completed += s.recs.size();
        s.recs.clear();
        s.busy = false;
        cv_done.notify_all();
      }
    }
    if (finished.empty() && to_launch.empty()) std::this_thread::yield();  // batches in flight
  }
}

namespace {

// Allocations made by inspire_pinned_alloc (base -> bytes).
std::mutex g_pinned_mu;
std::map<uintptr_t, size_t> g_pinned;

bool in_own_pinned(const void* p, size_t bytes) {
  const uintptr_t a = reinterpret_cast<uintptr_t>(p);
  std::lock_guard<std::mutex> lk(g_pinned_mu);
  auto it = g_pinned.upper_bound(a);
  if (it == g_pinned.begin()) return false;
  --it;
  return a >= it->first && bytes <= it->second && a - it->first <= it->second - bytes;
}

// cuPointerGetAttribute, reached through the runtime's driver entry point so
// that the library does not link against libcuda itself.
using PtrAttrFn = CUresult (*)(void*, CUpointer_attribute, CUdeviceptr);
PtrAttrFn ptr_attr_fn() {
  static const PtrAttrFn f = [] {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult st = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuPointerGetAttribute", &fn, 12000, cudaEnableDefault, &st) != cudaSuccess ||
        st != cudaDriverEntryPointSuccess) {
      cudaGetLastError();
      return static_cast<PtrAttrFn>(nullptr);
    }
    return reinterpret_cast<PtrAttrFn>(fn);
  }();
  return f;
}

// Whether [p, p + bytes) lies inside the one allocation that p belongs to,
// by the driver's record of that allocation's address range.
bool within_one_allocation(const void* p, size_t bytes) {
  const PtrAttrFn f = ptr_attr_fn();
  if (!f) return false;
  CUdeviceptr start = 0;
  size_t size = 0;
  const CUdeviceptr a = (CUdeviceptr) reinterpret_cast<uintptr_t>(p);
  if (f(&start, CU_POINTER_ATTRIBUTE_RANGE_START_ADDR, a) != CUDA_SUCCESS ||
      f(&size, CU_POINTER_ATTRIBUTE_RANGE_SIZE, a) != CUDA_SUCCESS)
    return false;
  return a >= start && bytes <= size && a - start <= size - bytes;
}

}  // namespace

namespace ighost {

// Device address of a page-locked host range [p, p + bytes), or null.  The
// whole range must lie in ONE page-locked allocation: checking its two ends
// alone would accept a range that spans two adjacent allocations with
// ordinary memory between them, which a kernel would then read.  Ranges in
// memory from inspire_pinned_alloc are checked against the library's own
// record of those allocations; other page-locked memory (cudaHostAlloc,
// cudaHostRegister) against the driver's record of the allocation's range.
// Anything unconfirmed is refused (callers then stage through device
// buffers, or report the error).
const uint8_t* mapped_range(const void* p, size_t bytes) {
  if (bytes == 0) return nullptr;
  cudaPointerAttributes a{}, b{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess || a.type != cudaMemoryTypeHost || !a.devicePointer) {
    cudaGetLastError();
    return nullptr;
  }
  const uint8_t* last = static_cast<const uint8_t*>(p) + bytes - 1;
  if (cudaPointerGetAttributes(&b, last) != cudaSuccess || b.type != cudaMemoryTypeHost || !b.devicePointer ||
      static_cast<const uint8_t*>(b.devicePointer) != static_cast<const uint8_t*>(a.devicePointer) + (bytes - 1)) {
    cudaGetLastError();
    return nullptr;
  }
  if (!in_own_pinned(p, bytes) && !within_one_allocation(p, bytes)) return nullptr;
  return static_cast<const uint8_t*>(a.devicePointer);
}

}  // namespace ighost

extern "C" {

void inspire_server_config_default(inspire_server_config* cfg) {
  if (!cfg) return;
  cfg->max_batch = 128;
  cfg->max_inflight = 4;
  cfg->capacity = 4096;
  cfg->device_budget = 0;
  cfg->batch_wait_us = 100;
  cfg->stage_wait_iters = STAGE_WAIT_ITERS_DEFAULT;
}

int64_t inspire_now_ns(void) { return now_ns(); }

int inspire_server_create(inspire_ctx* c, const inspire_server_config* cfg, inspire_server** out) {
  if (!c || !cfg || !out) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null argument");
  *out = nullptr;
  if (!c->has_crs) return fail(INSPIRE_ERR_NO_CRS, "no CRS loaded (inspire_crs_load)");
  if (cfg->max_batch < 1 || cfg->max_batch > 1024 || cfg->max_inflight < 1 || cfg->max_inflight > 64 ||
      cfg->capacity < cfg->max_batch || cfg->capacity >= (1u << TICKET_IDX_BITS))
    return fail(INSPIRE_ERR_INVALID_ARGUMENT, "server config out of range");
  uint32_t streams = cfg->max_inflight;
  const size_t slot_bytes = SLOT_BYTES_PER_QUERY * cfg->max_batch;
  if (cfg->device_budget) {
    const uint64_t fit = cfg->device_budget / slot_bytes;
    if (fit == 0) return fail(INSPIRE_ERR_OUT_OF_MEMORY, "device_budget is below one batch");
    if (fit < streams) streams = (uint32_t)fit;
  }
  if (int rc = set_device(c)) return rc;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device) != cudaSuccess || sms <= 0)
    return fail(INSPIRE_ERR_CUDA, "cannot read the SM count");
  inspire_server* s = new inspire_server();
  s->ctx = c;
  s->cfg = *cfg;
  s->sm_count = sms;
  auto bail = [&](int rc) {
    inspire_server_destroy(s);
    return rc;
  };
  cudaError_t e = cudaHostAlloc(reinterpret_cast<void**>(&s->pool), REC_BYTES * cfg->capacity,
                                cudaHostAllocMapped | cudaHostAllocPortable);
  if (e != cudaSuccess) {
    s->pool = nullptr;
    return bail(fail(INSPIRE_ERR_OUT_OF_MEMORY, std::string("pinned query pool: ") + cudaGetErrorString(e)));
  }
  if (cudaHostGetDevicePointer(reinterpret_cast<void**>(&s->dpool), s->pool, 0) != cudaSuccess)
    return bail(fail(INSPIRE_ERR_CUDA, "pinned query pool is not device-mapped"));
  s->recs.resize(cfg->capacity);
  for (uint32_t i = 0; i < cfg->capacity; i++) s->free_list.push_back((int)i);
  for (uint32_t i = 0; i < streams; i++) s->slots.push_back(std::make_unique<Slot>());
  const size_t B = cfg->max_batch;
  for (auto& slp : s->slots) {
    Slot& sl = *slp;
    if (cudaStreamCreateWithFlags(&sl.st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&sl.ev, cudaEventDisableTiming) != cudaSuccess ||
        cudaHostAlloc(reinterpret_cast<void**>(&sl.desc), sizeof(QueryDesc) * B, cudaHostAllocDefault) != cudaSuccess)
      return bail(fail(INSPIRE_ERR_CUDA, "serving stream setup failed"));
    sl.ddesc.ledger = c->ledger;
    if (sl.ddesc.ensure(sizeof(QueryDesc) * B))
      return bail(fail(INSPIRE_ERR_OUT_OF_MEMORY, alloc_failure(c, "serving slot buffers")));
  }
  s->worker = std::thread([s] { s->run(); });
  *out = s;
  return INSPIRE_OK;
}

void inspire_server_destroy(inspire_server* s) {
  if (!s) return;
  if (s->worker.joinable()) {
    {
      std::lock_guard<std::mutex> lk(s->mu);
      s->stop = true;
      s->pending.clear();  // queries never launched die with the loop
    }
    s->cv_work.notify_all();
    s->worker.join();
  }
  cudaSetDevice(s->ctx->device);
  for (auto& slp : s->slots) {
    Slot& sl = *slp;
    if (sl.st) cudaStreamSynchronize(sl.st);
    if (sl.ev) cudaEventDestroy(sl.ev);
    if (sl.st) cudaStreamDestroy(sl.st);
    if (sl.desc) cudaFreeHost(sl.desc);
  }
  if (s->pool) cudaFreeHost(s->pool);
  delete s;
}


int inspire_server_submit(inspire_server* s, uint32_t n, const inspire_db* const* dbs, const uint32_t* shard_ids,
                          const uint8_t* seeds, const uint64_t* b_rows, const int32_t* client_ids,
                          const int64_t* arrival_ns, uint32_t flags, uint64_t* tickets, uint32_t* accepted) {
  if (accepted) *accepted = 0;
  if (!s || !accepted || (n && (!dbs || !shard_ids || !seeds || !b_rows || !client_ids || !tickets)))
    return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null argument");
  if (flags & ~INSPIRE_SUBMIT_BORROW) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "unknown submit flags");
  const bool borrow = flags & INSPIRE_SUBMIT_BORROW;
  const size_t pw = poly_words();
  // borrowed b rows are read in place by the GPU; the seeds (96 bytes per
  // query) are copied into the batch's descriptors by the dispatcher
  const uint8_t* d_brows = nullptr;
  if (borrow && n) {
    // pointer attributes are looked up in this thread's current context
    if (int rc = set_device(s->ctx)) return rc;
    if (reinterpret_cast<uintptr_t>(b_rows) % 16)
      return fail(INSPIRE_ERR_INVALID_ARGUMENT, "borrowed b_rows must be 16-byte aligned");
    d_brows = mapped_range(b_rows, sizeof(uint64_t) * (size_t)n * 2 * ELL * pw);
    if (!d_brows)
      return fail(INSPIRE_ERR_INVALID_ARGUMENT, "borrowed query rows must lie in page-locked host memory");
  }
  const int64_t t_submit = now_ns();
  // validate in order; the first invalid query ends the accepted prefix
  uint32_t valid = n;
  int vrc = INSPIRE_OK;
  std::string vmsg;
  {
    std::lock_guard<std::mutex> lk(s->ctx->mu);
    for (uint32_t i = 0; i < n; i++) {
      const inspire_db* db = dbs[i];
      if (!db || db->device != s->ctx->device) {
        valid = i;
        vrc = INSPIRE_ERR_INVALID_ARGUMENT;
        vmsg = "query " + std::to_string(i) + ": null database or database of another device";
        break;
      }
      if (shard_ids[i] >= (uint32_t)db->nshards) {
        valid = i;
        vrc = INSPIRE_ERR_SHARD_NOT_FOUND;
        vmsg = "Shard " + std::to_string(shard_ids[i]) + " not found";
        break;
      }
      const int32_t id = client_ids[i];
      if (id < 0 || (size_t)id >= s->ctx->clients.size() || !s->ctx->clients[id]) {
        valid = i;
        vrc = INSPIRE_ERR_KEYS_MISSING;
        vmsg = "InspiRING client packing keys missing from query";
        break;
      }
    }
  }
  // reserve records
  std::vector<int> got;
  got.reserve(valid);
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "server is shutting down");
    while (got.size() < valid && !s->free_list.empty()) {
      got.push_back(s->free_list.front());
      s->free_list.pop_front();
    }
  }
  // rows ELL..2ELL-1 of each query: copied into its record, or borrowed in place
  for (size_t k = 0; k < got.size(); k++) {
    Rec& r = s->recs[got[k]];
    const size_t so = (size_t)k * 64 * ELL + 32 * ELL;                        // bytes into seeds
    const size_t bo = sizeof(uint64_t) * ((size_t)k * 2 * ELL + ELL) * pw;    // bytes into b_rows
    if (borrow) {
      r.seeds = seeds + so;
      r.brows = reinterpret_cast<const uint64_t*>(d_brows + bo);
    } else {
      uint8_t* p = s->rec_ptr(got[k]);
      memcpy(p + REC_SEEDS, seeds + so, 32 * ELL);
      memcpy(p + REC_BROWS, reinterpret_cast<const uint8_t*>(b_rows) + bo, sizeof(uint64_t) * ELL * pw);
      r.seeds = p + REC_SEEDS;
      r.brows = reinterpret_cast<const uint64_t*>(s->dev_rec_ptr(got[k]) + REC_BROWS);
    }
    r.db = dbs[k];
    r.shard = shard_ids[k];
    r.client = client_ids[k];
    r.t_arrival = arrival_ns ? arrival_ns[k] : t_submit;
    r.cuda_error = 0;
  }
  {
    std::lock_guard<std::mutex> lk(s->mu);
    const int64_t t_enq = now_ns();
    for (size_t k = 0; k < got.size(); k++) {
      s->recs[got[k]].state = PENDING;
      s->recs[got[k]].t_enqueue = t_enq;
      s->pending.push_back(got[k]);
      tickets[k] = s->ticket(got[k]);
    }
    s->n_submitted += got.size();
  }
  if (!got.empty()) s->cv_work.notify_one();
  *accepted = (uint32_t)got.size();
  if (got.size() < valid) return fail(INSPIRE_ERR_BUSY, "serving loop at capacity");
  if (vrc != INSPIRE_OK) return fail(vrc, vmsg);
  return INSPIRE_OK;
}

int inspire_pinned_alloc(size_t bytes, void** out) {
  if (!out) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null argument");
  *out = nullptr;
  if (bytes == 0) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "zero-size allocation");
  CUDA_TRY(cudaHostAlloc(out, bytes, cudaHostAllocMapped | cudaHostAllocPortable));
  std::lock_guard<std::mutex> lk(g_pinned_mu);
  g_pinned[reinterpret_cast<uintptr_t>(*out)] = bytes;
  return INSPIRE_OK;
}

void inspire_pinned_free(void* p) {
  if (!p) return;
  {
    std::lock_guard<std::mutex> lk(g_pinned_mu);
    g_pinned.erase(reinterpret_cast<uintptr_t>(p));
  }
  cudaFreeHost(p);
}

int inspire_server_poll(inspire_server* s, uint64_t ticket, uint64_t* out_ct, int64_t* done_ns, int32_t timeout_us) {
  if (!s) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null argument");
  const uint64_t idx = ticket & ((1ull << TICKET_IDX_BITS) - 1);
  std::unique_lock<std::mutex> lk(s->mu);
  if (idx >= s->recs.size() || s->recs[idx].gen != (ticket >> TICKET_IDX_BITS) || s->recs[idx].state == FREE)
    return fail(INSPIRE_ERR_INVALID_ARGUMENT, "unknown ticket");
  Rec& r = s->recs[idx];
  const uint64_t gen = r.gen;
  auto ready = [&] { return r.gen != gen || r.state == DONE || r.state == COLLECTING; };
  if (!ready()) {
    if (timeout_us == 0) return INSPIRE_PENDING;
    if (timeout_us < 0) {
      s->cv_done.wait(lk, ready);
    } else if (!s->cv_done.wait_for(lk, std::chrono::microseconds(timeout_us), ready)) {
      return INSPIRE_PENDING;
    }
  }
  if (r.gen != gen || r.state != DONE) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "ticket already collected");
  r.state = COLLECTING;  // this caller owns the record until it frees it
  const int cuda_error = r.cuda_error;
  const bool batch_lost = r.batch_lost;
  const int64_t t_done = r.t_done;
  lk.unlock();
  const uint8_t* p = s->rec_ptr((int)idx);
  const int32_t kstatus = *reinterpret_cast<const volatile int32_t*>(p + REC_STATUS);
  if (out_ct && !cuda_error && !kstatus && !batch_lost) memcpy(out_ct, p + REC_OUT, sizeof(uint64_t) * 4 * N);
  if (done_ns) *done_ns = t_done;
  lk.lock();
  r.gen++;
  r.state = FREE;
  s->free_list.push_back((int)idx);
  const std::string werr = s->worker_error;
  lk.unlock();
  if (cuda_error) return fail(INSPIRE_ERR_CUDA, werr.empty() ? "serving batch failed" : werr);
  if (batch_lost)
    return fail(INSPIRE_ERR_DEVICE_STATUS, "batch dropped: a query's rows were still being copied when its "
                                           "Respond CTA gave up waiting (ticket " + std::to_string(ticket) + ")");
  if (kstatus == ERR_STAGE)
    return fail(INSPIRE_ERR_DEVICE_STATUS, "query rows did not reach the GPU within stage_wait_iters (ticket " +
                                               std::to_string(ticket) + ")");
  if (kstatus)
    return fail(INSPIRE_ERR_DEVICE_STATUS, "respond kernel status " + std::to_string(kstatus) + " for ticket " +
                                               std::to_string(ticket));
  return INSPIRE_OK;
}

int inspire_server_poll_batch(inspire_server* s, uint32_t n, const uint64_t* tickets, uint64_t* out_ct,
                              int64_t* done_ns, int32_t timeout_us, uint32_t* collected) {
  if (collected) *collected = 0;
  if (!s || !collected || (n && !tickets)) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null argument");
  const int64_t deadline = timeout_us < 0 ? INT64_MAX : now_ns() + (int64_t)timeout_us * 1000;
  const size_t pw = poly_words();
  for (uint32_t k = 0; k < n; k++) {
    int32_t left = 0;
    if (timeout_us < 0) {
      left = -1;
    } else {
      const int64_t rem = deadline - now_ns();
      left = rem > 0 ? (int32_t)std::min<int64_t>(rem / 1000, INT32_MAX) : 0;
    }
    const int rc = inspire_server_poll(s, tickets[k], out_ct ? out_ct + (size_t)k * 2 * pw : nullptr,
                                       done_ns ? done_ns + k : nullptr, left);
    if (rc != INSPIRE_OK) return rc;
    *collected = k + 1;
  }
  return INSPIRE_OK;
}

int inspire_server_drive(inspire_server* s, uint32_t n, const inspire_db* const* dbs, const uint32_t* shard_ids,
                         const int32_t* client_ids, const uint8_t* pool_seeds, const uint64_t* pool_b_rows,
                         uint32_t pool_size, const int64_t* arrival_ns, uint32_t flags, uint32_t max_burst,
                         int64_t* submit_ns, int64_t* done_ns, uint32_t n_keep, uint64_t* out_keep) {
  if (!s || (n && (!dbs || !shard_ids || !client_ids || !pool_seeds || !pool_b_rows || !arrival_ns || !done_ns ||
                   pool_size == 0 || (n_keep && !out_keep))))
    return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null argument");
  if (n_keep > n) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "n_keep above n");
  for (uint32_t k = 1; k < n; k++)
    if (arrival_ns[k] < arrival_ns[k - 1]) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "arrivals not in order");
  if (max_burst == 0) max_burst = 256;
  const size_t pw = poly_words();
  const size_t seed_bytes = (size_t)64 * ELL, row_words = (size_t)2 * ELL * pw;
  std::vector<uint64_t> tickets(n);
  std::atomic<uint32_t> n_sub{0};
  std::atomic<int> stop_rc{INSPIRE_OK};   // the first failed query: the submitter stops
  std::atomic<bool> submit_end{false};    // the submitter has stopped (done or failed)
  std::string collector_err;
  // collector: every ticket in submission order, its completion time (the
  // serving loop's) and, for the first n_keep queries, the response.  A
  // failed query (its ticket is consumed all the same) or a rejected
  // submission stops the submissions, and the collector still collects every
  // ticket already accepted, so that none is left behind in the server.
  std::thread collector([&] {
    uint32_t k = 0;
    while (k < n) {
      if (k >= n_sub.load(std::memory_order_acquire)) {
        if (submit_end.load(std::memory_order_acquire) && k >= n_sub.load(std::memory_order_acquire)) break;
        std::this_thread::yield();
        continue;
      }
      const int rc = inspire_server_poll(s, tickets[k], k < n_keep ? out_keep + (size_t)k * 2 * pw : nullptr,
                                         done_ns + k, 2000);
      if (rc == INSPIRE_PENDING) continue;
      if (rc != INSPIRE_OK) {
        int expected = INSPIRE_OK;
        if (stop_rc.compare_exchange_strong(expected, rc)) collector_err = g_last_error;
        if (rc == INSPIRE_ERR_INVALID_ARGUMENT) break;  // the ticket was not ours to collect
      }
      k++;
    }
  });
  // submitter (this thread): each query at its arrival time, every query
  // already due in one call (one contiguous run of the pool), retrying on
  // backpressure
  uint32_t k = 0;
  int rc = INSPIRE_OK, submit_rc = INSPIRE_OK;
  std::string submit_err;
  while (k < n && stop_rc.load() == INSPIRE_OK) {
    const int64_t now = now_ns();
    if (arrival_ns[k] > now) {
      const int64_t gap = arrival_ns[k] - now;
      if (gap > 200000) std::this_thread::sleep_for(std::chrono::nanoseconds(gap - 100000));
      continue;  // spin the last 100 us
    }
    const uint32_t pk = k % pool_size;
    uint32_t j = k + 1;
    while (j < n && j - k < max_burst && j - k < pool_size - pk && arrival_ns[j] <= now) j++;
    uint32_t acc = 0;
    const int64_t t_call = now_ns();
    rc = inspire_server_submit(s, j - k, dbs + k, shard_ids + k, pool_seeds + (size_t)pk * seed_bytes,
                               pool_b_rows + (size_t)pk * row_words, client_ids + k, arrival_ns + k, flags,
                               tickets.data() + k, &acc);
    if (acc) {
      if (submit_ns)
        for (uint32_t i = k; i < k + acc; i++) submit_ns[i] = t_call;
      k += acc;
      n_sub.store(k, std::memory_order_release);
    }
    if (rc == INSPIRE_ERR_BUSY) {
      std::this_thread::yield();
      continue;
    }
    if (rc != INSPIRE_OK) {
      submit_err = g_last_error;
      submit_rc = rc;
      break;
    }
  }
  submit_end.store(true, std::memory_order_release);
  collector.join();
  if (submit_rc != INSPIRE_OK) return fail(submit_rc, "drive: " + submit_err);
  const int final_rc = stop_rc.load();
  if (final_rc != INSPIRE_OK) return fail(final_rc, "drive: " + collector_err);
  return INSPIRE_OK;
}

int inspire_server_get_stats(inspire_server* s, inspire_server_stats* out) {
  if (!s || !out) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null argument");
  std::lock_guard<std::mutex> lk(s->mu);
  out->submitted = s->n_submitted;
  out->completed = s->n_completed;
  out->batches = s->n_batches;
  out->pending = (uint32_t)s->pending.size();
  uint32_t busy = 0;
  for (const auto& sl : s->slots) busy += sl->busy;
  out->inflight_batches = busy;
  out->streams = (uint32_t)s->slots.size();
  return INSPIRE_OK;
}

}  // extern "C"
