// host.h -- host-side objects shared by the C ABI translation units
// (capi.cu, serve.cu): error reporting, device buffers, and the context and
// database handles.  Internal; not part of the public header.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "inspire_gpu.h"
#include "kernels.h"
#include "ledger.h"

namespace ighost {

using namespace ig;

inline thread_local std::string g_last_error;

inline int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

#define CUDA_TRY(expr)                                                                    \
  do {                                                                                    \
    cudaError_t _e = (expr);                                                              \
    if (_e != cudaSuccess)                                                                \
      return fail(_e == cudaErrorMemoryAllocation ? INSPIRE_ERR_OUT_OF_MEMORY : INSPIRE_ERR_CUDA, \
                  std::string(#expr) + ": " + cudaGetErrorString(_e));                   \
  } while (0)

// A device buffer that grows on demand.  Bound to a context's ledger, its
// bytes are reserved there before cudaMalloc (a refused reservation returns
// cudaErrorMemoryAllocation without allocating) and returned on release.
struct DevMem {
  void* p = nullptr;
  size_t bytes = 0;
  std::shared_ptr<Ledger> ledger;
  DevMem() = default;
  explicit DevMem(std::shared_ptr<Ledger> l) : ledger(std::move(l)) {}
  DevMem(const DevMem&) = delete;
  DevMem& operator=(const DevMem&) = delete;
  ~DevMem() { release(); }
  void release() {
    if (p) {
      cudaFree(p);
      if (ledger) ledger->release(bytes);
    }
    p = nullptr;
    bytes = 0;
  }
  cudaError_t ensure(size_t want) {
    if (want <= bytes) return cudaSuccess;
    release();
    if (ledger && !ledger->reserve(want)) return cudaErrorMemoryAllocation;
    cudaError_t e = cudaMalloc(&p, want);
    if (e == cudaSuccess) {
      bytes = want;
    } else {
      p = nullptr;
      if (ledger) ledger->release(want);
    }
    return e;
  }
  template <class T>
  T* as() const {
    return static_cast<T*>(p);
  }
};

}  // namespace ighost

namespace ighost {
// Page-locked, device-mapped host memory of at least `bytes` (grown on
// demand, contents not kept): the host-buffer calls' descriptors and status
// words, which the GPU reads by DMA and writes in place.
struct HostPinned {
  void* p = nullptr;  // host address
  void* d = nullptr;  // device address of the same memory
  size_t bytes = 0;
  cudaError_t ensure(size_t n) {
    if (n <= bytes) return cudaSuccess;
    release();
    cudaError_t e = cudaHostAlloc(&p, n, cudaHostAllocMapped | cudaHostAllocPortable);
    if (e != cudaSuccess) {
      p = nullptr;
      return e;
    }
    e = cudaHostGetDevicePointer(&d, p, 0);
    if (e != cudaSuccess) {
      cudaFreeHost(p);
      p = d = nullptr;
      return e;
    }
    bytes = n;
    return cudaSuccess;
  }
  void release() {
    if (p) cudaFreeHost(p);
    p = d = nullptr;
    bytes = 0;
  }
  template <class T>
  T* host() const {
    return static_cast<T*>(p);
  }
  template <class T>
  T* dev() const {
    return static_cast<T*>(d);
  }
  HostPinned() = default;
  HostPinned(const HostPinned&) = delete;
  HostPinned& operator=(const HostPinned&) = delete;
  ~HostPinned() { release(); }
};
}  // namespace ighost

struct inspire_ctx {
  std::mutex mu;
  // device-memory accounting of everything this context allocates
  std::shared_ptr<ighost::Ledger> ledger = std::make_shared<ighost::Ledger>();
  int device = 0;
  int mode = 0;
  int sm_count = 0;
  // batches of at most this many queries run on the two-CTA cluster kernel
  // (one SM per CRT residue; lower latency while the SMs are not all busy)
  std::atomic<int> pair_max{0};  // read by serving dispatchers without the lock
  inspire_params params{};
  uint64_t q = 0;  // composite modulus
  ig::DevParams P{};
  ighost::DevMem tables;
  // CRS
  bool has_crs = false;
  int gamma = 0;
  uint8_t w_seed[32] = {};
  uint64_t crs_a_count = 0;  // crs_a_vectors in the loaded crs.json
  ighost::DevMem what;   // rotated w_mask table (setup's precomputation reads it as is)
  ighost::DevMem what3;  // the same with the third gadget digit folded in (the Respond kernel's)
  ighost::DevMem wmask;  // [ELL][2][N] w_mask residues (client key generation)
  // tree packing: the CRS's Galois key table, the tree's work area and output
  bool has_galois = false;
  ighost::DevMem galois, tree_work, d_tree_out;
  // clients
  std::vector<ighost::DevMem*> clients;
  std::vector<const uint32_t*> client_ptrs;
  ighost::DevMem client_table;  // device copy of client_ptrs
  bool client_table_dirty = true;
  // client slot of the key table that queries carrying their own keys
  // (respond_*_inspiring) rebuild on every call, or -1
  int32_t inline_id = -1;
  // staging for host-buffer calls
  cudaStream_t stream = nullptr;
  ighost::DevMem d_shard, d_seeds, d_arows, d_brows, d_client, d_out, d_cols, d_status, d_keys, d_desc;
  std::vector<int32_t> h_status;
  ighost::HostPinned h_desc;    // descriptors of page-locked batch calls
  ighost::HostPinned h_qstatus; // status words of the batch calls, written by the kernel
  ighost::HostPinned h_stage;   // small batches' inputs, gathered for one DMA each
  ighost::HostPinned h_keys;    // client keys on their way to d_keys
  ighost::HostPinned h_out;     // responses of staged small batches, written by the kernel
  cudaEvent_t keys_ev = nullptr;  // recorded after the copy out of h_keys

  inspire_ctx() {
    for (ighost::DevMem* m : {&tables, &what, &what3, &wmask, &galois, &tree_work, &d_tree_out, &client_table, &d_shard,
                              &d_seeds, &d_arows, &d_brows, &d_client, &d_out, &d_cols, &d_status, &d_keys, &d_desc})
      m->ledger = ledger;
  }
  ~inspire_ctx() {
    for (ighost::DevMem* m : clients) delete m;
    if (keys_ev) cudaEventDestroy(keys_ev);
    if (stream) cudaStreamDestroy(stream);
  }
};

struct inspire_db {
  inspire_ctx* ctx = nullptr;  // never dereferenced after creation
  int device = 0;
  int gamma = 0;
  uint64_t n_entries = 0;
  uint32_t entry_size = 0;
  int nshards = 0;
  ighost::DevMem H, E;
};

namespace ighost {

inline size_t poly_words() { return (size_t)2 * N; }

// dbio.cu: a resident database from host raw columns [nshards][gamma][N].
// Device address of a page-locked host range [p, p + bytes) (cudaHostAlloc
// or cudaHostRegister memory, one mapping), or null for any other memory.
const uint8_t* mapped_range(const void* p, size_t bytes);
int db_from_host_columns(inspire_ctx* c, const uint16_t* Hh, int nshards, uint64_t n_entries, uint32_t entry_size,
                         inspire_db** out);

inline int sync_client_table(inspire_ctx* c) {
  if (!c->client_table_dirty) return INSPIRE_OK;
  // grown in steps of 256 entries: a reallocation (which waits for the
  // device) is rare while a serving loop has batches in flight
  const size_t bytes = sizeof(uint32_t*) * ((c->client_ptrs.size() + 256) & ~(size_t)255);
  CUDA_TRY(c->client_table.ensure(bytes));
  if (!c->client_ptrs.empty())
    CUDA_TRY(cudaMemcpy(c->client_table.p, c->client_ptrs.data(), sizeof(uint32_t*) * c->client_ptrs.size(),
                        cudaMemcpyHostToDevice));
  c->client_table_dirty = false;
  return INSPIRE_OK;
}

// Text of a refused or failed device allocation of `what`.
inline std::string alloc_failure(const inspire_ctx* c, const std::string& what) {
  const uint64_t budget = c->ledger->budget();
  if (!budget) return what + ": device out of memory";
  return what + ": does not fit the device budget (" + std::to_string(c->ledger->used()) + " of " +
         std::to_string(budget) + " bytes in use) or the device is out of memory";
}

inline int set_device(inspire_ctx* c) {
  CUDA_TRY(cudaSetDevice(c->device));
  return INSPIRE_OK;
}

}  // namespace ighost
