// capi.cu -- host side of the C ABI declared in include/inspire_gpu.h.
//
// Builds the per-context constants (the reference NttContext's psi and
// twiddles, CRT and Montgomery factors), owns the resident device objects
// (database, CRS key table, client key tables) and stages batched queries.
// Nothing here computes a response: every Respond result comes from the
// kernels in respond.cu.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "host.h"

using u128 = unsigned __int128;
using namespace ig;
using namespace ighost;

namespace {

uint64_t powmod(uint64_t b, uint64_t e, uint64_t m) {
  uint64_t r = 1;
  b %= m;
  while (e) {
    if (e & 1) r = (uint64_t)((u128)r * b % m);
    b = (uint64_t)((u128)b * b % m);
    e >>= 1;
  }
  return r;
}

uint64_t inv_prime(uint64_t a, uint64_t q) { return powmod(a % q, q - 2, q); }

uint32_t shoup(uint64_t w, uint64_t q) { return (uint32_t)(((u128)w << 32) / q); }

uint32_t brv(uint32_t x, int bits) {
  uint32_t r = 0;
  for (int i = 0; i < bits; i++) r |= ((x >> i) & 1u) << (bits - 1 - i);
  return r;
}

bool is_prime(uint64_t q) {
  if (q < 2) return false;
  for (uint64_t d = 2; d * d <= q; d++)
    if (q % d == 0) return false;
  return true;
}

// NttContext::find_primitive_root (src/math/ntt.rs:525-538)
uint64_t find_psi(uint64_t two_n, uint64_t q) {
  const uint64_t e = (q - 1) / two_n;
  for (uint64_t g = 2; g < q; g++) {
    uint64_t c = powmod(g, e, q);
    if (powmod(c, two_n, q) == 1 && powmod(c, two_n / 2, q) != 1) return c;
  }
  return 0;
}

// ChaCha20Rng::from_seed + next_u64 for generate_mask_from_seed
// (src/inspiring/inspiring2.rs:816-835), host side.
struct HostChaCha {
  uint32_t key[8];
  uint64_t ctr = 0;
  uint32_t buf[16];
  int idx = 16;
  explicit HostChaCha(const uint8_t seed[32]) {
    for (int i = 0; i < 8; i++)
      key[i] = (uint32_t)seed[4 * i] | ((uint32_t)seed[4 * i + 1] << 8) | ((uint32_t)seed[4 * i + 2] << 16) |
               ((uint32_t)seed[4 * i + 3] << 24);
  }
  static uint32_t rotl(uint32_t x, int k) { return (x << k) | (x >> (32 - k)); }
  void block() {
    uint32_t s[16] = {0x61707865u, 0x3320646eu, 0x79622d32u, 0x6b206574u};
    for (int i = 0; i < 8; i++) s[4 + i] = key[i];
    s[12] = (uint32_t)ctr;
    s[13] = (uint32_t)(ctr >> 32);
    s[14] = s[15] = 0;
    uint32_t x[16];
    memcpy(x, s, sizeof x);
    auto qr = [](uint32_t& a, uint32_t& b, uint32_t& c, uint32_t& d) {
      a += b; d ^= a; d = rotl(d, 16);
      c += d; b ^= c; b = rotl(b, 12);
      a += b; d ^= a; d = rotl(d, 8);
      c += d; b ^= c; b = rotl(b, 7);
    };
    for (int i = 0; i < 10; i++) {
      qr(x[0], x[4], x[8], x[12]);
      qr(x[1], x[5], x[9], x[13]);
      qr(x[2], x[6], x[10], x[14]);
      qr(x[3], x[7], x[11], x[15]);
      qr(x[0], x[5], x[10], x[15]);
      qr(x[1], x[6], x[11], x[12]);
      qr(x[2], x[7], x[8], x[13]);
      qr(x[3], x[4], x[9], x[14]);
    }
    for (int i = 0; i < 16; i++) buf[i] = x[i] + s[i];
    ctr++;
    idx = 0;
  }
  uint32_t next_u32() {
    if (idx >= 16) block();
    return buf[idx++];
  }
  uint64_t next_u64() {
    uint64_t lo = next_u32();
    uint64_t hi = next_u32();
    return lo | (hi << 32);
  }
};

}  // namespace

namespace {

// Build the client key table into m from y_body or y_all.  From y_body at
// gamma = 16 the table holds NTT(y_body) only (48 KiB, the Respond kernel
// forms each rotation in registers); from an explicit y_all, or at smaller
// gamma, all (gamma-1)*ELL rotated polys.  sync: wait for the build here
// (otherwise the launches that use the table follow on the same stream).
int build_key_table(inspire_ctx* c, const uint64_t* y_body, const uint64_t* y_all, DevMem& m, bool& body_form,
                    bool sync) {
  const int gamma = c->gamma;
  body_form = !y_all && gamma == MAX_GAMMA;
  const size_t tbl_words = (size_t)std::max(1, body_form ? ELL : (gamma - 1) * ELL) * poly_words();
  if (m.ensure(tbl_words * sizeof(uint32_t)) != cudaSuccess)
    return fail(INSPIRE_ERR_OUT_OF_MEMORY, alloc_failure(c, "client key table allocation"));
  const size_t in_polys = y_all ? (size_t)(gamma - 1) * ELL : ELL;
  if (gamma > 1) {
    const size_t in_bytes = in_polys * poly_words() * sizeof(uint64_t);
    if (c->d_keys.ensure(in_bytes) != cudaSuccess)
      return fail(INSPIRE_ERR_OUT_OF_MEMORY, alloc_failure(c, "client key upload buffer"));
    // through page-locked memory (one DMA), once the previous upload is out of it
    if (!c->keys_ev) CUDA_TRY(cudaEventCreateWithFlags(&c->keys_ev, cudaEventDisableTiming));
    CUDA_TRY(cudaEventSynchronize(c->keys_ev));
    CUDA_TRY(c->h_keys.ensure(in_bytes));
    memcpy(c->h_keys.p, y_all ? y_all : y_body, in_bytes);
    CUDA_TRY(cudaMemcpyAsync(c->d_keys.p, c->h_keys.p, in_bytes, cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(cudaEventRecord(c->keys_ev, c->stream));
    CUDA_TRY(y_all ? launch_client_from_yall(c->P, c->d_keys.as<uint64_t>(), m.as<uint32_t>(), c->stream)
                   : launch_client_from_ybody(c->P, c->d_keys.as<uint64_t>(), m.as<uint32_t>(),
                                              body_form ? 1 : gamma - 1, c->stream));
    // the Respond kernel multiplies the third key by R_{i+1} instead of NTT(d2)
    CUDA_TRY(launch_fold_third_digit(c->P, m.as<uint32_t>(), body_form ? 1 : gamma - 1, c->stream));
    if (sync) CUDA_TRY(cudaStreamSynchronize(c->stream));
  }
  return INSPIRE_OK;
}

// The device table entry of a key table: bit 0 marks a body table
// (allocations are 256-byte aligned).
const uint32_t* table_entry(const DevMem& m, bool body_form) {
  return reinterpret_cast<const uint32_t*>(reinterpret_cast<uintptr_t>(m.as<uint32_t>()) | (body_form ? 1u : 0u));
}

int32_t free_client_slot(inspire_ctx* c) {
  for (size_t i = 0; i < c->clients.size(); i++)
    if (!c->clients[i]) return (int32_t)i;
  c->clients.push_back(nullptr);
  c->client_ptrs.push_back(nullptr);
  return (int32_t)c->clients.size() - 1;
}

int register_keys(inspire_ctx* c, const uint64_t* y_body, const uint64_t* y_all, int32_t* id) {
  if (!y_body && !y_all)
    return fail(INSPIRE_ERR_KEYS_INVALID, "InspiRING packing keys invalid: y_all and y_body are both empty");
  std::unique_ptr<DevMem> m(new DevMem(c->ledger));  // freed (bytes returned) on every error path
  bool body_form = false;
  if (int rc = build_key_table(c, y_body, y_all, *m, body_form, true)) return rc;
  const int32_t slot = free_client_slot(c);
  c->clients[slot] = m.release();
  c->client_ptrs[slot] = table_entry(*c->clients[slot], body_form);
  c->client_table_dirty = true;
  *id = slot;
  return INSPIRE_OK;
}

// The keys a query carries (respond_*_inspiring): rebuilt on every call, as
// the crate derives them per request, into one table the context keeps for
// these calls (no allocation per call; the call's own launches follow the
// build on the context's stream, and the call waits for them).
int inline_keys(inspire_ctx* c, const uint64_t* y_body, const uint64_t* y_all, int32_t* id) {
  if (!y_body && !y_all)
    return fail(INSPIRE_ERR_KEYS_INVALID, "InspiRING packing keys invalid: y_all and y_body are both empty");
  if (c->inline_id < 0) {
    const int32_t slot = free_client_slot(c);
    c->clients[slot] = new DevMem(c->ledger);
    c->inline_id = slot;
  }
  DevMem& m = *c->clients[c->inline_id];
  bool body_form = false;
  if (int rc = build_key_table(c, y_body, y_all, m, body_form, false)) return rc;
  const uint32_t* entry = table_entry(m, body_form);
  if (c->client_ptrs[c->inline_id] != entry) {
    c->client_ptrs[c->inline_id] = entry;
    c->client_table_dirty = true;
  }
  *id = c->inline_id;
  return INSPIRE_OK;
}

void release_keys(inspire_ctx* c, int32_t id) {
  if (id < 0 || (size_t)id >= c->clients.size() || !c->clients[id]) return;
  delete c->clients[id];
  c->clients[id] = nullptr;
  c->client_ptrs[id] = nullptr;
  c->client_table_dirty = true;
  if (id == c->inline_id) c->inline_id = -1;
}

int finish_status(inspire_ctx* c, uint32_t n, const char* what);

// Batches up to this size stage their inputs through page-locked memory.
constexpr uint32_t STAGE_PINNED_MAX = 64;

// Seeded queries whose rows and responses are in page-locked host memory
// (device addresses d_rows, row_bytes apart, and d_out): the serving variant
// of the kernel reads each query's rows in place and writes its response
// straight to that memory, so nothing is staged or copied back.
int run_batch_mapped(inspire_ctx* c, const inspire_db* db, uint32_t n, const uint32_t* shard_ids, const uint8_t* seeds,
                     size_t seed_stride, const uint8_t* d_rows, size_t row_bytes, uint64_t* d_out,
                     const int32_t* client_ids) {
  const size_t pw = poly_words();
  // descriptors and status words in page-locked memory: the descriptors go
  // over by DMA, the kernel writes each status word in place
  CUDA_TRY(c->d_desc.ensure(sizeof(QueryDesc) * n));
  CUDA_TRY(c->h_desc.ensure(sizeof(QueryDesc) * n));
  CUDA_TRY(c->h_qstatus.ensure(sizeof(int32_t) * n));
  QueryDesc* hd = c->h_desc.host<QueryDesc>();
  int32_t* hs = c->h_qstatus.host<int32_t>();
  const DbView view{db->E.as<uint32_t>(), db->H.as<uint16_t>(), db->nshards, 0};
  for (uint32_t i = 0; i < n; i++) {
    QueryDesc& d = hd[i];
    memcpy(d.seeds, seeds + i * seed_stride, sizeof(d.seeds));
    d.brows = reinterpret_cast<const uint64_t*>(d_rows + i * row_bytes);
    d.out = d_out + (size_t)i * 2 * pw;
    d.status = c->h_qstatus.dev<int32_t>() + i;
    d.db = view;
    d.shard = shard_ids[i];
    d.client = client_ids[i];
    hs[i] = -1;
  }
  CUDA_TRY(cudaMemcpyAsync(c->d_desc.p, hd, sizeof(QueryDesc) * n, cudaMemcpyHostToDevice, c->stream));
  if (int rc = sync_client_table(c)) return rc;
  RespondArgs a{};
  a.P = c->P;
  a.nq = (int)n;
  a.yhat_table = c->client_table.as<const uint32_t*>();
  a.nclients = (int)c->client_ptrs.size();
  a.what = c->what3.as<uint32_t>();
  a.qdesc = c->d_desc.as<QueryDesc>();
  a.stage_wait_iters = STAGE_WAIT_ITERS_DEFAULT;
  CUDA_TRY(launch_respond(a, true, c->stream, 0, c->pair_max.load()));
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  for (uint32_t i = 0; i < n; i++)
    if (hs[i] != 0)
      return fail(INSPIRE_ERR_DEVICE_STATUS,
                  "respond kernel status " + std::to_string(hs[i]) + " for query " + std::to_string(i));
  return INSPIRE_OK;
}

// Stage n queries (rows ELL..2ELL-1 only) and run the Respond kernel.
// seeds/b_rows/a_rows use the full 2*ELL-row host layout.
// a_rows/b_rows point at the first needed poly of query 0 (ELL contiguous
// polys per query, query pitch `stride_polys`); seeds at the first needed seed
// (ELL contiguous seeds, query pitch `seed_stride` bytes).
int run_batch(inspire_ctx* c, const inspire_db* db, uint32_t n, const uint32_t* shard_ids, const uint8_t* seeds,
              size_t seed_stride, const uint64_t* a_rows, const uint64_t* b_rows, size_t stride_polys,
              const int32_t* client_ids, uint64_t* out_ct) {
  if (n == 0) return INSPIRE_OK;
  const size_t pw = poly_words();
  if (seeds) {
    // page-locked rows and responses (16-byte aligned): read and written in place
    const size_t row_bytes = sizeof(uint64_t) * stride_polys * pw;
    const size_t rows_span = row_bytes * (n - 1) + sizeof(uint64_t) * ELL * pw;
    const size_t out_span = sizeof(uint64_t) * n * 2 * pw;
    const uint8_t* d_rows = ((uintptr_t)b_rows % 16 == 0 && row_bytes % 16 == 0 && (uintptr_t)out_ct % 16 == 0)
                                ? mapped_range(b_rows, rows_span)
                                : nullptr;
    const uint8_t* d_outp = d_rows ? mapped_range(out_ct, out_span) : nullptr;
    if (d_rows && d_outp)
      return run_batch_mapped(c, db, n, shard_ids, seeds, seed_stride, d_rows, row_bytes,
                              const_cast<uint64_t*>(reinterpret_cast<const uint64_t*>(d_outp)), client_ids);
    if (n <= STAGE_PINNED_MAX) {
      // small batches in other memory: the rows gathered into page-locked
      // memory and read there in place, the responses written to page-locked
      // memory and copied out once (no copies to and from the device)
      const size_t rows_b = sizeof(uint64_t) * ELL * pw;
      CUDA_TRY(c->h_stage.ensure(rows_b * n));
      CUDA_TRY(c->h_out.ensure(out_span));
      uint8_t* hb = c->h_stage.host<uint8_t>();
      for (uint32_t i = 0; i < n; i++) memcpy(hb + rows_b * i, b_rows + i * stride_polys * pw, rows_b);
      if (int rc = run_batch_mapped(c, db, n, shard_ids, seeds, seed_stride, c->h_stage.dev<uint8_t>(), rows_b,
                                    c->h_out.dev<uint64_t>(), client_ids))
        return rc;
      memcpy(out_ct, c->h_out.host<uint64_t>(), out_span);
      return INSPIRE_OK;
    }
  }
  CUDA_TRY(c->d_shard.ensure(sizeof(uint32_t) * n));
  CUDA_TRY(c->d_client.ensure(sizeof(int32_t) * n));
  CUDA_TRY(c->d_brows.ensure(sizeof(uint64_t) * n * ELL * pw));
  CUDA_TRY(c->d_out.ensure(sizeof(uint64_t) * n * 2 * pw));
  const bool seeded = seeds != nullptr;
  const size_t rows_b = sizeof(uint64_t) * ELL * pw;  // rows ELL..2ELL-1 of one query, b (or a) polys
  if (seeded) CUDA_TRY(c->d_seeds.ensure((size_t)32 * ELL * n));
  else CUDA_TRY(c->d_arows.ensure(rows_b * n));
  CUDA_TRY(c->h_qstatus.ensure(sizeof(int32_t) * n));
  if (n <= STAGE_PINNED_MAX) {
    // small batches: the inputs are gathered into page-locked memory on the
    // host and go over by DMA without the driver's staging of pageable
    // copies; the kernel writes the status words in place
    const size_t a_b = seeded ? (size_t)32 * ELL * n : rows_b * n;
    CUDA_TRY(c->h_stage.ensure(rows_b * n + a_b + sizeof(uint32_t) * 2 * n));
    uint8_t* hb = c->h_stage.host<uint8_t>();
    uint8_t* ha = hb + rows_b * n;
    uint32_t* hsid = reinterpret_cast<uint32_t*>(ha + a_b);
    int32_t* hcid = reinterpret_cast<int32_t*>(hsid + n);
    for (uint32_t i = 0; i < n; i++) {
      memcpy(hb + rows_b * i, b_rows + i * stride_polys * pw, rows_b);
      if (seeded) memcpy(ha + (size_t)32 * ELL * i, seeds + i * seed_stride, (size_t)32 * ELL);
      else memcpy(ha + rows_b * i, a_rows + i * stride_polys * pw, rows_b);
      hsid[i] = shard_ids[i];
      hcid[i] = client_ids[i];
    }
    CUDA_TRY(cudaMemcpyAsync(c->d_brows.p, hb, rows_b * n, cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(cudaMemcpyAsync(seeded ? c->d_seeds.p : c->d_arows.p, ha, a_b, cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(cudaMemcpyAsync(c->d_shard.p, hsid, sizeof(uint32_t) * n, cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(cudaMemcpyAsync(c->d_client.p, hcid, sizeof(int32_t) * n, cudaMemcpyHostToDevice, c->stream));
  } else {
    CUDA_TRY(cudaMemcpyAsync(c->d_shard.p, shard_ids, sizeof(uint32_t) * n, cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(cudaMemcpyAsync(c->d_client.p, client_ids, sizeof(int32_t) * n, cudaMemcpyHostToDevice, c->stream));
    // b rows ELL..2ELL-1 of each query: one strided copy
    CUDA_TRY(cudaMemcpy2DAsync(c->d_brows.p, rows_b, b_rows, sizeof(uint64_t) * stride_polys * pw, rows_b, n,
                               cudaMemcpyHostToDevice, c->stream));
    if (seeded)
      CUDA_TRY(cudaMemcpy2DAsync(c->d_seeds.p, (size_t)32 * ELL, seeds, seed_stride, (size_t)32 * ELL, n,
                                 cudaMemcpyHostToDevice, c->stream));
    else
      CUDA_TRY(cudaMemcpy2DAsync(c->d_arows.p, rows_b, a_rows, sizeof(uint64_t) * stride_polys * pw, rows_b, n,
                                 cudaMemcpyHostToDevice, c->stream));
  }
  int rc = sync_client_table(c);
  if (rc) return rc;
  RespondArgs a{};
  a.P = c->P;
  a.nq = (int)n;
  a.shard = c->d_shard.as<uint32_t>();
  a.seeds = seeded ? c->d_seeds.as<uint8_t>() : nullptr;
  a.arows = seeded ? nullptr : c->d_arows.as<uint64_t>();
  a.brows = c->d_brows.as<uint64_t>();
  a.client = c->d_client.as<int32_t>();
  a.yhat_table = c->client_table.as<const uint32_t*>();
  a.nclients = (int)c->client_ptrs.size();
  a.nshards = db->nshards;
  a.E = db->E.as<uint32_t>();
  a.H = db->H.as<uint16_t>();
  a.what = c->what3.as<uint32_t>();
  a.out = c->d_out.as<uint64_t>();
  int32_t* hs = c->h_qstatus.host<int32_t>();
  for (uint32_t i = 0; i < n; i++) hs[i] = -1;
  a.status = c->h_qstatus.dev<int32_t>();
  CUDA_TRY(launch_respond(a, seeded, c->stream, 0, c->pair_max.load()));
  CUDA_TRY(cudaMemcpyAsync(out_ct, c->d_out.p, sizeof(uint64_t) * n * 2 * pw, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  for (uint32_t i = 0; i < n; i++)
    if (hs[i] != 0)
      return fail(INSPIRE_ERR_DEVICE_STATUS,
                  "respond kernel status " + std::to_string(hs[i]) + " for query " + std::to_string(i));
  return INSPIRE_OK;
}

// CTAs per query of the NoPacking kernel.  Few queries with column
// ciphertexts: each query's columns are split over CTAs (each expands the
// rows itself) so that a small batch fills the SMs; the combined
// ciphertexts are then summed from the columns.
int column_groups(const inspire_ctx* c, const inspire_db* db, uint32_t n, bool columns) {
  if (!columns || db->gamma <= 1 || n == 0) return 1;
  const int want = std::min(db->gamma, std::max(1, c->sm_count / (int)std::min<uint32_t>(n, 1u << 20)));
  const int per = (db->gamma + want - 1) / want;
  return (db->gamma + per - 1) / per;
}

// Stage n NoPacking queries (same row layout as run_batch) and run the
// NoPacking kernel; out_columns may be null.
// Stage n queries' rows and enqueue the NoPacking kernel on the context's
// stream: combined ciphertexts into d_out, and (columns) every column
// ciphertext into d_cols.
int enqueue_nopacking(inspire_ctx* c, const inspire_db* db, uint32_t n, const uint32_t* shard_ids,
                      const uint8_t* seeds, size_t seed_stride, const uint64_t* a_rows, const uint64_t* b_rows,
                      size_t stride_polys, bool columns) {
  const size_t pw = poly_words();
  const size_t col_words = (size_t)db->gamma * 2 * pw;
  CUDA_TRY(c->d_shard.ensure(sizeof(uint32_t) * n));
  CUDA_TRY(c->d_brows.ensure(sizeof(uint64_t) * n * ELL * pw));
  CUDA_TRY(c->d_out.ensure(sizeof(uint64_t) * n * 2 * pw));
  if (columns) CUDA_TRY(c->d_cols.ensure(sizeof(uint64_t) * n * col_words));
  CUDA_TRY(c->d_status.ensure(sizeof(int32_t) * n));
  CUDA_TRY(cudaMemcpyAsync(c->d_shard.p, shard_ids, sizeof(uint32_t) * n, cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(cudaMemcpy2DAsync(c->d_brows.p, sizeof(uint64_t) * ELL * pw, b_rows, sizeof(uint64_t) * stride_polys * pw,
                             sizeof(uint64_t) * ELL * pw, n, cudaMemcpyHostToDevice, c->stream));
  const bool seeded = seeds != nullptr;
  if (seeded) {
    CUDA_TRY(c->d_seeds.ensure((size_t)32 * ELL * n));
    CUDA_TRY(cudaMemcpy2DAsync(c->d_seeds.p, (size_t)32 * ELL, seeds, seed_stride, (size_t)32 * ELL, n,
                               cudaMemcpyHostToDevice, c->stream));
  } else {
    CUDA_TRY(c->d_arows.ensure(sizeof(uint64_t) * n * ELL * pw));
    CUDA_TRY(cudaMemcpy2DAsync(c->d_arows.p, sizeof(uint64_t) * ELL * pw, a_rows, sizeof(uint64_t) * stride_polys * pw,
                               sizeof(uint64_t) * ELL * pw, n, cudaMemcpyHostToDevice, c->stream));
  }
  NoPackingArgs a{};
  a.P = c->P;
  a.nq = (int)n;
  a.col_groups = column_groups(c, db, n, columns);
  a.shard = c->d_shard.as<uint32_t>();
  a.seeds = seeded ? c->d_seeds.as<uint8_t>() : nullptr;
  a.arows = seeded ? nullptr : c->d_arows.as<uint64_t>();
  a.brows = c->d_brows.as<uint64_t>();
  a.nshards = db->nshards;
  a.H = db->H.as<uint16_t>();
  a.out = c->d_out.as<uint64_t>();
  a.out_columns = columns ? c->d_cols.as<uint64_t>() : nullptr;
  a.status = c->d_status.as<int>();
  CUDA_TRY(launch_nopacking(a, seeded, c->stream));
  return INSPIRE_OK;
}

// Copy the n query statuses back, wait for the stream, and turn a nonzero
// status into an error.
int finish_status(inspire_ctx* c, uint32_t n, const char* what) {
  c->h_status.resize(n);
  CUDA_TRY(cudaMemcpyAsync(c->h_status.data(), c->d_status.p, sizeof(int32_t) * n, cudaMemcpyDeviceToHost,
                           c->stream));
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  for (uint32_t i = 0; i < n; i++)
    if (c->h_status[i] != 0)
      return fail(INSPIRE_ERR_DEVICE_STATUS,
                  std::string(what) + " kernel status " + std::to_string(c->h_status[i]) + " for query " +
                      std::to_string(i));
  return INSPIRE_OK;
}

int run_nopacking(inspire_ctx* c, const inspire_db* db, uint32_t n, const uint32_t* shard_ids, const uint8_t* seeds,
                  size_t seed_stride, const uint64_t* a_rows, const uint64_t* b_rows, size_t stride_polys,
                  uint64_t* out_ct, uint64_t* out_columns) {
  if (n == 0) return INSPIRE_OK;
  const size_t pw = poly_words();
  const size_t col_words = (size_t)db->gamma * 2 * pw;
  if (int rc = enqueue_nopacking(c, db, n, shard_ids, seeds, seed_stride, a_rows, b_rows, stride_polys,
                                 out_columns != nullptr))
    return rc;
  CUDA_TRY(cudaMemcpyAsync(out_ct, c->d_out.p, sizeof(uint64_t) * n * 2 * pw, cudaMemcpyDeviceToHost, c->stream));
  if (out_columns)
    CUDA_TRY(cudaMemcpyAsync(out_columns, c->d_cols.p, sizeof(uint64_t) * n * col_words, cudaMemcpyDeviceToHost,
                             c->stream));
  return finish_status(c, n, "nopacking");
}

// respond_one_packing (src/pir/respond.rs:213-268) of n queries: column
// products on the GPU (the NoPacking kernel, columns kept on the device),
// then pack_lwes with the CRS's Galois keys (tree.cu).  Query i's packed a
// goes to out_a[i] (one poly) and its b to out_b[i] (room for two polys):
// *b_words words, one poly, or two in compat mode (the crate's
// dimension-2d b polynomial).
int run_tree(inspire_ctx* c, const inspire_db* db, uint32_t n, const uint32_t* shard_ids, const uint8_t* seeds,
             size_t seed_stride, const uint64_t* a_rows, const uint64_t* b_rows, size_t stride_polys, uint64_t* out_a,
             uint64_t* out_b, uint32_t* b_words) {
  const size_t pw = poly_words();
  if (!c->has_galois) return fail(INSPIRE_ERR_NO_CRS, "no Galois keys loaded (inspire_crs_load_galois_keys)");
  const uint32_t words = (c->mode == MODE_COMPAT && db->gamma > 1) ? (uint32_t)(2 * pw) : (uint32_t)pw;
  *b_words = words;
  if (n == 0) return INSPIRE_OK;
  if (int rc = enqueue_nopacking(c, db, n, shard_ids, seeds, seed_stride, a_rows, b_rows, stride_polys, true))
    return rc;
  CUDA_TRY(c->tree_work.ensure(sizeof(uint32_t) * tree_work_words_per_query() * n));
  CUDA_TRY(c->d_tree_out.ensure(sizeof(uint64_t) * 3 * pw * n));
  TreeArgs t{};
  t.P = c->P;
  t.nq = (int)n;
  t.ncols = db->gamma;
  t.mode = c->mode;
  t.cols = c->d_cols.as<uint64_t>();
  t.ks = c->galois.as<uint32_t>();
  t.work = c->tree_work.as<uint32_t>();
  t.out_a = c->d_tree_out.as<uint64_t>();
  t.out_b = t.out_a + pw * n;
  CUDA_TRY(launch_pack_tree(t, c->stream));
  CUDA_TRY(cudaMemcpyAsync(out_a, t.out_a, sizeof(uint64_t) * pw * n, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(cudaMemcpyAsync(out_b, t.out_b, sizeof(uint64_t) * 2 * pw * n, cudaMemcpyDeviceToHost, c->stream));
  return finish_status(c, n, "nopacking");
}

// Validation order of respond_inspiring (src/pir/respond.rs:295-305, 365-370).
int single_query(inspire_ctx* c, const inspire_db* db, uint32_t shard_id, const uint8_t* seeds,
                 const uint64_t* rgsw_full, const uint64_t* b_rows, int32_t has_keys, const uint64_t* y_body,
                 const uint64_t* y_all, uint64_t* out_ct) {
  if (!c || !db || !out_ct) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null argument");
  if (!c->has_crs) return fail(INSPIRE_ERR_NO_CRS, "no CRS loaded (inspire_crs_load)");
  if (!has_keys) return fail(INSPIRE_ERR_KEYS_MISSING, "InspiRING client packing keys missing from query");
  if (shard_id >= (uint32_t)db->nshards)
    return fail(INSPIRE_ERR_SHARD_NOT_FOUND, "Shard " + std::to_string(shard_id) + " not found");
  if (!y_all && !y_body)
    return fail(INSPIRE_ERR_KEYS_INVALID, "InspiRING packing keys invalid: y_all and y_body are both empty");
  int32_t id = -1;
  int rc = inline_keys(c, y_body, y_all, &id);
  if (rc) return rc;
  if (seeds) {
    rc = run_batch(c, db, 1, &shard_id, seeds + 32 * ELL, (size_t)64 * ELL, nullptr, b_rows + (size_t)ELL * poly_words(),
                   2 * ELL, &id, out_ct);
  } else {
    // rgsw_full holds 2*ELL rows of (a, b): row r's a is poly 2r, its b poly 2r+1
    const size_t pw = poly_words();
    std::vector<uint64_t> ar((size_t)ELL * pw), br((size_t)ELL * pw);
    for (int t = 0; t < ELL; t++) {
      memcpy(ar.data() + t * pw, rgsw_full + (size_t)(2 * (ELL + t)) * pw, pw * sizeof(uint64_t));
      memcpy(br.data() + t * pw, rgsw_full + (size_t)(2 * (ELL + t) + 1) * pw, pw * sizeof(uint64_t));
    }
    rc = run_batch(c, db, 1, &shard_id, nullptr, 0, ar.data(), br.data(), ELL, &id, out_ct);
  }
  return rc;
}

}  // namespace

extern "C" {

const char* inspire_last_error(void) { return g_last_error.c_str(); }

const char* inspire_version(void) { return "inspire-gb300 0.1.0 (sm_103a)"; }

void inspire_params_default(inspire_params* out) {
  if (!out) return;
  memset(out, 0, sizeof(*out));
  out->ring_dim = 2048;
  out->crt_count = 2;
  out->crt_moduli[0] = 268369921ULL;
  out->crt_moduli[1] = 249561089ULL;
  out->p = 1ULL << 16;
  out->sigma = 6.4;
  out->gadget_base = 1ULL << 20;
  out->gadget_len = 3;
}

int inspire_ctx_create(const inspire_params* prm, int device, int mode, inspire_ctx** out) {
  if (!prm || !out) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null argument");
  *out = nullptr;
  if (mode != INSPIRE_MODE_COMPAT && mode != INSPIRE_MODE_CRT_FIXED)
    return fail(INSPIRE_ERR_INVALID_ARGUMENT, "mode must be INSPIRE_MODE_COMPAT or INSPIRE_MODE_CRT_FIXED");
  // InspireParams::validate (params.rs:348-387) + the GPU path's envelope
  if (prm->ring_dim == 0 || (prm->ring_dim & (prm->ring_dim - 1)))
    return fail(INSPIRE_ERR_INVALID_ARGUMENT, "ring_dim must be a power of two");
  if (prm->crt_count != 2 || prm->ring_dim != (uint32_t)N || prm->gadget_base != (1ULL << ZBITS) ||
      prm->gadget_len != (uint32_t)ELL)
    return fail(INSPIRE_ERR_UNSUPPORTED,
                "GPU path supports ring_dim=2048, two CRT moduli, gadget_base=2^20, gadget_len=3");
  const uint64_t q0 = prm->crt_moduli[0], q1 = prm->crt_moduli[1];
  for (uint64_t qm : {q0, q1}) {
    if (qm % (2 * N) != 1) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "CRT moduli must be = 1 (mod 2d) for NTT");
    // below 2^28: the lazily reduced transforms keep values below 16 q_i < 2^32
    if (qm >= (1ULL << 28) || qm <= (1ULL << ZBITS) || !is_prime(qm))
      return fail(INSPIRE_ERR_UNSUPPORTED, "GPU path needs prime CRT moduli in (2^20, 2^28)");
  }
  if (q0 == q1) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "CRT moduli must be coprime");
  if (q0 >= 2 * q1) return fail(INSPIRE_ERR_UNSUPPORTED, "GPU path needs q0 < 2 q1");
  const uint64_t q = q0 * q1;
  if (q < prm->p || prm->p < 2) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "q must be >= p");
  // ceil(log2(q)/20) must be the gadget length (params.rs:224)
  if (q >= (1ULL << (ZBITS * ELL)) || q < (1ULL << (ZBITS * (ELL - 1))))
    return fail(INSPIRE_ERR_UNSUPPORTED, "gadget_len 3 does not cover q");

  inspire_ctx* c = new inspire_ctx();
  c->device = device;
  c->mode = mode;
  c->params = *prm;
  c->q = q;
  if (int rc = set_device(c)) {
    delete c;
    return rc;
  }
  cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete c;
    return fail(INSPIRE_ERR_CUDA, std::string("cudaStreamCreate: ") + cudaGetErrorString(e));
  }
  if (cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
      c->sm_count <= 0) {
    delete c;
    return fail(INSPIRE_ERR_CUDA, "cannot read the SM count");
  }
  c->pair_max.store(c->sm_count / 2);
  // tables per residue: fwd pairs (2N words), inv pairs (2N words), psi_pow (2N)
  const size_t per = 6 * (size_t)N;
  std::vector<uint32_t> host(2 * per);
  DevParams& P = c->P;
  memset(&P, 0, sizeof(P));
  for (int r = 0; r < 2; r++) {
    const uint64_t qm = prm->crt_moduli[r];
    uint32_t* t = host.data() + r * per;
    const uint64_t psi = find_psi(2 * N, qm), psi_inv = inv_prime(psi, qm);
    for (int k = 1; k < N; k++) {
      const uint64_t w = powmod(psi, brv(k, LOGN), qm), wi = powmod(psi_inv, brv(k, LOGN), qm);
      t[2 * k] = (uint32_t)w;
      t[2 * k + 1] = shoup(w, qm);
      t[2 * N + 2 * k] = (uint32_t)wi;
      t[2 * N + 2 * k + 1] = shoup(wi, qm);
    }
    uint64_t pw = 1;
    for (int k = 0; k < 2 * N; k++) {
      t[4 * N + k] = (uint32_t)pw;
      pw = (uint64_t)((u128)pw * psi % qm);
    }
    ResidueConsts& C = P.r[r];
    C.q = (uint32_t)qm;
    uint32_t inv = (uint32_t)qm;  // Newton: q^-1 mod 2^32
    for (int it = 0; it < 5; it++) inv *= 2u - (uint32_t)qm * inv;
    C.qinv = 0u - inv;
    const uint64_t r64 = (uint64_t)(((u128)1 << 64) % qm);
    const uint64_t r32 = (1ULL << 32) % qm;
    const uint64_t ninv = inv_prime(N, qm), r64inv = inv_prime(r64, qm);
    C.r64 = (uint32_t)r64;
    C.r64_p = shoup(r64, qm);
    const uint64_t ris = (uint64_t)((u128)ninv * r64inv % qm);
    C.ref_inv_scale = (uint32_t)ris;
    C.ref_inv_scale_p = shoup(ris, qm);
    const uint64_t nm = (uint64_t)((u128)ninv * r32 % qm);
    C.ninv_mont = (uint32_t)nm;
    C.ninv_mont_p = shoup(nm, qm);
    C.mont = (uint32_t)r32;
    C.mont_p = shoup(r32, qm);
    const uint64_t zinv = inv_prime((1ULL << ZBITS) % qm, qm), z2inv = (uint64_t)((u128)zinv * zinv % qm);
    const uint64_t nz2 = (uint64_t)((u128)N * z2inv % qm);
    C.d2_nz2 = (uint32_t)nz2;
    C.d2_nz2_p = shoup(nz2, qm);
    C.d2_z2 = (uint32_t)z2inv;
    C.d2_z2_p = shoup(z2inv, qm);
    C.d2_z1 = (uint32_t)zinv;
    C.d2_z1_p = shoup(zinv, qm);
    int lz = __builtin_clzll(qm);
    C.zone = (qm << lz) - 1;
  }
  P.q0inv_q1 = (uint32_t)inv_prime(q0, q1);
  P.q0inv_q1_p = shoup(P.q0inv_q1, q1);
  {
    const uint64_t r64_0 = (uint64_t)(((u128)1 << 64) % q0), r64_1 = (uint64_t)(((u128)1 << 64) % q1);
    const uint64_t a = (uint64_t)((u128)N * r64_0 % q0);
    const uint64_t b = (uint64_t)((u128)inv_prime(r64_1, q1) * inv_prime(N, q1) % q1);
    P.conv_a = (uint32_t)a;
    P.conv_a_p = shoup(a, q0);
    P.conv_b = (uint32_t)b;
    P.conv_b_p = shoup(b, q1);
    P.conv0_a = (uint32_t)r64_0;
    P.conv0_a_p = shoup(r64_0, q0);
    const uint64_t b0 = inv_prime(r64_1, q1);
    P.conv0_b = (uint32_t)b0;
    P.conv0_b_p = shoup(b0, q1);
  }
  P.delta = q / prm->p;
  P.mode = mode;
  P.one = 1;
  e = c->tables.ensure(host.size() * sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMemcpy(c->tables.p, host.data(), host.size() * sizeof(uint32_t), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    delete c;
    return fail(INSPIRE_ERR_CUDA, std::string("table upload: ") + cudaGetErrorString(e));
  }
  for (int r = 0; r < 2; r++) {
    const uint32_t* base = c->tables.as<uint32_t>() + r * per;
    P.r[r].fwd = reinterpret_cast<const uint2*>(base);
    P.r[r].inv = reinterpret_cast<const uint2*>(base + 2 * N);
    P.r[r].psi_pow = base + 4 * N;
  }
  e = prepare_respond_kernels();
  if (e == cudaSuccess) e = prepare_respond_pair_kernels();
  if (e == cudaSuccess) e = prepare_nopacking_kernels();
  if (e == cudaSuccess) e = prepare_ops_kernels();
  if (e == cudaSuccess) e = prepare_setup_kernels();
  if (e == cudaSuccess) e = prepare_client_kernels();
  if (e == cudaSuccess) e = prepare_tree_kernels();
  if (e != cudaSuccess) {
    delete c;
    return fail(INSPIRE_ERR_CUDA, std::string("kernel setup: ") + cudaGetErrorString(e));
  }
  *out = c;
  return INSPIRE_OK;
}

void inspire_ctx_destroy(inspire_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  delete c;
}

int inspire_crs_load(inspire_ctx* c, const uint8_t w_seed[32], uint32_t num_columns) {
  if (!c || !w_seed) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null argument");
  std::lock_guard<std::mutex> lk(c->mu);
  if (int rc = set_device(c)) return rc;
  if (num_columns == 0 || num_columns > (uint32_t)MAX_GAMMA || (num_columns & (num_columns - 1)))
    return fail(INSPIRE_ERR_UNSUPPORTED, "GPU path supports num_columns in {1, 2, 4, 8, 16}");
  const int gamma = (int)num_columns;
  c->gamma = gamma;
  c->crs_a_count = 0;
  memcpy(c->w_seed, w_seed, 32);
  c->P.gamma = gamma;
  for (int r = 0; r < 2; r++) {
    const uint64_t qm = c->params.crt_moduli[r];
    const uint64_t r96 = (uint64_t)(((u128)1 << 96) % qm);
    const uint64_t k = (uint64_t)((u128)((u128)inv_prime(gamma, qm) * inv_prime(N, qm) % qm) * r96 % qm);
    c->P.r[r].e_scale = (uint32_t)k;
    c->P.r[r].e_scale_p = shoup(k, qm);
  }
  // w_mask = generate_mask_from_seed(w_seed) (inspiring2.rs:816-835): next_u64 % q, CRT split
  std::vector<uint32_t> wm((size_t)ELL * 2 * N);
  HostChaCha rng(w_seed);
  for (int k = 0; k < ELL; k++)
    for (int i = 0; i < N; i++) {
      const uint64_t v = rng.next_u64() % c->q;
      wm[((size_t)k * 2 + 0) * N + i] = (uint32_t)(v % c->params.crt_moduli[0]);
      wm[((size_t)k * 2 + 1) * N + i] = (uint32_t)(v % c->params.crt_moduli[1]);
    }
  CUDA_TRY(c->wmask.ensure(wm.size() * sizeof(uint32_t)));
  CUDA_TRY(cudaMemcpy(c->wmask.p, wm.data(), wm.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
  CUDA_TRY(c->what.ensure(sizeof(uint32_t) * (size_t)std::max(1, (gamma - 1) * ELL) * 2 * N));
  CUDA_TRY(launch_crs_what(c->P, c->wmask.as<uint32_t>(), c->what.as<uint32_t>(), c->stream));
  CUDA_TRY(c->what3.ensure(c->what.bytes));
  CUDA_TRY(cudaMemcpyAsync(c->what3.p, c->what.p, c->what.bytes, cudaMemcpyDeviceToDevice, c->stream));
  CUDA_TRY(launch_fold_third_digit(c->P, c->what3.as<uint32_t>(), gamma - 1, c->stream));
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  // key tables of registered clients were built for the previous gamma
  for (size_t i = 0; i < c->clients.size(); i++) release_keys(c, (int32_t)i);
  c->has_crs = true;
  return INSPIRE_OK;
}

int inspire_db_create(inspire_ctx* c, const uint8_t* raw, uint64_t n_entries, uint32_t entry_size,
                      inspire_db** out) {
  if (!c || !out || (!raw && n_entries && entry_size)) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null argument");
  std::lock_guard<std::mutex> lk(c->mu);
  *out = nullptr;
  if (!c->has_crs) return fail(INSPIRE_ERR_NO_CRS, "no CRS loaded (inspire_crs_load)");
  if (int rc = set_device(c)) return rc;
  inspire_db* db = new inspire_db();
  db->H.ledger = db->E.ledger = c->ledger;
  db->ctx = c;
  db->device = c->device;
  db->n_entries = n_entries;
  db->entry_size = entry_size;
  // encode_database returns no shard for an empty database (encode_db.rs:112-114)
  const uint64_t nshards64 = (entry_size == 0 || n_entries == 0) ? 0 : (n_entries + N - 1) / N;
  if (nshards64 > 0x7fffffffULL) {
    delete db;
    return fail(INSPIRE_ERR_INVALID_ARGUMENT, "too many shards");
  }
  db->nshards = (int)nshards64;
  const int gamma = entry_size ? (int)((entry_size * 8 + 15) / 16) : c->gamma;
  if (db->nshards > 0 && gamma != c->gamma) {
    delete db;
    return fail(INSPIRE_ERR_INVALID_ARGUMENT, "ceil(entry_size/2) must equal the CRS num_columns");
  }
  db->gamma = c->gamma;
  if (db->nshards > 0) {
    const size_t hbytes = sizeof(uint16_t) * (size_t)db->nshards * gamma * N;
    const size_t ebytes = sizeof(uint32_t) * (size_t)db->nshards * 2 * ELL * gamma * N;
    cudaError_t e = db->H.ensure(hbytes);
    if (e == cudaSuccess) e = db->E.ensure(ebytes);
    if (e != cudaSuccess) {
      delete db;
      return fail(INSPIRE_ERR_OUT_OF_MEMORY, alloc_failure(c, "database allocation"));
    }
    // raw bytes in chunks of whole shards
    const uint64_t shards_per_chunk = std::max<uint64_t>(1, (256ULL << 20) / ((uint64_t)N * entry_size));
    DevMem stage(c->ledger);
    for (uint64_t s0 = 0; s0 < (uint64_t)db->nshards; s0 += shards_per_chunk) {
      const uint64_t s1 = std::min<uint64_t>(db->nshards, s0 + shards_per_chunk);
      const uint64_t e0 = s0 * N, e1 = std::min<uint64_t>(n_entries, s1 * N);
      const size_t bytes = (size_t)(e1 - e0) * entry_size;
      cudaError_t ce = stage.ensure(std::max<size_t>(bytes, 1));
      if (ce == cudaSuccess) ce = cudaMemcpy(stage.p, raw + e0 * entry_size, bytes, cudaMemcpyHostToDevice);
      if (ce == cudaSuccess)
        ce = launch_columns_from_raw(stage.as<uint8_t>(), e1 - e0, (int)entry_size, gamma, (int)(s1 - s0),
                                     db->H.as<uint16_t>() + s0 * gamma * N, c->stream);
      if (ce == cudaSuccess) ce = cudaStreamSynchronize(c->stream);
      if (ce != cudaSuccess) {
        delete db;
        return fail(INSPIRE_ERR_CUDA, std::string("database upload: ") + cudaGetErrorString(ce));
      }
    }
    cudaError_t ce = launch_encode_E(c->P, db->H.as<uint16_t>(), db->nshards, db->E.as<uint32_t>(), c->stream);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(c->stream);
    if (ce != cudaSuccess) {
      delete db;
      return fail(INSPIRE_ERR_CUDA, std::string("database encode: ") + cudaGetErrorString(ce));
    }
  }
  *out = db;
  return INSPIRE_OK;
}

void inspire_db_destroy(inspire_db* db) {
  if (!db) return;
  cudaSetDevice(db->device);
  delete db;
}

int inspire_ctx_set_device_budget(inspire_ctx* c, uint64_t bytes) {
  if (!c) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null argument");
  if (!c->ledger->set_budget(bytes))
    return fail(INSPIRE_ERR_INVALID_ARGUMENT, "device budget below the " + std::to_string(c->ledger->used()) +
                                                  " bytes already in use");
  return INSPIRE_OK;
}

int inspire_ctx_set_pair_threshold(inspire_ctx* c, uint32_t max_queries) {
  if (!c) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null argument");
  if (max_queries > (1u << 30)) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "max_queries out of range");
  std::lock_guard<std::mutex> lk(c->mu);
  c->pair_max.store((int)max_queries);
  return INSPIRE_OK;
}

uint32_t inspire_ctx_pair_threshold(const inspire_ctx* c) { return c ? (uint32_t)c->pair_max.load() : 0; }

int inspire_ctx_device_memory(inspire_ctx* c, uint64_t* used, uint64_t* budget) {
  if (!c) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null argument");
  if (used) *used = c->ledger->used();
  if (budget) *budget = c->ledger->budget();
  return INSPIRE_OK;
}

uint32_t inspire_db_num_shards(const inspire_db* db) { return db ? (uint32_t)db->nshards : 0; }

uint64_t inspire_db_device_bytes(const inspire_db* db) { return db ? (uint64_t)(db->H.bytes + db->E.bytes) : 0; }

int inspire_client_register(inspire_ctx* c, const uint64_t* y_body, const uint64_t* y_all, int32_t* id) {
  if (!c || !id) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null argument");
  std::lock_guard<std::mutex> lk(c->mu);
  if (!c->has_crs) return fail(INSPIRE_ERR_NO_CRS, "no CRS loaded (inspire_crs_load)");
  if (int rc = set_device(c)) return rc;
  if (int rc = register_keys(c, y_body, y_all, id)) return rc;
  // the device client table is brought up to date here, so that later
  // launches make no copy (they can be captured in a CUDA graph); if it
  // cannot grow, the registration is undone
  if (int rc = sync_client_table(c)) {
    const std::string msg = g_last_error;
    release_keys(c, *id);
    *id = -1;
    return fail(rc, msg);
  }
  return INSPIRE_OK;
}

int inspire_client_release(inspire_ctx* c, int32_t id) {
  if (!c) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null argument");
  std::lock_guard<std::mutex> lk(c->mu);
  if (id < 0 || (size_t)id >= c->clients.size() || !c->clients[id])
    return fail(INSPIRE_ERR_INVALID_ARGUMENT, "unknown client id");
  if (int rc = set_device(c)) return rc;
  release_keys(c, id);
  return sync_client_table(c);
}

int inspire_respond_seeded_inspiring(inspire_ctx* c, const inspire_db* db, const inspire_seeded_query* qy,
                                     uint64_t* out_ct) {
  if (!c || !qy) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null argument");
  if (!qy->seeds || !qy->b_rows) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null query rows");
  std::lock_guard<std::mutex> lk(c->mu);
  if (int rc = set_device(c)) return rc;
  return single_query(c, db, qy->shard_id, qy->seeds, nullptr, qy->b_rows, qy->has_packing_keys, qy->y_body,
                      qy->y_all, out_ct);
}

int inspire_respond_inspiring(inspire_ctx* c, const inspire_db* db, const inspire_query* qy, uint64_t* out_ct) {
  if (!c || !qy) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null argument");
  if (!qy->rgsw) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null query rows");
  std::lock_guard<std::mutex> lk(c->mu);
  if (int rc = set_device(c)) return rc;
  return single_query(c, db, qy->shard_id, nullptr, qy->rgsw, nullptr, qy->has_packing_keys, qy->y_body,
                      qy->y_all, out_ct);
}

int inspire_respond_seeded(inspire_ctx* c, const inspire_db* db, const inspire_seeded_query* qy, uint64_t* out_ct,
                           uint64_t* out_columns) {
  if (!c || !db || !qy || !out_ct) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null argument");
  if (!qy->seeds || !qy->b_rows) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null query rows");
  std::lock_guard<std::mutex> lk(c->mu);
  if (!c->has_crs) return fail(INSPIRE_ERR_NO_CRS, "no CRS loaded (inspire_crs_load)");
  if (qy->shard_id >= (uint32_t)db->nshards)
    return fail(INSPIRE_ERR_SHARD_NOT_FOUND, "Shard " + std::to_string(qy->shard_id) + " not found");
  if (int rc = set_device(c)) return rc;
  return run_nopacking(c, db, 1, &qy->shard_id, qy->seeds + 32 * ELL, (size_t)64 * ELL, nullptr,
                       qy->b_rows + (size_t)ELL * poly_words(), 2 * ELL, out_ct, out_columns);
}

int inspire_respond(inspire_ctx* c, const inspire_db* db, const inspire_query* qy, uint64_t* out_ct,
                    uint64_t* out_columns) {
  if (!c || !db || !qy || !out_ct) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null argument");
  if (!qy->rgsw) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null query rows");
  std::lock_guard<std::mutex> lk(c->mu);
  if (!c->has_crs) return fail(INSPIRE_ERR_NO_CRS, "no CRS loaded (inspire_crs_load)");
  if (qy->shard_id >= (uint32_t)db->nshards)
    return fail(INSPIRE_ERR_SHARD_NOT_FOUND, "Shard " + std::to_string(qy->shard_id) + " not found");
  if (int rc = set_device(c)) return rc;
  // rgsw holds 2*ELL rows of (a, b): row r's a is poly 2r, its b poly 2r+1
  const size_t pw = poly_words();
  std::vector<uint64_t> ar((size_t)ELL * pw), br((size_t)ELL * pw);
  for (int t = 0; t < ELL; t++) {
    memcpy(ar.data() + t * pw, qy->rgsw + (size_t)(2 * (ELL + t)) * pw, pw * sizeof(uint64_t));
    memcpy(br.data() + t * pw, qy->rgsw + (size_t)(2 * (ELL + t) + 1) * pw, pw * sizeof(uint64_t));
  }
  return run_nopacking(c, db, 1, &qy->shard_id, nullptr, 0, ar.data(), br.data(), ELL, out_ct, out_columns);
}

int inspire_crs_info(inspire_ctx* c, uint8_t* w_seed, uint32_t* num_columns, int32_t* has_galois_keys) {
  if (!c || !w_seed || !num_columns || !has_galois_keys) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null argument");
  std::lock_guard<std::mutex> lk(c->mu);
  if (!c->has_crs) return fail(INSPIRE_ERR_NO_CRS, "no CRS loaded (inspire_crs_load)");
  memcpy(w_seed, c->w_seed, 32);
  *num_columns = (uint32_t)c->gamma;
  *has_galois_keys = c->has_galois ? 1 : 0;
  return INSPIRE_OK;
}

int inspire_crs_load_galois_keys(inspire_ctx* c, const uint64_t* keys, uint32_t nkeys) {
  if (!c || !keys) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null argument");
  if (nkeys != (uint32_t)LOGN)
    return fail(INSPIRE_ERR_INVALID_ARGUMENT, "expected log2(ring_dim) = " + std::to_string(LOGN) + " Galois keys");
  const size_t pw = poly_words();
  const size_t npolys = (size_t)nkeys * 2 * ELL;
  for (size_t p = 0; p < npolys; p++)
    for (int r = 0; r < 2; r++)
      for (int i = 0; i < N; i++)
        if (keys[p * pw + (size_t)r * N + i] >= c->params.crt_moduli[r])
          return fail(INSPIRE_ERR_INVALID_ARGUMENT, "Galois key coefficients must be reduced mod each CRT modulus");
  std::lock_guard<std::mutex> lk(c->mu);
  if (int rc = set_device(c)) return rc;
  DevMem staged(c->ledger);
  CUDA_TRY(staged.ensure(sizeof(uint64_t) * npolys * pw));
  CUDA_TRY(cudaMemcpyAsync(staged.p, keys, sizeof(uint64_t) * npolys * pw, cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(c->galois.ensure(sizeof(uint32_t) * npolys * pw));
  CUDA_TRY(launch_galois_prep(c->P, staged.as<uint64_t>(), (int)npolys, c->galois.as<uint32_t>(), c->stream));
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  c->has_galois = true;
  return INSPIRE_OK;
}

int inspire_respond_one_packing(inspire_ctx* c, const inspire_db* db, const inspire_query* qy, uint64_t* out_a,
                                uint64_t* out_b, uint32_t* b_words) {
  if (!c || !db || !qy || !out_a || !out_b || !b_words) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null argument");
  if (!qy->rgsw) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null query rows");
  std::lock_guard<std::mutex> lk(c->mu);
  if (!c->has_crs) return fail(INSPIRE_ERR_NO_CRS, "no CRS loaded (inspire_crs_load)");
  if (qy->shard_id >= (uint32_t)db->nshards)
    return fail(INSPIRE_ERR_SHARD_NOT_FOUND, "Shard " + std::to_string(qy->shard_id) + " not found");
  if (int rc = set_device(c)) return rc;
  const size_t pw = poly_words();
  std::vector<uint64_t> ar((size_t)ELL * pw), br((size_t)ELL * pw);
  for (int t = 0; t < ELL; t++) {
    memcpy(ar.data() + t * pw, qy->rgsw + (size_t)(2 * (ELL + t)) * pw, pw * sizeof(uint64_t));
    memcpy(br.data() + t * pw, qy->rgsw + (size_t)(2 * (ELL + t) + 1) * pw, pw * sizeof(uint64_t));
  }
  std::vector<uint64_t> ob(2 * pw);
  if (int rc = run_tree(c, db, 1, &qy->shard_id, nullptr, 0, ar.data(), br.data(), ELL, out_a, ob.data(), b_words))
    return rc;
  memcpy(out_b, ob.data(), sizeof(uint64_t) * *b_words);
  return INSPIRE_OK;
}

int inspire_respond_seeded_packed(inspire_ctx* c, const inspire_db* db, const inspire_seeded_query* qy,
                                  uint64_t* out_a, uint64_t* out_b, uint32_t* b_words) {
  if (!c || !db || !qy || !out_a || !out_b || !b_words) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null argument");
  if (!qy->seeds || !qy->b_rows) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null query rows");
  std::lock_guard<std::mutex> lk(c->mu);
  if (!c->has_crs) return fail(INSPIRE_ERR_NO_CRS, "no CRS loaded (inspire_crs_load)");
  if (qy->shard_id >= (uint32_t)db->nshards)
    return fail(INSPIRE_ERR_SHARD_NOT_FOUND, "Shard " + std::to_string(qy->shard_id) + " not found");
  if (int rc = set_device(c)) return rc;
  std::vector<uint64_t> ob(2 * poly_words());
  if (int rc = run_tree(c, db, 1, &qy->shard_id, qy->seeds + 32 * ELL, (size_t)64 * ELL, nullptr,
                        qy->b_rows + (size_t)ELL * poly_words(), 2 * ELL, out_a, ob.data(), b_words))
    return rc;
  memcpy(out_b, ob.data(), sizeof(uint64_t) * *b_words);
  return INSPIRE_OK;
}

int inspire_respond_seeded_packed_batch(inspire_ctx* c, const inspire_db* db, uint32_t n, const uint32_t* shard_ids,
                                        const uint8_t* seeds, const uint64_t* b_rows, uint64_t* out_a,
                                        uint64_t* out_b, uint32_t* b_words) {
  if (!c || !db || !b_words || (n && (!shard_ids || !seeds || !b_rows || !out_a || !out_b)))
    return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null argument");
  std::lock_guard<std::mutex> lk(c->mu);
  if (!c->has_crs) return fail(INSPIRE_ERR_NO_CRS, "no CRS loaded (inspire_crs_load)");
  for (uint32_t i = 0; i < n; i++)
    if (shard_ids[i] >= (uint32_t)db->nshards)
      return fail(INSPIRE_ERR_SHARD_NOT_FOUND, "Shard " + std::to_string(shard_ids[i]) + " not found");
  if (int rc = set_device(c)) return rc;
  return run_tree(c, db, n, shard_ids, seeds + 32 * ELL, (size_t)64 * ELL, nullptr, b_rows + (size_t)ELL * poly_words(),
                  2 * ELL, out_a, out_b, b_words);
}


int inspire_respond_seeded_nopacking_batch(inspire_ctx* c, const inspire_db* db, uint32_t n,
                                           const uint32_t* shard_ids, const uint8_t* seeds, const uint64_t* b_rows,
                                           uint64_t* out_ct) {
  if (!c || !db || (n && (!shard_ids || !seeds || !b_rows || !out_ct)))
    return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null argument");
  std::lock_guard<std::mutex> lk(c->mu);
  if (!c->has_crs) return fail(INSPIRE_ERR_NO_CRS, "no CRS loaded (inspire_crs_load)");
  for (uint32_t i = 0; i < n; i++)
    if (shard_ids[i] >= (uint32_t)db->nshards)
      return fail(INSPIRE_ERR_SHARD_NOT_FOUND, "Shard " + std::to_string(shard_ids[i]) + " not found");
  if (int rc = set_device(c)) return rc;
  return run_nopacking(c, db, n, shard_ids, seeds + 32 * ELL, (size_t)64 * ELL, nullptr,
                       b_rows + (size_t)ELL * poly_words(), 2 * ELL, out_ct, nullptr);
}

int inspire_respond_seeded_batch(inspire_ctx* c, const inspire_db* db, uint32_t n, const uint32_t* shard_ids,
                                 const uint8_t* seeds, const uint64_t* b_rows, const int32_t* client_ids,
                                 uint64_t* out_ct) {
  if (!c || !db || (n && (!shard_ids || !seeds || !b_rows || !client_ids || !out_ct)))
    return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null argument");
  std::lock_guard<std::mutex> lk(c->mu);
  if (!c->has_crs) return fail(INSPIRE_ERR_NO_CRS, "no CRS loaded (inspire_crs_load)");
  if (int rc = set_device(c)) return rc;
  for (uint32_t i = 0; i < n; i++) {
    if (shard_ids[i] >= (uint32_t)db->nshards)
      return fail(INSPIRE_ERR_SHARD_NOT_FOUND, "Shard " + std::to_string(shard_ids[i]) + " not found");
    const int32_t id = client_ids[i];
    if (id < 0 || (size_t)id >= c->clients.size() || !c->clients[id])
      return fail(INSPIRE_ERR_KEYS_MISSING, "InspiRING client packing keys missing from query");
  }
  return run_batch(c, db, n, shard_ids, seeds + 32 * ELL, (size_t)64 * ELL, nullptr, b_rows + (size_t)ELL * poly_words(),
                   2 * ELL, client_ids, out_ct);
}

int inspire_respond_batch(inspire_ctx* c, const inspire_db* db, uint32_t n, const uint32_t* shard_ids,
                          const uint64_t* rgsw, const int32_t* client_ids, uint64_t* out_ct) {
  if (!c || !db || (n && (!shard_ids || !rgsw || !client_ids || !out_ct)))
    return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null argument");
  std::lock_guard<std::mutex> lk(c->mu);
  if (!c->has_crs) return fail(INSPIRE_ERR_NO_CRS, "no CRS loaded (inspire_crs_load)");
  if (int rc = set_device(c)) return rc;
  for (uint32_t i = 0; i < n; i++) {
    if (shard_ids[i] >= (uint32_t)db->nshards)
      return fail(INSPIRE_ERR_SHARD_NOT_FOUND, "Shard " + std::to_string(shard_ids[i]) + " not found");
    const int32_t id = client_ids[i];
    if (id < 0 || (size_t)id >= c->clients.size() || !c->clients[id])
      return fail(INSPIRE_ERR_KEYS_MISSING, "InspiRING client packing keys missing from query");
  }
  // rows ELL..2ELL-1 of each query, split into their a and b polys
  const size_t pw = poly_words();
  std::vector<uint64_t> ar((size_t)n * ELL * pw), br((size_t)n * ELL * pw);
  for (uint32_t i = 0; i < n; i++)
    for (int t = 0; t < ELL; t++) {
      const uint64_t* row = rgsw + ((size_t)i * 2 * ELL + ELL + t) * 2 * pw;
      memcpy(ar.data() + ((size_t)i * ELL + t) * pw, row, pw * sizeof(uint64_t));
      memcpy(br.data() + ((size_t)i * ELL + t) * pw, row + pw, pw * sizeof(uint64_t));
    }
  return run_batch(c, db, n, shard_ids, nullptr, 0, ar.data(), br.data(), ELL, client_ids, out_ct);
}

int inspire_respond_seeded_batch_device(inspire_ctx* c, const inspire_db* db, uint32_t n, const uint32_t* d_shard_ids,
                                        const uint8_t* d_seeds, const uint64_t* d_b_rows, const int32_t* d_client_ids,
                                        uint64_t* d_out_ct, int32_t* d_status, void* stream) {
  return inspire_respond_seeded_batch_device_grid(c, db, n, d_shard_ids, d_seeds, d_b_rows, d_client_ids, d_out_ct,
                                                  d_status, 0, stream);
}

int inspire_respond_seeded_batch_device_grid(inspire_ctx* c, const inspire_db* db, uint32_t n,
                                             const uint32_t* d_shard_ids, const uint8_t* d_seeds,
                                             const uint64_t* d_b_rows, const int32_t* d_client_ids, uint64_t* d_out_ct,
                                             int32_t* d_status, uint32_t max_ctas, void* stream) {
  if (!c || !db || (n && (!d_shard_ids || !d_seeds || !d_b_rows || !d_client_ids || !d_out_ct || !d_status)))
    return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null argument");
  if (reinterpret_cast<uintptr_t>(d_b_rows) % 16)
    return fail(INSPIRE_ERR_INVALID_ARGUMENT, "d_b_rows must be 16-byte aligned");
  if (max_ctas > 0x7fffffffu) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "max_ctas out of range");
  std::lock_guard<std::mutex> lk(c->mu);
  if (!c->has_crs) return fail(INSPIRE_ERR_NO_CRS, "no CRS loaded (inspire_crs_load)");
  if (int rc = set_device(c)) return rc;
  if (int rc = sync_client_table(c)) return rc;
  RespondArgs a{};
  a.P = c->P;
  a.nq = (int)n;
  a.shard = d_shard_ids;
  a.seeds = d_seeds;
  a.arows = nullptr;
  a.brows = d_b_rows;
  a.client = d_client_ids;
  a.yhat_table = c->client_table.as<const uint32_t*>();
  a.nclients = (int)c->client_ptrs.size();
  a.nshards = db->nshards;
  a.E = db->E.as<uint32_t>();
  a.H = db->H.as<uint16_t>();
  a.what = c->what3.as<uint32_t>();
  a.out = d_out_ct;
  a.status = d_status;
  CUDA_TRY(launch_respond(a, true, (cudaStream_t)stream, (int)max_ctas, c->pair_max.load()));
  return INSPIRE_OK;
}

int inspire_ntt_forward_device(inspire_ctx* c, uint32_t* d_polys, uint32_t npolys, void* stream) {
  if (!c || (npolys && !d_polys)) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null argument");
  if (int rc = set_device(c)) return rc;
  CUDA_TRY(launch_ntt_ref(c->P, d_polys, (int)npolys, false, (cudaStream_t)stream));
  return INSPIRE_OK;
}

int inspire_ntt_inverse_device(inspire_ctx* c, uint32_t* d_polys, uint32_t npolys, void* stream) {
  if (!c || (npolys && !d_polys)) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null argument");
  if (int rc = set_device(c)) return rc;
  CUDA_TRY(launch_ntt_ref(c->P, d_polys, (int)npolys, true, (cudaStream_t)stream));
  return INSPIRE_OK;
}

int inspire_extract_inspiring_device(inspire_ctx* c, const uint64_t* d_sk, const uint64_t* d_ct, uint32_t n,
                                     uint32_t entry_size, uint8_t* d_entries, void* stream) {
  if (!c || (n && (!d_sk || !d_ct || !d_entries))) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null argument");
  if (entry_size == 0 || entry_size > 32) return fail(INSPIRE_ERR_UNSUPPORTED, "entry_size must be 1..32 on the GPU path");
  if (int rc = set_device(c)) return rc;
  CUDA_TRY(launch_extract(c->P, c->params.p, d_sk, d_ct, (int)n, (int)entry_size, d_entries, (cudaStream_t)stream));
  return INSPIRE_OK;
}

}  // extern "C"

namespace {

// Client-side randomness tables: the discrete Gaussian on [-T, T],
// T = ceil(6 sigma) (math/gaussian.rs:31-38, 88-104), as cdt[j] =
// floor(2^63 P(|e| <= j)) for j < T, and the gadget powers z^i mod q_r
// (rgsw/types.rs:67-90, Poly::scalar_mul poly.rs:466-486).
template <class Args>
int client_tables(const inspire_ctx* c, const uint8_t* key, Args& a) {
  if (!(c->params.sigma > 0.0)) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "sigma must be positive");
  const int T = (int)std::ceil(c->params.sigma * 6.0);
  if (T + 1 > MAX_CDT) return fail(INSPIRE_ERR_UNSUPPORTED, "sigma too large for the device error table");
  a.P = c->P;
  for (int i = 0; i < 8; i++)
    a.key[i] = (uint32_t)key[4 * i] | ((uint32_t)key[4 * i + 1] << 8) | ((uint32_t)key[4 * i + 2] << 16) |
               ((uint32_t)key[4 * i + 3] << 24);
  for (int r = 0; r < 2; r++) {
    const uint64_t q = c->params.crt_moduli[r];
    uint64_t zp = 1;
    for (int i = 0; i < ELL; i++) {
      a.zpow[r][i] = (uint32_t)zp;
      a.zpow_p[r][i] = shoup(zp, q);
      zp = (uint64_t)((u128)zp * (c->params.gadget_base % q) % q);
    }
  }
  const double s2 = 2.0 * c->params.sigma * c->params.sigma;
  double total = 0.0;
  for (int x = -T; x <= T; x++) total += std::exp(-(double)x * x / s2);
  double cum = 0.0;
  for (int j = 0; j < T; j++) {
    cum += (j ? 2.0 : 1.0) * std::exp(-(double)j * j / s2) / total;
    a.cdt[j] = (uint64_t)std::ldexp(std::fmin(cum, 1.0), 63);
  }
  a.cdt_len = T + 1;
  return INSPIRE_OK;
}

}  // namespace

extern "C" {

int inspire_query_seeded_device(inspire_ctx* c, const uint64_t* d_sk, const uint8_t* key, uint64_t first_query,
                                uint32_t n, const uint32_t* d_local_idx, uint8_t* d_seeds, uint64_t* d_b_rows,
                                int32_t* d_status, void* stream) {
  if (!c || !key || (n && (!d_sk || !d_local_idx || !d_seeds || !d_b_rows || !d_status)))
    return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null argument");
  // seed blocks Q * 16 + row stay below the error blocks' base 2^40
  if (first_query > (1ull << 36) || first_query + n > (1ull << 36))
    return fail(INSPIRE_ERR_INVALID_ARGUMENT, "first_query + n must be <= 2^36");
  QueryGenArgs a{};
  if (int rc = client_tables(c, key, a)) return rc;
  if (int rc = set_device(c)) return rc;
  a.first_query = first_query;
  a.local_idx = d_local_idx;
  a.sk = d_sk;
  a.seeds = d_seeds;
  a.b_rows = d_b_rows;
  a.status = d_status;
  CUDA_TRY(launch_query_gen(a, (int)n, (cudaStream_t)stream));
  return INSPIRE_OK;
}

int inspire_client_keygen_device(inspire_ctx* c, const uint8_t* key, uint64_t first_client, uint32_t n,
                                 uint64_t* d_sk, uint64_t* d_y_body, void* stream) {
  if (!c || !key || (n && (!d_sk || !d_y_body))) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null argument");
  if (first_client > (1ull << 30) || first_client + n > (1ull << 30))
    return fail(INSPIRE_ERR_INVALID_ARGUMENT, "first_client + n must be <= 2^30");
  std::lock_guard<std::mutex> lk(c->mu);
  if (!c->has_crs) return fail(INSPIRE_ERR_NO_CRS, "no CRS loaded (inspire_crs_load)");
  KeyGenArgs a{};
  if (int rc = client_tables(c, key, a)) return rc;
  if (int rc = set_device(c)) return rc;
  a.first_client = first_client;
  a.wmask = c->wmask.as<uint32_t>();
  a.sk = d_sk;
  a.y_body = d_y_body;
  CUDA_TRY(launch_client_keys(a, (int)n, (cudaStream_t)stream));
  return INSPIRE_OK;
}

int inspire_respond_seeded_packed_noalloc_device(inspire_ctx* c, const inspire_db* db, uint32_t n,
                                                 const uint32_t* d_shard_ids, const uint8_t* d_seeds,
                                                 const uint64_t* d_b_rows, uint64_t* d_out_a, uint64_t* d_out_b,
                                                 int32_t* d_status, uint32_t* b_words, void* stream) {
  if (!c || !db || !b_words || (n && (!d_shard_ids || !d_seeds || !d_b_rows || !d_out_a || !d_out_b || !d_status)))
    return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null argument");
  if (n > (uint32_t)TREE_NOALLOC_MAX_QUERIES)
    return fail(INSPIRE_ERR_INVALID_ARGUMENT,
                "at most " + std::to_string(TREE_NOALLOC_MAX_QUERIES) + " queries per allocation-free call");
  std::lock_guard<std::mutex> lk(c->mu);
  if (!c->has_crs) return fail(INSPIRE_ERR_NO_CRS, "no CRS loaded (inspire_crs_load)");
  if (!c->has_galois) return fail(INSPIRE_ERR_NO_CRS, "no Galois keys loaded (inspire_crs_load_galois_keys)");
  const size_t pw = poly_words();
  *b_words = (c->mode == MODE_COMPAT && db->gamma > 1) ? (uint32_t)(2 * pw) : (uint32_t)pw;
  if (n == 0) return INSPIRE_OK;
  if (int rc = set_device(c)) return rc;
  void* scratch = nullptr;
  CUDA_TRY(tree_noalloc_scratch(c->device, &scratch));
  // carve: columns [n][gamma][2][poly] u64, combined [n][2][poly] u64, tree work (u32)
  uint64_t* cols = static_cast<uint64_t*>(scratch);
  uint64_t* comb = cols + (size_t)n * db->gamma * 2 * pw;
  uint32_t* work = reinterpret_cast<uint32_t*>(comb + (size_t)n * 2 * pw);
  NoPackingArgs a{};
  a.P = c->P;
  a.nq = (int)n;
  a.shard = d_shard_ids;
  a.seeds = d_seeds;
  a.arows = nullptr;
  a.brows = d_b_rows;
  a.nshards = db->nshards;
  a.H = db->H.as<uint16_t>();
  a.out = comb;
  a.out_columns = cols;
  a.status = d_status;
  a.col_groups = column_groups(c, db, n, true);
  CUDA_TRY(launch_nopacking(a, true, (cudaStream_t)stream));
  TreeArgs t{};
  t.P = c->P;
  t.nq = (int)n;
  t.ncols = db->gamma;
  t.mode = c->mode;
  t.cols = cols;
  t.ks = c->galois.as<uint32_t>();
  t.work = work;
  t.out_a = d_out_a;
  t.out_b = d_out_b;
  CUDA_TRY(launch_pack_tree(t, (cudaStream_t)stream));
  return INSPIRE_OK;
}

int inspire_galois_keygen_device(inspire_ctx* c, const uint8_t* key, const uint64_t* d_sk, uint64_t* d_keys,
                                 int32_t* d_status, void* stream) {
  if (!c || !key || !d_sk || !d_keys || !d_status) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null argument");
  GaloisGenArgs a{};
  if (int rc = client_tables(c, key, a)) return rc;
  if (int rc = set_device(c)) return rc;
  a.sk = d_sk;
  a.keys = d_keys;
  a.status = d_status;
  CUDA_TRY(launch_ks_matrices(a, LOGN, (cudaStream_t)stream));
  return INSPIRE_OK;
}

int inspire_setup_keygen_device(inspire_ctx* c, const uint8_t* key, const uint64_t* d_sk, uint64_t* d_ks,
                                uint64_t* d_crs_a, int32_t* d_status, void* stream) {
  if (!c || !key || !d_sk || !d_ks || !d_status) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null argument");
  GaloisGenArgs a{};
  if (int rc = client_tables(c, key, a)) return rc;
  if (int rc = set_device(c)) return rc;
  a.sk = d_sk;
  a.keys = d_ks;
  a.status = d_status;
  const cudaStream_t st = (cudaStream_t)stream;
  CUDA_TRY(launch_ks_matrices(a, LOGN + 4, st));
  a.status = d_status + LOGN + 4;
  CUDA_TRY(cudaMemsetAsync(a.status, 0, sizeof(int32_t), st));
  if (d_crs_a) CUDA_TRY(launch_crs_a(a, N, d_crs_a, st));
  return INSPIRE_OK;
}

int inspire_mulmod_rate_device(inspire_ctx* c, uint32_t blocks, uint32_t iters, uint32_t* d_sink, void* stream) {
  if (!c || (blocks && !d_sink)) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null argument");
  if (int rc = set_device(c)) return rc;
  CUDA_TRY(launch_mulmod_rate(c->P, (int)blocks, (int)iters, d_sink, (cudaStream_t)stream));
  return INSPIRE_OK;
}

int inspire_int8_mma_rate_device(inspire_ctx* c, uint32_t blocks, uint32_t iters, const int8_t* d_a, const int8_t* d_b,
                                 int32_t* d_out, void* stream) {
  if (!c || !d_a || !d_b || !d_out) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null argument");
  if (blocks == 0 || blocks > (1u << 20) || iters == 0 || iters > 4096)
    return fail(INSPIRE_ERR_INVALID_ARGUMENT, "blocks in [1, 2^20] and iters in [1, 4096]");
  if (int rc = set_device(c)) return rc;
  CUDA_TRY(launch_int8_mma_rate(d_a, d_b, (int)blocks, (int)iters, d_out, (cudaStream_t)stream));
  return INSPIRE_OK;
}

int inspire_external_product_device(inspire_ctx* c, const uint32_t* d_ct, const uint32_t* d_rgsw, uint32_t* d_out,
                                    uint32_t npairs, void* stream) {
  if (!c || (npairs && (!d_ct || !d_rgsw || !d_out))) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null argument");
  if (int rc = set_device(c)) return rc;
  CUDA_TRY(launch_external_product(c->P, d_ct, d_rgsw, d_out, (int)npairs, (cudaStream_t)stream));
  return INSPIRE_OK;
}

}  // extern "C"
