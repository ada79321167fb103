// wire.cu -- native codecs for the crate's wire formats (host code only).
//
// JSON follows serde's derived layouts with serde_json's compact output:
//   Poly (src/math/poly.rs:63-77)
//     {"coeffs":[..],"moduli":[..],"q":Q,"dim":D,"crt_q0_inv_mod_q1":I,"is_ntt":false}
//   SeededRlweCiphertext (rlwe/types.rs:165-171) {"seed":[32 bytes],"b":Poly}
//   GadgetVector (rgsw/types.rs:37-45) {"base":B,"len":L,"q":Q}
//   SeededRgswCiphertext (rgsw/types.rs:225-231) {"rows":[..],"gadget":G}
//   ClientPackingKeys (inspiring/inspiring2.rs:603-628)
//     {"y_body":[..],"z_body":[..] (omitted when empty),"full_key":b,"num_to_pack":n}
//   SeededClientQuery (pir/query.rs:138-150)
//     {"shard_id":s,"rgsw_ciphertext":R,"packing_mode":"inspiring"|"tree",
//      "inspiring_packing_keys":K (omitted when None)}
//   RlweCiphertext {"a":Poly,"b":Poly}; ServerResponse (pir/respond.rs:31-37)
//     {"ciphertext":C,"column_ciphertexts":[..]}
//   the server's QueryResponse (src/bin/server.rs:88-92)
//     {"response":ServerResponse,"processing_time_ms":t}
// bincode 1.3's default encoding (fixed-width little-endian integers, u64
// sequence lengths, bool as one byte) for ServerResponse::to_binary
// (pir/respond.rs:43-50).
#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include <unistd.h>

#include "host.h"
#include "json_codec.h"

using namespace ighost;
using namespace igjson;

namespace {

// A Poly's "coeffs" array whose parse is deferred: the structural pass of a
// large query records where each array lies and the checks its Poly needs,
// and the arrays (independent of one another) are then parsed in parallel.
struct PolyJob {
  const char* lb;  // its '['
  const char* rb;  // its ']' (the first after lb; anything else fails the job)
  uint64_t* dst;
  size_t plen;
  uint64_t moduli[2];
  uint32_t ring_dim;
};

bool run_poly_job(const PolyJob& jb) {
  Json j{jb.lb, jb.rb + 1, "", jb.lb};
  size_t n = 0;
  if (!j.u64_array_into(jb.dst, jb.plen, &n) || j.p != jb.rb + 1 || n != jb.plen) return false;
  for (size_t r = 0; r < 2; r++) {
    const uint64_t m = jb.moduli[r], *d = jb.dst + r * jb.ring_dim;
    uint64_t bad = 0;
    for (size_t i = 0; i < jb.ring_dim; i++) bad |= (uint64_t)(d[i] >= m);
    if (bad) return false;
  }
  return true;
}

// Worker threads for the deferred arrays, shared by every caller; a caller
// that finds them busy parses its arrays itself.
class ParsePool {
 public:
  // Up to 8 workers (a seeded query with keys has 9 arrays: with the caller
  // they parse in one round), leaving two cores to the rest of the process.
  ParsePool() : pid_(getpid()) {
    const unsigned hw = std::max(3u, std::thread::hardware_concurrency());
    const unsigned n = std::min(8u, hw - 2);
    for (unsigned i = 0; i < n; i++) workers_.emplace_back([this] { work(); });
  }
  // Runs every job; true if all succeeded.
  bool run(const std::vector<PolyJob>& jobs) {
    std::unique_lock<std::mutex> busy(run_mu_, std::try_to_lock);
    // (a forked child has none of the workers: it parses on its own)
    if (!busy.owns_lock() || jobs.size() < 2 || getpid() != pid_) {
      bool ok = true;
      for (const PolyJob& jb : jobs) ok &= run_poly_job(jb);
      return ok;
    }
    {
      std::lock_guard<std::mutex> lk(mu_);
      jobs_ = &jobs;
      next_.store(0);
      failed_.store(false);
      pending_ = (int)workers_.size();
      gen_++;
    }
    cv_.notify_all();
    drain();
    std::unique_lock<std::mutex> lk(mu_);
    done_cv_.wait(lk, [&] { return pending_ == 0; });
    jobs_ = nullptr;
    return !failed_.load();
  }

 private:
  void drain() {
    const std::vector<PolyJob>& jobs = *jobs_;
    for (size_t k; (k = next_.fetch_add(1)) < jobs.size();)
      if (!run_poly_job(jobs[k])) failed_.store(true);
  }
  void work() {
    uint64_t seen = 0;
    for (;;) {
      {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [&] { return gen_ != seen; });
        seen = gen_;
      }
      drain();
      std::lock_guard<std::mutex> lk(mu_);
      if (--pending_ == 0) done_cv_.notify_one();
    }
  }
  std::mutex run_mu_, mu_;
  std::condition_variable cv_, done_cv_;
  std::vector<std::thread> workers_;
  const std::vector<PolyJob>* jobs_ = nullptr;
  std::atomic<size_t> next_{0};
  std::atomic<bool> failed_{false};
  int pending_ = 0;
  uint64_t gen_ = 0;
  pid_t pid_;
};

ParsePool& parse_pool() {
  // never destroyed: its threads outlive every caller
  static ParsePool* pool = new ParsePool();
  return *pool;
}

// Queries at least this large have their coefficient arrays parsed in
// parallel (a SeededClientQuery with keys is ~355 KB).
constexpr size_t PARALLEL_PARSE_MIN_BYTES = 64 * 1024;

// Poly in coefficient form over the context's moduli, into dst[2N].  With
// `jobs`, the coefficient array is located but parsed later (PolyJob); the
// array's own checks then run with it.
bool parse_poly(Json& j, const inspire_params& P, uint64_t* dst, const std::string& what,
                std::vector<PolyJob>* jobs = nullptr) {
  const size_t plen = 2 * (size_t)P.ring_dim;
  uint64_t moduli[3] = {0, 0, 0};
  size_t ncoeffs = 0, nmod = 0;
  uint64_t dim = 0;
  bool is_ntt = false, have_coeffs = false, have_moduli = false;
  size_t job = SIZE_MAX;
  const bool ok = j.object([&](const std::string& k) {
    if (k == "coeffs") {
      if (have_coeffs) return j.fail("duplicate field `coeffs`");  // as serde's derive
      have_coeffs = true;
      if (jobs) {
        if (!j.eat('[')) return j.fail("expected '['");
        const char* lb = j.p - 1;
        const char* rb = static_cast<const char*>(memchr(j.p, ']', (size_t)(j.end - j.p)));
        if (!rb) return j.fail("unterminated array");
        job = jobs->size();
        jobs->push_back({lb, rb, dst, plen, {0, 0}, P.ring_dim});
        j.p = rb + 1;
        ncoeffs = plen;
        return true;
      }
      return j.u64_array_into(dst, plen, &ncoeffs);  // parsed in place, checked below
    }
    if (k == "moduli") {
      if (have_moduli) return j.fail("duplicate field `moduli`");
      have_moduli = true;
      return j.u64_array_into(moduli, 3, &nmod);
    }
    if (k == "dim") return j.u64(dim);
    if (k == "is_ntt") return j.boolean(is_ntt);
    return j.skip();  // q, crt_q0_inv_mod_q1 are derived from the moduli
  });
  if (!ok) return false;
  if (!have_coeffs || !have_moduli) return j.fail(what + ": missing coeffs or moduli");
  if (nmod != 2 || moduli[0] != P.crt_moduli[0] || moduli[1] != P.crt_moduli[1])
    return j.fail(what + ": moduli differ from the context");
  if (dim != P.ring_dim || ncoeffs != plen) return j.fail(what + ": dimension mismatch");
  if (is_ntt) return j.fail(what + ": expected coefficient form (is_ntt false)");
  if (job != SIZE_MAX) {  // count and residues are checked by the job
    (*jobs)[job].moduli[0] = moduli[0];
    (*jobs)[job].moduli[1] = moduli[1];
    return true;
  }
  for (size_t r = 0; r < 2; r++) {  // residue-major: coefficient i of residue r at r * ring_dim + i
    const uint64_t m = moduli[r], *d = dst + r * P.ring_dim;
    uint64_t bad = 0;
    for (size_t i = 0; i < (size_t)P.ring_dim; i++) bad |= (uint64_t)(d[i] >= m);
    if (bad) return j.fail(what + ": residue not reduced");
  }
  return true;
}


uint64_t q0_inv_q1(uint64_t q0, uint64_t q1) {
  // Poly::init_moduli's cached q0^-1 mod q1 (q1 prime): q0^(q1-2) mod q1
  unsigned __int128 r = 1, b = q0 % q1;
  uint64_t e = q1 - 2;
  while (e) {
    if (e & 1) r = r * b % q1;
    b = b * b % q1;
    e >>= 1;
  }
  return (uint64_t)r;
}

void poly_json(Out& o, const inspire_params& P, const uint64_t* c) {
  const size_t n = 2 * (size_t)P.ring_dim;
  o.lit("{\"coeffs\":[");
  o.nums(c, n);
  o.lit("],\"moduli\":[");
  o.num(P.crt_moduli[0]);
  o.ch(',');
  o.num(P.crt_moduli[1]);
  o.lit("],\"q\":");
  o.num(P.crt_moduli[0] * P.crt_moduli[1]);
  o.lit(",\"dim\":");
  o.num(P.ring_dim);
  o.lit(",\"crt_q0_inv_mod_q1\":");
  o.num(q0_inv_q1(P.crt_moduli[0], P.crt_moduli[1]));
  o.lit(",\"is_ntt\":false}");
}

// Poly of `dim` coefficients per residue (dim may differ from ring_dim: the
// crate's compat tree-packing b has dimension 2 ring_dim).
void poly_json_dim(Out& o, const inspire_params& P, const uint64_t* c, size_t dim) {
  o.lit("{\"coeffs\":[");
  o.nums(c, 2 * dim);
  o.lit("],\"moduli\":[");
  o.num(P.crt_moduli[0]);
  o.ch(',');
  o.num(P.crt_moduli[1]);
  o.lit("],\"q\":");
  o.num(P.crt_moduli[0] * P.crt_moduli[1]);
  o.lit(",\"dim\":");
  o.num(dim);
  o.lit(",\"crt_q0_inv_mod_q1\":");
  o.num(q0_inv_q1(P.crt_moduli[0], P.crt_moduli[1]));
  o.lit(",\"is_ntt\":false}");
}

// An f64 as serde_json writes it: the shortest decimal that reads back to
// the same value, with ".0" on integral values.
void f64_json(Out& o, double v) {
  char b[40];
  for (int prec = 1; prec <= 17; prec++) {
    snprintf(b, sizeof b, "%.*g", prec, v);
    if (strtod(b, nullptr) == v) break;
  }
  std::string t(b);
  const size_t e = t.find('e');
  if (e != std::string::npos) {  // 1e-07 -> 1e-7, 1e+21 -> 1e21
    std::string m = t.substr(0, e), x = t.substr(e + 1);
    bool neg = !x.empty() && x[0] == '-';
    if (!x.empty() && (x[0] == '-' || x[0] == '+')) x = x.substr(1);
    while (x.size() > 1 && x[0] == '0') x = x.substr(1);
    t = m + "e" + (neg ? "-" : "") + x;
  } else if (t.find('.') == std::string::npos) {
    t += ".0";
  }
  o.lit(t.c_str());
}

void gadget_json(Out& o, const inspire_params& P) {
  o.lit("{\"base\":");
  o.num(P.gadget_base);
  o.lit(",\"len\":");
  o.num(P.gadget_len);
  o.lit(",\"q\":");
  o.num(P.crt_moduli[0] * P.crt_moduli[1]);
  o.ch('}');
}

void rlwe_json(Out& o, const inspire_params& P, const uint64_t* ct);

// KeySwitchingMatrix {rows: [RlweCiphertext; gadget_len], gadget} (ks/setup.rs:40-46)
// from rows [gadget_len][a, b][poly].
void ksm_json(Out& o, const inspire_params& P, const uint64_t* m) {
  o.lit("{\"rows\":[");
  for (uint32_t k = 0; k < P.gadget_len; k++) {
    if (k) o.ch(',');
    rlwe_json(o, P, m + (size_t)k * 4 * P.ring_dim);
  }
  o.lit("],\"gadget\":");
  gadget_json(o, P);
  o.ch('}');
}

void seed_json(Out& o, const uint8_t* s) {
  o.ch('[');
  for (int i = 0; i < 32; i++) {
    if (i) o.ch(',');
    o.num(s[i]);
  }
  o.ch(']');
}

void rlwe_json(Out& o, const inspire_params& P, const uint64_t* ct) {
  o.lit("{\"a\":");
  poly_json(o, P, ct);
  o.lit(",\"b\":");
  poly_json(o, P, ct + 2 * (size_t)P.ring_dim);
  o.ch('}');
}

template <class T>
void le(std::string& s, T v) {
  for (size_t i = 0; i < sizeof(T); i++) s.push_back((char)(uint8_t)(v >> (8 * i)));
}

bool host_is_le() {
  const uint32_t one = 1;
  uint8_t b;
  memcpy(&b, &one, 1);
  return b == 1;
}

void poly_bincode(std::string& s, const inspire_params& P, const uint64_t* c) {
  const uint64_t n = 2 * (uint64_t)P.ring_dim;
  le<uint64_t>(s, n);
  if (host_is_le()) {
    const size_t at = s.size();
    s.resize(at + 8 * n);
    memcpy(&s[at], c, 8 * n);
  } else {
    for (uint64_t i = 0; i < n; i++) le<uint64_t>(s, c[i]);
  }
  le<uint64_t>(s, 2);
  le<uint64_t>(s, P.crt_moduli[0]);
  le<uint64_t>(s, P.crt_moduli[1]);
  le<uint64_t>(s, P.crt_moduli[0] * P.crt_moduli[1]);
  le<uint64_t>(s, P.ring_dim);
  le<uint64_t>(s, q0_inv_q1(P.crt_moduli[0], P.crt_moduli[1]));
  s.push_back(0);  // is_ntt
}

int copy_out(const char* data, size_t size, char* buf, size_t cap, size_t* len) {
  *len = size;
  if (!buf) return INSPIRE_OK;  // size query
  if (cap < size) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "output buffer too small");
  memcpy(buf, data, size);
  return INSPIRE_OK;
}
int copy_out(const std::string& s, char* buf, size_t cap, size_t* len) { return copy_out(s.data(), s.size(), buf, cap, len); }
int copy_out(const Out& o, char* buf, size_t cap, size_t* len) { return copy_out(o.data(), o.n, buf, cap, len); }

bool params_ok(const inspire_params* P) {
  return P && P->ring_dim > 0 && P->crt_count == 2 && P->gadget_len > 0 && P->crt_moduli[0] > 1 &&
         P->crt_moduli[1] > 1;
}

}  // namespace

namespace {

// SeededClientQuery (seeded rows {seed, b}) or ClientQuery (full rows
// {a, b}, RgswCiphertext rgsw/types.rs:100-110) JSON; see the header.
int query_from_json_pass(const inspire_params* P, const char* json, size_t len, bool seeded, uint32_t* shard_id,
                         uint8_t* seeds, uint64_t* rows, int32_t* packing_mode, int32_t* has_keys, uint64_t* y_body,
                         std::vector<PolyJob>* jobs) {
  const char* what_q = seeded ? "SeededClientQuery JSON: " : "ClientQuery JSON: ";
  if (!params_ok(P) || !json || !shard_id || (seeded && !seeds) || !rows || !packing_mode || !has_keys)
    return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null argument or unsupported parameters");
  const size_t plen = 2 * (size_t)P->ring_dim;
  const uint32_t rows_want = 2 * P->gadget_len;
  Json j{json, json + len, "", json};
  uint64_t sid = 0;
  bool have_sid = false, have_rgsw = false;
  int mode = 0;
  int keys = 0;
  const bool ok = j.object([&](const std::string& k) -> bool {
    if (k == "shard_id") {
      have_sid = true;
      return j.u64(sid) && (sid <= 0xffffffffULL || j.fail("shard_id out of range"));
    }
    if (k == "rgsw_ciphertext") {
      have_rgsw = true;
      uint32_t nrows = 0;
      return j.object([&](const std::string& rk) -> bool {
        if (rk == "rows")
          return j.array([&](size_t i) -> bool {
            if (i >= rows_want) return j.fail("too many RGSW rows");
            nrows = (uint32_t)i + 1;
            bool have_first = false, have_b = false;
            const bool rok = j.object([&](const std::string& fk) -> bool {
              if (seeded && fk == "seed") {
                have_first = true;
                size_t nb = 0;
                return j.array([&](size_t bi) -> bool {
                  uint64_t v;
                  if (bi >= 32 || !j.u64(v) || v > 255) return j.fail("seed must be 32 bytes");
                  seeds[i * 32 + bi] = (uint8_t)v;
                  nb = bi + 1;
                  return true;
                }) && (nb == 32 || j.fail("seed must be 32 bytes"));
              }
              if (!seeded && fk == "a") {
                have_first = true;
                return parse_poly(j, *P, rows + (2 * i) * plen, "rgsw row a", jobs);
              }
              if (fk == "b") {
                have_b = true;
                return parse_poly(j, *P, rows + (seeded ? i : 2 * i + 1) * plen, "rgsw row b", jobs);
              }
              return j.skip();
            });
            return rok && ((have_first && have_b) || j.fail(seeded ? "RGSW row needs seed and b" : "RGSW row needs a and b"));
          }) && (nrows == rows_want || j.fail("expected 2*gadget_len RGSW rows"));
        if (rk == "gadget") {
          uint64_t base = 0, glen = 0;
          return j.object([&](const std::string& gk) -> bool {
            if (gk == "base") return j.u64(base);
            if (gk == "len") return j.u64(glen);
            return j.skip();
          }) && ((base == P->gadget_base && glen == P->gadget_len) || j.fail("gadget differs from the context"));
        }
        return j.skip();
      });
    }
    if (k == "packing_mode") {
      std::string m;
      if (!j.str(m)) return false;
      if (m == "inspiring") mode = 0;
      else if (m == "tree") mode = 1;
      else return j.fail("unknown packing_mode");
      return true;
    }
    if (k == "inspiring_packing_keys") {
      if (j.null()) return true;  // Option::None
      size_t ny = 0;
      const bool kok = j.object([&](const std::string& kk) -> bool {
        if (kk == "y_body")
          return j.array([&](size_t i) -> bool {
            if (i >= P->gadget_len) return j.fail("too many y_body polynomials");
            ny = i + 1;
            if (!y_body) return j.skip();
            return parse_poly(j, *P, y_body + i * plen, "y_body", jobs);
          }) && (ny == 0 || ny == P->gadget_len || j.fail("y_body must hold gadget_len polynomials"));
        return j.skip();  // z_body, full_key, num_to_pack
      });
      keys = ny ? 1 : 2;  // 2: keys present with an empty y_body (rejected by respond)
      return kok;
    }
    return j.skip();
  });
  if (!ok) return fail(INSPIRE_ERR_INVALID_ARGUMENT, what_q + j.err);
  j.ws();
  if (j.p != j.end) return fail(INSPIRE_ERR_INVALID_ARGUMENT, std::string(what_q) + "trailing data");
  if (!have_sid || !have_rgsw)
    return fail(INSPIRE_ERR_INVALID_ARGUMENT, std::string(what_q) + "missing shard_id or rgsw_ciphertext");
  *shard_id = (uint32_t)sid;
  *packing_mode = mode;
  *has_keys = keys;
  return INSPIRE_OK;
}

// Large queries: a structural pass that defers the coefficient arrays, which
// are then parsed in parallel.  Any failure re-parses the query in one pass,
// which reports the first error exactly as the sequential parser does.
int query_from_json(const inspire_params* P, const char* json, size_t len, bool seeded, uint32_t* shard_id,
                    uint8_t* seeds, uint64_t* rows, int32_t* packing_mode, int32_t* has_keys, uint64_t* y_body) {
  if (len >= PARALLEL_PARSE_MIN_BYTES && json) {
    std::vector<PolyJob> jobs;
    jobs.reserve(16);
    if (query_from_json_pass(P, json, len, seeded, shard_id, seeds, rows, packing_mode, has_keys, y_body, &jobs) ==
            INSPIRE_OK &&
        parse_pool().run(jobs))
      return INSPIRE_OK;
  }
  return query_from_json_pass(P, json, len, seeded, shard_id, seeds, rows, packing_mode, has_keys, y_body, nullptr);
}

}  // namespace

extern "C" {

int inspire_seeded_query_from_json(const inspire_params* P, const char* json, size_t len, uint32_t* shard_id,
                                   uint8_t* seeds, uint64_t* b_rows, int32_t* packing_mode, int32_t* has_keys,
                                   uint64_t* y_body) {
  return query_from_json(P, json, len, true, shard_id, seeds, b_rows, packing_mode, has_keys, y_body);
}

int inspire_query_from_json(const inspire_params* P, const char* json, size_t len, uint32_t* shard_id,
                            uint64_t* rgsw, int32_t* packing_mode, int32_t* has_keys, uint64_t* y_body) {
  return query_from_json(P, json, len, false, shard_id, nullptr, rgsw, packing_mode, has_keys, y_body);
}

int inspire_query_response_to_json(const inspire_params* P, const uint64_t* ct, uint32_t n_columns,
                                   const uint64_t* columns, uint64_t processing_time_ms, char* buf, size_t cap,
                                   size_t* len) {
  if (!params_ok(P) || !ct || !len || (n_columns && !columns)) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null argument");
  Out o;
  // every coefficient array's worst-case reservation fits without growing
  o.reserve((size_t)(2 + 2 * n_columns) * 2 * P->ring_dim * 21 + 512);
  o.lit("{\"response\":{\"ciphertext\":");
  rlwe_json(o, *P, ct);
  o.lit(",\"column_ciphertexts\":[");
  for (uint32_t c = 0; c < n_columns; c++) {
    if (c) o.ch(',');
    rlwe_json(o, *P, columns + (size_t)c * 4 * P->ring_dim);
  }
  o.lit("]},\"processing_time_ms\":");
  o.num(processing_time_ms);
  o.ch('}');
  return copy_out(o, buf, cap, len);
}

int inspire_server_response_to_bincode(const inspire_params* P, const uint64_t* ct, uint32_t n_columns,
                                       const uint64_t* columns, uint8_t* buf, size_t cap, size_t* len) {
  if (!params_ok(P) || !ct || !len || (n_columns && !columns)) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null argument");
  std::string s;
  const size_t plen = 2 * (size_t)P->ring_dim;
  s.reserve((2 + 2 * (size_t)n_columns) * (8 * plen + 64) + 8);
  poly_bincode(s, *P, ct);
  poly_bincode(s, *P, ct + plen);
  le<uint64_t>(s, n_columns);
  for (uint32_t c = 0; c < n_columns; c++) {
    poly_bincode(s, *P, columns + (size_t)c * 2 * plen);
    poly_bincode(s, *P, columns + (size_t)c * 2 * plen + plen);
  }
  return copy_out(s, reinterpret_cast<char*>(buf), cap, len);
}

int inspire_crs_load_json(inspire_ctx* c, const char* json, size_t len) {
  if (!c || !json) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null argument");
  const inspire_params P = c->params;
  Json j{json, json + len, "", json};
  uint8_t w_seed[32] = {};
  size_t nseed = 0;
  uint64_t num_columns = 0;
  bool have_seed = false, have_cols = false, have_params = false;
  std::vector<uint64_t> keys;  // [matrix][row][a, b][poly]
  size_t nmat = 0;
  uint64_t n_crs_a = 0;
  const size_t pw = 2 * (size_t)P.ring_dim;
  const bool ok = j.object([&](const std::string& k) {
    if (k == "params") {
      have_params = true;
      uint64_t ring_dim = 0, q = 0, p = 0, gbase = 0, glen = 0;
      uint64_t mod[3] = {0, 0, 0};
      size_t nmod = 0;
      const bool pok = j.object([&](const std::string& f) {
        if (f == "ring_dim") return j.u64(ring_dim);
        if (f == "q") return j.u64(q);
        if (f == "crt_moduli") return j.u64_array_into(mod, 3, &nmod);
        if (f == "p") return j.u64(p);
        if (f == "gadget_base") return j.u64(gbase);
        if (f == "gadget_len") return j.u64(glen);
        return j.skip();  // sigma, security_level
      });
      if (!pok) return false;
      if (ring_dim != P.ring_dim || nmod != 2 || mod[0] != P.crt_moduli[0] || mod[1] != P.crt_moduli[1] ||
          p != P.p || gbase != P.gadget_base || glen != P.gadget_len)
        return j.fail("params differ from the context's");
      return true;
    }
    if (k == "galois_keys") {
      return j.array([&](size_t) {  // KeySwitchingMatrix {rows, gadget}
        size_t nrows = 0;
        keys.resize((nmat + 1) * 2 * ELL * pw);
        const bool mok = j.object([&](const std::string& f) {
          if (f == "rows") {
            return j.array([&](size_t) {  // RlweCiphertext {a, b}
              if (nrows >= (size_t)ELL) return j.fail("a Galois key has more than gadget_len rows");
              const bool rok = j.object([&](const std::string& g) {
                if (g == "a" || g == "b") {
                  uint64_t* dst = keys.data() + ((nmat * ELL + nrows) * 2 + (g == "b")) * pw;
                  return parse_poly(j, P, dst, "Galois key " + std::to_string(nmat) + " row " + std::to_string(nrows));
                }
                return j.skip();
              });
              nrows++;
              return rok;
            });
          }
          return j.skip();  // gadget
        });
        if (!mok) return false;
        if (nrows != (size_t)ELL) return j.fail("a Galois key has fewer than gadget_len rows");
        nmat++;
        return true;
      });
    }
    if (k == "inspiring_w_seed") {
      have_seed = true;
      uint64_t v[32];
      if (!j.u64_array_into(v, 32, &nseed)) return false;
      for (size_t i = 0; i < nseed; i++) {
        if (v[i] > 255) return j.fail("inspiring_w_seed bytes must be < 256");
        w_seed[i] = (uint8_t)v[i];
      }
      return nseed == 32 || j.fail("inspiring_w_seed must hold 32 bytes");
    }
    if (k == "inspiring_num_columns") {
      have_cols = true;
      return j.u64(num_columns);
    }
    if (k == "crs_a_vectors")  // counted (the server's /params reports it), not kept
      return j.array([&](size_t) {
        n_crs_a++;
        return j.skip();
      });
    return j.skip();  // k_g, k_h, rgsw_gadget, packing_k_*, inspiring_precomp, inspiring_v_seed
  });
  if (ok) j.ws();
  if (!ok || j.p != j.end)
    return fail(INSPIRE_ERR_INVALID_ARGUMENT, "ServerCrs JSON: " + (j.err.empty() ? std::string("trailing characters") : j.err));
  if (!have_params || !have_seed || !have_cols)
    return fail(INSPIRE_ERR_INVALID_ARGUMENT, "ServerCrs JSON: missing params, inspiring_w_seed or inspiring_num_columns");
  if (num_columns > 0xffffffffull) return fail(INSPIRE_ERR_UNSUPPORTED, "GPU path supports num_columns in {1, 2, 4, 8, 16}");
  if (int rc = inspire_crs_load(c, w_seed, (uint32_t)num_columns)) return rc;
  c->crs_a_count = n_crs_a;
  // galois_keys is empty in CRSs made without tree packing; a tree-packing
  // call then reports the missing keys
  if (nmat > 0) return inspire_crs_load_galois_keys(c, keys.data(), (uint32_t)nmat);
  return INSPIRE_OK;
}

int inspire_db_load_json(inspire_ctx* c, const char* json, size_t len, inspire_db** out) {
  if (!c || !json || !out) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null argument");
  std::lock_guard<std::mutex> lk(c->mu);
  *out = nullptr;
  if (!c->has_crs) return fail(INSPIRE_ERR_NO_CRS, "no CRS loaded (inspire_crs_load)");
  const int gamma = c->gamma;
  const inspire_params& P = c->params;
  Json j{json, json + len, "", json};
  std::vector<uint16_t> H;
  std::vector<uint64_t> poly(2 * (size_t)N);
  uint64_t entry_size = 0, total_entries = 0;
  bool have_shards = false, have_config = false;
  int nshards = 0;
  const bool ok = j.object([&](const std::string& k) {
    if (k == "shards") {
      have_shards = true;
      return j.array([&](size_t) {
        uint64_t id = ~0ull;
        int npolys = 0;
        const bool sok = j.object([&](const std::string& f) {
          if (f == "id") return j.u64(id);
          if (f == "polynomials") {
            return j.array([&](size_t) {
              const std::string what = "shard " + std::to_string(nshards) + " polynomial " + std::to_string(npolys);
              if (npolys >= gamma) return j.fail(what + ": the CRS packs " + std::to_string(gamma) + " columns");
              if (!parse_poly(j, P, poly.data(), what)) return false;
              H.resize((size_t)(nshards + 1) * gamma * N);
              uint16_t* dst = H.data() + ((size_t)nshards * gamma + npolys) * N;
              for (int i = 0; i < N; i++) {
                if (poly[i] >= 65536 || poly[N + i] != poly[i])
                  return j.fail(what + ": not an encoded 16-bit column (coefficient " + std::to_string(i) + ")");
                dst[i] = (uint16_t)poly[i];
              }
              npolys++;
              return true;
            });
          }
          return j.skip();
        });
        if (!sok) return false;
        if (id != (uint64_t)nshards) return j.fail("shard ids must be 0, 1, ... in order");
        if (npolys != gamma)
          return j.fail("shard " + std::to_string(nshards) + ": " + std::to_string(npolys) +
                        " polynomials, the CRS packs " + std::to_string(gamma));
        if (nshards == 0x7fffffff) return j.fail("too many shards");
        nshards++;
        return true;
      });
    }
    if (k == "config") {
      have_config = true;
      return j.object([&](const std::string& f) {
        if (f == "entry_size_bytes") return j.u64(entry_size);
        if (f == "total_entries") return j.u64(total_entries);
        return j.skip();  // shard_size_bytes
      });
    }
    return j.skip();
  });
  if (ok) j.ws();
  if (!ok || j.p != j.end)
    return fail(INSPIRE_ERR_INVALID_ARGUMENT,
                "EncodedDatabase JSON: " + (j.err.empty() ? std::string("trailing characters") : j.err));
  if (!have_shards || !have_config) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "EncodedDatabase JSON: missing shards or config");
  if ((entry_size * 8 + 15) / 16 != (uint64_t)gamma)
    return fail(INSPIRE_ERR_INVALID_ARGUMENT, "ceil(entry_size/2) must equal the CRS num_columns");
  if (total_entries > (uint64_t)nshards * N)
    return fail(INSPIRE_ERR_INVALID_ARGUMENT, "total_entries exceeds the shards' capacity");
  if (int rc = set_device(c)) return rc;
  return db_from_host_columns(c, H.data(), nshards, total_entries, (uint32_t)entry_size, out);
}

uint64_t inspire_crs_a_vectors_count(const inspire_ctx* c) { return c ? c->crs_a_count : 0; }

int inspire_packed_response_to_json(const inspire_params* P, const uint64_t* a, const uint64_t* b, uint32_t b_words,
                                    uint64_t processing_time_ms, char* buf, size_t cap, size_t* len) {
  if (!params_ok(P) || !a || !b || !len) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null argument");
  if (b_words == 0 || b_words % 2) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "b_words must be a positive even count");
  Out o;
  o.reserve((size_t)(2 * P->ring_dim + b_words) * 21 + 1024);
  o.lit("{\"response\":{\"ciphertext\":{\"a\":");
  poly_json_dim(o, *P, a, P->ring_dim);
  o.lit(",\"b\":");
  poly_json_dim(o, *P, b, b_words / 2);
  o.lit("},\"column_ciphertexts\":[]},\"processing_time_ms\":");
  o.num(processing_time_ms);
  o.ch('}');
  return copy_out(o, buf, cap, len);
}

int inspire_crs_write_json(const inspire_params* P, const inspire_server_crs* crs, const char* path) {
  if (!params_ok(P) || !crs || !path) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null argument");
  if (!crs->k_g || !crs->k_h || (crs->n_galois && !crs->galois_keys) || (crs->n_crs_a && !crs->crs_a_vectors) ||
      (crs->precomp_a_hat && crs->inspiring_num_columns > 1 && !crs->precomp_bold_t))
    return fail(INSPIRE_ERR_INVALID_ARGUMENT, "missing ServerCrs part");
  const size_t pw = 2 * (size_t)P->ring_dim;
  FILE* f = fopen(path, "wb");
  if (!f) return fail(INSPIRE_ERR_INVALID_ARGUMENT, std::string("cannot create ") + path);
  Out o;
  o.reserve(1 << 24);
  bool io_ok = true;
  auto flush = [&](bool force) {
    if (o.n >= (1u << 23) || (force && o.n)) {
      io_ok &= fwrite(o.data(), 1, o.n, f) == o.n;
      o.n = 0;
    }
  };
  const uint64_t q = P->crt_moduli[0] * P->crt_moduli[1];
  o.lit("{\"params\":{\"ring_dim\":");
  o.num(P->ring_dim);
  o.lit(",\"q\":");
  o.num(q);
  o.lit(",\"crt_moduli\":[");
  o.num(P->crt_moduli[0]);
  o.ch(',');
  o.num(P->crt_moduli[1]);
  o.lit("],\"p\":");
  o.num(P->p);
  o.lit(",\"sigma\":");
  f64_json(o, P->sigma);
  o.lit(",\"gadget_base\":");
  o.num(P->gadget_base);
  o.lit(",\"gadget_len\":");
  o.num(P->gadget_len);
  o.lit(",\"security_level\":\"Bits128\"},\"k_g\":");
  ksm_json(o, *P, crs->k_g);
  o.lit(",\"k_h\":");
  ksm_json(o, *P, crs->k_h);
  o.lit(",\"galois_keys\":[");
  for (uint32_t i = 0; i < crs->n_galois; i++) {
    if (i) o.ch(',');
    ksm_json(o, *P, crs->galois_keys + (size_t)i * P->gadget_len * 2 * pw);
    flush(false);
  }
  o.lit("],\"rgsw_gadget\":");
  gadget_json(o, *P);
  o.lit(",\"crs_a_vectors\":[");
  for (uint32_t i = 0; i < crs->n_crs_a; i++) {
    if (i) o.ch(',');
    o.ch('[');
    const uint64_t* v = crs->crs_a_vectors + (size_t)i * pw;
    for (size_t t = 0; t < pw; t++) {
      if (t) o.ch(',');
      o.num(v[t]);
    }
    o.ch(']');
    flush(false);
  }
  o.lit("],\"packing_k_g\":");
  if (crs->packing_k_g) ksm_json(o, *P, crs->packing_k_g);
  else o.lit("null");
  o.lit(",\"packing_k_h\":");
  if (crs->packing_k_h) ksm_json(o, *P, crs->packing_k_h);
  else o.lit("null");
  o.lit(",\"inspiring_precomp\":");
  if (crs->precomp_a_hat) {
    // PrecompInsPIR (inspiring/inspiring2.rs:357-375; bold_t_ntt is not serialised)
    o.lit("{\"a_hat\":");
    poly_json_dim(o, *P, crs->precomp_a_hat, P->ring_dim);
    o.lit(",\"bold_t\":[");
    const uint32_t nt = crs->inspiring_num_columns > 0 ? crs->inspiring_num_columns - 1 : 0;
    for (uint32_t i = 0; i < nt; i++) {
      if (i) o.ch(',');
      o.ch('[');
      for (uint32_t k = 0; k < P->gadget_len; k++) {
        if (k) o.ch(',');
        poly_json_dim(o, *P, crs->precomp_bold_t + ((size_t)i * P->gadget_len + k) * pw, P->ring_dim);
      }
      o.ch(']');
      flush(false);
    }
    o.lit("],\"bold_t_bar\":[],\"bold_t_hat\":[],\"num_to_pack\":");
    o.num(crs->inspiring_num_columns);
    o.lit(",\"ring_dim\":");
    o.num(P->ring_dim);
    o.lit(",\"q\":");
    o.num(q);
    o.ch('}');
  } else {
    o.lit("null");
  }
  o.lit(",\"inspiring_w_seed\":");
  seed_json(o, crs->inspiring_w_seed);
  o.lit(",\"inspiring_v_seed\":");
  seed_json(o, crs->inspiring_v_seed);
  o.lit(",\"inspiring_num_columns\":");
  o.num(crs->inspiring_num_columns);
  o.ch('}');
  flush(true);
  io_ok &= fclose(f) == 0;
  if (!io_ok) return fail(INSPIRE_ERR_INVALID_ARGUMENT, std::string("write failed: ") + path);
  return INSPIRE_OK;
}

}  // extern "C"
