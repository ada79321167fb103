// http.cu -- native HTTP front end of the Respond path (host code only):
// the routes, JSON shapes, status codes and error texts of the crate's
// server binary (src/bin/server.rs:88-236, 311-317) over the C ABI:
//
//   GET  /health        {"status":"ok","version":"0.1.2"}
//   GET  /params        ParamsResponse (:106-118)
//   GET  /crs           the crs.json the server was started with
//   POST /query         ClientQuery        -> QueryResponse (:120-177)
//   POST /query_seeded  SeededClientQuery  -> QueryResponse (:179-236)
//
// One thread per connection (HTTP/1.1 keep-alive; request bodies by
// Content-Length or chunked).  Seeded InspiRING queries go through the
// serving loop given at start (inspire_server_submit / poll), so the
// queries of all connections share GPU batches; the other kinds use the
// synchronous entry points.  The packing keys in each query are kept
// resident: clients are keyed by a 128-bit hash of y_body, registered on
// first use, evicted least-recently-used beyond max_clients or when the
// context's device budget refuses a new one.
#include <arpa/inet.h>
#include <netinet/in.h>
#include <netinet/tcp.h>
#include <sys/socket.h>
#include <unistd.h>

#include <atomic>
#include <chrono>
#include <cstring>
#include <list>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "host.h"
#include "json_codec.h"

using namespace ighost;

namespace {

constexpr const char* KEYS_MISSING = "InspiRING packing keys missing (set packing_mode=tree to use tree packing)";

std::string json_escape(const std::string& s) {
  std::string o;
  for (char c : s) {
    if (c == '"' || c == '\\') {
      o.push_back('\\');
      o.push_back(c);
    } else if ((unsigned char)c < 0x20) {
      char b[8];
      snprintf(b, sizeof b, "\\u%04x", (unsigned char)c);
      o += b;
    } else {
      o.push_back(c);
    }
  }
  return o;
}

struct Hash128 {
  uint64_t a, b;
  bool operator==(const Hash128& o) const { return a == o.a && b == o.b; }
};
struct Hash128H {
  size_t operator()(const Hash128& h) const { return (size_t)(h.a ^ (h.b * 0x9E3779B97F4A7C15ull)); }
};

uint64_t mix64(uint64_t x) {
  x ^= x >> 30;
  x *= 0xBF58476D1CE4E5B9ull;
  x ^= x >> 27;
  x *= 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// Two independent 64-bit running hashes over the words of y_body.
Hash128 hash_words(const uint64_t* w, size_t n) {
  uint64_t a = 0x6A09E667F3BCC908ull, b = 0xBB67AE8584CAA73Bull;
  for (size_t i = 0; i < n; i++) {
    a = mix64(a ^ w[i]) + i;
    b = mix64(b + w[i] * 0xD6E8FEB86659FD93ull) ^ (b >> 17);
  }
  return {mix64(a ^ n), mix64(b + n)};
}

}  // namespace

struct inspire_http_server {
  inspire_ctx* ctx = nullptr;
  const inspire_db* db = nullptr;
  inspire_server* srv = nullptr;
  inspire_http_config cfg{};
  std::string crs_json, version;
  uint64_t entry_count = 0, shard_count = 0;
  int listen_fd = -1;
  uint16_t port = 0;
  std::atomic<bool> stop{false};
  std::thread acceptor;
  // connections: each thread closes its socket when done; the acceptor
  // joins finished threads
  struct Conn {
    std::thread t;
    int fd;
    std::shared_ptr<std::atomic<bool>> done;
  };
  std::mutex conn_mu;
  std::list<Conn> conns;
  // resident client keys: hash -> (client id, queries in flight), LRU order
  struct Client {
    int32_t id;
    int inflight;
    std::list<Hash128>::iterator lru;
  };
  std::mutex keys_mu;
  std::unordered_map<Hash128, Client, Hash128H> clients;
  std::list<Hash128> lru;  // most recent at the back

  void accept_loop();
  void serve(int fd);
  bool handle(int fd, const std::string& method, const std::string& path, const std::string& ctype,
              const std::string& body, bool keep_alive);
  int acquire_client(const uint64_t* y_body, Hash128* h, int32_t* id);
  void release_client(const Hash128& h);
};

namespace {

bool send_all(int fd, const char* p, size_t n) {
  while (n) {
    const ssize_t k = ::send(fd, p, n, MSG_NOSIGNAL);
    if (k <= 0) return false;
    p += k;
    n -= (size_t)k;
  }
  return true;
}

bool reply(int fd, int status, const char* reason, const std::string& ctype, const char* body, size_t n,
           bool keep_alive) {
  std::string h = "HTTP/1.1 " + std::to_string(status) + " " + reason + "\r\ncontent-type: " + ctype +
                  "\r\ncontent-length: " + std::to_string(n) + "\r\n" +
                  (keep_alive ? "" : "connection: close\r\n") + "\r\n";
  return send_all(fd, h.data(), h.size()) && send_all(fd, body, n);
}
bool reply(int fd, int status, const char* reason, const std::string& ctype, const std::string& body,
           bool keep_alive) {
  return reply(fd, status, reason, ctype, body.data(), body.size(), keep_alive);
}

const char* JSON = "application/json";
const char* TEXT = "text/plain; charset=utf-8";

std::string lower(std::string s) {
  for (char& c : s) c = (char)tolower((unsigned char)c);
  return s;
}

// A buffered reader over a socket.
struct Reader {
  int fd;
  std::string buf;
  size_t pos = 0;
  bool fill() {
    if (pos > 0 && pos == buf.size()) {
      buf.clear();
      pos = 0;
    }
    char tmp[65536];
    const ssize_t k = ::recv(fd, tmp, sizeof tmp, 0);
    if (k <= 0) return false;
    buf.append(tmp, (size_t)k);
    return true;
  }
  bool line(std::string& out) {  // without the CRLF
    for (;;) {
      const size_t e = buf.find('\n', pos);
      if (e != std::string::npos) {
        out.assign(buf, pos, e - pos);
        if (!out.empty() && out.back() == '\r') out.pop_back();
        pos = e + 1;
        return true;
      }
      if (buf.size() - pos > (1u << 16)) return false;  // header line too long
      if (!fill()) return false;
    }
  }
  // n bytes into `out`: what is buffered, then received straight into it (a
  // query body of ~355 KB is not copied through the line buffer, and a
  // connection's requests of one size reuse the string without refilling it)
  bool bytes(size_t n, std::string& out) {
    const size_t have = std::min(n, buf.size() - pos);
    out.resize(n);
    if (have) memcpy(&out[0], buf.data() + pos, have);
    pos += have;
    for (size_t got = have; got < n;) {
      const ssize_t k = ::recv(fd, &out[got], n - got, 0);
      if (k <= 0) return false;
      got += (size_t)k;
    }
    return true;
  }
};

}  // namespace

int inspire_http_server::acquire_client(const uint64_t* y_body, Hash128* h, int32_t* id) {
  const size_t words = (size_t)ELL * poly_words();
  *h = hash_words(y_body, words);
  {
    std::lock_guard<std::mutex> lk(keys_mu);
    auto it = clients.find(*h);
    if (it != clients.end()) {
      it->second.inflight++;
      lru.splice(lru.end(), lru, it->second.lru);
      *id = it->second.id;
      return INSPIRE_OK;
    }
  }
  int32_t cid = -1;
  for (;;) {
    const int rc = inspire_client_register(ctx, y_body, nullptr, &cid);
    if (rc == INSPIRE_OK) break;
    if (rc != INSPIRE_ERR_OUT_OF_MEMORY) return rc;
    // the device budget refused the keys: evict the least recently used idle client
    int32_t victim = -1;
    {
      std::lock_guard<std::mutex> lk(keys_mu);
      for (auto it = lru.begin(); it != lru.end(); ++it) {
        auto c = clients.find(*it);
        if (c->second.inflight == 0) {
          victim = c->second.id;
          clients.erase(c);
          lru.erase(it);
          break;
        }
      }
    }
    if (victim < 0) return rc;
    inspire_client_release(ctx, victim);
  }
  std::vector<int32_t> evict;
  {
    std::lock_guard<std::mutex> lk(keys_mu);
    auto it = clients.find(*h);
    if (it != clients.end()) {  // registered meanwhile by another connection
      it->second.inflight++;
      *id = it->second.id;
      evict.push_back(cid);
    } else {
      lru.push_back(*h);
      clients.emplace(*h, Client{cid, 1, std::prev(lru.end())});
      *id = cid;
      for (auto l = lru.begin(); l != lru.end() && clients.size() > cfg.max_clients;) {
        auto c = clients.find(*l);
        if (c->second.inflight == 0) {
          evict.push_back(c->second.id);
          clients.erase(c);
          l = lru.erase(l);
        } else {
          ++l;
        }
      }
    }
  }
  for (int32_t e : evict) inspire_client_release(ctx, e);
  return INSPIRE_OK;
}

void inspire_http_server::release_client(const Hash128& h) {
  std::lock_guard<std::mutex> lk(keys_mu);
  auto it = clients.find(h);
  if (it != clients.end()) it->second.inflight--;
}

bool inspire_http_server::handle(int fd, const std::string& method, const std::string& path, const std::string& ctype,
                                 const std::string& body, bool ka) {
  const inspire_params& P = ctx->params;
  if (path == "/health" || path == "/params" || path == "/crs") {
    if (method != "GET") return reply(fd, 405, "Method Not Allowed", TEXT, "", ka);
    if (path == "/health") return reply(fd, 200, "OK", JSON, "{\"status\":\"ok\",\"version\":\"0.1.2\"}", ka);
    if (path == "/params") {
      const uint64_t q = P.crt_moduli[0] * P.crt_moduli[1];
      const std::string b = "{\"version\":\"" + json_escape(version) + "\",\"ring_dim\":" + std::to_string(P.ring_dim) +
                            ",\"modulus\":\"" + std::to_string(q) + "\",\"plaintext_modulus\":" + std::to_string(P.p) +
                            ",\"gadget_base\":" + std::to_string(P.gadget_base) + ",\"gadget_len\":" +
                            std::to_string(P.gadget_len) + ",\"entry_count\":" + std::to_string(entry_count) +
                            ",\"shard_count\":" + std::to_string(shard_count) + ",\"crs_a_vectors_count\":" +
                            std::to_string(inspire_crs_a_vectors_count(ctx)) + "}";
      return reply(fd, 200, "OK", JSON, b, ka);
    }
    if (crs_json.empty())
      return reply(fd, 404, "Not Found", JSON, "{\"error\":\"this server was started without a crs.json\"}", ka);
    return reply(fd, 200, "OK", JSON, crs_json, ka);
  }
  const bool seeded = path == "/query_seeded";
  if (!seeded && path != "/query") return reply(fd, 404, "Not Found", TEXT, "", ka);
  if (method != "POST") return reply(fd, 405, "Method Not Allowed", TEXT, "", ka);
  const std::string ct = lower(ctype.substr(0, ctype.find(';')));
  std::string ctt = ct;
  while (!ctt.empty() && ctt.back() == ' ') ctt.pop_back();
  while (!ctt.empty() && ctt.front() == ' ') ctt.erase(0, 1);
  const bool json_ct = ctt == "application/json" ||
                       (ctt.rfind("application/", 0) == 0 && ctt.size() > 5 && ctt.substr(ctt.size() - 5) == "+json");
  if (!json_ct) return reply(fd, 415, "Unsupported Media Type", TEXT, "Expected request with `Content-Type: application/json`", ka);
  const size_t pw = poly_words();
  // per connection thread, reused by its requests (no zero fill per request;
  // the parser writes every word that is used)
  thread_local std::vector<uint64_t> rows, y_body, ct2;
  thread_local std::string out;
  rows.resize((seeded ? 1 : 2) * (size_t)2 * ELL * pw);
  y_body.resize((size_t)ELL * pw);
  uint8_t seeds[2 * ELL * 32];
  uint32_t sid = 0;
  int32_t mode = 0, keys = 0;
  const int prc = seeded ? inspire_seeded_query_from_json(&P, body.data(), body.size(), &sid, seeds, rows.data(), &mode,
                                                           &keys, y_body.data())
                         : inspire_query_from_json(&P, body.data(), body.size(), &sid, rows.data(), &mode, &keys,
                                                   y_body.data());
  if (prc != INSPIRE_OK) {
    // axum's Json extractor: 400 for a body that is not JSON, 422 for JSON
    // that does not deserialise into the target type
    const std::string err = inspire_last_error();
    igjson::Json j{body.data(), body.data() + body.size(), "", body.data()};
    const bool is_json = j.skip() && (j.ws(), j.p == j.end);
    if (!is_json)
      return reply(fd, 400, "Bad Request", TEXT, "Failed to parse the request body as JSON: " + j.err, ka);
    return reply(fd, 422, "Unprocessable Entity", TEXT,
                 "Failed to deserialize the JSON body into the target type: " + err, ka);
  }
  const auto t0 = std::chrono::steady_clock::now();
  const std::string prefix = seeded ? "Seeded query processing failed: " : "Query processing failed: ";
  auto ms_since = [&] {
    return (uint64_t)std::chrono::duration_cast<std::chrono::milliseconds>(std::chrono::steady_clock::now() - t0)
        .count();
  };
  auto fail_reply = [&](const std::string& msg) {
    return reply(fd, 400, "Bad Request", JSON, "{\"error\":\"" + json_escape(prefix + msg) + "\"}", ka);
  };
  size_t len = 0;
  if (mode == 1) {  // tree packing
    std::vector<uint64_t> a(pw), b(2 * pw);
    uint32_t words = 0;
    int rc;
    if (seeded) {
      inspire_seeded_query q{sid, seeds, rows.data(), 0, nullptr, nullptr};
      rc = inspire_respond_seeded_packed(ctx, db, &q, a.data(), b.data(), &words);
    } else {
      inspire_query q{sid, rows.data(), 0, nullptr, nullptr};
      rc = inspire_respond_one_packing(ctx, db, &q, a.data(), b.data(), &words);
    }
    if (rc != INSPIRE_OK) return fail_reply(inspire_last_error());
    const uint64_t ms = ms_since();
    if (out.size() < (pw + words) * 21 + 1024) out.resize((pw + words) * 21 + 1024);
    if (inspire_packed_response_to_json(&P, a.data(), b.data(), words, ms, &out[0], out.size(), &len) != INSPIRE_OK)
      return reply(fd, 500, "Internal Server Error", TEXT, inspire_last_error(), ka);
    return reply(fd, 200, "OK", JSON, out.data(), len, ka);
  }
  if (keys == 0) return reply(fd, 400, "Bad Request", JSON, std::string("{\"error\":\"") + KEYS_MISSING + "\"}", ka);
  ct2.resize(2 * pw);
  if (keys == 2 || !seeded || !srv) {
    // keys with an empty y_body (the crate's "keys invalid"), full queries,
    // or no serving loop: the synchronous call, keys in the query
    int rc;
    if (seeded) {
      inspire_seeded_query q{sid, seeds, rows.data(), 1, keys == 1 ? y_body.data() : nullptr, nullptr};
      rc = inspire_respond_seeded_inspiring(ctx, db, &q, ct2.data());
    } else {
      inspire_query q{sid, rows.data(), 1, keys == 1 ? y_body.data() : nullptr, nullptr};
      rc = inspire_respond_inspiring(ctx, db, &q, ct2.data());
    }
    if (rc != INSPIRE_OK) return fail_reply(inspire_last_error());
  } else {
    Hash128 h{};
    int32_t cid = -1;
    if (sid >= inspire_db_num_shards(db))  // the crate's lookup error, before any key work
      return fail_reply("Shard " + std::to_string(sid) + " not found");
    if (int rc = acquire_client(y_body.data(), &h, &cid)) {
      (void)rc;
      return fail_reply(inspire_last_error());
    }
    uint64_t ticket = 0;
    uint32_t acc = 0;
    int rc;
    const inspire_db* dbs[1] = {db};
    for (;;) {
      rc = inspire_server_submit(srv, 1, dbs, &sid, seeds, rows.data(), &cid, nullptr, 0, &ticket, &acc);
      if (!(rc == INSPIRE_ERR_BUSY && acc == 0)) break;
      std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
    if (acc == 1) rc = inspire_server_poll(srv, ticket, ct2.data(), nullptr, -1);
    release_client(h);
    if (rc != INSPIRE_OK) return fail_reply(inspire_last_error());
  }
  const uint64_t ms = ms_since();
  if (out.size() < 2 * pw * 21 + 1024) out.resize(2 * pw * 21 + 1024);
  if (inspire_query_response_to_json(&P, ct2.data(), 0, nullptr, ms, &out[0], out.size(), &len) != INSPIRE_OK)
    return reply(fd, 500, "Internal Server Error", TEXT, inspire_last_error(), ka);
  return reply(fd, 200, "OK", JSON, out.data(), len, ka);
}

void inspire_http_server::serve(int fd) {
  Reader r{fd};
  std::string line, body;
  for (;;) {
    if (!r.line(line)) break;
    if (line.empty()) continue;  // stray CRLF between requests
    const size_t s1 = line.find(' '), s2 = line.find(' ', s1 + 1);
    if (s1 == std::string::npos || s2 == std::string::npos) break;
    const std::string method = line.substr(0, s1);
    std::string path = line.substr(s1 + 1, s2 - s1 - 1);
    const std::string proto = line.substr(s2 + 1);
    const size_t qm = path.find('?');
    if (qm != std::string::npos) path.resize(qm);
    size_t clen = 0;
    bool chunked = false, ka = proto != "HTTP/1.0", bad = false;
    std::string ctype;
    for (;;) {
      if (!r.line(line)) return;
      if (line.empty()) break;
      const size_t c = line.find(':');
      if (c == std::string::npos) continue;
      const std::string k = lower(line.substr(0, c));
      size_t v0 = c + 1;
      while (v0 < line.size() && line[v0] == ' ') v0++;
      const std::string v = line.substr(v0);
      if (k == "content-length") {
        char* e = nullptr;
        const unsigned long long n = strtoull(v.c_str(), &e, 10);
        bad |= e == v.c_str();
        clen = (size_t)n;
      } else if (k == "transfer-encoding") {
        chunked = lower(v).find("chunked") != std::string::npos;
      } else if (k == "content-type") {
        ctype = v;
      } else if (k == "connection") {
        const std::string lv = lower(v);
        if (lv.find("close") != std::string::npos) ka = false;
        if (lv.find("keep-alive") != std::string::npos) ka = true;
      }
    }
    if (bad) {
      reply(fd, 400, "Bad Request", TEXT, "bad content-length", false);
      break;
    }
    if (chunked) {
      body.clear();
      for (;;) {
        if (!r.line(line)) return;
        const size_t n = strtoull(line.c_str(), nullptr, 16);
        if (n == 0) {
          while (r.line(line) && !line.empty()) {
          }
          break;
        }
        if (body.size() + n > cfg.max_body) {
          reply(fd, 413, "Payload Too Large", TEXT, "length limit exceeded", false);
          return;
        }
        std::string part;
        if (!r.bytes(n, part) || !r.line(line)) return;
        body += part;
      }
    } else {
      if (clen > cfg.max_body) {
        reply(fd, 413, "Payload Too Large", TEXT, "length limit exceeded", false);
        break;
      }
      if (!clen) body.clear();
      else if (!r.bytes(clen, body)) break;
    }
    if (!handle(fd, method, path, ctype, body, ka) || !ka) break;
  }
}

void inspire_http_server::accept_loop() {
  while (!stop.load()) {
    sockaddr_in a{};
    socklen_t al = sizeof a;
    const int fd = ::accept(listen_fd, reinterpret_cast<sockaddr*>(&a), &al);
    if (fd < 0) {
      if (stop.load()) break;
      continue;
    }
    int one = 1;
    setsockopt(fd, IPPROTO_TCP, TCP_NODELAY, &one, sizeof one);
    std::lock_guard<std::mutex> lk(conn_mu);
    for (auto it = conns.begin(); it != conns.end();) {  // reap finished connections
      if (it->done->load()) {
        it->t.join();
        it = conns.erase(it);
      } else {
        ++it;
      }
    }
    auto done = std::make_shared<std::atomic<bool>>(false);
    conns.push_back(Conn{std::thread([this, fd, done] {
                           cudaSetDevice(ctx->device);
                           serve(fd);
                           ::shutdown(fd, SHUT_RDWR);
                           done->store(true);
                         }),
                         fd, done});
  }
}

extern "C" {

void inspire_http_config_default(inspire_http_config* cfg) {
  if (!cfg) return;
  memset(cfg, 0, sizeof *cfg);
  cfg->host = "127.0.0.1";
  cfg->port = 0;
  cfg->max_clients = 4096;
  cfg->max_body = 64ull << 20;
  cfg->version = "1.0.0";
}

int inspire_http_start(inspire_ctx* ctx, const inspire_db* db, inspire_server* srv, const inspire_http_config* cfg,
                       const char* crs_json, size_t crs_len, inspire_http_server** out) {
  if (!ctx || !db || !cfg || !out || !cfg->host) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null argument");
  *out = nullptr;
  if (!ctx->has_crs) return fail(INSPIRE_ERR_NO_CRS, "no CRS loaded (inspire_crs_load)");
  auto s = std::make_unique<inspire_http_server>();
  s->ctx = ctx;
  s->db = db;
  s->srv = srv;
  s->cfg = *cfg;
  if (!s->cfg.max_clients) s->cfg.max_clients = 4096;
  if (!s->cfg.max_body) s->cfg.max_body = 64ull << 20;
  s->version = cfg->version ? cfg->version : "1.0.0";
  s->entry_count = cfg->entry_count;
  s->shard_count = cfg->shard_count;
  if (crs_json && crs_len) s->crs_json.assign(crs_json, crs_len);
  s->listen_fd = ::socket(AF_INET, SOCK_STREAM, 0);
  if (s->listen_fd < 0) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "socket() failed");
  int one = 1;
  setsockopt(s->listen_fd, SOL_SOCKET, SO_REUSEADDR, &one, sizeof one);
  sockaddr_in a{};
  a.sin_family = AF_INET;
  a.sin_port = htons(cfg->port);
  if (inet_pton(AF_INET, cfg->host, &a.sin_addr) != 1) {
    ::close(s->listen_fd);
    return fail(INSPIRE_ERR_INVALID_ARGUMENT, std::string("bad bind address ") + cfg->host);
  }
  if (::bind(s->listen_fd, reinterpret_cast<sockaddr*>(&a), sizeof a) != 0 || ::listen(s->listen_fd, 512) != 0) {
    ::close(s->listen_fd);
    return fail(INSPIRE_ERR_INVALID_ARGUMENT, std::string("cannot listen on ") + cfg->host + ":" +
                                                  std::to_string(cfg->port) + ": " + strerror(errno));
  }
  socklen_t al = sizeof a;
  getsockname(s->listen_fd, reinterpret_cast<sockaddr*>(&a), &al);
  s->port = ntohs(a.sin_port);
  inspire_http_server* raw = s.get();
  raw->acceptor = std::thread([raw] { raw->accept_loop(); });
  *out = s.release();
  return INSPIRE_OK;
}

uint16_t inspire_http_port(const inspire_http_server* s) { return s ? s->port : 0; }

void inspire_http_stop(inspire_http_server* s) {
  if (!s) return;
  s->stop.store(true);
  ::shutdown(s->listen_fd, SHUT_RDWR);
  ::close(s->listen_fd);
  if (s->acceptor.joinable()) s->acceptor.join();
  std::list<inspire_http_server::Conn> conns;
  {
    std::lock_guard<std::mutex> lk(s->conn_mu);
    for (auto& c : s->conns) ::shutdown(c.fd, SHUT_RDWR);  // ends each connection's blocking read
    conns.swap(s->conns);
  }
  for (auto& c : conns) {
    if (c.t.joinable()) c.t.join();
    ::close(c.fd);
  }
  for (auto& kv : s->clients) inspire_client_release(s->ctx, kv.second.id);
  delete s;
}

}  // extern "C"
