// dbio.cu -- the crate's binary shard files <-> the resident database.
//
// File format (save_shards_binary / load_shard_binary, src/pir/mmap.rs:19-87),
// one file per shard, `shard-{id:04}.bin`, little-endian:
//   u32 id, u32 num_polys, u32 ring_dim, u32 crt_count, u64 moduli[crt_count],
//   then num_polys polynomials of ring_dim * crt_count u64 residues
//   (residue-major, the layout of Poly::coeffs).
// A directory is read the way MmapDatabase::open counts it (mmap.rs:97-111):
// every file whose name starts with "shard-" is one shard, and shards are
// looked up by id as shard-{id:04}.bin, so ids 0..n-1 must all exist.
//
// The encoded database's polynomials hold one 16-bit column value per
// coefficient (encode_database, src/pir/encode_db.rs:106-164), identical in
// every residue; the loader checks that, keeps the raw columns and builds the
// Respond kernel's contracted form on the GPU exactly as inspire_db_create.
#include <dirent.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "host.h"

using namespace ig;
using namespace ighost;

namespace {

std::string shard_path(const std::string& dir, uint32_t id) {
  char name[32];
  snprintf(name, sizeof(name), "shard-%04u.bin", id);
  return dir + "/" + name;
}

template <class T>
bool read_le(FILE* f, T* v) {
  uint8_t b[sizeof(T)];
  if (fread(b, 1, sizeof(T), f) != sizeof(T)) return false;
  T x = 0;
  for (size_t i = 0; i < sizeof(T); i++) x |= (T)b[i] << (8 * i);
  *v = x;
  return true;
}

template <class T>
void put_le(std::vector<uint8_t>& out, T v) {
  for (size_t i = 0; i < sizeof(T); i++) out.push_back((uint8_t)(v >> (8 * i)));
}

struct FileCloser {
  FILE* f;
  ~FileCloser() {
    if (f) fclose(f);
  }
};

// One shard file into H_host[gamma][N]; returns an error text or "".
std::string read_shard(const std::string& path, uint32_t want_id, const inspire_ctx* c, uint16_t* H_host) {
  FILE* f = fopen(path.c_str(), "rb");
  if (!f) return "Shard " + std::to_string(want_id) + " not found";  // MmapDatabase::get_shard, mmap.rs:115-118
  FileCloser fc{f};
  uint32_t id, num_polys, ring_dim, crt_count;
  if (!read_le(f, &id) || !read_le(f, &num_polys) || !read_le(f, &ring_dim) || !read_le(f, &crt_count))
    return path + ": truncated header";
  if (id != want_id) return path + ": header id " + std::to_string(id) + " differs from the file name";
  if (num_polys == 0) return path + ": empty shard (not supported on the GPU path)";
  if (num_polys != (uint32_t)c->gamma)
    return path + ": " + std::to_string(num_polys) + " polynomials, the CRS packs " + std::to_string(c->gamma);
  if (ring_dim != (uint32_t)N || crt_count != 2) return path + ": ring_dim / crt_count differ from the context";
  for (uint32_t r = 0; r < 2; r++) {
    uint64_t m;
    if (!read_le(f, &m)) return path + ": truncated header";
    if (m != c->params.crt_moduli[r]) return path + ": moduli differ from the context";
  }
  std::vector<uint8_t> buf(sizeof(uint64_t) * 2 * N * num_polys);
  if (fread(buf.data(), 1, buf.size(), f) != buf.size()) return path + ": truncated polynomial data";
  auto word = [&](size_t i) {  // little-endian u64 i of the polynomial data
    uint64_t x = 0;
    for (int b = 0; b < 8; b++) x |= (uint64_t)buf[8 * i + b] << (8 * b);
    return x;
  };
  for (uint32_t p = 0; p < num_polys; p++) {
    const size_t base = (size_t)p * 2 * N;
    for (int k = 0; k < N; k++) {
      const uint64_t v0 = word(base + k), v1 = word(base + N + k);
      if (v0 >= 65536 || v1 != v0)
        return path + ": polynomial " + std::to_string(p) + " is not an encoded 16-bit column (coefficient " +
               std::to_string(k) + ")";
      H_host[(size_t)p * N + k] = (uint16_t)v0;
    }
  }
  return "";
}

}  // namespace

namespace ighost {

// A resident database from host raw columns Hh[nshards][gamma][N] (gamma = the
// context's CRS columns): upload, then the contracted form on the GPU.
int db_from_host_columns(inspire_ctx* c, const uint16_t* Hh, int nshards, uint64_t n_entries, uint32_t entry_size,
                         inspire_db** out) {
  const int gamma = c->gamma;
  inspire_db* db = new inspire_db();
  db->H.ledger = db->E.ledger = c->ledger;
  db->ctx = c;
  db->device = c->device;
  db->gamma = gamma;
  db->nshards = nshards;
  db->n_entries = n_entries;
  db->entry_size = entry_size;
  if (nshards > 0) {
    cudaError_t e = db->H.ensure(sizeof(uint16_t) * (size_t)nshards * gamma * N);
    if (e == cudaSuccess) e = db->E.ensure(sizeof(uint32_t) * (size_t)nshards * 2 * ELL * gamma * N);
    if (e != cudaSuccess) {
      delete db;
      return fail(INSPIRE_ERR_OUT_OF_MEMORY, alloc_failure(c, "database allocation"));
    }
    e = cudaMemcpy(db->H.p, Hh, sizeof(uint16_t) * (size_t)nshards * gamma * N, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = launch_encode_E(c->P, db->H.as<uint16_t>(), nshards, db->E.as<uint32_t>(), c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) {
      delete db;
      return fail(INSPIRE_ERR_CUDA, std::string("database upload / encode: ") + cudaGetErrorString(e));
    }
  }
  *out = db;
  return INSPIRE_OK;
}

}  // namespace ighost

extern "C" {

int inspire_db_load_shards(inspire_ctx* c, const char* dir, inspire_db** out) {
  if (!c || !dir || !out) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null argument");
  std::lock_guard<std::mutex> lk(c->mu);
  *out = nullptr;
  if (!c->has_crs) return fail(INSPIRE_ERR_NO_CRS, "no CRS loaded (inspire_crs_load)");
  DIR* d = opendir(dir);
  if (!d) return fail(INSPIRE_ERR_INVALID_ARGUMENT, std::string("cannot open shard directory ") + dir);
  uint64_t count = 0;
  while (dirent* e = readdir(d))
    if (strncmp(e->d_name, "shard-", 6) == 0) count++;
  closedir(d);
  if (count > 0x7fffffffULL) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "too many shards");
  if (int rc = set_device(c)) return rc;
  const int gamma = c->gamma;
  const int nshards = (int)count;
  inspire_db* db = new inspire_db();
  db->H.ledger = db->E.ledger = c->ledger;
  db->ctx = c;
  db->device = c->device;
  db->gamma = gamma;
  db->nshards = nshards;
  db->n_entries = (uint64_t)nshards * N;
  db->entry_size = 2 * (uint32_t)gamma;
  if (nshards > 0) {
    cudaError_t e = db->H.ensure(sizeof(uint16_t) * (size_t)nshards * gamma * N);
    if (e == cudaSuccess) e = db->E.ensure(sizeof(uint32_t) * (size_t)nshards * 2 * ELL * gamma * N);
    if (e != cudaSuccess) {
      delete db;
      return fail(INSPIRE_ERR_OUT_OF_MEMORY, alloc_failure(c, "database allocation"));
    }
    // shards in chunks of up to 256 MiB of raw columns
    const int per_chunk = std::max(1, (int)((256u << 20) / (sizeof(uint16_t) * gamma * N)));
    std::vector<uint16_t> Hh((size_t)std::min(per_chunk, nshards) * gamma * N);
    // the files of a chunk are read by up to 16 host threads; the error
    // reported is the one of the lowest shard id, as a serial read would give
    const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
    std::vector<std::string> errs((size_t)std::min(per_chunk, nshards));
    for (int s0 = 0; s0 < nshards; s0 += per_chunk) {
      const int s1 = std::min(nshards, s0 + per_chunk);
      const int nt = std::min({16, hw, s1 - s0});
      auto work = [&](int t) {
        for (int s = s0 + t; s < s1; s += nt)
          errs[(size_t)(s - s0)] = read_shard(shard_path(dir, (uint32_t)s), (uint32_t)s, c,
                                              Hh.data() + (size_t)(s - s0) * gamma * N);
      };
      std::vector<std::thread> pool;
      for (int t = 1; t < nt; t++) pool.emplace_back(work, t);
      work(0);
      for (std::thread& th : pool) th.join();
      for (int s = s0; s < s1; s++) {
        const std::string& err = errs[(size_t)(s - s0)];
        if (!err.empty()) {
          delete db;
          return fail(err.rfind("Shard ", 0) == 0 ? INSPIRE_ERR_SHARD_NOT_FOUND : INSPIRE_ERR_INVALID_ARGUMENT, err);
        }
      }
      cudaError_t ce = cudaMemcpy(db->H.as<uint16_t>() + (size_t)s0 * gamma * N, Hh.data(),
                                  sizeof(uint16_t) * (size_t)(s1 - s0) * gamma * N, cudaMemcpyHostToDevice);
      if (ce != cudaSuccess) {
        delete db;
        return fail(INSPIRE_ERR_CUDA, std::string("database upload: ") + cudaGetErrorString(ce));
      }
    }
    cudaError_t ce = launch_encode_E(c->P, db->H.as<uint16_t>(), nshards, db->E.as<uint32_t>(), c->stream);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(c->stream);
    if (ce != cudaSuccess) {
      delete db;
      return fail(INSPIRE_ERR_CUDA, std::string("database encode: ") + cudaGetErrorString(ce));
    }
  }
  *out = db;
  return INSPIRE_OK;
}

int inspire_db_save_shards(const inspire_db* db, const inspire_params* params, const char* dir) {
  if (!db || !params || !dir) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null argument");
  const int gamma = db->gamma;
  std::vector<uint16_t> Hh((size_t)gamma * N);
  std::vector<uint8_t> bytes;
  if (cudaSetDevice(db->device) != cudaSuccess) return fail(INSPIRE_ERR_CUDA, "cudaSetDevice failed");
  for (int s = 0; s < db->nshards; s++) {
    cudaError_t ce = cudaMemcpy(Hh.data(), db->H.as<uint16_t>() + (size_t)s * gamma * N,
                                sizeof(uint16_t) * Hh.size(), cudaMemcpyDeviceToHost);
    if (ce != cudaSuccess) return fail(INSPIRE_ERR_CUDA, std::string("database download: ") + cudaGetErrorString(ce));
    bytes.clear();
    put_le<uint32_t>(bytes, (uint32_t)s);
    put_le<uint32_t>(bytes, (uint32_t)gamma);
    put_le<uint32_t>(bytes, (uint32_t)N);
    put_le<uint32_t>(bytes, 2u);
    put_le<uint64_t>(bytes, params->crt_moduli[0]);
    put_le<uint64_t>(bytes, params->crt_moduli[1]);
    for (int p = 0; p < gamma; p++)
      for (int r = 0; r < 2; r++)
        for (int k = 0; k < N; k++) put_le<uint64_t>(bytes, (uint64_t)Hh[(size_t)p * N + k]);
    const std::string path = shard_path(dir, (uint32_t)s);
    FILE* f = fopen(path.c_str(), "wb");
    if (!f) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "cannot create " + path);
    const bool ok = fwrite(bytes.data(), 1, bytes.size(), f) == bytes.size();
    if (fclose(f) != 0 || !ok) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "cannot write " + path);
  }
  return INSPIRE_OK;
}

}  // extern "C"
