// kernels.h -- launch interfaces of the InsPIRe GB300 kernels (internal).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "common.cuh"

namespace ig {

constexpr int ERR_EXPAND = 1;  // seeded expansion exceeded its iteration bound
constexpr int ERR_INDEX = 2;   // shard or client id out of range
constexpr int ERR_STAGE = 3;   // the query's rows did not arrive in shared memory within the wait bound
// ... and the copies were still in flight after the drain wait: results of
// the whole launch are unreliable (a later CTA on the SM may have received
// the late copies in its shared memory)
constexpr int ERR_STAGE_LOST = 4;
constexpr uint32_t STAGE_WAIT_ITERS_DEFAULT = 1u << 20;
constexpr uint32_t STAGE_DRAIN_ITERS = 1u << 22;

// One resident database as the Respond kernel sees it.
struct DbView {
  const uint32_t* E;  // [nshards][2][gamma][ELL][N] contracted database, by recursion step
  const uint16_t* H;  // [nshards][gamma][N] raw 16-bit columns
  int nshards;
  int pad;
};

// One admitted query of the serving loop.  The descriptor itself -- with the
// query's seeds inline -- is copied to device memory per batch; the rows and
// the response live in pinned host memory that the Respond kernel reads and
// writes directly.
struct QueryDesc {
  uint8_t seeds[ELL * 32];  // seeds of rows ELL..2ELL-1
  const uint64_t* brows;  // [ELL][2][N] b-polys of rows ELL..2ELL-1 (16-byte aligned)
  uint64_t* out;          // [2][2][N] response destination (16-byte aligned)
  int32_t* status;        // kernel status destination
  DbView db;
  uint32_t shard;
  int32_t client;
};

struct RespondArgs {
  DevParams P;
  int nq;
  const uint32_t* shard;         // [nq] shard index (validated by the host)
  const uint8_t* seeds;          // [nq][ELL][32]   seeds of RGSW rows ELL..2ELL-1
  const uint64_t* arows;         // [nq][ELL][2][N] a-polys of rows ELL..2ELL-1 (unseeded queries) or null
  const uint64_t* brows;         // [nq][ELL][2][N] b-polys of rows ELL..2ELL-1
  const int32_t* client;         // [nq] client id
  // [nclients] -> client key table: [(gamma-1)][ELL][2][N] rotated keys,
  // or, when the pointer's bit 0 is set (gamma = 16 only), the body table
  // [ELL][2][N] whose rotations the kernel forms; third digit folded in
  const uint32_t* const* yhat_table;
  int nclients, nshards;
  const uint32_t* E;             // [nshards][2][gamma][ELL][N] contracted database, by recursion step
  const uint16_t* H;             // [nshards][gamma][N] raw 16-bit columns
  const uint32_t* what;          // [(gamma-1)][ELL][2][N] rotated w_mask (CRS), third digit folded in
  uint64_t* out;                 // [nq][2][2][N] response (a_hat, b) residues
  int* status;                   // [nq]
  // Serving loop: per-query descriptors in device memory (override shard,
  // client, seeds, brows, E/H/nshards, out and status; rows are read from and
  // responses written to the pinned host memory they point at), or null.
  const struct QueryDesc* qdesc;
  // Serving loop: bound of the wait for a query's staged rows, in wait
  // iterations (0: give up at once)
  uint32_t stage_wait_iters;
};

// NoPacking respond (respond.rs:71-115): per query the combined ciphertext
// out[nq][2][2][N] and, if out_columns is set, every column ciphertext
// out_columns[nq][gamma][2][2][N].
struct NoPackingArgs {
  DevParams P;
  int nq;
  const uint32_t* shard;
  const uint8_t* seeds;          // [nq][ELL][32] or null
  const uint64_t* arows;         // [nq][ELL][2][N] or null
  const uint64_t* brows;         // [nq][ELL][2][N]
  int nshards;
  const uint16_t* H;             // [nshards][gamma][N]
  uint64_t* out;
  uint64_t* out_columns;
  int* status;
  // CTAs per query, each answering ceil(gamma / col_groups) of its columns
  // (1: one CTA per query).  Above 1, out_columns is required and the
  // combined ciphertexts are summed from the columns by a second launch.
  int col_groups;
};

// Seeded query generation (client side): query first_query + i asks for
// local index local_idx[i] under the secret key sk[2][N].
constexpr int MAX_CDT = 64;  // |error| table entries (tail cut ceil(6 sigma) + 1)
struct QueryGenArgs {
  DevParams P;
  uint64_t first_query;
  const uint32_t* local_idx;  // [n]
  const uint64_t* sk;         // [2][N] residues
  uint32_t key[8];            // ChaCha20 key of the query stream
  uint32_t zpow[2][ELL], zpow_p[2][ELL];  // z^i mod q_r and Shoup companions
  uint64_t cdt[MAX_CDT];      // cdt[j] = 2^63 P(|e| <= j), j < cdt_len - 1
  int cdt_len;
  uint8_t* seeds;             // [n][2 ELL][32]
  uint64_t* b_rows;           // [n][2 ELL][2][N]
  int* status;                // [n]
};

// Client key generation: client first_client + i gets secret key sk[i][2][N]
// and packing key body y_body[i][ELL][2][N] against the CRS mask wmask.
struct KeyGenArgs {
  DevParams P;
  uint64_t first_client;
  uint32_t key[8];
  uint32_t zpow[2][ELL], zpow_p[2][ELL];
  uint64_t cdt[MAX_CDT];
  int cdt_len;
  const uint32_t* wmask;      // [ELL][2][N] w_mask residues
  uint64_t* sk;               // [n][2][N]
  uint64_t* y_body;           // [n][ELL][2][N]
};

// Galois key-switching matrices of the secret key sk[2][N]: keys[i][k][a, b][2][N]
// for i < nmat (t = N / 2^i + 1), k < ELL.
struct GaloisGenArgs {
  DevParams P;
  uint32_t key[8];
  uint32_t zpow[2][ELL], zpow_p[2][ELL];
  uint64_t cdt[MAX_CDT];
  int cdt_len;
  const uint64_t* sk;
  uint64_t* keys;
  int* status;  // [nmat]
};

// Tree packing (respond_one_packing) of nq queries' column ciphertexts.
struct TreeArgs {
  DevParams P;
  int nq, ncols;
  int mode;
  const uint64_t* cols;  // [nq][ncols][2 (a, b)][2][N] column ciphertexts
  const uint32_t* ks;    // [log2 N][ELL][2 (a, b)][2][N] Galois keys, NTT domain x n^-1 2^32
  uint32_t* work;        // [nq][tree_work_words_per_query()] ciphertexts of the tree
  uint64_t* out_a;       // [nq][2][N]
  uint64_t* out_b;       // [nq][4][N]: 2 residues x N, or 4 N words in compat mode
};

// Set the kernels' dynamic shared-memory limits on the current device (once
// per device, before any launch; launches then make no configuration call).
cudaError_t prepare_respond_kernels();
cudaError_t prepare_nopacking_kernels();
cudaError_t prepare_ops_kernels();
cudaError_t prepare_setup_kernels();
cudaError_t prepare_client_kernels();

size_t query_gen_smem_bytes();
cudaError_t launch_query_gen(const QueryGenArgs& a, int n, cudaStream_t st);
// Allocation-free tree packing: a static device array holds the scratch of
// up to TREE_NOALLOC_MAX_QUERIES queries.
constexpr int TREE_NOALLOC_MAX_QUERIES = 2;
size_t tree_noalloc_query_bytes();
cudaError_t tree_noalloc_scratch(int device, void** ptr);
size_t tree_smem_bytes();
size_t tree_work_words_per_query();
cudaError_t prepare_tree_kernels();
cudaError_t launch_pack_tree(const TreeArgs& a, cudaStream_t st);
cudaError_t launch_galois_prep(const DevParams& P, const uint64_t* keys, int npolys, uint32_t* ks, cudaStream_t st);
size_t galois_keys_smem_bytes();
// Key-switching matrices 0 .. nmat-1 (nmat <= LOGN + 4): the LOGN Galois
// matrices, k_g, k_h, packing_k_g, packing_k_h.
cudaError_t launch_ks_matrices(const GaloisGenArgs& a, int nmat, cudaStream_t st);
// nvec uniform polys [nvec][2][N] u64 (setup's crs_a_vectors).
cudaError_t launch_crs_a(const GaloisGenArgs& a, int nvec, uint64_t* out, cudaStream_t st);
size_t client_keys_smem_bytes();
cudaError_t launch_client_keys(const KeyGenArgs& a, int n, cudaStream_t st);

size_t nopacking_smem_bytes();
cudaError_t launch_nopacking(const NoPackingArgs& a, bool seeded, cudaStream_t st);

size_t respond_smem_bytes(int mode, bool qdb);
// max_ctas > 0 caps the grid: each CTA then answers several queries in turn.
// Otherwise batches of at most pair_max queries run on the two-CTA cluster
// kernel (respond_pair.cu), larger ones on the one-CTA kernel.
cudaError_t launch_respond(const RespondArgs& a, bool seeded, cudaStream_t st, int max_ctas = 0, int pair_max = 0);
size_t respond_pair_smem_bytes();
cudaError_t prepare_respond_pair_kernels();
cudaError_t launch_respond_pair(const RespondArgs& a, bool seeded, cudaStream_t st);

// setup-time kernels
cudaError_t launch_columns_from_raw(const uint8_t* raw, uint64_t n_entries, int entry_size,
                                    int gamma, int nshards, uint16_t* H, cudaStream_t st);
cudaError_t launch_encode_E(const DevParams& P, const uint16_t* H, int nshards, uint32_t* E,
                            cudaStream_t st);
cudaError_t launch_crs_what(const DevParams& P, const uint32_t* wmask, uint32_t* what,
                            cudaStream_t st);
// Fold the third gadget digit into ngroups key triples [g][k<3][2][N] in
// place (k0 - z^-2 k2, k1 - z^-1 k2, n z^-2 k2): the Respond kernel then
// multiplies the third key by R_{i+1} instead of by NTT(d2).
cudaError_t launch_fold_third_digit(const DevParams& P, uint32_t* tbl, int ngroups, cudaStream_t st);
// The first nrot rotations y_all[0..nrot) of the client key table (nrot =
// gamma - 1: the full table; 1: the body table the Respond kernel rotates).
cudaError_t launch_client_from_ybody(const DevParams& P, const uint64_t* ybody, uint32_t* yhat, int nrot,
                                     cudaStream_t st);
cudaError_t launch_client_from_yall(const DevParams& P, const uint64_t* yall, uint32_t* yhat,
                                    cudaStream_t st);

// kernel-level operations
// decrypt + extract_inspiring of n responses ct[n][2][2][N] (u64) with the
// secret key sk[2][N] (u64); entries[n][entry_size] (entry_size <= 32).
cudaError_t launch_extract(const DevParams& P, uint64_t p, const uint64_t* sk, const uint64_t* ct, int n,
                           int entry_size, uint8_t* entries, cudaStream_t st);
// blocks x 256 threads x 8 chains x iters lazy Shoup multiplies; sink[blocks * 256].
cudaError_t launch_mulmod_rate(const DevParams& P, int blocks, int iters, uint32_t* sink, cudaStream_t st);
// blocks x 8 warps x 4 chains x iters INT8 MMAs (m16n8k32); out[4][16][8]
// receives warp 0's accumulators (= iters * A B for iters <= 4096).
cudaError_t launch_int8_mma_rate(const int8_t* A, const int8_t* B, int blocks, int iters, int32_t* out,
                                 cudaStream_t st);
cudaError_t launch_ntt_ref(const DevParams& P, uint32_t* polys, int npolys, bool inverse,
                           cudaStream_t st);
cudaError_t launch_external_product(const DevParams& P, const uint32_t* ct, const uint32_t* rgsw,
                                    uint32_t* out, int npairs, cudaStream_t st);

}  // namespace ig
