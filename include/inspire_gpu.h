/*
 * inspire_gpu.h -- C ABI of the GB300-native InsPIRe server Respond path.
 *
 * This is the drop-in boundary for the Respond path of the Rust crate
 * igor53627/inspire-rs v0.1.2: every entry point below replaces one public
 * item of that crate (cited per declaration as crate-relative file:line), so a
 * thin `-sys` binding can route the crate's API onto the GPU.  Plain pointers
 * and sizes only; no C++ or torch types cross this boundary.
 *
 * Conventions
 *  - A polynomial is `crt_count * ring_dim` u64 values, residue-major
 *    ([residues mod q0..., residues mod q1...]), each canonical (< its modulus):
 *    the layout of the crate's `Poly::coeffs` (src/math/poly.rs:64-77).
 *  - Functions return INSPIRE_OK (0) or a positive inspire_status; the text of
 *    the last error of the calling thread is inspire_last_error().  Texts of
 *    the errors the crate reports follow its `PirError` messages
 *    (src/pir/respond.rs:82, 141-143, 299, 367-369).
 *  - `*_device` functions take device pointers and a cudaStream_t (as void*)
 *    and are asynchronous; all other functions take host pointers and return
 *    when the result is in host memory.
 *  - One context owns one GPU.  Host-pointer calls on one context are
 *    serialised internally; they may be made from several threads.
 */
#ifndef INSPIRE_GPU_H
#define INSPIRE_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  INSPIRE_OK = 0,
  INSPIRE_ERR_INVALID_ARGUMENT = 1,
  INSPIRE_ERR_SHARD_NOT_FOUND = 2,  /* "Shard {id} not found" (respond.rs:301-305) */
  INSPIRE_ERR_KEYS_MISSING = 3,     /* "InspiRING client packing keys missing from query" (respond.rs:296-299) */
  INSPIRE_ERR_KEYS_INVALID = 4,     /* "InspiRING packing keys invalid: y_all and y_body are both empty" (respond.rs:365-370) */
  INSPIRE_ERR_UNSUPPORTED = 5,      /* parameters outside the GPU path (ring_dim 2048, two CRT primes, gadget 2^20 x 3, num_columns <= 16) */
  INSPIRE_ERR_CUDA = 6,
  INSPIRE_ERR_OUT_OF_MEMORY = 7,
  INSPIRE_ERR_NO_CRS = 8,
  INSPIRE_ERR_DEVICE_STATUS = 9,    /* a kernel reported a failed bounded loop or a bad index */
  INSPIRE_PENDING = 10,             /* serving loop: the ticket's response is not ready yet */
  INSPIRE_ERR_BUSY = 11             /* serving loop: no free query slot; retry after polling */
} inspire_status;

/* NTT-domain automorphism semantics of InspiRING packing
 * (src/inspiring/inspiring2.rs:279-296).  COMPAT is the crate's behaviour,
 * bit for bit: only the residue-0 slice is permuted and residue 1 is rebuilt
 * from it.  With two CRT moduli those responses do not decrypt.  CRT_FIXED
 * permutes every residue; its responses decrypt. */
typedef enum { INSPIRE_MODE_COMPAT = 0, INSPIRE_MODE_CRT_FIXED = 1 } inspire_mode;

/* InspireParams (src/params.rs:135-185).  The GPU path requires
 * ring_dim = 2048, two CRT primes in (2^20, 2^28) with q_i = 1 mod 4096 and q0 < 2 q1,
 * gadget_base = 2^20 and gadget_len = 3 (secure_128_d2048, params.rs:213-230;
 * p may be 65537 or 2^16). */
typedef struct {
  uint32_t ring_dim;
  uint32_t crt_count;
  uint64_t crt_moduli[2];
  uint64_t p;
  double sigma;
  uint64_t gadget_base;
  uint32_t gadget_len;
} inspire_params;

typedef struct inspire_ctx inspire_ctx;
typedef struct inspire_db inspire_db;

/* Text of the calling thread's last error ("" if none). */
const char *inspire_last_error(void);
/* Library version string. */
const char *inspire_version(void);

/* InspireParams::secure_128_d2048 with p = 2^16 (params.rs:213-230). */
void inspire_params_default(inspire_params *out);

/* Create a context on CUDA device `device`: validates parameters
 * (InspireParams::validate, params.rs:348-387), builds NTT twiddles and
 * constants (NttContext::with_moduli, src/math/ntt.rs:116-164) in HBM. */
int inspire_ctx_create(const inspire_params *params, int device, int mode, inspire_ctx **out);
void inspire_ctx_destroy(inspire_ctx *ctx);

/* Admission by device memory.  Every device buffer of a context -- its
 * tables, CRS and Galois key tables, resident databases, client key tables,
 * serving-loop slots, staging buffers -- is accounted against an optional
 * budget (0, the default: no limit).  A registration, database load or
 * server creation that would exceed it fails with
 * INSPIRE_ERR_OUT_OF_MEMORY before anything is allocated, and leaves the
 * context usable; freeing objects returns their bytes.  A budget below the
 * bytes already in use is refused. */
int inspire_ctx_set_device_budget(inspire_ctx *ctx, uint64_t bytes);
/* Bytes accounted now and the budget (0: none). */
int inspire_ctx_device_memory(inspire_ctx *ctx, uint64_t *used, uint64_t *budget);

/* Respond launches of at most `max_queries` queries (batch calls, device
 * batches, serving-loop batches) run each query on a cluster of two CTAs, one
 * per CRT residue, which halves a lone query's latency; larger launches use
 * one CTA per query, which needs half the SMs per query.  Both give the same
 * responses bit for bit.  Default: half the device's SM count (every query of
 * the launch then has its two SMs); 0 turns the cluster kernel off.  The
 * capped-grid call (inspire_respond_seeded_batch_device_grid with max_ctas)
 * always uses one CTA per query. */
int inspire_ctx_set_pair_threshold(inspire_ctx *ctx, uint32_t max_queries);
uint32_t inspire_ctx_pair_threshold(const inspire_ctx *ctx);

/* Load the InspiRING part of ServerCrs (src/pir/setup.rs:52-87): the shared
 * seed `inspiring_w_seed` and `inspiring_num_columns` (gamma).  Builds the
 * rotated w_mask table of OfflinePackingKeys::generate
 * (src/inspiring/inspiring2.rs:448-506) once; the crate rebuilds it and
 * PackParams::new on every query (respond.rs:360-361).  gamma must be a power
 * of two <= 16 on the GPU path. */
int inspire_crs_load(inspire_ctx *ctx, const uint8_t w_seed[32], uint32_t num_columns);

/* Encode a raw database resident in HBM: encode_database
 * (src/pir/encode_db.rs:106-164) with shards of ring_dim entries
 * (setup.rs:149-153), plus the per-shard contracted form the Respond kernel
 * reads.  `raw` holds n_entries * entry_size bytes (host memory).
 * ceil(entry_size / 2) must equal the CRS num_columns. */
int inspire_db_create(inspire_ctx *ctx, const uint8_t *raw, uint64_t n_entries, uint32_t entry_size,
                      inspire_db **out);
void inspire_db_destroy(inspire_db *db);

/* Load the crate's binary shard files from `dir` straight into HBM:
 * save_shards_binary's format (src/pir/mmap.rs:19-53, shard-{id:04}.bin),
 * read as MmapDatabase::open / get_shard / load_shard_binary read it
 * (mmap.rs:56-122): every "shard-*" file is one shard and ids 0..n-1 must all
 * exist ("Shard {id} not found" otherwise).  Each shard must hold num_columns
 * encoded 16-bit column polynomials over this context's moduli.  The result
 * equals inspire_db_create on the raw entries the files encode. */
int inspire_db_load_shards(inspire_ctx *ctx, const char *dir, inspire_db **out);

/* The loaded CRS's inspiring_w_seed (32 bytes), inspiring_num_columns, and
 * whether Galois keys are loaded. */
int inspire_crs_info(inspire_ctx *ctx, uint8_t *w_seed, uint32_t *num_columns, int32_t *has_galois_keys);

/* The server's crs.json (src/bin/server.rs:255-264): serde_json of ServerCrs
 * (src/pir/setup.rs:52-87).  params must equal the context's; the InspiRING
 * part (inspiring_w_seed, inspiring_num_columns) is loaded as
 * inspire_crs_load does and galois_keys, if present, as
 * inspire_crs_load_galois_keys; the other fields (k_g, k_h, crs_a_vectors,
 * packing_k_*, inspiring_precomp, ...) are not read by the Respond paths and
 * are skipped. */
int inspire_crs_load_json(inspire_ctx *ctx, const char *json, size_t len);

/* setup's InspiRING offline precomputation (src/pir/setup.rs:194-224):
 * packing_offline (src/inspiring/inspiring2.rs:926-1041) over the CRS's
 * num_columns a-polys a_polys [num_columns][poly] (coefficient form; setup
 * takes the first num_columns crs_a_vectors), with the loaded CRS's
 * OfflinePackingKeys.  a_hat receives PrecompInsPIR.a_hat [poly] and bold_t
 * PrecompInsPIR.bold_t [(num_columns-1)][gadget_len][poly], both in
 * coefficient form (the crate's layout; bold_t may be NULL when
 * num_columns = 1).  Computed on the GPU, host buffers, synchronous. */
int inspire_inspiring_precomp(inspire_ctx *ctx, const uint64_t *a_polys, uint64_t *a_hat, uint64_t *bold_t);

/* Number of crs_a_vectors in the crs.json last loaded with
 * inspire_crs_load_json (the server's /params reports it,
 * src/bin/server.rs:99-118); 0 for a CRS loaded otherwise. */
uint64_t inspire_crs_a_vectors_count(const inspire_ctx *ctx);

/* The parts of ServerCrs (src/pir/setup.rs:52-87) for writing crs.json.
 * Key-switching matrices are [gadget_len][a, b][poly] (the layout
 * inspire_setup_keygen_device writes); NULL optional parts are written as
 * null (packing_k_g, packing_k_h, inspiring_precomp). */
typedef struct {
  const uint64_t *k_g;
  const uint64_t *k_h;
  const uint64_t *galois_keys;   /* [n_galois][gadget_len][a, b][poly] */
  uint32_t n_galois;
  const uint64_t *crs_a_vectors; /* [n_crs_a][poly] */
  uint32_t n_crs_a;
  const uint64_t *packing_k_g;
  const uint64_t *packing_k_h;
  const uint64_t *precomp_a_hat;  /* PrecompInsPIR.a_hat [poly], or NULL */
  const uint64_t *precomp_bold_t; /* [(num_columns-1)][gadget_len][poly] */
  uint8_t inspiring_w_seed[32];
  uint8_t inspiring_v_seed[32];
  uint32_t inspiring_num_columns;
} inspire_server_crs;

/* Write crs.json at `path` as setup's binary writes it (serde_json::to_writer
 * of ServerCrs, src/bin/setup.rs:183-190): serde's field order and compact
 * form, the skipped fields (inspiring_pack_params, inspiring_packing_key,
 * PrecompInsPIR.bold_t_ntt) left out.  params.security_level is written as
 * Bits128 (inspire_params has no such field; secure_128_d2048's value).
 * inspire_crs_load_json reads the file back. */
int inspire_crs_write_json(const inspire_params *params, const inspire_server_crs *crs, const char *path);

/* The server's encoded_db.json (src/bin/server.rs:292-301): serde_json of
 * EncodedDatabase {shards: [ShardData {id, polynomials: [Poly]}], config:
 * ShardConfig} (src/pir/setup.rs:104-120, src/params.rs:432-450) made
 * resident like inspire_db_create.  Shard ids must be 0, 1, ... in order,
 * each with the CRS's num_columns polynomials of encoded 16-bit columns. */
int inspire_db_load_json(inspire_ctx *ctx, const char *json, size_t len, inspire_db **out);

/* Write a resident database as the crate's binary shard files into `dir`
 * (which must exist), in save_shards_binary's format, with the moduli of
 * `params`. */
int inspire_db_save_shards(const inspire_db *db, const inspire_params *params, const char *dir);
uint32_t inspire_db_num_shards(const inspire_db *db);
/* Device bytes held by the database. */
uint64_t inspire_db_device_bytes(const inspire_db *db);

/* Register per-client packing keys (ClientPackingKeys,
 * src/inspiring/inspiring2.rs:604-628) resident in HBM.  Give y_body
 * (gadget_len polys; the server derives y_all with generate_rotations,
 * inspiring2.rs:1309-1323, as respond.rs:365-377 does for wire queries) or
 * y_all ((num_columns-1) * gadget_len polys, the in-process form).  y_all
 * takes precedence.  Both NULL -> INSPIRE_ERR_KEYS_INVALID. */
int inspire_client_register(inspire_ctx *ctx, const uint64_t *y_body, const uint64_t *y_all,
                            int32_t *client_id);
int inspire_client_release(inspire_ctx *ctx, int32_t client_id);

/* SeededClientQuery (src/pir/query.rs:138-150) with its RGSW rows flattened:
 * seeds = 2*gadget_len seeds of 32 bytes, b_rows = 2*gadget_len polys. */
typedef struct {
  uint32_t shard_id;
  const uint8_t *seeds;
  const uint64_t *b_rows;
  /* inspiring_packing_keys: has_packing_keys = 0 is Option::None. */
  int32_t has_packing_keys;
  const uint64_t *y_body; /* gadget_len polys or NULL */
  const uint64_t *y_all;  /* (num_columns-1)*gadget_len polys or NULL */
} inspire_seeded_query;

/* ClientQuery (query.rs:119-132): rgsw = 2*gadget_len rows of (a, b) polys. */
typedef struct {
  uint32_t shard_id;
  const uint64_t *rgsw;
  int32_t has_packing_keys;
  const uint64_t *y_body;
  const uint64_t *y_all;
} inspire_query;

/* respond_seeded_inspiring (src/pir/respond.rs:391-398): out_ct receives
 * ServerResponse.ciphertext as [a poly, b poly] (column_ciphertexts is empty
 * for InspiRING, respond.rs:382-385). */
int inspire_respond_seeded_inspiring(inspire_ctx *ctx, const inspire_db *db, const inspire_seeded_query *query,
                                     uint64_t *out_ct);

/* respond_inspiring (src/pir/respond.rs:284-386). */
int inspire_respond_inspiring(inspire_ctx *ctx, const inspire_db *db, const inspire_query *query,
                              uint64_t *out_ct);

/* respond (src/pir/respond.rs:71-115), the NoPacking variant: one external
 * product of trivial_encrypt(column) with the query's RGSW per shard column.
 * out_ct receives ServerResponse.ciphertext (the sum of the column
 * ciphertexts) as [a poly, b poly]; out_columns, if not NULL, receives
 * column_ciphertexts as [num_columns][a, b][poly].  Packing keys in the query
 * are ignored, as in the crate. */
int inspire_respond(inspire_ctx *ctx, const inspire_db *db, const inspire_query *query, uint64_t *out_ct,
                    uint64_t *out_columns);

/* ServerCrs.galois_keys (src/pir/setup.rs:164-173) for tree packing: nkeys =
 * log2(ring_dim) key-switching matrices, matrix i for the automorphism
 * X -> X^(ring_dim / 2^i + 1), each 2*gadget_len polys [row 0 a, row 0 b,
 * row 1 a, ...] (u64, residue-major, reduced).  Kept in HBM in NTT form. */
int inspire_crs_load_galois_keys(inspire_ctx *ctx, const uint64_t *keys, uint32_t nkeys);

/* respond_one_packing (src/pir/respond.rs:213-268), the tree-packing
 * variant: the column products, the LWEs at their coefficient 0, and
 * pack_lwes (src/inspiring/automorph_pack.rs:418-485) with the Galois keys.
 * out_a receives the packed a (one poly); out_b (room for two polys) receives
 * *b_words words: one poly, or -- in compat mode with more than one column --
 * the crate's b polynomial of dimension 2*ring_dim (2 polys' words).
 * Packing keys in the query are ignored, as in the crate. */
int inspire_respond_one_packing(inspire_ctx *ctx, const inspire_db *db, const inspire_query *query,
                                uint64_t *out_a, uint64_t *out_b, uint32_t *b_words);

/* respond_seeded_packed (src/pir/respond.rs:428-435): expand, then
 * respond_one_packing. */
int inspire_respond_seeded_packed(inspire_ctx *ctx, const inspire_db *db, const inspire_seeded_query *query,
                                  uint64_t *out_a, uint64_t *out_b, uint32_t *b_words);

/* A batch of respond_seeded_packed calls: query i (shard_ids[i], seeds
 * [n][2*gadget_len][32], b_rows [n][2*gadget_len][poly]) is answered into
 * out_a[i] (one poly) and out_b[i] (two polys' room; *b_words words used). */
int inspire_respond_seeded_packed_batch(inspire_ctx *ctx, const inspire_db *db, uint32_t n, const uint32_t *shard_ids,
                                        const uint8_t *seeds, const uint64_t *b_rows, uint64_t *out_a,
                                        uint64_t *out_b, uint32_t *b_words);

/* respond_seeded (src/pir/respond.rs:408-415): SeededClientQuery::expand then
 * respond. */
int inspire_respond_seeded(inspire_ctx *ctx, const inspire_db *db, const inspire_seeded_query *query,
                           uint64_t *out_ct, uint64_t *out_columns);

/* Batched respond_seeded (combined ciphertexts only), host buffers laid out
 * as for inspire_respond_seeded_batch: shard_ids[n], seeds[n][2*gadget_len][32],
 * b_rows[n][2*gadget_len][poly], out_ct[n][2][poly]. */
int inspire_respond_seeded_nopacking_batch(inspire_ctx *ctx, const inspire_db *db, uint32_t n,
                                           const uint32_t *shard_ids, const uint8_t *seeds, const uint64_t *b_rows,
                                           uint64_t *out_ct);

/* Batched respond_seeded_inspiring over n queries with registered client
 * keys, host buffers: shard_ids[n], seeds[n][2*gadget_len][32],
 * b_rows[n][2*gadget_len][poly], client_ids[n], out_ct[n][2][poly].  Queries
 * may name different shards.  Each result is the one respond_seeded_inspiring
 * returns for that query alone.  When b_rows and out_ct are page-locked
 * (inspire_pinned_alloc, cudaHostAlloc or cudaHostRegister memory) and
 * 16-byte aligned, the GPU reads the rows and writes the responses in place
 * (no staging copies); other memory is staged through device buffers. */
int inspire_respond_seeded_batch(inspire_ctx *ctx, const inspire_db *db, uint32_t n, const uint32_t *shard_ids,
                                 const uint8_t *seeds, const uint64_t *b_rows, const int32_t *client_ids,
                                 uint64_t *out_ct);

/* Batched respond_inspiring (full, unseeded queries, src/pir/respond.rs:284-386)
 * over n queries with registered client keys, host buffers: shard_ids[n],
 * rgsw[n][2*gadget_len][2][poly] (rows of (a, b)), client_ids[n],
 * out_ct[n][2][poly].  Each result is the one respond_inspiring returns for
 * that query alone. */
int inspire_respond_batch(inspire_ctx *ctx, const inspire_db *db, uint32_t n, const uint32_t *shard_ids,
                          const uint64_t *rgsw, const int32_t *client_ids, uint64_t *out_ct);

/* Same on device buffers, asynchronous on `stream`.  seeds holds only rows
 * gadget_len..2*gadget_len-1 ([n][gadget_len][32]) and b_rows only those rows
 * ([n][gadget_len][poly], 16-byte aligned); d_status[n] receives 0 or a
 * nonzero kernel status (unknown shard or client id, exhausted expansion
 * bound).  Two launches: the b side of every query, parked in the last 128
 * bytes of its d_out_ct slot, then the Respond kernel, which overwrites the
 * slot with the response (a slot whose status is nonzero holds no response).
 * No allocation and no configuration call: the call can be captured in a
 * CUDA graph. */
int inspire_respond_seeded_batch_device(inspire_ctx *ctx, const inspire_db *db, uint32_t n,
                                        const uint32_t *d_shard_ids, const uint8_t *d_seeds,
                                        const uint64_t *d_b_rows, const int32_t *d_client_ids, uint64_t *d_out_ct,
                                        int32_t *d_status, void *stream);

/* The same with the grid capped at max_ctas CTAs (0: one CTA per query):
 * CTA b answers queries b, b + max_ctas, ... in turn, so one call can answer
 * a large batch with one CTA per SM and no SM idles until the last round. */
int inspire_respond_seeded_batch_device_grid(inspire_ctx *ctx, const inspire_db *db, uint32_t n,
                                             const uint32_t *d_shard_ids, const uint8_t *d_seeds,
                                             const uint64_t *d_b_rows, const int32_t *d_client_ids,
                                             uint64_t *d_out_ct, int32_t *d_status, uint32_t max_ctas, void *stream);

/* ---- Serving loop ----
 * The crate serves each HTTP request with one synchronous respond call on a
 * tokio worker (src/bin/server.rs:179-236).  The serving loop replaces that
 * with continuous batching on the GPU: queries are submitted from any thread
 * and admitted into pinned query slots; a dispatcher thread launches each
 * batch of pending queries (up to max_batch, any shards, any registered
 * clients, any databases of this context) on one of max_inflight CUDA streams
 * as soon as a stream is free, so batches overlap on the device; the GPU reads
 * the queries and writes the responses in pinned host memory directly.  Each
 * response equals respond_seeded_inspiring of that query alone. */
typedef struct inspire_server inspire_server;

typedef struct {
  uint32_t max_batch;     /* queries per launch (1..1024) */
  uint32_t max_inflight;  /* batches on the device at once, one stream each */
  uint32_t capacity;      /* queries submitted and not yet polled, at most */
  uint64_t device_budget; /* device bytes for in-flight batches; 0 = no limit.
                             Fewer streams are used if max_inflight batches do not fit. */
  uint32_t batch_wait_us; /* while at least one query per SM is in flight, a free
                             stream waits up to this long for a full batch */
  uint32_t stage_wait_iters; /* bound of the Respond kernel's wait for a query's rows,
                             copied from pinned host memory into shared memory, in
                             wait iterations.  When it runs out the query fails
                             (INSPIRE_ERR_DEVICE_STATUS) and the next batches are
                             served as usual; 0 gives up at once (a test of that
                             path).  If the copies are still in flight after a
                             second, longer wait, every query of that batch fails. */
} inspire_server_config;

typedef struct {
  uint64_t submitted, completed, batches; /* totals since creation */
  uint32_t pending, inflight_batches;     /* now */
  uint32_t streams;                       /* streams in use (after the device budget) */
} inspire_server_stats;

/* max_batch 128, max_inflight 4, capacity 4096, device_budget 0, batch_wait_us 100,
 * stage_wait_iters 2^20. */
void inspire_server_config_default(inspire_server_config *cfg);
int inspire_server_create(inspire_ctx *ctx, const inspire_server_config *cfg, inspire_server **out);
/* Waits for batches in flight, then frees the loop.  Unpolled tickets die. */
void inspire_server_destroy(inspire_server *srv);

/* Submission flag: read the query b rows in place instead of copying them.
 * b_rows must then lie in page-locked host memory (for instance from
 * inspire_pinned_alloc), 16-byte aligned; seeds and b_rows must stay
 * unchanged until every ticket of the call has been collected (the seeds are
 * read when the query's batch is launched). */
#define INSPIRE_SUBMIT_BORROW 1u

/* Submit n seeded InspiRING queries; query i asks database dbs[i] (any
 * database of this context), laid out as for inspire_respond_seeded_batch
 * (full 2*gadget_len-row seeds and b_rows).  Without INSPIRE_SUBMIT_BORROW
 * the needed rows are copied, so the buffers are free on return.  arrival_ns
 * (may be NULL: the submit time) stamps each query for latency accounting on
 * the inspire_now_ns clock.  tickets[n] receive one ticket per accepted query.
 * Validation as inspire_respond_seeded_batch ("Shard {id} not found", keys
 * missing); queries are accepted in order until the first invalid one (its
 * error is returned) or until capacity is reached (INSPIRE_ERR_BUSY);
 * *accepted counts the accepted ones. */
int inspire_server_submit(inspire_server *srv, uint32_t n, const inspire_db *const *dbs, const uint32_t *shard_ids,
                          const uint8_t *seeds, const uint64_t *b_rows, const int32_t *client_ids,
                          const int64_t *arrival_ns, uint32_t flags, uint64_t *tickets, uint32_t *accepted);

/* Page-locked, device-mapped host memory for borrowed submissions. */
int inspire_pinned_alloc(size_t bytes, void **out);
void inspire_pinned_free(void *p);

/* Collect a ticket: waits up to timeout_us (0 = do not wait, < 0 = no
 * limit).  INSPIRE_OK: out_ct (may be NULL) receives [a poly, b poly],
 * done_ns (may be NULL) the completion time, and the ticket is consumed.
 * INSPIRE_PENDING: not ready.  Unknown or consumed tickets:
 * INSPIRE_ERR_INVALID_ARGUMENT. */
int inspire_server_poll(inspire_server *srv, uint64_t ticket, uint64_t *out_ct, int64_t *done_ns,
                        int32_t timeout_us);

/* Collect tickets[0..n) in order, as inspire_server_poll each (out_ct, may
 * be NULL, receives n responses of [a poly, b poly]; done_ns, may be NULL, n
 * times), waiting for all of them up to timeout_us in total.  Stops at the
 * first ticket still pending (INSPIRE_PENDING) or failing (its error);
 * *collected counts the tickets consumed. */
int inspire_server_poll_batch(inspire_server *srv, uint32_t n, const uint64_t *tickets, uint64_t *out_ct,
                              int64_t *done_ns, int32_t timeout_us, uint32_t *collected);

/* Open-loop load driven natively (no reference counterpart; for measuring the
 * loop without a scripting-language load generator's own delays): query k
 * (k < n) is submitted at arrival_ns[k] (the inspire_now_ns clock, in
 * non-decreasing order) by the calling thread, which spins on the clock and
 * puts every query already due into one inspire_server_submit call (at most
 * max_burst, 0 = 256), retrying on backpressure; a second thread collects
 * the tickets in order.  Query k's rows are entry k mod pool_size of the
 * pool (pool_seeds: pool_size x 2*gadget_len x 32 bytes; pool_b_rows:
 * pool_size x 2*gadget_len x 2N u64; flags as for inspire_server_submit);
 * dbs, shard_ids and client_ids are per query.  done_ns[k] receives each
 * completion time, submit_ns[k] (may be NULL) the time of its submission
 * call, and out_keep the responses of the first n_keep queries (n_keep x
 * [a poly, b poly]).  Latency from arrival is done_ns - arrival_ns.  A
 * rejected query (an unknown shard or client, as inspire_server_submit
 * reports it) or a query that fails on the device (as inspire_server_poll
 * reports it) ends the submissions; every query accepted until then is
 * still collected, then the first error is returned. */
int inspire_server_drive(inspire_server *srv, uint32_t n, const inspire_db *const *dbs, const uint32_t *shard_ids,
                         const int32_t *client_ids, const uint8_t *pool_seeds, const uint64_t *pool_b_rows,
                         uint32_t pool_size, const int64_t *arrival_ns, uint32_t flags, uint32_t max_burst,
                         int64_t *submit_ns, int64_t *done_ns, uint32_t n_keep, uint64_t *out_keep);

int inspire_server_get_stats(inspire_server *srv, inspire_server_stats *out);

/* Monotonic clock of the serving loop's timestamps (CLOCK_MONOTONIC, ns). */
int64_t inspire_now_ns(void);

/* ---- Wire codecs (host only; need no GPU) ----
 * JSON as serde_json writes the crate's derived layouts (Poly,
 * src/math/poly.rs:63-77; SeededRlweCiphertext, rlwe/types.rs:165-171;
 * SeededRgswCiphertext + GadgetVector, rgsw/types.rs:37-45, 225-231;
 * ClientPackingKeys, inspiring/inspiring2.rs:603-628; SeededClientQuery,
 * pir/query.rs:138-150; ServerResponse, pir/respond.rs:31-37; the server's
 * QueryResponse, src/bin/server.rs:88-92); bincode 1.3's default encoding for
 * ServerResponse::to_binary (pir/respond.rs:43-50). */

/* Parse a SeededClientQuery JSON body (the server's /query_seeded request,
 * src/bin/server.rs:179-236) into the inspire_seeded_query layout:
 * seeds[2*gadget_len][32], b_rows[2*gadget_len][poly], *packing_mode 0 =
 * inspiring / 1 = tree, *has_keys = 0 when inspiring_packing_keys is absent
 * or null, 1 when it carries y_body (gadget_len polys into y_body, which may
 * be NULL to skip them), 2 when its y_body is empty (respond then reports
 * the keys invalid).  Polynomials must be in coefficient form over the
 * parameters' moduli; numbers follow serde_json's grammar (no leading
 * zeros). */
int inspire_seeded_query_from_json(const inspire_params *params, const char *json, size_t len, uint32_t *shard_id,
                                   uint8_t *seeds, uint64_t *b_rows, int32_t *packing_mode, int32_t *has_keys,
                                   uint64_t *y_body);

/* Parse a ClientQuery JSON body (the server's /query request,
 * src/bin/server.rs:120-177; ClientQuery, src/pir/query.rs:119-132): rgsw
 * receives the 2*gadget_len RGSW rows as [row][a, b][poly] (the
 * inspire_query layout); the other outputs as for
 * inspire_seeded_query_from_json. */
int inspire_query_from_json(const inspire_params *params, const char *json, size_t len, uint32_t *shard_id,
                            uint64_t *rgsw, int32_t *packing_mode, int32_t *has_keys, uint64_t *y_body);

/* The server's JSON reply {"response": ServerResponse, "processing_time_ms": t}
 * for ciphertext ct[2][poly] and n_columns column ciphertexts
 * columns[n][2][poly].  buf NULL: *len receives the size only. */
int inspire_query_response_to_json(const inspire_params *params, const uint64_t *ct, uint32_t n_columns,
                                   const uint64_t *columns, uint64_t processing_time_ms, char *buf, size_t cap,
                                   size_t *len);

/* The server's JSON reply for a tree-packing response (respond_one_packing,
 * src/pir/respond.rs:213-268): ciphertext (a [poly], b [b_words words], the
 * b polynomial's dimension being b_words / 2 -- 2*ring_dim for the crate's
 * compat-mode b), no column ciphertexts.  buf NULL: *len receives the size
 * only. */
int inspire_packed_response_to_json(const inspire_params *params, const uint64_t *a, const uint64_t *b,
                                    uint32_t b_words, uint64_t processing_time_ms, char *buf, size_t cap,
                                    size_t *len);

/* ServerResponse::to_binary (bincode) of the same response. */
int inspire_server_response_to_bincode(const inspire_params *params, const uint64_t *ct, uint32_t n_columns,
                                       const uint64_t *columns, uint8_t *buf, size_t cap, size_t *len);

/* ---- HTTP front end ----
 * The crate's server binary (src/bin/server.rs:242-337) over this ABI: the
 * routes GET /health, GET /params, GET /crs, POST /query, POST /query_seeded
 * with the crate's JSON shapes, status codes and error texts (QueryResponse
 * {response, processing_time_ms}; 400 {"error": ...}; 400/422/415 for bodies
 * that are not JSON, not the target type, or not application/json).  One
 * thread per connection, HTTP/1.1 keep-alive.  Seeded InspiRING queries go
 * through `srv` (a serving loop on `ctx`; NULL: the synchronous call), the
 * other kinds through the synchronous entry points on (ctx, db).  The client
 * keys of each query stay registered, keyed by a hash of y_body, evicted
 * least-recently-used beyond max_clients or when the context's device budget
 * refuses new keys.  ctx, db and srv must outlive the server. */
typedef struct inspire_http_server inspire_http_server;

typedef struct {
  const char *host;     /* IPv4 address to bind ("0.0.0.0", "127.0.0.1") */
  uint16_t port;        /* 0: any free port (inspire_http_port tells which) */
  uint32_t max_clients; /* resident client keys kept */
  uint64_t max_body;    /* request body limit in bytes (413 beyond) */
  const char *version;  /* /params: metadata.json's version, entry_count, shard_count */
  uint64_t entry_count;
  uint64_t shard_count;
} inspire_http_config;

/* host 127.0.0.1, port 0, max_clients 4096, max_body 64 MiB, version "1.0.0". */
void inspire_http_config_default(inspire_http_config *cfg);
/* Start serving (accepting in a thread of its own); crs_json (may be NULL)
 * is what GET /crs returns. */
int inspire_http_start(inspire_ctx *ctx, const inspire_db *db, inspire_server *srv, const inspire_http_config *cfg,
                       const char *crs_json, size_t crs_len, inspire_http_server **out);
uint16_t inspire_http_port(const inspire_http_server *http);
/* Stop accepting, close every connection (requests in progress finish
 * first), release the cached client keys, free the server. */
void inspire_http_stop(inspire_http_server *http);

/* Batched NttContext::forward / inverse (src/math/ntt.rs:223-325) on device
 * data polys[npolys][2][ring_dim] (u32 residues), in place.  Forward outputs
 * the crate's NTT-domain values (Montgomery form, R = 2^64, bit-reversed slot
 * order); inverse takes them and returns coefficients. */
int inspire_ntt_forward_device(inspire_ctx *ctx, uint32_t *d_polys, uint32_t npolys, void *stream);
int inspire_ntt_inverse_device(inspire_ctx *ctx, uint32_t *d_polys, uint32_t npolys, void *stream);

/* Batched external_product (src/rgsw/external_product.rs:88-150) on device
 * data: ct[n][2][2][ring_dim], rgsw[n][2*gadget_len][2][2][ring_dim],
 * out[n][2][2][ring_dim] (u32 residues). */
int inspire_external_product_device(inspire_ctx *ctx, const uint32_t *d_ct, const uint32_t *d_rgsw,
                                    uint32_t *d_out, uint32_t npairs, void *stream);

/* Client side, for verification at scale: RlweCiphertext::decrypt
 * (src/rlwe/enc.rs:90-108) + extract_inspiring (src/pir/extract.rs:155-182,
 * reconstruct_entry src/pir/encode_db.rs:186-201) of n packed responses on
 * the device.  d_sk: the client's RLWE secret key [poly] (u64, residue-major);
 * d_ct: [n][2][poly] (u64, as the Respond calls return them); d_entries
 * receives [n][entry_size] bytes (entry_size <= 32). */
int inspire_extract_inspiring_device(inspire_ctx *ctx, const uint64_t *d_sk, const uint64_t *d_ct, uint32_t n,
                                     uint32_t entry_size, uint8_t *d_entries, void *stream);

/* Allocation-free tree packing on device buffers; no reference counterpart.
 * Answers n <= 2 seeded queries like inspire_respond_seeded_packed_batch, but
 * takes device pointers (d_shard_ids [n], d_seeds [n][gadget_len][32] and
 * d_b_rows [n][gadget_len][poly] of RGSW rows gadget_len..2*gadget_len-1,
 * as inspire_respond_seeded_batch_device takes them; d_out_a [n][poly],
 * d_out_b [n][2 polys], d_status [n]) and enqueues its work on `stream`
 * without allocating: its scratch (column ciphertexts, combined ciphertext,
 * the tree's work area; 2.0 MiB per query) is one static device array per
 * device, whose address is looked up with cudaGetSymbolAddress on every
 * call.  The first call on a device may load the library's device code into
 * that device's context (CUDA's lazy loading), so make it before any stream
 * capture.  n > 2 is rejected.
 * Calls that overlap on the device (from several host threads, or on
 * streams that run concurrently) race on that array: issue them on one
 * stream, or wait for one to finish before the next starts.  A query whose
 * status is nonzero has undefined outputs.  *b_words is set as for the
 * other tree-packing calls. */
int inspire_respond_seeded_packed_noalloc_device(inspire_ctx *ctx, const inspire_db *db, uint32_t n,
                                                 const uint32_t *d_shard_ids, const uint8_t *d_seeds,
                                                 const uint64_t *d_b_rows, uint64_t *d_out_a, uint64_t *d_out_b,
                                                 int32_t *d_status, uint32_t *b_words, void *stream);

/* Setup side: the log2(ring_dim) Galois key-switching matrices of the
 * secret key d_sk [poly] (ServerCrs.galois_keys, src/pir/setup.rs:164-173;
 * generate_automorphism_ks_matrix, src/ks/setup.rs:218-245): matrix i for
 * t = ring_dim / 2^i + 1, row k = (a, -a s + e + tau_t(s) z^k), written to
 * d_keys [log2(ring_dim)][2*gadget_len][poly] in the layout
 * inspire_crs_load_galois_keys reads; d_status [log2(ring_dim)].  a is
 * uniform (Poly::from_seed_moduli of a seed) and e the crate's discrete
 * Gaussian, both from a ChaCha20 stream keyed by `key`, disjoint from the
 * query and client-key streams of the same key; the crate's thread_rng draws
 * are not reproduced. */
int inspire_galois_keygen_device(inspire_ctx *ctx, const uint8_t *key, const uint64_t *d_sk, uint64_t *d_keys,
                                 int32_t *d_status, void *stream);

/* Setup side: every public key of setup (src/pir/setup.rs:151-200) for the
 * secret key d_sk [poly].  d_ks receives log2(ring_dim) + 4 key-switching
 * matrices [.][2*gadget_len][poly], row k = (a, -a s + e + s_i z^k):
 *   i < log2(ring_dim): galois_keys, equal to inspire_galois_keygen_device's
 *     output for the same key;
 *   i = log2(ring_dim): k_g, s_i = tau_3(s); i = log2(ring_dim) + 1: k_h,
 *     s_i = tau_{2 ring_dim - 1}(s) (generate_automorphism_ks_matrix,
 *     src/ks/setup.rs:218-245; galois_generators, src/rlwe/galois.rs:80-91);
 *   i = log2(ring_dim) + 2, + 3: packing_k_g, packing_k_h, s_i the LWE key
 *     of s (generate_packing_ks_matrix, src/ks/setup.rs:183-205;
 *     LweSecretKey::from_rlwe, src/lwe/enc.rs:53-66).
 * d_crs_a (may be NULL) receives crs_a_vectors (setup.rs:175-180):
 * ring_dim uniform polys [ring_dim][poly].  d_status [log2(ring_dim) + 5]:
 * one per matrix, the last for crs_a_vectors.  Uniform polys and errors come
 * from the ChaCha20 stream keyed by `key` (as inspire_galois_keygen_device);
 * the crate's thread_rng draws are not reproduced. */
int inspire_setup_keygen_device(inspire_ctx *ctx, const uint8_t *key, const uint64_t *d_sk, uint64_t *d_ks,
                                uint64_t *d_crs_a, int32_t *d_status, void *stream);

/* Client side, for load generation at served rates: keys of n clients,
 * numbered first_client + i.  d_sk receives each RlweSecretKey::generate
 * (src/rlwe/enc.rs:14-17) [n][poly] and d_y_body each ClientPackingKeys
 * body (generate_ksk_body, src/inspiring/inspiring2.rs:846-902: tau_g(s) z^k
 * - s w_mask[k] + e_k, g = gen_pows[1], w_mask of the loaded CRS's w_seed)
 * [n][gadget_len][poly] (u64, residue-major); register the bodies with
 * inspire_client_register.  Secret-key and error coefficients are the crate's
 * discrete Gaussian drawn by inverse table from a ChaCha20 stream keyed by
 * `key` (32 bytes), disjoint from the query streams of the same key; the
 * crate's own randomness is not reproduced.  Requires a loaded CRS and
 * first_client + n <= 2^30. */
int inspire_client_keygen_device(inspire_ctx *ctx, const uint8_t *key, uint64_t first_client, uint32_t n,
                                 uint64_t *d_sk, uint64_t *d_y_body, void *stream);

/* Client side, for load generation at served rates: n seeded queries
 * (query_seeded, src/pir/query.rs:43-85; SeededRgswCiphertext::encrypt,
 * src/rgsw/types.rs:233-300) of the inverse monomials X^-k, k =
 * d_local_idx[i] mod ring_dim, under the secret key d_sk [poly] (u64,
 * residue-major).  Row seeds come from a ChaCha20 stream keyed by `key` (32
 * bytes), indexed by query number first_query + i, and the errors are the
 * crate's discrete Gaussian (sigma, tail cut ceil(6 sigma)) drawn by inverse
 * table from the same stream; the crate's own randomness (thread_rng and a
 * rejection sampler) is not reproduced.  Outputs in the crate's row order:
 * d_seeds [n][2*gadget_len][32], d_b_rows [n][2*gadget_len][poly],
 * d_status [n] (0, or 1 if a seed's expansion hit its bound).  Requires
 * first_query + n <= 2^36. */
int inspire_query_seeded_device(inspire_ctx *ctx, const uint64_t *d_sk, const uint8_t *key, uint64_t first_query,
                                uint32_t n, const uint32_t *d_local_idx, uint8_t *d_seeds, uint64_t *d_b_rows,
                                int32_t *d_status, void *stream);

/* Rate probe with no crate counterpart: blocks x 256 threads x 8
 * independent chains x iters exact 28-bit modular multiplies (Shoup's
 * method, the operation the transforms and products are built from) on
 * `stream`; d_sink receives blocks * 256 u32.  Timing it gives the integer
 * roofline denominator of the integer-bound kernels. */
int inspire_mulmod_rate_device(inspire_ctx *ctx, uint32_t blocks, uint32_t iters, uint32_t *d_sink, void *stream);

/* Rate probe with no crate counterpart: the integer tensor-core rate that an
 * 8-bit-limb contraction would run at.  blocks x 8 warps x 4 chains x iters
 * INT8 MMAs (mma.sync m16n8k32, s8 x s8 -> s32; 8192 operations each) of
 * d_a (16 x 32 s8, row-major) by d_b (32 x 8 s8, row-major) on `stream`.
 * d_out [4][16][8] receives the first warp's four accumulators, each exactly
 * iters * (A B).  iters <= 4096 (no INT32 overflow). */
int inspire_int8_mma_rate_device(inspire_ctx *ctx, uint32_t blocks, uint32_t iters, const int8_t *d_a,
                                 const int8_t *d_b, int32_t *d_out, void *stream);

#ifdef __cplusplus
}
#endif
#endif
