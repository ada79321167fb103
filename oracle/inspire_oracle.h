/*
 * inspire_oracle.h -- CPU oracle for the InsPIRe server Respond path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * crate igor53627/inspire-rs (v0.1.2) for the Respond path, used as the
 * checker of the CUDA library and as the timed CPU baseline.  Only tests/,
 * __graft_entry__.smoke() and bench.py (cpu_baseline and --impl reference)
 * may load it.  The product library never links, loads or calls it.
 *
 * Parity status: the modular arithmetic (NTT, Montgomery, CRT, gadget,
 * external product, InspiRING packing) is pinned against the reference's own
 * known-answer tests (src/math/ntt.rs:590-749, src/math/poly.rs:936-1116,
 * src/rgsw/external_product.rs:171-365, src/inspiring/inspiring2.rs:1689-1806,
 * tests/e2e_pir.rs:464-535).  The ChaCha20 block is pinned by the RFC 8439
 * known-answer blocks.  The rand 0.8 / rand_chacha 0.3 stream semantics
 * (gen_range rejection sampling, next_u64 word order) are restated from the
 * published algorithms; no golden vector of the reference pins them, so
 * bit parity of *seed-expanded* polynomials is unpinned at that boundary
 * (everything downstream of the expanded polynomials is pinned).
 *
 * Layout conventions follow the reference Poly (src/math/poly.rs:64-77):
 * a polynomial is `crt * n` u64 values, residue-major ([mod0 coeffs..., mod1
 * coeffs...]), each canonical (< its modulus).  NTT-domain values are the
 * reference's Montgomery form (R = 2^64).
 */
#ifndef INSPIRE_ORACLE_H
#define INSPIRE_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Automorphism-in-NTT-domain semantics (src/inspiring/inspiring2.rs:279-296).
 * IO_MODE_COMPAT reproduces the reference exactly: only the residue-0 slice is
 * permuted and residue 1 is rebuilt as (residue-0 Montgomery value mod q1).
 * IO_MODE_CRT_FIXED applies the same permutation to every residue slice. */
#define IO_MODE_COMPAT 0
#define IO_MODE_CRT_FIXED 1

typedef struct io_ctx io_ctx;
typedef struct io_pack io_pack;
typedef struct io_sampler io_sampler;
typedef struct io_rng io_rng;

/* ---- parameters + NTT context (params.rs:135-298, ntt.rs:116-164) ---- */
io_ctx *io_ctx_new(int n, int crt, const uint64_t *moduli, uint64_t p,
                   double sigma, uint64_t gadget_base, int gadget_len);
void io_ctx_free(io_ctx *ctx);
uint64_t io_ctx_q(const io_ctx *ctx);
uint64_t io_ctx_delta(const io_ctx *ctx);
uint64_t io_ctx_psi(const io_ctx *ctx, int r);
/* forward/inverse twiddle tables of residue r (n entries each, Montgomery) */
void io_ctx_twiddles(const io_ctx *ctx, int r, uint64_t *fwd, uint64_t *inv);

/* ---- NTT / Poly (ntt.rs:223-379, poly.rs:426-630) ---- */
void io_ntt_forward(const io_ctx *ctx, uint64_t *polys, int npolys);
void io_ntt_inverse(const io_ctx *ctx, uint64_t *polys, int npolys);
void io_poly_mul(const io_ctx *ctx, const uint64_t *a, const uint64_t *b,
                 uint64_t *out);
uint64_t io_poly_coeff(const io_ctx *ctx, const uint64_t *poly, int i);
void io_poly_from_composite(const io_ctx *ctx, const uint64_t *coeffs,
                            uint64_t *out);

/* ---- RGSW / RLWE (rgsw/external_product.rs:16-150, rlwe/enc.rs, rlwe/galois.rs) ---- */
void io_gadget_decompose(const io_ctx *ctx, const uint64_t *poly,
                         uint64_t *out);
void io_gadget_reconstruct(const io_ctx *ctx, const uint64_t *digits,
                           uint64_t *out);
/* ct = [a poly, b poly]; rgsw = 2*ell rows of [a poly, b poly] */
void io_external_product(const io_ctx *ctx, const uint64_t *ct,
                         const uint64_t *rgsw, uint64_t *out);
void io_automorphism(const io_ctx *ctx, const uint64_t *poly, int t,
                     uint64_t *out);

/* ---- ChaCha20 / rand 0.8 restatement ---- */
/* One ChaCha20 block with state words 12..15 given by ctr_nonce. */
void io_chacha20_block(const uint32_t key[8], const uint32_t ctr_nonce[4],
                       uint32_t out[16]);
io_rng *io_rng_from_seed(const uint8_t seed[32]);   /* ChaCha20Rng::from_seed */
io_rng *io_rng_seed_from_u64(uint64_t state);       /* SeedableRng::seed_from_u64 */
void io_rng_free(io_rng *rng);
uint32_t io_rng_next_u32(io_rng *rng);
uint64_t io_rng_next_u64(io_rng *rng);
uint64_t io_rng_gen_range_u64(io_rng *rng, uint64_t low, uint64_t high);
/* Poly::from_seed_moduli (poly.rs:278-281) */
void io_poly_from_seed(const io_ctx *ctx, const uint8_t seed[32],
                       uint64_t *out);
/* generate_mask_from_seed (inspiring2.rs:816-835): ell polys */
void io_mask_from_seed(const io_ctx *ctx, const uint8_t seed[32], int count,
                       uint64_t *out);

/* ---- InspiRING (inspiring2.rs) ---- */
/* Automorphism table for odd t: closed form.  out[j] = source slot. */
void io_automorph_table_closed(int n, int t, int32_t *out);
/* Brute-force search exactly as generate_automorph_tables (:208-263). */
void io_automorph_table_brute(const io_ctx *ctx, int t, io_rng *rng,
                              int32_t *out);
/* PackParams::new + OfflinePackingKeys::generate.  brute=1 builds the
 * automorphism tables by the reference's brute-force search and the monomial
 * NTTs by transforming every monomial (the reference's per-query cost);
 * brute=0 uses the closed forms (identical values). */
io_pack *io_pack_new(const io_ctx *ctx, int gamma, const uint8_t w_seed[32],
                     int mode, int brute, uint64_t rng_seed);
void io_pack_free(io_pack *pk);
int io_pack_generator(const io_pack *pk);
void io_pack_gen_pows(const io_pack *pk, int32_t *out); /* n entries */
uint64_t io_pack_mod_inv_gamma(const io_pack *pk);
/* w_all_ntt: (gamma-1)*ell polys, Montgomery NTT form */
void io_pack_w_all_ntt(const io_pack *pk, uint64_t *out);
/* packing_offline (:926-1041): a_ct = gamma coefficient polys.
 * out_a_hat: 1 poly; out_bold_t: (gamma-1)*ell polys (coefficient form). */
void io_packing_offline(const io_pack *pk, const uint64_t *a_ct,
                        uint64_t *out_a_hat, uint64_t *out_bold_t);
/* generate_rotations (:1309-1323): y_body ell polys -> (gamma-1)*ell polys */
void io_generate_rotations(const io_pack *pk, const uint64_t *y_body,
                           uint64_t *y_all);
/* packing_online (:1185-1222) */
void io_packing_online(const io_pack *pk, const uint64_t *a_hat,
                       const uint64_t *bold_t, const uint64_t *y_all,
                       const uint64_t *b_poly, uint64_t *out_ct);

/* ---- Respond (pir/respond.rs:284-398) ---- */
/* respond_inspiring.  shard = gamma column polys; rgsw = full expanded RGSW
 * (2*ell rows of [a, b]).  Exactly one of y_all / y_body non-NULL (y_all takes
 * precedence as in respond.rs:365-377).  pk == NULL rebuilds PackParams and
 * OfflinePackingKeys per call with brute-force tables, as respond.rs:360-361
 * do; otherwise pk (built for this gamma, w_seed and mode) is reused.
 * Returns 0 on success, negative on error.  out_ct = [a_hat, b]. */
int io_respond_inspiring(const io_ctx *ctx, const io_pack *pk, int mode,
                         const uint8_t w_seed[32], const uint64_t *shard,
                         int gamma, const uint64_t *rgsw,
                         const uint64_t *y_body, const uint64_t *y_all,
                         uint64_t *out_ct, int nthreads);
/* SeededRgswCiphertext::expand (rgsw/types.rs:315-318): seeds 2*ell x 32 B,
 * b_rows 2*ell polys -> rgsw 2*ell rows of [a, b]. */
void io_expand_rgsw(const io_ctx *ctx, const uint8_t *seeds,
                    const uint64_t *b_rows, uint64_t *rgsw);
/* respond (NoPacking) (:71-115): out = combined ct [a,b]; out_cols may be
 * NULL, else ncols cts. */
int io_respond_nopacking(const io_ctx *ctx, const uint64_t *shard, int ncols,
                         const uint64_t *rgsw, uint64_t *out_ct,
                         uint64_t *out_cols, int nthreads);

/* ---- database encoding (pir/encode_db.rs:80-201) ---- */
int io_num_columns(int entry_size);
/* encode one shard: entries [shard_id*n, ...) of db; out = ncols polys */
void io_encode_shard(const io_ctx *ctx, const uint8_t *db, uint64_t db_len,
                     int entry_size, uint32_t shard_id, uint64_t *out);
void io_inverse_monomial(const io_ctx *ctx, int k, uint64_t *out);

/* ---- client side (for fixtures; pir/query.rs, extract.rs) ---- */
io_sampler *io_sampler_new(double sigma, uint64_t seed);
void io_sampler_free(io_sampler *s);
int64_t io_sampler_sample(io_sampler *s);
void io_sk_generate(const io_ctx *ctx, io_sampler *s, uint64_t *sk);
/* RLWE encryption of Delta*msg with a fresh uniform a (rlwe/enc.rs:32-51) */
void io_rlwe_encrypt(const io_ctx *ctx, io_sampler *s, io_rng *rng,
                     const uint64_t *sk, const uint64_t *msg, uint64_t *ct);
/* RgswCiphertext::encrypt (rgsw/types.rs:133-187): msg poly */
void io_rgsw_encrypt(const io_ctx *ctx, io_sampler *s, io_rng *rng,
                     const uint64_t *sk, const uint64_t *msg, uint64_t *rgsw);
/* SeededRgswCiphertext::encrypt of X^-local_idx (rgsw/types.rs:235-300) */
void io_query_seeded(const io_ctx *ctx, io_sampler *s, io_rng *rng,
                     const uint64_t *sk, int local_idx, uint8_t *seeds,
                     uint64_t *b_rows);
/* ClientPackingKeys::generate (inspiring2.rs:640-707): y_body ell polys;
 * y_all (gamma-1)*ell polys built with the pack's mode. */
void io_client_packing_keys(const io_pack *pk, io_sampler *s,
                            const uint64_t *sk, uint64_t *y_body,
                            uint64_t *y_all);
/* tree packing (respond_one_packing, pir/respond.rs:213-268) */
void io_automorphism_ks_matrix(const io_ctx *ctx, io_sampler *s, io_rng *g,
                               const uint64_t *sk, int t, uint64_t *ks);
void io_galois_keys(const io_ctx *ctx, io_sampler *s, io_rng *g,
                    const uint64_t *sk, uint64_t *keys);
int io_pack_lwes(const io_ctx *ctx, const uint64_t *leaf_a, const uint64_t *bval,
                 int nlwe, const uint64_t *keys, int mode, uint64_t *out_a,
                 uint64_t *out_b);
int io_respond_one_packing(const io_ctx *ctx, const uint64_t *shard, int ncols,
                           const uint64_t *rgsw, const uint64_t *keys,
                           int mode, uint64_t *out_a, uint64_t *out_b,
                           int nthreads);
void io_extract_packed(const io_ctx *ctx, const uint64_t *sk, const uint64_t *ct,
                       int entry_size, uint8_t *out);
void io_decrypt(const io_ctx *ctx, const uint64_t *sk, const uint64_t *ct,
                uint64_t *out);
void io_extract_inspiring(const io_ctx *ctx, const uint64_t *sk,
                          const uint64_t *ct, int entry_size, uint8_t *out);

#ifdef __cplusplus
}
#endif
#endif
