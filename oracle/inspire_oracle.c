/*
 * inspire_oracle.c -- CPU oracle for the InsPIRe server Respond path.
 *
 * TEST INFRASTRUCTURE ONLY (see inspire_oracle.h).  Each function restates
 * the reference crate igor53627/inspire-rs v0.1.2 and cites the file:line it
 * follows.  Structure and operation order follow the reference so that the
 * timed CPU baseline does the reference's work, and so that every NTT-domain
 * value is the reference's Montgomery (R = 2^64) value.
 */
#include "inspire_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef unsigned __int128 u128;

/* ===================================================================== */
/* scalar helpers                                                          */
/* ===================================================================== */

static uint64_t powmod(uint64_t b, uint64_t e, uint64_t m) {
  /* ntt.rs:511-522 */
  uint64_t r = 1;
  b %= m;
  while (e) {
    if (e & 1) r = (uint64_t)(((u128)r * b) % m);
    e >>= 1;
    b = (uint64_t)(((u128)b * b) % m);
  }
  return r;
}

static uint64_t modinv(uint64_t a, uint64_t m) {
  /* crt.rs:10-35 (extended Euclid over i128) */
  __int128 t = 0, nt = 1, r = (__int128)m, nr = (__int128)a;
  while (nr != 0) {
    __int128 qq = r / nr, tmp;
    tmp = t - qq * nt; t = nt; nt = tmp;
    tmp = r - qq * nr; r = nr; nr = tmp;
  }
  if (r != 1) return 0;
  if (t < 0) t += (__int128)m;
  return (uint64_t)t;
}

/* ===================================================================== */
/* context: params + NTT tables                                            */
/* ===================================================================== */

struct io_ctx {
  int n, crt;
  uint64_t mod[2];
  uint64_t q;      /* composite */
  uint64_t q0inv;  /* q0^-1 mod q1 (poly.rs:74) */
  uint64_t p, zbase, delta;
  int ell;
  double sigma;
  uint64_t qinvneg[2], r2[2], psi[2], ninv_m[2];
  uint64_t *psi_pow[2], *psi_inv_pow[2];
};

static inline uint64_t mont_mul(uint64_t a, uint64_t b, uint64_t q,
                                uint64_t qin) {
  /* ntt.rs:468-479 */
  u128 ab = (u128)a * b;
  uint64_t m = (uint64_t)ab * qin;
  uint64_t t = (uint64_t)((ab + (u128)m * q) >> 64);
  return t >= q ? t - q : t;
}

static uint64_t q_inv_neg(uint64_t q) {
  /* ntt.rs:497-504 */
  uint64_t y = 1;
  for (int i = 1; i < 64; i++) y |= (y * q) & (1ULL << i);
  return (uint64_t)(0 - y);
}

static uint64_t find_primitive_root(uint64_t order, uint64_t q) {
  /* ntt.rs:525-538: first g >= 2 whose g^((q-1)/order) has exact order */
  uint64_t e = (q - 1) / order;
  for (uint64_t g = 2; g < q; g++) {
    uint64_t c = powmod(g, e, q);
    if (powmod(c, order, q) == 1 && powmod(c, order / 2, q) != 1) return c;
  }
  return 0;
}

static void twiddles(int n, uint64_t psi_m, uint64_t q, uint64_t qin,
                     uint64_t r2, uint64_t *f) {
  /* ntt.rs:541-583 */
  uint64_t one_m = mont_mul(1, r2, q, qin);
  memset(f, 0, sizeof(uint64_t) * (size_t)n);
  f[1] = one_m;
  for (int m = 1; m < n; m++) {
    if ((m & (m - 1)) == 0) {
      int e = n / (2 * m);
      uint64_t pw = one_m;
      for (int k = 0; k < e; k++) pw = mont_mul(pw, psi_m, q, qin);
      f[m] = pw;
    } else {
      f[m] = mont_mul(f[m & (m - 1)], f[m & (-m)], q, qin);
    }
  }
}

io_ctx *io_ctx_new(int n, int crt, const uint64_t *moduli, uint64_t p,
                   double sigma, uint64_t gadget_base, int gadget_len) {
  /* params.rs:135-185, 296-298; ntt.rs:116-164 */
  if (crt < 1 || crt > 2 || n < 2 || (n & (n - 1))) return NULL;
  io_ctx *c = (io_ctx *)calloc(1, sizeof(io_ctx));
  c->n = n;
  c->crt = crt;
  c->q = 1;
  for (int r = 0; r < crt; r++) {
    c->mod[r] = moduli[r];
    c->q *= moduli[r];
  }
  c->q0inv = crt == 2 ? modinv(moduli[0], moduli[1]) : 0;
  c->p = p;
  c->sigma = sigma;
  c->zbase = gadget_base;
  c->ell = gadget_len;
  c->delta = c->q / p;
  for (int r = 0; r < crt; r++) {
    uint64_t q = moduli[r];
    c->qinvneg[r] = q_inv_neg(q);
    uint64_t rm = (uint64_t)(((u128)1 << 64) % q);
    c->r2[r] = (uint64_t)(((u128)rm * rm) % q);
    uint64_t psi = find_primitive_root(2 * (uint64_t)n, q);
    c->psi[r] = psi;
    uint64_t psi_m = mont_mul(psi, c->r2[r], q, c->qinvneg[r]);
    c->psi_pow[r] = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)n);
    c->psi_inv_pow[r] = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)n);
    twiddles(n, psi_m, q, c->qinvneg[r], c->r2[r], c->psi_pow[r]);
    uint64_t psi_inv = powmod(psi, q - 2, q);
    uint64_t psi_inv_m = mont_mul(psi_inv, c->r2[r], q, c->qinvneg[r]);
    twiddles(n, psi_inv_m, q, c->qinvneg[r], c->r2[r], c->psi_inv_pow[r]);
    uint64_t ninv = powmod((uint64_t)n, q - 2, q);
    c->ninv_m[r] = mont_mul(ninv, c->r2[r], q, c->qinvneg[r]);
  }
  return c;
}

void io_ctx_free(io_ctx *c) {
  if (!c) return;
  for (int r = 0; r < c->crt; r++) {
    free(c->psi_pow[r]);
    free(c->psi_inv_pow[r]);
  }
  free(c);
}

uint64_t io_ctx_q(const io_ctx *c) { return c->q; }
uint64_t io_ctx_delta(const io_ctx *c) { return c->delta; }
uint64_t io_ctx_psi(const io_ctx *c, int r) { return c->psi[r]; }

void io_ctx_twiddles(const io_ctx *c, int r, uint64_t *fwd, uint64_t *inv) {
  memcpy(fwd, c->psi_pow[r], sizeof(uint64_t) * (size_t)c->n);
  memcpy(inv, c->psi_inv_pow[r], sizeof(uint64_t) * (size_t)c->n);
}

#define PLEN(c) ((size_t)(c)->n * (size_t)(c)->crt)

/* ===================================================================== */
/* NTT (ntt.rs:223-379)                                                    */
/* ===================================================================== */

static void fwd_at(const io_ctx *c, uint64_t *a, int r) {
  /* ntt.rs:269-294 (Cooley-Tukey DIT) */
  int n = c->n;
  uint64_t q = c->mod[r], qin = c->qinvneg[r];
  const uint64_t *w = c->psi_pow[r];
  int t = n;
  for (int m = 1; m < n; m <<= 1) {
    t >>= 1;
    for (int i = 0; i < m; i++) {
      int j1 = 2 * i * t;
      uint64_t wi = w[m + i];
      for (int j = j1; j < j1 + t; j++) {
        uint64_t u = a[j];
        uint64_t v = mont_mul(a[j + t], wi, q, qin);
        a[j] = u + v >= q ? u + v - q : u + v;
        a[j + t] = u >= v ? u - v : q - v + u;
      }
    }
  }
}

static void inv_at(const io_ctx *c, uint64_t *a, int r) {
  /* ntt.rs:348-379 (Gentleman-Sande DIF) */
  int n = c->n;
  uint64_t q = c->mod[r], qin = c->qinvneg[r];
  const uint64_t *w = c->psi_inv_pow[r];
  int t = 1;
  for (int m = n; m > 1;) {
    m >>= 1;
    for (int i = 0; i < m; i++) {
      int j2 = i * 2 * t;
      uint64_t wi = w[m + i];
      for (int j = j2; j < j2 + t; j++) {
        uint64_t u = a[j], v = a[j + t];
        a[j] = u + v >= q ? u + v - q : u + v;
        uint64_t d = u >= v ? u - v : q - v + u;
        a[j + t] = mont_mul(d, wi, q, qin);
      }
    }
    t <<= 1;
  }
  for (int j = 0; j < n; j++) a[j] = mont_mul(a[j], c->ninv_m[r], q, qin);
}

static void ntt_fwd1(const io_ctx *c, uint64_t *poly) {
  /* ntt.rs:223-246: to Montgomery, then forward */
  for (int r = 0; r < c->crt; r++) {
    uint64_t *a = poly + (size_t)r * c->n;
    for (int j = 0; j < c->n; j++)
      a[j] = mont_mul(a[j], c->r2[r], c->mod[r], c->qinvneg[r]);
    fwd_at(c, a, r);
  }
}

static void ntt_inv1(const io_ctx *c, uint64_t *poly) {
  /* ntt.rs:308-325: inverse then out of Montgomery */
  for (int r = 0; r < c->crt; r++) {
    uint64_t *a = poly + (size_t)r * c->n;
    inv_at(c, a, r);
    for (int j = 0; j < c->n; j++)
      a[j] = mont_mul(a[j], 1, c->mod[r], c->qinvneg[r]);
  }
}

void io_ntt_forward(const io_ctx *c, uint64_t *polys, int np) {
  for (int i = 0; i < np; i++) ntt_fwd1(c, polys + (size_t)i * PLEN(c));
}

void io_ntt_inverse(const io_ctx *c, uint64_t *polys, int np) {
  for (int i = 0; i < np; i++) ntt_inv1(c, polys + (size_t)i * PLEN(c));
}

/* pointwise ops on NTT (Montgomery) values: ntt.rs:394-417, poly.rs:613-630 */
static void pw_mul(const io_ctx *c, const uint64_t *a, const uint64_t *b,
                   uint64_t *o) {
  for (int r = 0; r < c->crt; r++) {
    size_t s = (size_t)r * c->n;
    for (int i = 0; i < c->n; i++)
      o[s + i] = mont_mul(a[s + i], b[s + i], c->mod[r], c->qinvneg[r]);
  }
}

static void pw_mac(const io_ctx *c, uint64_t *acc, const uint64_t *a,
                   const uint64_t *b) {
  for (int r = 0; r < c->crt; r++) {
    size_t s = (size_t)r * c->n;
    uint64_t q = c->mod[r];
    for (int i = 0; i < c->n; i++) {
      uint64_t pr = mont_mul(a[s + i], b[s + i], q, c->qinvneg[r]);
      uint64_t sm = acc[s + i] + pr;
      acc[s + i] = sm >= q ? sm - q : sm;
    }
  }
}

/* poly.rs:710-735 (add), 758-785 (sub), 807-829 (neg) */
static void p_add(const io_ctx *c, const uint64_t *a, const uint64_t *b,
                  uint64_t *o) {
  for (int r = 0; r < c->crt; r++) {
    size_t s = (size_t)r * c->n;
    uint64_t q = c->mod[r];
    for (int i = 0; i < c->n; i++) {
      uint64_t sm = a[s + i] + b[s + i];
      o[s + i] = sm >= q ? sm - q : sm;
    }
  }
}

static void p_neg(const io_ctx *c, const uint64_t *a, uint64_t *o) {
  for (int r = 0; r < c->crt; r++) {
    size_t s = (size_t)r * c->n;
    for (int i = 0; i < c->n; i++)
      o[s + i] = a[s + i] == 0 ? 0 : c->mod[r] - a[s + i];
  }
}

static void p_scalar(const io_ctx *c, const uint64_t *a, uint64_t k,
                     uint64_t *o) {
  /* poly.rs:466-485 */
  for (int r = 0; r < c->crt; r++) {
    size_t s = (size_t)r * c->n;
    uint64_t q = c->mod[r], km = k % q;
    for (int i = 0; i < c->n; i++)
      o[s + i] = (uint64_t)(((u128)a[s + i] * km) % q);
  }
}

void io_poly_mul(const io_ctx *c, const uint64_t *a, const uint64_t *b,
                 uint64_t *out) {
  /* poly.rs:505-532 */
  size_t L = PLEN(c);
  uint64_t *x = (uint64_t *)malloc(8 * L), *y = (uint64_t *)malloc(8 * L);
  memcpy(x, a, 8 * L);
  memcpy(y, b, 8 * L);
  ntt_fwd1(c, x);
  ntt_fwd1(c, y);
  pw_mul(c, x, y, out);
  ntt_inv1(c, out);
  free(x);
  free(y);
}

/* ===================================================================== */
/* CRT (crt.rs:41-56, poly.rs:127-159, 359-388)                            */
/* ===================================================================== */

static inline uint64_t crt_compose(const io_ctx *c, uint64_t a0, uint64_t a1) {
  uint64_t q0 = c->mod[0], q1 = c->mod[1];
  uint64_t a0m = a0 % q1;
  uint64_t diff = a1 >= a0m ? a1 - a0m : (a1 + q1) - a0m;
  uint64_t t = (uint64_t)(((u128)diff * c->q0inv) % q1);
  return a0 + q0 * t;
}

uint64_t io_poly_coeff(const io_ctx *c, const uint64_t *poly, int i) {
  if (c->crt == 1) return poly[i];
  return crt_compose(c, poly[i], poly[i + c->n]) % c->q;
}

static inline void set_coeff(const io_ctx *c, uint64_t *poly, int i,
                             uint64_t v) {
  for (int r = 0; r < c->crt; r++) poly[(size_t)r * c->n + i] = v % c->mod[r];
}

void io_poly_from_composite(const io_ctx *c, const uint64_t *coeffs,
                            uint64_t *out) {
  for (int i = 0; i < c->n; i++) set_coeff(c, out, i, coeffs[i]);
}

/* ===================================================================== */
/* gadget + external product (rgsw/external_product.rs:16-150)             */
/* ===================================================================== */

void io_gadget_decompose(const io_ctx *c, const uint64_t *poly,
                         uint64_t *out) {
  /* external_product.rs:16-37 */
  size_t L = PLEN(c);
  memset(out, 0, 8 * L * (size_t)c->ell);
  for (int j = 0; j < c->n; j++) {
    uint64_t v = io_poly_coeff(c, poly, j);
    for (int i = 0; i < c->ell; i++) {
      set_coeff(c, out + (size_t)i * L, j, v % c->zbase);
      v /= c->zbase;
    }
  }
}

void io_gadget_reconstruct(const io_ctx *c, const uint64_t *digits,
                           uint64_t *out) {
  /* external_product.rs:43-75; GadgetVector::powers (rgsw/types.rs:79-90) */
  size_t L = PLEN(c);
  uint64_t *tmp = (uint64_t *)malloc(8 * L);
  memset(out, 0, 8 * L);
  u128 pw = 1;
  for (int i = 0; i < c->ell; i++) {
    p_scalar(c, digits + (size_t)i * L, (uint64_t)pw, tmp);
    p_add(c, out, tmp, out);
    pw = (pw * c->zbase) % c->q;
  }
  free(tmp);
}

void io_external_product(const io_ctx *c, const uint64_t *ct,
                         const uint64_t *rgsw, uint64_t *out) {
  /* external_product.rs:88-150: 4*ell mul_ntt, coefficient-domain sums */
  size_t L = PLEN(c);
  int ell = c->ell;
  uint64_t *ad = (uint64_t *)malloc(8 * L * ell);
  uint64_t *bd = (uint64_t *)malloc(8 * L * ell);
  uint64_t *tmp = (uint64_t *)malloc(8 * L);
  io_gadget_decompose(c, ct, ad);
  io_gadget_decompose(c, ct + L, bd);
  uint64_t *ra = out, *rb = out + L;
  memset(out, 0, 16 * L);
  for (int i = 0; i < ell; i++) {
    const uint64_t *rowa = rgsw + (size_t)(2 * i) * L;
    const uint64_t *rowb = rgsw + (size_t)(2 * (ell + i)) * L;
    io_poly_mul(c, ad + i * L, rowa, tmp);
    p_add(c, ra, tmp, ra);
    io_poly_mul(c, ad + i * L, rowa + L, tmp);
    p_add(c, rb, tmp, rb);
    io_poly_mul(c, bd + i * L, rowb, tmp);
    p_add(c, ra, tmp, ra);
    io_poly_mul(c, bd + i * L, rowb + L, tmp);
    p_add(c, rb, tmp, rb);
  }
  free(ad);
  free(bd);
  free(tmp);
}

void io_automorphism(const io_ctx *c, const uint64_t *poly, int g,
                     uint64_t *out) {
  /* rlwe/galois.rs:22-55 on composite coefficients; mod_add/mod_sub :126-141 */
  int d = c->n;
  uint64_t q = c->q;
  uint64_t *rc = (uint64_t *)calloc((size_t)d, 8);
  for (int i = 0; i < d; i++) {
    uint64_t co = io_poly_coeff(c, poly, i);
    if (co == 0) continue;
    long long ni = ((long long)g * i) % (2 * d);
    if (ni < d) {
      rc[ni] = (uint64_t)(((u128)rc[ni] + co) % q);
    } else {
      uint64_t a = rc[ni - d];
      rc[ni - d] = a >= co ? a - co : q - co + a;
    }
  }
  io_poly_from_composite(c, rc, out);
  free(rc);
}

/* ===================================================================== */
/* ChaCha20 (RFC 8439 block) + rand_core / rand 0.8 semantics              */
/* ===================================================================== */

#define ROTL(x, k) (((x) << (k)) | ((x) >> (32 - (k))))
#define QR(a, b, c, d)                                                        \
  a += b; d ^= a; d = ROTL(d, 16); c += d; b ^= c; b = ROTL(b, 12);          \
  a += b; d ^= a; d = ROTL(d, 8);  c += d; b ^= c; b = ROTL(b, 7);

void io_chacha20_block(const uint32_t key[8], const uint32_t cn[4],
                       uint32_t out[16]) {
  uint32_t s[16] = {0x61707865u, 0x3320646eu, 0x79622d32u, 0x6b206574u};
  for (int i = 0; i < 8; i++) s[4 + i] = key[i];
  for (int i = 0; i < 4; i++) s[12 + i] = cn[i];
  uint32_t x[16];
  memcpy(x, s, sizeof x);
  for (int i = 0; i < 10; i++) {
    QR(x[0], x[4], x[8], x[12]);
    QR(x[1], x[5], x[9], x[13]);
    QR(x[2], x[6], x[10], x[14]);
    QR(x[3], x[7], x[11], x[15]);
    QR(x[0], x[5], x[10], x[15]);
    QR(x[1], x[6], x[11], x[12]);
    QR(x[2], x[7], x[8], x[13]);
    QR(x[3], x[4], x[9], x[14]);
  }
  for (int i = 0; i < 16; i++) out[i] = x[i] + s[i];
}

/* ChaCha20Rng (rand_chacha 0.3): key = seed, 64-bit block counter in state
 * words 12-13 starting at 0, stream id 0 in words 14-15.  Output words are
 * consumed in keystream order; next_u64 = lo | hi << 32 (rand_core 0.6
 * BlockRng::next_u64, which stays in keystream order across refills). */
struct io_rng {
  uint32_t key[8];
  uint64_t ctr;
  uint32_t buf[16];
  int idx;
};

static io_rng *rng_new_key(const uint8_t seed[32]) {
  io_rng *g = (io_rng *)calloc(1, sizeof(io_rng));
  for (int i = 0; i < 8; i++)
    g->key[i] = (uint32_t)seed[4 * i] | ((uint32_t)seed[4 * i + 1] << 8) |
                ((uint32_t)seed[4 * i + 2] << 16) |
                ((uint32_t)seed[4 * i + 3] << 24);
  g->idx = 16;
  return g;
}

io_rng *io_rng_from_seed(const uint8_t seed[32]) { return rng_new_key(seed); }

io_rng *io_rng_seed_from_u64(uint64_t state) {
  /* rand_core 0.6 SeedableRng::seed_from_u64: PCG32 fills the seed */
  uint8_t seed[32];
  for (int k = 0; k < 8; k++) {
    state = state * 6364136223846793005ULL + 11634580027462260723ULL;
    uint64_t st = state;
    uint32_t xs = (uint32_t)(((st >> 18) ^ st) >> 27);
    uint32_t rot = (uint32_t)(st >> 59);
    uint32_t x = (xs >> rot) | (xs << ((32 - rot) & 31));
    seed[4 * k] = (uint8_t)x;
    seed[4 * k + 1] = (uint8_t)(x >> 8);
    seed[4 * k + 2] = (uint8_t)(x >> 16);
    seed[4 * k + 3] = (uint8_t)(x >> 24);
  }
  return rng_new_key(seed);
}

void io_rng_free(io_rng *g) { free(g); }

uint32_t io_rng_next_u32(io_rng *g) {
  if (g->idx >= 16) {
    uint32_t cn[4] = {(uint32_t)g->ctr, (uint32_t)(g->ctr >> 32), 0, 0};
    io_chacha20_block(g->key, cn, g->buf);
    g->ctr++;
    g->idx = 0;
  }
  return g->buf[g->idx++];
}

uint64_t io_rng_next_u64(io_rng *g) {
  uint64_t lo = io_rng_next_u32(g);
  uint64_t hi = io_rng_next_u32(g);
  return lo | (hi << 32);
}

static void rng_fill_bytes(io_rng *g, uint8_t *out, int len) {
  for (int i = 0; i < len; i += 4) {
    uint32_t w = io_rng_next_u32(g);
    for (int k = 0; k < 4 && i + k < len; k++) out[i + k] = (uint8_t)(w >> (8 * k));
  }
}

static inline int clz64(uint64_t x) { return x ? __builtin_clzll(x) : 64; }

uint64_t io_rng_gen_range_u64(io_rng *g, uint64_t low, uint64_t high) {
  /* rand 0.8 UniformInt::<u64>::sample_single(low, high) ->
   * sample_single_inclusive(low, high - 1): widening-multiply rejection with
   * zone = (range << leading_zeros(range)) - 1. */
  uint64_t range = high - low;
  if (range == 0) return io_rng_next_u64(g);
  uint64_t zone = (range << clz64(range)) - 1;
  for (;;) {
    uint64_t v = io_rng_next_u64(g);
    u128 m = (u128)v * range;
    uint64_t hi = (uint64_t)(m >> 64), lo = (uint64_t)m;
    if (lo <= zone) return low + hi;
  }
}

static int64_t gen_range_i64_incl(io_rng *g, int64_t low, int64_t high) {
  /* rand 0.8 UniformInt::<i64>::sample_single_inclusive */
  uint64_t range = (uint64_t)(high - low) + 1;
  if (range == 0) return (int64_t)io_rng_next_u64(g);
  uint64_t zone = (range << clz64(range)) - 1;
  for (;;) {
    uint64_t v = io_rng_next_u64(g);
    u128 m = (u128)v * range;
    uint64_t hi = (uint64_t)(m >> 64), lo = (uint64_t)m;
    if (lo <= zone) return (int64_t)((uint64_t)low + hi);
  }
}

static double gen_f64(io_rng *g) {
  /* rand 0.8 Standard for f64: 53 high bits scaled by 2^-53 */
  return (double)(io_rng_next_u64(g) >> 11) * (1.0 / 9007199254740992.0);
}

static void random_poly(const io_ctx *c, io_rng *g, uint64_t *out) {
  /* poly.rs:251-268: residue-major gen_range(0..modulus) */
  for (int r = 0; r < c->crt; r++)
    for (int i = 0; i < c->n; i++)
      out[(size_t)r * c->n + i] = io_rng_gen_range_u64(g, 0, c->mod[r]);
}

void io_poly_from_seed(const io_ctx *c, const uint8_t seed[32],
                       uint64_t *out) {
  io_rng *g = io_rng_from_seed(seed);
  random_poly(c, g, out);
  io_rng_free(g);
}

void io_mask_from_seed(const io_ctx *c, const uint8_t seed[32], int count,
                       uint64_t *out) {
  /* inspiring2.rs:816-835: next_u64() % q (composite), then CRT split */
  io_rng *g = io_rng_from_seed(seed);
  uint64_t *co = (uint64_t *)malloc(8 * (size_t)c->n);
  for (int k = 0; k < count; k++) {
    for (int i = 0; i < c->n; i++) co[i] = io_rng_next_u64(g) % c->q;
    io_poly_from_composite(c, co, out + (size_t)k * PLEN(c));
  }
  free(co);
  io_rng_free(g);
}

/* ===================================================================== */
/* InspiRING (inspiring2.rs)                                               */
/* ===================================================================== */

static int bitrev(int x, int logn) {
  int r = 0;
  for (int i = 0; i < logn; i++) r |= ((x >> i) & 1) << (logn - 1 - i);
  return r;
}

void io_automorph_table_closed(int n, int t, int32_t *out) {
  /* NTT slot j of the reference forward transform holds a(psi^(2*brv(j)+1))
   * (checked against direct evaluation in the oracle tests), so tau_t moves
   * slot source i with 2*brv(i)+1 = t*(2*brv(j)+1) mod 2n into slot j. */
  int logn = 0;
  while ((1 << logn) < n) logn++;
  for (int j = 0; j < n; j++) {
    long long e = (long long)t * (2 * bitrev(j, logn) + 1) % (2 * n);
    out[j] = bitrev((int)((e - 1) / 2), logn);
  }
}

void io_automorph_table_brute(const io_ctx *c, int t, io_rng *g,
                              int32_t *out) {
  /* inspiring2.rs:208-263, one odd t: compare residue-0 NTT values */
  int n = c->n;
  size_t L = PLEN(c);
  uint64_t *a = (uint64_t *)malloc(8 * L), *an = (uint64_t *)malloc(8 * L);
  uint64_t *b = (uint64_t *)malloc(8 * L);
  for (;;) {
    random_poly(c, g, a);
    io_automorphism(c, a, t, b);
    memcpy(an, a, 8 * L);
    ntt_fwd1(c, an);
    ntt_fwd1(c, b);
    int redo = 0;
    for (int i = 0; i < n && !redo; i++) {
      uint64_t ov = an[i];
      int cnt = 0, found = -1;
      for (int j = 0; j < n; j++)
        if (b[j] == ov) {
          cnt++;
          found = j;
        }
      if (cnt != 1) redo = 1;
      else out[found] = i;
    }
    if (!redo) break;
  }
  free(a);
  free(an);
  free(b);
}

struct io_pack {
  const io_ctx *c;
  int n;  /* ring dimension, kept so io_pack_free never touches c */
  int gamma, gen, mode;
  uint8_t w_seed[32];
  int32_t *gen_pows;       /* n */
  uint64_t mod_inv_gamma;
  uint64_t *mod_inv_ntt;   /* 1 poly, Montgomery NTT */
  uint64_t *mono_ntt;      /* 2n polys: NTT(X^e), e in [0, 2n) */
  int32_t **tables;        /* n tables (odd t), lazily filled */
  uint64_t *w_all_ntt;     /* (gamma-1)*ell polys */
};

static const int32_t *pack_table(const io_pack *pk, int t) {
  return pk->tables[(t - 1) / 2]; /* PackParams::table_index :188-191 */
}

static void apply_auto_ntt(const io_ctx *c, int mode, const uint64_t *src,
                           const int32_t *tab, uint64_t *out) {
  /* inspiring2.rs:279-296 */
  int n = c->n;
  if (mode == IO_MODE_COMPAT || c->crt == 1) {
    /* result_coeffs[i] = src[table[i]] over the first n words only, then
     * Poly::from_coeffs_moduli re-splits each word into residues. */
    uint64_t *rc = (uint64_t *)malloc(8 * (size_t)n);
    for (int i = 0; i < n; i++) rc[i] = src[tab[i]];
    io_poly_from_composite(c, rc, out);
    free(rc);
  } else {
    for (int r = 0; r < c->crt; r++)
      for (int i = 0; i < n; i++)
        out[(size_t)r * n + i] = src[(size_t)r * n + tab[i]];
  }
}

io_pack *io_pack_new(const io_ctx *c, int gamma, const uint8_t w_seed[32],
                     int mode, int brute, uint64_t rng_seed) {
  /* PackParams::new (inspiring2.rs:107-182) */
  int n = c->n, two_n = 2 * n;
  size_t L = PLEN(c);
  if (gamma < 1) return NULL;
  io_pack *pk = (io_pack *)calloc(1, sizeof(io_pack));
  pk->c = c;
  pk->n = n;
  pk->gamma = gamma;
  pk->mode = mode;
  memcpy(pk->w_seed, w_seed, 32);
  pk->gen = gamma < n ? two_n / gamma + 1 : 5;
  pk->gen_pows = (int32_t *)malloc(4 * (size_t)n);
  long long v = 1;
  for (int i = 0; i < n; i++) {
    pk->gen_pows[i] = (int32_t)v;
    v = (v * pk->gen) % two_n;
  }
  pk->mod_inv_gamma = modinv((uint64_t)gamma, c->q);
  pk->mod_inv_ntt = (uint64_t *)calloc(L, 8);
  set_coeff(c, pk->mod_inv_ntt, 0, pk->mod_inv_gamma);
  ntt_fwd1(c, pk->mod_inv_ntt);
  /* monomials (:143-158): NTT(X^j) and NTT(-X^j) = NTT(X^(j+n)) */
  pk->mono_ntt = (uint64_t *)calloc(L * (size_t)two_n, 8);
  if (brute) {
    for (int j = 0; j < n; j++) {
      uint64_t *pp = pk->mono_ntt + (size_t)j * L;
      uint64_t *pn = pk->mono_ntt + (size_t)(j + n) * L;
      set_coeff(c, pp, j, 1);
      set_coeff(c, pn, j, c->q - 1);
      ntt_fwd1(c, pp);
      ntt_fwd1(c, pn);
    }
  } else {
    /* closed form: slot s of NTT(X^e) = R * psi^(e*(2*brv(s)+1)) */
    int logn = 0;
    while ((1 << logn) < n) logn++;
    for (int r = 0; r < c->crt; r++) {
      uint64_t q = c->mod[r];
      uint64_t *pw = (uint64_t *)malloc(8 * (size_t)two_n);
      uint64_t rm = (uint64_t)(((u128)1 << 64) % q);
      pw[0] = rm;
      for (int k = 1; k < two_n; k++)
        pw[k] = (uint64_t)(((u128)pw[k - 1] * c->psi[r]) % q);
      for (int e = 0; e < two_n; e++) {
        uint64_t *pp = pk->mono_ntt + (size_t)e * L + (size_t)r * n;
        for (int s = 0; s < n; s++)
          pp[s] = pw[(long long)e * (2 * bitrev(s, logn) + 1) % two_n];
      }
      free(pw);
    }
  }
  /* automorphism tables (:208-263) for every odd t < 2n */
  pk->tables = (int32_t **)calloc((size_t)n, sizeof(int32_t *));
  io_rng *g = brute ? io_rng_seed_from_u64(rng_seed) : NULL;
  for (int t = 1; t < two_n; t += 2) {
    int32_t *tab = (int32_t *)malloc(4 * (size_t)n);
    if (brute) io_automorph_table_brute(c, t, g, tab);
    else io_automorph_table_closed(n, t, tab);
    pk->tables[(t - 1) / 2] = tab;
  }
  if (g) io_rng_free(g);
  /* OfflinePackingKeys::generate (:448-506) */
  int ell = c->ell;
  uint64_t *wm = (uint64_t *)malloc(8 * L * (size_t)ell);
  io_mask_from_seed(c, w_seed, ell, wm);
  io_ntt_forward(c, wm, ell);
  pk->w_all_ntt = (uint64_t *)malloc(8 * L * (size_t)(gamma > 1 ? (gamma - 1) * ell : 1));
  for (int i = 0; i < gamma - 1; i++)
    for (int k = 0; k < ell; k++)
      apply_auto_ntt(c, mode, wm + (size_t)k * L, pack_table(pk, pk->gen_pows[i]),
                     pk->w_all_ntt + ((size_t)i * ell + k) * L);
  free(wm);
  return pk;
}

void io_pack_free(io_pack *pk) {
  if (!pk) return;
  for (int i = 0; i < pk->n; i++) free(pk->tables[i]);
  free(pk->tables);
  free(pk->gen_pows);
  free(pk->mod_inv_ntt);
  free(pk->mono_ntt);
  free(pk->w_all_ntt);
  free(pk);
}

int io_pack_generator(const io_pack *pk) { return pk->gen; }
void io_pack_gen_pows(const io_pack *pk, int32_t *out) {
  memcpy(out, pk->gen_pows, 4 * (size_t)pk->c->n);
}
uint64_t io_pack_mod_inv_gamma(const io_pack *pk) { return pk->mod_inv_gamma; }
void io_pack_w_all_ntt(const io_pack *pk, uint64_t *out) {
  memcpy(out, pk->w_all_ntt,
         8 * PLEN(pk->c) * (size_t)((pk->gamma - 1) * pk->c->ell));
}

void io_packing_offline(const io_pack *pk, const uint64_t *a_ct,
                        uint64_t *out_a_hat, uint64_t *out_bold_t) {
  /* inspiring2.rs:926-1041 */
  const io_ctx *c = pk->c;
  int n = c->n, gamma = pk->gamma, ell = c->ell;
  size_t L = PLEN(c);
  uint64_t *a_ntt = (uint64_t *)malloc(8 * L * (size_t)gamma);
  memcpy(a_ntt, a_ct, 8 * L * (size_t)gamma);
  io_ntt_forward(c, a_ntt, gamma);
  uint64_t *r_all = (uint64_t *)malloc(8 * L * (size_t)gamma);
  uint64_t *acc = (uint64_t *)malloc(8 * L), *sc = (uint64_t *)malloc(8 * L);
  for (int i = 0; i < gamma; i++) {
    memset(acc, 0, 8 * L); /* zero poly to_ntt is zero */
    for (int j = 0; j < gamma; j++) {
      int exp_index = (n - i) % n;
      long long index = ((long long)j * pk->gen_pows[exp_index]) % (2 * n);
      pw_mac(c, acc, pk->mono_ntt + (size_t)index * L, a_ntt + (size_t)j * L);
    }
    pw_mul(c, acc, pk->mod_inv_ntt, sc);
    apply_auto_ntt(c, pk->mode, sc, pack_table(pk, pk->gen_pows[i]),
                   r_all + (size_t)i * L);
  }
  uint64_t *rc = (uint64_t *)malloc(8 * L);
  uint64_t *tk = (uint64_t *)malloc(8 * L);
  for (int i = gamma - 2; i >= 0; i--) {
    memcpy(rc, r_all + (size_t)(i + 1) * L, 8 * L);
    ntt_inv1(c, rc);
    uint64_t *bt = out_bold_t + (size_t)i * ell * L;
    io_gadget_decompose(c, rc, bt);
    for (int k = 0; k < ell; k++) {
      memcpy(tk, bt + (size_t)k * L, 8 * L);
      ntt_fwd1(c, tk);
      pw_mac(c, r_all + (size_t)i * L, tk,
             pk->w_all_ntt + ((size_t)i * ell + k) * L);
    }
  }
  memcpy(out_a_hat, r_all, 8 * L);
  ntt_inv1(c, out_a_hat);
  free(a_ntt);
  free(r_all);
  free(acc);
  free(sc);
  free(rc);
  free(tk);
}

void io_generate_rotations(const io_pack *pk, const uint64_t *y_body,
                           uint64_t *y_all) {
  /* inspiring2.rs:1309-1323 */
  const io_ctx *c = pk->c;
  size_t L = PLEN(c);
  for (int i = 0; i < pk->gamma - 1; i++)
    for (int k = 0; k < c->ell; k++)
      io_automorphism(c, y_body + (size_t)k * L, pk->gen_pows[i],
                      y_all + ((size_t)i * c->ell + k) * L);
}

void io_packing_online(const io_pack *pk, const uint64_t *a_hat,
                       const uint64_t *bold_t, const uint64_t *y_all,
                       const uint64_t *b_poly, uint64_t *out_ct) {
  /* inspiring2.rs:1185-1222 */
  const io_ctx *c = pk->c;
  size_t L = PLEN(c);
  uint64_t *sum = (uint64_t *)calloc(L, 8);
  uint64_t *y = (uint64_t *)malloc(8 * L), *t = (uint64_t *)malloc(8 * L);
  for (int i = 0; i < pk->gamma - 1; i++)
    for (int k = 0; k < c->ell; k++) {
      size_t o = ((size_t)i * c->ell + k) * L;
      memcpy(y, y_all + o, 8 * L);
      memcpy(t, bold_t + o, 8 * L);
      ntt_fwd1(c, y);
      ntt_fwd1(c, t);
      pw_mac(c, sum, y, t);
    }
  ntt_inv1(c, sum);
  memcpy(out_ct, a_hat, 8 * L);
  p_add(c, b_poly, sum, out_ct + L);
  free(sum);
  free(y);
  free(t);
}

/* ===================================================================== */
/* Respond (pir/respond.rs)                                                */
/* ===================================================================== */

static void column_products(const io_ctx *c, const uint64_t *shard, int ncols,
                            const uint64_t *rgsw, uint64_t *cols,
                            int nthreads) {
  /* respond.rs:316-324: trivial_encrypt (rlwe/enc.rs:174-182) then
   * external_product per column, columns in parallel */
  size_t L = PLEN(c);
#ifdef _OPENMP
  if (nthreads < 1) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
#endif
  for (int col = 0; col < ncols; col++) {
    uint64_t *ct = (uint64_t *)calloc(2 * L, 8);
    p_scalar(c, shard + (size_t)col * L, c->delta, ct + L);
    io_external_product(c, ct, rgsw, cols + (size_t)col * 2 * L);
    free(ct);
  }
  (void)nthreads;
}

int io_respond_inspiring(const io_ctx *c, const io_pack *pk_in, int mode,
                         const uint8_t w_seed[32], const uint64_t *shard,
                         int gamma, const uint64_t *rgsw,
                         const uint64_t *y_body, const uint64_t *y_all,
                         uint64_t *out_ct, int nthreads) {
  size_t L = PLEN(c);
  int n = c->n, ell = c->ell;
  if (!y_all && !y_body) return -2; /* respond.rs:365-370 */
  if (gamma <= 0) {                 /* respond.rs:307-313 */
    memset(out_ct, 0, 16 * L);
    return 1;
  }
  uint64_t *cols = (uint64_t *)malloc(8 * 2 * L * (size_t)gamma);
  column_products(c, shard, gamma, rgsw, cols, nthreads);
  /* sample_extract_coeff0 b values -> b_poly (respond.rs:326-356) */
  uint64_t *bco = (uint64_t *)calloc((size_t)n, 8);
  for (int i = 0; i < gamma && i < n; i++)
    bco[i] = io_poly_coeff(c, cols + (size_t)i * 2 * L + L, 0);
  uint64_t *b_poly = (uint64_t *)malloc(8 * L);
  io_poly_from_composite(c, bco, b_poly);
  uint64_t *a_ct = (uint64_t *)malloc(8 * L * (size_t)gamma);
  for (int i = 0; i < gamma; i++)
    memcpy(a_ct + (size_t)i * L, cols + (size_t)i * 2 * L, 8 * L);
  /* respond.rs:360-362 */
  io_pack *own = NULL;
  const io_pack *pk = pk_in;
  if (!pk) pk = own = io_pack_new(c, gamma, w_seed, mode, 1, 0x5eedULL);
  uint64_t *a_hat = (uint64_t *)malloc(8 * L);
  size_t nb = (size_t)(gamma > 1 ? (gamma - 1) * ell : 1);
  uint64_t *bold_t = (uint64_t *)malloc(8 * L * nb);
  io_packing_offline(pk, a_ct, a_hat, bold_t);
  const uint64_t *ya = y_all;
  uint64_t *derived = NULL;
  if (!ya) {
    derived = (uint64_t *)malloc(8 * L * nb);
    io_generate_rotations(pk, y_body, derived);
    ya = derived;
  }
  io_packing_online(pk, a_hat, bold_t, ya, b_poly, out_ct);
  free(derived);
  free(bold_t);
  free(a_hat);
  if (own) io_pack_free(own);
  free(a_ct);
  free(b_poly);
  free(bco);
  free(cols);
  return 0;
}

void io_expand_rgsw(const io_ctx *c, const uint8_t *seeds,
                    const uint64_t *b_rows, uint64_t *rgsw) {
  size_t L = PLEN(c);
  for (int r = 0; r < 2 * c->ell; r++) {
    io_poly_from_seed(c, seeds + 32 * r, rgsw + (size_t)2 * r * L);
    memcpy(rgsw + (size_t)(2 * r + 1) * L, b_rows + (size_t)r * L, 8 * L);
  }
}

int io_respond_nopacking(const io_ctx *c, const uint64_t *shard, int ncols,
                         const uint64_t *rgsw, uint64_t *out_ct,
                         uint64_t *out_cols, int nthreads) {
  /* respond.rs:71-115 */
  size_t L = PLEN(c);
  if (ncols <= 0) {
    memset(out_ct, 0, 16 * L);
    return 1;
  }
  uint64_t *cols = (uint64_t *)malloc(8 * 2 * L * (size_t)ncols);
  column_products(c, shard, ncols, rgsw, cols, nthreads);
  memcpy(out_ct, cols, 16 * L);
  for (int i = 1; i < ncols; i++) {
    p_add(c, out_ct, cols + (size_t)i * 2 * L, out_ct);
    p_add(c, out_ct + L, cols + (size_t)i * 2 * L + L, out_ct + L);
  }
  if (out_cols) memcpy(out_cols, cols, 8 * 2 * L * (size_t)ncols);
  free(cols);
  return 0;
}

/* ===================================================================== */
/* database encoding (pir/encode_db.rs)                                    */
/* ===================================================================== */

int io_num_columns(int entry_size) { return (entry_size * 8 + 15) / 16; }

void io_encode_shard(const io_ctx *c, const uint8_t *db, uint64_t db_len,
                     int entry_size, uint32_t shard_id, uint64_t *out) {
  /* encode_db.rs:106-181 (entries_per_shard = n, setup.rs:149-153) */
  int n = c->n, ncols = io_num_columns(entry_size);
  uint64_t total = db_len / (uint64_t)entry_size;
  uint64_t first = (uint64_t)shard_id * (uint64_t)n;
  size_t L = PLEN(c);
  memset(out, 0, 8 * L * (size_t)ncols);
  for (int col = 0; col < ncols; col++) {
    for (int k = 0; k < n; k++) {
      uint64_t e = first + (uint64_t)k;
      if (e >= total) break;
      const uint8_t *ent = db + e * (uint64_t)entry_size;
      int bo = col * 2;
      uint64_t v = 0;
      if (bo + 1 < entry_size) v = ent[bo] | ((uint64_t)ent[bo + 1] << 8);
      else if (bo < entry_size) v = ent[bo];
      set_coeff(c, out + (size_t)col * L, k, v % c->q);
    }
  }
}

void io_inverse_monomial(const io_ctx *c, int k, uint64_t *out) {
  /* encode_db.rs:80-91 */
  memset(out, 0, 8 * PLEN(c));
  if (k == 0) set_coeff(c, out, 0, 1);
  else set_coeff(c, out, c->n - k, c->q - 1);
}

/* ===================================================================== */
/* client side (fixtures): gaussian.rs, rlwe/enc.rs, rgsw/types.rs,        */
/* inspiring2.rs:640-707, 846-904, extract.rs:155-182                      */
/* ===================================================================== */

struct io_sampler {
  double sigma;
  int tailcut;
  io_rng *g;
};

io_sampler *io_sampler_new(double sigma, uint64_t seed) {
  /* gaussian.rs:26-40 */
  io_sampler *s = (io_sampler *)calloc(1, sizeof(io_sampler));
  s->sigma = sigma;
  s->tailcut = (int)ceil(sigma * 6.0);
  s->g = io_rng_seed_from_u64(seed);
  return s;
}

void io_sampler_free(io_sampler *s) {
  if (!s) return;
  io_rng_free(s->g);
  free(s);
}

int64_t io_sampler_sample(io_sampler *s) {
  /* gaussian.rs:88-105 */
  double ss2 = 2.0 * s->sigma * s->sigma;
  int64_t b = s->tailcut;
  for (;;) {
    int64_t x = gen_range_i64_incl(s->g, -b, b);
    double prob = exp(-(double)(x * x) / ss2);
    double u = gen_f64(s->g);
    if (u < prob) return x;
  }
}

static uint64_t from_signed(int64_t v, uint64_t q) {
  /* modular.rs:110-117 */
  if (v >= 0) return (uint64_t)v % q;
  uint64_t a = (uint64_t)(-v);
  return q - (a % q);
}

static void gaussian_poly(const io_ctx *c, io_sampler *s, uint64_t *out) {
  /* poly.rs:208-232 */
  int64_t *smp = (int64_t *)malloc(8 * (size_t)c->n);
  for (int i = 0; i < c->n; i++) smp[i] = io_sampler_sample(s);
  for (int r = 0; r < c->crt; r++)
    for (int i = 0; i < c->n; i++)
      out[(size_t)r * c->n + i] = from_signed(smp[i], c->mod[r]);
  free(smp);
}

void io_sk_generate(const io_ctx *c, io_sampler *s, uint64_t *sk) {
  gaussian_poly(c, s, sk); /* rlwe/enc.rs:14-17 */
}

void io_rlwe_encrypt(const io_ctx *c, io_sampler *s, io_rng *g,
                     const uint64_t *sk, const uint64_t *msg, uint64_t *ct) {
  /* rlwe/enc.rs:32-51 with a = Poly::random_moduli */
  size_t L = PLEN(c);
  uint64_t *e = (uint64_t *)malloc(8 * L), *t = (uint64_t *)malloc(8 * L);
  random_poly(c, g, ct);
  gaussian_poly(c, s, e);
  io_poly_mul(c, ct, sk, t);
  p_neg(c, t, t);
  p_add(c, t, e, t);
  p_scalar(c, msg, c->delta, e);
  p_add(c, t, e, ct + L);
  free(e);
  free(t);
}

void io_rgsw_encrypt(const io_ctx *c, io_sampler *s, io_rng *g,
                     const uint64_t *sk, const uint64_t *msg, uint64_t *rgsw) {
  /* rgsw/types.rs:133-187 */
  size_t L = PLEN(c);
  int ell = c->ell;
  uint64_t *e = (uint64_t *)malloc(8 * L), *t = (uint64_t *)malloc(8 * L);
  uint64_t *m = (uint64_t *)malloc(8 * L);
  u128 pw = 1;
  for (int half = 0; half < 2; half++) {
    pw = 1;
    for (int i = 0; i < ell; i++) {
      uint64_t *ra = rgsw + (size_t)(2 * (half * ell + i)) * L, *rb = ra + L;
      random_poly(c, g, ra);
      gaussian_poly(c, s, e);
      io_poly_mul(c, ra, sk, t);
      p_neg(c, t, t);
      p_add(c, t, e, rb);
      p_scalar(c, msg, (uint64_t)pw, m);
      if (half == 0) p_add(c, ra, m, ra);
      else p_add(c, rb, m, rb);
      pw = (pw * c->zbase) % c->q;
    }
  }
  free(e);
  free(t);
  free(m);
}

void io_query_seeded(const io_ctx *c, io_sampler *s, io_rng *g,
                     const uint64_t *sk, int local_idx, uint8_t *seeds,
                     uint64_t *b_rows) {
  /* query.rs:43-85 (RGSW part) -> SeededRgswCiphertext::encrypt
   * (rgsw/types.rs:235-300) of inverse_monomial(local_idx) */
  size_t L = PLEN(c);
  int ell = c->ell;
  uint64_t *msg = (uint64_t *)malloc(8 * L), *a = (uint64_t *)malloc(8 * L);
  uint64_t *e = (uint64_t *)malloc(8 * L), *t = (uint64_t *)malloc(8 * L);
  uint64_t *m = (uint64_t *)malloc(8 * L);
  io_inverse_monomial(c, local_idx, msg);
  for (int half = 0; half < 2; half++) {
    u128 pw = 1;
    for (int i = 0; i < ell; i++) {
      int row = half * ell + i;
      uint8_t *seed = seeds + 32 * row;
      uint64_t *b = b_rows + (size_t)row * L;
      rng_fill_bytes(g, seed, 32);
      io_poly_from_seed(c, seed, a);
      gaussian_poly(c, s, e);
      io_poly_mul(c, a, sk, t);
      p_neg(c, t, t);
      p_add(c, t, e, b);
      p_scalar(c, msg, (uint64_t)pw, m);
      if (half == 0) {
        io_poly_mul(c, m, sk, t);
        p_add(c, b, t, b);
      } else {
        p_add(c, b, m, b);
      }
      pw = (pw * c->zbase) % c->q;
    }
  }
  free(msg);
  free(a);
  free(e);
  free(t);
  free(m);
}

void io_client_packing_keys(const io_pack *pk, io_sampler *s,
                            const uint64_t *sk, uint64_t *y_body,
                            uint64_t *y_all) {
  /* ClientPackingKeys::generate (inspiring2.rs:640-707) with
   * generate_ksk_body (:846-904) */
  const io_ctx *c = pk->c;
  size_t L = PLEN(c);
  int n = c->n, ell = c->ell;
  uint64_t *wm = (uint64_t *)malloc(8 * L * (size_t)ell);
  io_mask_from_seed(c, pk->w_seed, ell, wm);
  uint64_t *tau_s = (uint64_t *)malloc(8 * L), *s_ntt = (uint64_t *)malloc(8 * L);
  uint64_t *t1 = (uint64_t *)malloc(8 * L), *t2 = (uint64_t *)malloc(8 * L);
  uint64_t *err = (uint64_t *)malloc(8 * (size_t)n);
  io_automorphism(c, sk, pk->gen_pows[1], tau_s);
  memcpy(s_ntt, sk, 8 * L);
  ntt_fwd1(c, s_ntt);
  u128 gp = 1;
  for (int k = 0; k < ell; k++) {
    uint64_t *yk = y_body + (size_t)k * L;
    p_scalar(c, tau_s, (uint64_t)gp, yk);
    memcpy(t1, wm + (size_t)k * L, 8 * L);
    ntt_fwd1(c, t1);
    pw_mul(c, s_ntt, t1, t2);
    ntt_inv1(c, t2);
    p_neg(c, t2, t2);
    p_add(c, yk, t2, yk);
    for (int i = 0; i < n; i++) {
      int64_t smp = io_sampler_sample(s);
      err[i] = smp >= 0 ? (uint64_t)smp % c->q
                        : (uint64_t)((int64_t)c->q + (smp % (int64_t)c->q));
    }
    io_poly_from_composite(c, err, t1);
    p_add(c, yk, t1, yk);
    gp = (gp * c->zbase) % c->q;
  }
  uint64_t *yb_ntt = (uint64_t *)malloc(8 * L * (size_t)ell);
  memcpy(yb_ntt, y_body, 8 * L * (size_t)ell);
  io_ntt_forward(c, yb_ntt, ell);
  for (int i = 0; i < pk->gamma - 1; i++)
    for (int k = 0; k < ell; k++) {
      uint64_t *o = y_all + ((size_t)i * ell + k) * L;
      apply_auto_ntt(c, pk->mode, yb_ntt + (size_t)k * L,
                     pack_table(pk, pk->gen_pows[i]), o);
      ntt_inv1(c, o);
    }
  free(yb_ntt);
  free(wm);
  free(tau_s);
  free(s_ntt);
  free(t1);
  free(t2);
  free(err);
}

void io_decrypt(const io_ctx *c, const uint64_t *sk, const uint64_t *ct,
                uint64_t *out) {
  /* rlwe/enc.rs:90-108 */
  size_t L = PLEN(c);
  uint64_t *t = (uint64_t *)malloc(8 * L);
  io_poly_mul(c, ct, sk, t);
  p_add(c, t, ct + L, t);
  uint64_t half = c->delta / 2;
  for (int i = 0; i < c->n; i++) {
    uint64_t v = io_poly_coeff(c, t, i);
    uint64_t rounded = (uint64_t)(((u128)v + half) / c->delta);
    out[i] = rounded % c->p;
  }
  free(t);
}

void io_extract_inspiring(const io_ctx *c, const uint64_t *sk,
                          const uint64_t *ct, int entry_size, uint8_t *out) {
  /* extract.rs:155-182 + reconstruct_entry (encode_db.rs:186-201) */
  uint64_t *m = (uint64_t *)malloc(8 * (size_t)c->n);
  io_decrypt(c, sk, ct, m);
  int ncols = io_num_columns(entry_size);
  memset(out, 0, (size_t)entry_size);
  for (int col = 0; col < ncols; col++) {
    uint64_t v = m[col];
    int bo = col * 2;
    if (bo < entry_size) out[bo] = (uint8_t)(v & 0xFF);
    if (bo + 1 < entry_size) out[bo + 1] = (uint8_t)((v >> 8) & 0xFF);
  }
  free(m);
}

/* ===================================================================== */
/* tree packing: respond_one_packing (pir/respond.rs:213-268) with        */
/* pack_lwes (inspiring/automorph_pack.rs:171-485) and the Galois keys of */
/* setup (pir/setup.rs:164-173; ks/setup.rs:118-245)                       */
/* ===================================================================== */

static int log2i(int n) {
  int l = 0;
  while ((1 << l) < n) l++;
  return l;
}

void io_automorphism_ks_matrix(const io_ctx *c, io_sampler *s, io_rng *g,
                               const uint64_t *sk, int t, uint64_t *ks) {
  /* generate_automorphism_ks_matrix (ks/setup.rs:218-245): tau_t(s), then
   * generate_ks_matrix (:118-162) row i = (a_i, -a_i*s + e_i + tau_t(s)*z^i) */
  size_t L = PLEN(c);
  uint64_t *as = (uint64_t *)malloc(8 * L), *e = (uint64_t *)malloc(8 * L);
  uint64_t *tmp = (uint64_t *)malloc(8 * L);
  io_automorphism(c, sk, t, as);
  u128 pw = 1; /* GadgetVector::powers (rgsw/types.rs:79-90) */
  for (int i = 0; i < c->ell; i++) {
    uint64_t *a = ks + (size_t)(2 * i) * L, *b = a + L;
    random_poly(c, g, a);
    gaussian_poly(c, s, e);
    io_poly_mul(c, a, sk, tmp);
    p_neg(c, tmp, tmp);
    p_add(c, tmp, e, tmp);
    p_scalar(c, as, (uint64_t)pw, e);
    p_add(c, tmp, e, b);
    pw = (pw * c->zbase) % c->q;
  }
  free(as);
  free(e);
  free(tmp);
}

void io_galois_keys(const io_ctx *c, io_sampler *s, io_rng *g,
                    const uint64_t *sk, uint64_t *keys) {
  /* setup.rs:164-173: keys[i] for t = d / 2^i + 1, i < log2(d) */
  size_t L = PLEN(c);
  int ld = log2i(c->n);
  for (int i = 0; i < ld; i++)
    io_automorphism_ks_matrix(c, s, g, sk, (c->n >> i) + 1,
                              keys + (size_t)i * 2 * c->ell * L);
}

static void homomorphic_automorph(const io_ctx *c, const uint64_t *ct, int t,
                                  const uint64_t *ks, uint64_t *out) {
  /* automorph_pack.rs:33-79 */
  size_t L = PLEN(c);
  uint64_t *aa = (uint64_t *)malloc(8 * L), *ab = (uint64_t *)malloc(8 * L);
  uint64_t *dg = (uint64_t *)malloc(8 * L * (size_t)c->ell);
  uint64_t *tmp = (uint64_t *)malloc(8 * L);
  io_automorphism(c, ct, t, aa);
  io_automorphism(c, ct + L, t, ab);
  io_gadget_decompose(c, aa, dg);
  memset(out, 0, 8 * L);
  memcpy(out + L, ab, 8 * L);
  for (int i = 0; i < c->ell; i++) {
    const uint64_t *row = ks + (size_t)(2 * i) * L;
    io_poly_mul(c, dg + (size_t)i * L, row, tmp);
    p_add(c, out, tmp, out);
    io_poly_mul(c, dg + (size_t)i * L, row + L, tmp);
    p_add(c, out + L, tmp, out + L);
  }
  free(aa);
  free(ab);
  free(dg);
  free(tmp);
}

static void monomial(const io_ctx *c, int k, int negative, uint64_t *out) {
  /* YConstants::generate (automorph_pack.rs:103-132): X^k, or (q-1) X^k */
  uint64_t *co = (uint64_t *)calloc((size_t)c->n, 8);
  co[k] = negative ? c->q - 1 : 1;
  io_poly_from_composite(c, co, out);
  free(co);
}

/* pack_lwes_inner (automorph_pack.rs:171-255).  Subtrees whose leaves are
 * all zero padding return NULL: every step maps an all-zero ciphertext to
 * an all-zero ciphertext (0 + 0, y * 0, tau(0), gadget digits of 0), so
 * skipping them gives the same bits. */
static uint64_t *pack_inner(const io_ctx *c, int ell, int start,
                            const uint64_t *leaves, int nreal,
                            const uint64_t *keys, int log_n) {
  size_t L = PLEN(c);
  if (start >= nreal) return NULL;
  if (ell == 0) {
    uint64_t *r = (uint64_t *)malloc(16 * L);
    memcpy(r, leaves + (size_t)start * 2 * L, 16 * L);
    return r;
  }
  int step = 1 << (log_n - ell);
  uint64_t *even = pack_inner(c, ell - 1, start, leaves, nreal, keys, log_n);
  uint64_t *odd = pack_inner(c, ell - 1, start + step, leaves, nreal, keys, log_n);
  uint64_t *s0 = (uint64_t *)malloc(16 * L), *s1 = (uint64_t *)malloc(16 * L);
  memcpy(s0, even, 16 * L);
  memcpy(s1, even, 16 * L);
  if (odd) {
    uint64_t *y = (uint64_t *)malloc(8 * L), *ny = (uint64_t *)malloc(8 * L);
    uint64_t *tmp = (uint64_t *)malloc(8 * L);
    monomial(c, c->n >> ell, 0, y);
    monomial(c, c->n >> ell, 1, ny);
    for (int h = 0; h < 2; h++) { /* RlweCiphertext::poly_mul (rlwe/enc.rs:147-152) */
      io_poly_mul(c, odd + (size_t)h * L, y, tmp);
      p_add(c, s0 + (size_t)h * L, tmp, s0 + (size_t)h * L);
      io_poly_mul(c, odd + (size_t)h * L, ny, tmp);
      p_add(c, s1 + (size_t)h * L, tmp, s1 + (size_t)h * L);
    }
    free(y);
    free(ny);
    free(tmp);
  }
  int ld = log2i(c->n);
  uint64_t *au = (uint64_t *)malloc(16 * L);
  homomorphic_automorph(c, s1, (1 << ell) + 1,
                        keys + (size_t)(ld - ell) * 2 * c->ell * L, au);
  p_add(c, s0, au, s0);
  p_add(c, s0 + L, au + L, s0 + L);
  free(au);
  free(s1);
  free(even);
  free(odd);
  return s0;
}

int io_pack_lwes(const io_ctx *c, const uint64_t *leaf_a, const uint64_t *bval_in,
                 int nlwe, const uint64_t *keys, int mode, uint64_t *out_a,
                 uint64_t *out_b) {
  /* pack_lwes (automorph_pack.rs:418-485) on LWEs given as their prepped
   * form: leaf_a[i] = invert_sample_extract(lwe_i.a) as a polynomial (for a
   * sample_extract_coeff0 output that is the RLWE a itself,
   * automorph_pack.rs:349-405), bval_in[i] = lwe_i.b (composite).  out_b
   * holds 2 PLEN words in MODE_COMPAT with two moduli: the crate adds
   * b_val * d to the first d words of the residue-major vector and rebuilds
   * the polynomial from all 2d words with Poly::from_coeffs_moduli
   * (poly.rs:127-159), giving ring dimension 2d.  MODE_CRT_FIXED adds
   * b_val * d to composite coefficient z.  Returns the words written to out_b
   * (PLEN or 2 PLEN), or -1 for no LWE (the zero ciphertext). */
  size_t L = PLEN(c);
  int n = c->n;
  if (nlwe <= 0) {
    memset(out_a, 0, 8 * L);
    memset(out_b, 0, 8 * L);
    return -1;
  }
  if (nlwe == 1) { /* automorph_pack.rs:439-446: (a, b_val at coefficient 0) */
    memcpy(out_a, leaf_a, 8 * L);
    uint64_t *bco = (uint64_t *)calloc((size_t)n, 8);
    bco[0] = bval_in[0];
    io_poly_from_composite(c, bco, out_b);
    free(bco);
    return (int)L;
  }
  uint64_t *leaves = (uint64_t *)calloc(2 * L * (size_t)nlwe, 8);
  uint64_t *bval = (uint64_t *)calloc((size_t)n, 8);
  for (int i = 0; i < nlwe; i++) {
    memcpy(leaves + (size_t)i * 2 * L, leaf_a + (size_t)i * L, 8 * L);
    if (i < n) bval[i] = bval_in[i];
  }
  int ld = log2i(n);
  uint64_t *packed = pack_inner(c, ld, 0, leaves, nlwe, keys, ld);
  memcpy(out_a, packed, 8 * L);
  const uint64_t q = c->q;
  int words = (int)L;
  if (mode == IO_MODE_COMPAT && c->crt == 2) {
    /* automorph_pack.rs:474-484 on the residue-major vector of 2d words */
    uint64_t *bc = (uint64_t *)malloc(8 * L);
    memcpy(bc, packed + L, 8 * L);
    for (int z = 0; z < n; z++) {
      uint64_t sc = (uint64_t)(((u128)bval[z] * (uint64_t)n) % q);
      bc[z] = (uint64_t)(((u128)bc[z] + sc) % q);
    }
    for (size_t w = 0; w < L; w++) {
      out_b[w] = bc[w] % c->mod[0];
      out_b[L + w] = bc[w] % c->mod[1];
    }
    free(bc);
    words = (int)(2 * L);
  } else {
    for (int z = 0; z < n; z++) {
      uint64_t v = io_poly_coeff(c, packed + L, z);
      uint64_t sc = (uint64_t)(((u128)bval[z] * (uint64_t)n) % q);
      set_coeff(c, out_b, z, (uint64_t)(((u128)v + sc) % q));
    }
  }
  free(packed);
  free(bval);
  free(leaves);
  return words;
}

int io_respond_one_packing(const io_ctx *c, const uint64_t *shard, int ncols,
                           const uint64_t *rgsw, const uint64_t *keys,
                           int mode, uint64_t *out_a, uint64_t *out_b,
                           int nthreads) {
  /* respond.rs:213-268: column products, sample_extract_coeff0 of each
   * (rlwe/enc.rs:195-208), pack_lwes */
  size_t L = PLEN(c);
  if (ncols <= 0) { /* the zero response (respond.rs:230-236) */
    memset(out_a, 0, 8 * L);
    memset(out_b, 0, 8 * L);
    return -1;
  }
  uint64_t *cols = (uint64_t *)malloc(8 * 2 * L * (size_t)ncols);
  column_products(c, shard, ncols, rgsw, cols, nthreads);
  uint64_t *la = (uint64_t *)malloc(8 * L * (size_t)ncols);
  uint64_t *bv = (uint64_t *)malloc(8 * (size_t)ncols);
  for (int i = 0; i < ncols; i++) {
    memcpy(la + (size_t)i * L, cols + (size_t)i * 2 * L, 8 * L);
    bv[i] = io_poly_coeff(c, cols + (size_t)i * 2 * L + L, 0);
  }
  int words = io_pack_lwes(c, la, bv, ncols, keys, mode, out_a, out_b);
  free(bv);
  free(la);
  free(cols);
  return words;
}

void io_extract_packed(const io_ctx *c, const uint64_t *sk, const uint64_t *ct,
                       int entry_size, uint8_t *out) {
  /* extract_packed (pir/extract.rs:113-148): decrypt, then column values
   * times d^-1 mod p (1 when d has no inverse), reconstruct_entry */
  uint64_t *m = (uint64_t *)malloc(8 * (size_t)c->n);
  io_decrypt(c, sk, ct, m);
  uint64_t p = c->p, dinv = 1;
  if (p % 2 == 1) dinv = powmod((uint64_t)c->n % p, p - 2, p); /* p prime here (65537) */
  int ncols = io_num_columns(entry_size);
  memset(out, 0, (size_t)entry_size);
  for (int col = 0; col < ncols; col++) {
    uint64_t v = (uint64_t)(((u128)m[col] * dinv) % p);
    int bo = col * 2;
    if (bo < entry_size) out[bo] = (uint8_t)(v & 0xFF);
    if (bo + 1 < entry_size) out[bo + 1] = (uint8_t)((v >> 8) & 0xFF);
  }
  free(m);
}
