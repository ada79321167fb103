// tree.cu -- tree packing (respond_one_packing / respond_seeded_packed,
// src/pir/respond.rs:213-268, 428-435) of one query's column ciphertexts on
// the GPU: pack_lwes (src/inspiring/automorph_pack.rs:418-485) over the
// LWEs sample-extracted at coefficient 0 (rlwe/enc.rs:195-208), with the
// CRS's log2(d) Galois key-switching matrices (pir/setup.rs:164-173).
//
// pack_lwes_inner (automorph_pack.rs:171-255) at d = 2048 has 11 levels;
// node (l, s) combines its children (l-1, s) and (l-1, s + 2^(11-l)):
//   s0 = even + X^(d >> l) odd,  s1 = even - X^(d >> l) odd,
//   node = s0 + homomorphic_automorph(s1, 2^l + 1, key[11 - l])
// and a child whose start is past the last LWE is absent (then s0 = s1 =
// even; all-zero subtrees contribute nothing, bit for bit).  With at most 16
// LWEs, levels 1..7 are a chain per LWE and levels 8..11 combine pairs.
//
// homomorphic_automorph (automorph_pack.rs:33-79): tau_t of both parts,
// gadget digits (base 2^20, 3 digits) of tau_t(a), and
//   out = (sum_k digit_k * K[k].a, tau_t(b) + sum_k digit_k * K[k].b).
//
// 768 threads per CTA (six groups: CRT residue r x digit k).  The per-LWE
// chains of levels 1..7 run one CTA per (query, LWE), side by side; each of
// levels 8..11 is one launch with one CTA per (query, node).  Per combine: [K1] every thread gathers s1 for its source coefficients,
// applies tau_t (a scattered write in shared memory) and splits the
// composite coefficient into digits; [K3] group (r,k) transforms digit k mod
// q_r and multiplies it into both key parts; [K4] groups (r,0) / (r,1) sum
// and inverse-transform the a / b products and write node = s0 + out.
// Ciphertexts of the tree live in a per-query global work area (31 buffers
// of 2 polys x 2 residues, L2-resident); the key switch works in shared
// memory.

#include "kernels.h"

namespace ig {
namespace {

constexpr int TT = 6 * NTT_GT;   // 768 threads
constexpr int CT_WORDS = 4 * N;  // one ciphertext: a (2 residues), b (2 residues)

// shared-memory layout, u32 words
constexpr int S_TB = 0;                      // [2][N] tau_t(b), coefficient order
constexpr int S_D = S_TB + 2 * N;            // [3][N] digits of tau_t(a)
constexpr int S_PA = S_D + 3 * N;            // [6][N] group products with K[k].a (slot layout, swizzled)
constexpr int S_PB = S_PA + 6 * N;           // [6][N] group products with K[k].b
constexpr int S_SC = S_PB + 6 * N;           // [6][NTT_SCRATCH]
constexpr int S_TOTAL = S_SC + 6 * NTT_SCRATCH;

__device__ __forceinline__ uint32_t neg_mod(uint32_t v, uint32_t q) { return v ? q - v : 0; }

// node R = E + X^k O + homomorphic_automorph(E - X^k O, 2^l + 1, key[11 - l]);
// O may be null (absent child).  R may alias E.
__device__ void combine(const TreeArgs& A, uint32_t* sm, const uint32_t* E, const uint32_t* O, uint32_t* R, int l) {
  const DevParams& P = A.P;
  const int tid = threadIdx.x, g = tid >> 7, x = tid & 127;
  const int r = g / 3, kd = g - 3 * r;
  const int k = N >> l;
  const uint32_t t = (1u << l) + 1u;
  const int key = 11 - l;
  uint32_t* TB = sm + S_TB;
  uint32_t* D = sm + S_D;
  // [K1] s1 = E - X^k O at source i, tau_t: i -> i t mod 2N (negated past N),
  //      digits of the composite a coefficient, tau_t(b) kept
  for (int i = tid; i < N; i += TT) {
    uint32_t sa[2], sb[2];
#pragma unroll
    for (int rr = 0; rr < 2; rr++) {
      const uint32_t q = P.r[rr].q;
      uint32_t ea = E[rr * N + i], eb = E[2 * N + rr * N + i];
      if (O) {
        const int src = (i - k) & (N - 1);
        const bool wrap = i < k;  // X^k X^src = -X^i when src + k >= N
        uint32_t oa = O[rr * N + src], ob = O[2 * N + rr * N + src];
        if (wrap) {
          oa = neg_mod(oa, q);
          ob = neg_mod(ob, q);
        }
        ea = sub_mod(ea, oa, q);
        eb = sub_mod(eb, ob, q);
      }
      sa[rr] = ea;
      sb[rr] = eb;
    }
    const uint32_t j2 = ((uint32_t)i * t) & (2 * N - 1);
    const bool neg = j2 >= (uint32_t)N;
    const int j = (int)(j2 & (N - 1));
#pragma unroll
    for (int rr = 0; rr < 2; rr++) {
      if (neg) {
        sa[rr] = neg_mod(sa[rr], P.r[rr].q);
        sb[rr] = neg_mod(sb[rr], P.r[rr].q);
      }
      TB[rr * N + j] = sb[rr];
    }
    const uint64_t c = crt_compose(P, sa[0], sa[1]);
    D[j] = (uint32_t)c & 0xFFFFFu;
    D[N + j] = (uint32_t)(c >> 20) & 0xFFFFFu;
    D[2 * N + j] = (uint32_t)(c >> 40);
  }
  __syncthreads();
  // [K3] group (r, kd): NTT of digit kd mod q_r, products with both key parts
  {
    const uint32_t q = P.r[r].q, qinv = P.r[r].qinv;
    const size_t base = ((size_t)(key * ELL + kd) * 2 * 2) * N;  // [key][kd][part][r][N]
    const uint4* ka4 = reinterpret_cast<const uint4*>(A.ks + base + (size_t)(0 * 2 + r) * N + 16 * x);
    const uint4* kb4 = reinterpret_cast<const uint4*>(A.ks + base + (size_t)(1 * 2 + r) * N + 16 * x);
    uint4 ka[4], kb[4];
#pragma unroll
    for (int r4 = 0; r4 < 4; r4++) {
      ka[r4] = __ldg(ka4 + r4);
      kb[r4] = __ldg(kb4 + r4);
    }
    uint32_t v[16];
#pragma unroll
    for (int j = 0; j < 16; j++) v[j] = D[kd * N + x + 128 * j];
    ntt_fwd<false>(v, sm + S_SC + g * NTT_SCRATCH, fwd_tw(P.r[r]), q, x, 1 + g);
    uint32_t pa[16], pb[16];
#pragma unroll
    for (int r4 = 0; r4 < 4; r4++) {
      const uint32_t aa[4] = {ka[r4].x, ka[r4].y, ka[r4].z, ka[r4].w};
      const uint32_t bb[4] = {kb[r4].x, kb[r4].y, kb[r4].z, kb[r4].w};
#pragma unroll
      for (int e = 0; e < 4; e++) {
        pa[4 * r4 + e] = redc_lazy((uint64_t)v[4 * r4 + e] * aa[e], q, qinv);  // [0, 2q)
        pb[4 * r4 + e] = redc_lazy((uint64_t)v[4 * r4 + e] * bb[e], q, qinv);
      }
    }
    store16(sm + S_PA + g * N, x, pa);
    store16(sm + S_PB + g * N, x, pb);
  }
  __syncthreads();
  // [K4] groups (r,0) / (r,1): a / b part of the key switch, node = s0 + out
  if (kd < 2) {
    const uint32_t q = P.r[r].q, q2 = 2 * q;
    const uint32_t* src = sm + (kd == 0 ? S_PA : S_PB) + 3 * r * N;
    uint32_t u[16], b1[16], b2[16];
    load16(src, x, u);
    load16(src + N, x, b1);
    load16(src + 2 * N, x, b2);
#pragma unroll
    for (int j = 0; j < 16; j++) {
      uint32_t s = u[j] + b1[j] + b2[j];  // < 6q
      s = min(s, s - 4 * q);
      u[j] = min(s, s - q2);
    }
    ntt_inv_noscale(u, sm + S_SC + g * NTT_SCRATCH, inv_tw(P.r[r]), q, x, 1 + g);
    const int po = kd * 2 * N + r * N;  // this group's part and residue in a ciphertext
#pragma unroll
    for (int j = 0; j < 16; j++) {
      const int c = x + 128 * j;
      uint32_t val = canon2(u[j], q);
      if (kd == 1) val = add_mod(val, TB[r * N + c], q);
      uint32_t e = E[po + c];
      if (O) {
        const int srcc = (c - k) & (N - 1);
        uint32_t o = O[po + srcc];
        if (c < k) o = neg_mod(o, q);
        e = add_mod(e, o, q);
      }
      R[po + c] = add_mod(e, val, q);
    }
  }
  __syncthreads();
}

// Work area of one query: the node (l, s) of levels 7..11 in buffer
// level_base(l) + s: 0..15 level 7 (each LWE's key-switch chain), 16..23
// level 8, 24..27 level 9, 28..29 level 10, 30 the root.
constexpr int TREE_BUFS = 31;
__host__ __device__ constexpr int level_base(int l) { return l == 7 ? 0 : l == 8 ? 16 : l == 9 ? 24 : l == 10 ? 28 : 30; }

// Levels 1..7 for one LWE: node(l, s) = node(l-1, s) + homomorphic_automorph
// (its odd child is absent), one CTA per (query, LWE), so the 16 chains of a
// query run side by side.
__global__ void __launch_bounds__(TT, 1) tree_chain_kernel(const __grid_constant__ TreeArgs A) {
  extern __shared__ __align__(16) uint32_t sm[];
  const int nreal = A.ncols;
  const int qi = blockIdx.x / nreal, leaf = blockIdx.x - qi * nreal, tid = threadIdx.x;
  const uint64_t* ca = A.cols + ((size_t)qi * nreal + leaf) * 2 * 2 * N;  // the column's a, residues
  uint32_t* c = A.work + ((size_t)qi * TREE_BUFS + leaf) * CT_WORDS;
  for (int w = tid; w < 2 * N; w += TT) {  // leaf ciphertext (a of the column, b = 0)
    c[w] = (uint32_t)ca[w];
    c[2 * N + w] = 0;
  }
  __syncthreads();
  for (int l = 1; l <= 7; l++) combine(A, sm, c, nullptr, c, l);
}

// Level l (8..11) of the tree: one CTA per (query, node s < 2^(11-l)); node
// (l, s) combines (l-1, s) and (l-1, s + 2^(11-l)), absent past the last LWE.
__global__ void __launch_bounds__(TT, 1) tree_level_kernel(const __grid_constant__ TreeArgs A, int l) {
  extern __shared__ __align__(16) uint32_t sm[];
  const int nn = 1 << (11 - l), nreal = A.ncols;
  const int qi = blockIdx.x / nn, s = blockIdx.x - qi * nn;
  if (s >= nreal) return;  // absent node (uniform over the CTA)
  uint32_t* W = A.work + (size_t)qi * TREE_BUFS * CT_WORDS;
  auto buf = [&](int b) { return W + (size_t)b * CT_WORDS; };
  const int cb = level_base(l - 1);
  combine(A, sm, buf(cb + s), s + nn < nreal ? buf(cb + s + nn) : nullptr, buf(level_base(l) + s), l);
}

// pack_lwes' result: the root, or the single LWE unpacked.
__global__ void __launch_bounds__(TT, 1) pack_tree_kernel(const __grid_constant__ TreeArgs A) {
  const DevParams& P = A.P;
  const int qi = blockIdx.x, tid = threadIdx.x;
  const int nreal = A.ncols;
  const uint64_t* cols = A.cols + (size_t)qi * nreal * 2 * 2 * N;  // [col][a/b][r][N]
  uint64_t* out_a = A.out_a + (size_t)qi * 2 * N;
  uint64_t* out_b = A.out_b + (size_t)qi * 4 * N;
  if (nreal == 1) {  // automorph_pack.rs:439-446: (a, b_val at coefficient 0)
    for (int w = tid; w < 2 * N; w += TT) {
      out_a[w] = cols[w];
      out_b[w] = (w & (N - 1)) == 0 ? cols[2 * N + w] : 0;
    }
    return;
  }
  uint32_t* W = A.work + (size_t)qi * TREE_BUFS * CT_WORDS;
  auto buf = [&](int b) { return W + (size_t)b * CT_WORDS; };
  // pack_lwes' last step (automorph_pack.rs:466-484): b_val_z * d added at
  // coefficient z < nreal
  const uint32_t* root = buf(level_base(11));
  const uint32_t q0 = P.r[0].q, q1 = P.r[1].q;
  for (int w = tid; w < 2 * N; w += TT) out_a[w] = root[w];
  if (A.mode == MODE_CRT_FIXED) {
    for (int w = tid; w < 2 * N; w += TT) {
      const int rr = w >> LOGN, z = w & (N - 1);
      uint32_t b = root[2 * N + w];
      if (z < nreal) {
        const uint32_t q = P.r[rr].q;
        const uint32_t bv = (uint32_t)cols[((size_t)z * 2 + 1) * 2 * N + (size_t)rr * N];  // b_val_z mod q_r
        b = add_mod(b, (uint32_t)((uint64_t)bv * (uint64_t)(N % q) % q), q);
      }
      out_b[w] = b;
    }
  } else {
    // compat: the crate adds b_val_z * d to the first d words of the
    // residue-major b vector and rebuilds a polynomial of dimension 2d from
    // all 2d words (Poly::from_coeffs_moduli, math/poly.rs:127-159)
    const uint64_t qc = (uint64_t)q0 * q1;
    for (int w = tid; w < 2 * N; w += TT) {
      uint64_t bc = root[2 * N + w];
      if (w < nreal) {
        uint64_t bv = crt_compose(P, (uint32_t)cols[((size_t)w * 2 + 1) * 2 * N],
                                  (uint32_t)cols[((size_t)w * 2 + 1) * 2 * N + N]);
        for (int s = 0; s < LOGN; s++) {  // b_val * d mod q by doubling (q < 2^56)
          bv <<= 1;
          if (bv >= qc) bv -= qc;
        }
        bc += bv;
        if (bc >= qc) bc -= qc;
      }
      out_b[w] = bc % q0;
      out_b[2 * N + w] = bc % q1;
    }
  }
}

// Galois key table: each of the log2(d) matrices' ELL rows (a, b), per
// residue, NTT-transformed and scaled by n^-1 2^32 (products then come out of
// Montgomery reduction already divided by n).
__global__ void __launch_bounds__(BLOCK) galois_prep_kernel(const DevParams P, const uint64_t* __restrict__ keys,
                                                            uint32_t* __restrict__ ks) {
  __shared__ uint32_t SC[2][NTT_SCRATCH];
  const int p = blockIdx.x, tid = threadIdx.x, g = tid >> 7, x = tid & 127;
  const ResidueConsts& C = P.r[g];
  uint32_t v[16];
#pragma unroll
  for (int j = 0; j < 16; j++) v[j] = (uint32_t)keys[((size_t)p * 2 + g) * N + x + 128 * j];
  ntt_fwd<false>(v, SC[g], fwd_tw(C), C.q, x, 1 + g);
#pragma unroll
  for (int j = 0; j < 16; j++) ks[((size_t)p * 2 + g) * N + 16 * x + j] = mul_shoup(v[j], C.ninv_mont, C.ninv_mont_p, C.q);
}

// Static scratch of the allocation-free tree-packing entry: per query the
// column ciphertexts (MAX_GAMMA columns, u64), the combined NoPacking
// ciphertext (u64) and the tree's work area (u32).
constexpr size_t NOALLOC_QUERY_BYTES =
    sizeof(uint64_t) * ((size_t)MAX_GAMMA * 2 * 2 * N + 2 * 2 * N) + sizeof(uint32_t) * (size_t)TREE_BUFS * CT_WORDS;
__device__ __align__(256) unsigned char g_tree_noalloc_scratch[TREE_NOALLOC_MAX_QUERIES * NOALLOC_QUERY_BYTES];

}  // namespace

size_t tree_noalloc_query_bytes() { return NOALLOC_QUERY_BYTES; }

// Device address of the static scratch in the current device's context.
// Looked up on every call rather than cached: the lookup is cheap and
// allocates nothing, and a cached address would go stale if the context were
// destroyed and re-created (cudaDeviceReset) within the process.
cudaError_t tree_noalloc_scratch(int device, void** ptr) {
  int cur = -1;
  cudaError_t e = cudaGetDevice(&cur);
  if (e != cudaSuccess) return e;
  if (cur != device) return cudaErrorInvalidDevice;  // the caller makes `device` current first
  return cudaGetSymbolAddress(ptr, g_tree_noalloc_scratch);
}

size_t tree_smem_bytes() { return sizeof(uint32_t) * (size_t)S_TOTAL; }
size_t tree_work_words_per_query() { return (size_t)TREE_BUFS * CT_WORDS; }

cudaError_t prepare_tree_kernels() {
  cudaError_t e = cudaFuncSetAttribute(pack_tree_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)tree_smem_bytes());
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(tree_chain_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tree_smem_bytes());
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(tree_level_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tree_smem_bytes());
  return e;
}

cudaError_t launch_pack_tree(const TreeArgs& a, cudaStream_t st) {
  if (a.nq <= 0) return cudaSuccess;
  if (a.ncols > 1) {
    tree_chain_kernel<<<a.nq * a.ncols, TT, tree_smem_bytes(), st>>>(a);
    cudaError_t e = cudaGetLastError();
    for (int l = 8; l <= 11 && e == cudaSuccess; l++) {
      tree_level_kernel<<<a.nq << (11 - l), TT, tree_smem_bytes(), st>>>(a, l);
      e = cudaGetLastError();
    }
    if (e != cudaSuccess) return e;
  }
  pack_tree_kernel<<<a.nq, TT, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_galois_prep(const DevParams& P, const uint64_t* keys, int npolys, uint32_t* ks, cudaStream_t st) {
  if (npolys <= 0) return cudaSuccess;
  galois_prep_kernel<<<npolys, BLOCK, 0, st>>>(P, keys, ks);
  return cudaGetLastError();
}

}  // namespace ig
