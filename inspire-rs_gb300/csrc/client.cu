// client.cu -- client-side seeded query generation on the device, for load
// generation at served rates.
//
// query_seeded (src/pir/query.rs:43-85) builds SeededRgswCiphertext::encrypt
// (src/rgsw/types.rs:233-300) of m = inverse_monomial(k) (X^-k,
// src/pir/encode_db.rs:80-91) under the secret key s: for row i < ELL,
// b = -a s + e + (m z^i) s; for row ELL + i, b = -a s + e + m z^i, where a is
// Poly::from_seed_moduli of the row's 32-byte seed (the same expansion the
// server runs) and z = 2^20.
//
// client_keys_kernel: RlweSecretKey::generate (src/rlwe/enc.rs:14-17) and
// ClientPackingKeys::generate's y_body (src/inspiring/inspiring2.rs:640-660,
// generate_ksk_body :846-902): y_body[k] = tau_g(s) z^k - s w_mask[k] + e_k
// with g = gen_pows[1] and w_mask the CRS mask of w_seed.
//
// ks_matrices_kernel: the key-switching matrices of setup
// (src/pir/setup.rs:151-200; generate_ks_matrix, src/ks/setup.rs:118-162):
// row k of matrix i = (a, -a s + e + s_i z^k) with a uniform, where the
// source key s_i is
//   i < LOGN:        tau_t(s), t = N / 2^i + 1 (galois_keys, setup.rs:164-173;
//                    generate_automorphism_ks_matrix, ks/setup.rs:218-245)
//   i = LOGN:        tau_3(s)     (k_g; galois_generators, rlwe/galois.rs:80-91)
//   i = LOGN + 1:    tau_{2N-1}(s) (k_h)
//   i = LOGN + 2, 3: the LWE key of s, s_lwe[0] = s[0], s_lwe[j] = -s[j]
//                    (packing_k_g, packing_k_h; generate_packing_ks_matrix,
//                    ks/setup.rs:183-205; LweSecretKey::from_rlwe,
//                    lwe/enc.rs:53-66)
// crs_a_kernel: setup's crs_a_vectors (setup.rs:175-180), N uniform polys.
//
// Randomness: the crate draws seeds from thread_rng and errors from a
// rejection sampler over ChaCha20.  Here both come from ChaCha20 keyed by a
// caller key, each error coefficient a discrete Gaussian of the parameters'
// sigma drawn by inverse cumulative table from one 64-bit word (8 per block).
// Block layout of one key's stream:
//   query Q, row r: seed = first 8 words of block Q * 16 + r; errors from
//     blocks 2^40 + (Q * 2 ELL + r) * 256 + j / 8          (Q < 2^36)
//   client C: secret key from blocks 2^48 + C * 1024 + j / 8; y_body[k]
//     errors from blocks 2^48 + C * 1024 + 256 (k + 1) + j / 8  (C < 2^30)
//   key-switching matrix i, row k (m = 3 i + k): a from the seed = first 8
//     words of block 2^52 + m (Poly::from_seed_moduli of it), errors from
//     blocks 2^52 + 2^20 + m * 256 + j / 8
//   crs_a vector v: Poly::from_seed_moduli of the first 8 words of block
//     2^53 + v
// The outputs are valid keys and queries (responses decrypt to the queried
// entries) but are not the crate's random draws.
#include "expand.cuh"
#include "kernels.h"

namespace ig {
namespace {

constexpr int CT = 256;  // threads per query: one expansion sub-block, two NTT groups

// Thread t (of 256) fills err[8t .. 8t+7] with discrete Gaussian samples from
// keystream block `blk + t`.
__device__ __forceinline__ void gaussian8(const uint32_t key[8], uint64_t blk, uint32_t one, const uint64_t* cdt,
                                          int cdt_len, int t, int32_t* err) {
  uint32_t w[16];
  chacha20_block(key, blk + (uint64_t)t, one, w);
#pragma unroll
  for (int e = 0; e < 8; e++) {
    const uint64_t u = (uint64_t)w[2 * e] | ((uint64_t)w[2 * e + 1] << 32);
    const uint64_t mag = u & 0x7fffffffffffffffull;
    int j = 0;
    while (j < cdt_len - 1 && mag >= cdt[j]) j++;
    err[8 * t + e] = (j != 0 && (u >> 63)) ? -j : j;
  }
}

__device__ __forceinline__ uint32_t signed_mod(int32_t e, uint32_t q) {
  return e >= 0 ? (uint32_t)e : q - (uint32_t)(-e);
}

__global__ void __launch_bounds__(CT) query_gen_kernel(const __grid_constant__ QueryGenArgs A) {
  extern __shared__ __align__(16) uint32_t smem[];
  uint64_t* cand = reinterpret_cast<uint64_t*>(smem);        // [N] expansion candidates
  uint32_t* a0 = smem + 2 * N;                               // [2][N] expanded a (residue 0, 1)
  uint32_t* shat = a0 + 2 * N;                               // [2][N] NTT(s) * n^-1 2^32, slot layout
  uint32_t* sco = shat + 2 * N;                              // [2][N] s, coefficients
  int32_t* err = reinterpret_cast<int32_t*>(sco + 2 * N);    // [N] signed error
  uint32_t* SC = reinterpret_cast<uint32_t*>(err + N);       // [2][NTT_SCRATCH]
  uint64_t* cdt = reinterpret_cast<uint64_t*>(SC + 2 * NTT_SCRATCH);  // [MAX_CDT]
  int* ws = reinterpret_cast<int*>(cdt + MAX_CDT);           // [20]
  uint32_t* seed_w = reinterpret_cast<uint32_t*>(ws + 20);   // [8]
  const DevParams& P = A.P;
  const int tid = threadIdx.x, g = tid >> 7, x = tid & 127;
  const int qi = blockIdx.x;
  const uint64_t Q = A.first_query + (uint64_t)qi;
  const uint32_t k = A.local_idx[qi] & (N - 1);
  const uint32_t q = P.r[g].q, qinv = P.r[g].qinv;
  const int cdt_len = A.cdt_len;
  if (tid < MAX_CDT) cdt[tid] = A.cdt[tid];
  if (tid == 0) A.status[qi] = 0;

  // s (both residues) and its transform, once per query
  {
    uint32_t v[16];
#pragma unroll
    for (int j = 0; j < 16; j++) {
      const uint32_t sv = (uint32_t)A.sk[(size_t)g * N + x + 128 * j];
      sco[g * N + x + 128 * j] = sv;
      v[j] = sv;
    }
    ntt_fwd(v, SC + g * NTT_SCRATCH, fwd_tw(P.r[g]), q, x, 1 + g);
#pragma unroll
    for (int j = 0; j < 16; j++)
      shat[g * N + 16 * x + j] = mul_shoup(v[j], P.r[g].ninv_mont, P.r[g].ninv_mont_p, q);
  }
  uint32_t key[8];
#pragma unroll
  for (int i = 0; i < 8; i++) key[i] = A.key[i];

  for (int row = 0; row < 2 * ELL; row++) {
    __syncthreads();  // previous row's buffers are free
    if (tid == 0) {
      uint32_t w[16];
      chacha20_block(key, Q * 16 + (uint64_t)row, P.one, w);
#pragma unroll
      for (int i = 0; i < 8; i++) seed_w[i] = w[i];
    }
    gaussian8(key, (1ull << 40) + (Q * 2 * ELL + (uint64_t)row) * (N / 8), P.one, cdt, cdt_len, tid, err);
    __syncthreads();
    uint8_t* seed_out = A.seeds + ((size_t)qi * 2 * ELL + row) * 32;
    if (tid < 32) seed_out[tid] = (uint8_t)(seed_w[tid >> 2] >> (8 * (tid & 3)));
    // a = Poly::from_seed_moduli(seed) (poly.rs:251-281)
    const bool ok = expand_seeded_row<2>(P, reinterpret_cast<const uint8_t*>(seed_w), cand, a0, a0 + N, ws, 3, tid);
    if (!ok && tid == 0) A.status[qi] = ERR_EXPAND;
    __syncthreads();
    // a s by the NTT (n^-1 folded into s_hat), one residue per group
    uint32_t v[16];
#pragma unroll
    for (int j = 0; j < 16; j++) v[j] = a0[g * N + x + 128 * j];
    ntt_fwd(v, SC + g * NTT_SCRATCH, fwd_tw(P.r[g]), q, x, 1 + g);
#pragma unroll
    for (int j = 0; j < 16; j++) v[j] = redc_lazy((uint64_t)v[j] * shat[g * N + 16 * x + j], q, qinv);  // [0, 2q)
    ntt_inv_noscale(v, SC + g * NTT_SCRATCH, inv_tw(P.r[g]), q, x, 1 + g);
    const int i = row < ELL ? row : row - ELL;
    const uint32_t zp = A.zpow[g][i], zp_p = A.zpow_p[g][i];  // z^i mod q_g, Shoup companion
    uint64_t* brow = A.b_rows + ((size_t)qi * 2 * ELL + row) * 2 * N + (size_t)g * N;
#pragma unroll
    for (int j = 0; j < 16; j++) {
      const int c = x + 128 * j;
      uint32_t b = canon2(v[j], q);  // a s
      b = b ? q - b : 0;             // -a s
      b = add_mod(b, signed_mod(err[c], q), q);
      uint32_t msg;  // row < ELL: (m s)[c] = (X^-k s)[c]; else m[c]
      if (row < ELL) {
        const int src = c + (int)k;
        msg = src < N ? sco[g * N + src] : (sco[g * N + src - N] ? q - sco[g * N + src - N] : 0);
      } else {
        msg = (k == 0) ? (c == 0 ? 1u : 0u) : (c == N - (int)k ? q - 1 : 0u);
      }
      b = add_mod(b, mul_shoup(msg, zp, zp_p, q), q);
      brow[c] = b;
    }
  }
}

__global__ void __launch_bounds__(CT) client_keys_kernel(const __grid_constant__ KeyGenArgs A) {
  extern __shared__ __align__(16) uint32_t smem[];
  int32_t* sk = reinterpret_cast<int32_t*>(smem);            // [N] signed secret key
  int32_t* tau = sk + N;                                     // [N] tau_g(s), signed
  uint32_t* shat = reinterpret_cast<uint32_t*>(tau + N);     // [2][N] NTT(s) * n^-1 2^32, slot layout
  int32_t* err = reinterpret_cast<int32_t*>(shat + 2 * N);   // [N]
  uint32_t* SC = reinterpret_cast<uint32_t*>(err + N);       // [2][NTT_SCRATCH]
  uint64_t* cdt = reinterpret_cast<uint64_t*>(SC + 2 * NTT_SCRATCH);  // [MAX_CDT]
  const DevParams& P = A.P;
  const int tid = threadIdx.x, g = tid >> 7, x = tid & 127;
  const uint64_t C = A.first_client + blockIdx.x;
  const uint32_t q = P.r[g].q, qinv = P.r[g].qinv;
  const int cdt_len = A.cdt_len;
  if (tid < MAX_CDT) cdt[tid] = A.cdt[tid];
  uint32_t key[8];
#pragma unroll
  for (int i = 0; i < 8; i++) key[i] = A.key[i];
  const uint64_t base = (1ull << 48) + C * 4 * (N / 8);
  __syncthreads();
  // s = Poly::sample_gaussian_moduli (math/poly.rs:208-232)
  gaussian8(key, base, P.one, cdt, cdt_len, tid, sk);
  __syncthreads();
  uint64_t* sk_out = A.sk + (size_t)blockIdx.x * 2 * N + (size_t)g * N;
  const uint32_t gen = gen_pow(P.gamma, 1);  // gen_pows[1] (inspiring2.rs:652-654)
  for (int i = tid; i < N; i += CT) {
    // apply_automorphism (rlwe/galois.rs:22-55): X^i -> X^(i g mod 2n), negated past n
    const uint32_t j = ((uint32_t)i * gen) & (2 * N - 1);
    if (j < (uint32_t)N) tau[j] = sk[i];
    else tau[j - N] = -sk[i];
  }
  {
    uint32_t v[16];
#pragma unroll
    for (int j = 0; j < 16; j++) {
      v[j] = signed_mod(sk[x + 128 * j], q);
      sk_out[x + 128 * j] = v[j];
    }
    ntt_fwd(v, SC + g * NTT_SCRATCH, fwd_tw(P.r[g]), q, x, 1 + g);
#pragma unroll
    for (int j = 0; j < 16; j++)
      shat[g * N + 16 * x + j] = mul_shoup(v[j], P.r[g].ninv_mont, P.r[g].ninv_mont_p, q);
  }
  for (int k = 0; k < ELL; k++) {
    __syncthreads();  // tau complete; previous k's errors consumed
    gaussian8(key, base + (uint64_t)(k + 1) * (N / 8), P.one, cdt, cdt_len, tid, err);
    // s w_mask[k] by the NTT (generate_ksk_body, inspiring2.rs:874-884)
    uint32_t v[16];
#pragma unroll
    for (int j = 0; j < 16; j++) v[j] = A.wmask[((size_t)k * 2 + g) * N + x + 128 * j];
    ntt_fwd(v, SC + g * NTT_SCRATCH, fwd_tw(P.r[g]), q, x, 1 + g);
#pragma unroll
    for (int j = 0; j < 16; j++) v[j] = redc_lazy((uint64_t)v[j] * shat[g * N + 16 * x + j], q, qinv);
    ntt_inv_noscale(v, SC + g * NTT_SCRATCH, inv_tw(P.r[g]), q, x, 1 + g);
    __syncthreads();  // errors visible
    const uint32_t zp = A.zpow[g][k], zp_p = A.zpow_p[g][k];
    uint64_t* y = A.y_body + ((size_t)blockIdx.x * ELL + k) * 2 * N + (size_t)g * N;
#pragma unroll
    for (int j = 0; j < 16; j++) {
      const int c = x + 128 * j;
      const uint32_t sw = canon2(v[j], q);
      uint32_t b = mul_shoup(signed_mod(tau[c], q), zp, zp_p, q);  // tau_g(s) z^k
      b = sub_mod(b, sw, q);
      b = add_mod(b, signed_mod(err[c], q), q);
      y[c] = b;
    }
  }
}

// Source key of matrix mi: t > 0 for tau_t(s), 0 for the LWE key of s.
__device__ __forceinline__ uint32_t ks_source(int mi) {
  return mi < LOGN ? (uint32_t)(N >> mi) + 1u : mi == LOGN ? 3u : mi == LOGN + 1 ? 2u * N - 1u : 0u;
}

__global__ void __launch_bounds__(CT) ks_matrices_kernel(const __grid_constant__ GaloisGenArgs A) {
  extern __shared__ __align__(16) uint32_t smem[];
  uint64_t* cand = reinterpret_cast<uint64_t*>(smem);        // [N] expansion candidates
  uint32_t* a0 = smem + 2 * N;                               // [2][N] a (residue 0, 1)
  uint32_t* shat = a0 + 2 * N;                               // [2][N] NTT(s) * n^-1 2^32, slot layout
  uint32_t* tau = shat + 2 * N;                              // [2][N] tau_t(s), residues
  int32_t* err = reinterpret_cast<int32_t*>(tau + 2 * N);    // [N]
  uint32_t* SC = reinterpret_cast<uint32_t*>(err + N);       // [2][NTT_SCRATCH]
  uint64_t* cdt = reinterpret_cast<uint64_t*>(SC + 2 * NTT_SCRATCH);  // [MAX_CDT]
  int* ws = reinterpret_cast<int*>(cdt + MAX_CDT);           // [20]
  uint32_t* seed_w = reinterpret_cast<uint32_t*>(ws + 20);   // [8]
  const DevParams& P = A.P;
  const int tid = threadIdx.x, g = tid >> 7, x = tid & 127;
  const int mi = blockIdx.x;
  const uint32_t t = ks_source(mi);
  const uint32_t q = P.r[g].q, qinv = P.r[g].qinv;
  const int cdt_len = A.cdt_len;
  if (tid < MAX_CDT) cdt[tid] = A.cdt[tid];
  if (tid == 0) A.status[mi] = 0;
  uint32_t key[8];
#pragma unroll
  for (int i = 0; i < 8; i++) key[i] = A.key[i];
  // the source key per residue: tau_t(s) (rlwe/galois.rs:22-55) or s_lwe
  for (int c = tid; c < N; c += CT) {
    const uint32_t j = t ? ((uint32_t)c * t) & (2 * N - 1) : (c ? (uint32_t)(c + N) : 0u);
#pragma unroll
    for (int rr = 0; rr < 2; rr++) {
      const uint32_t sv = (uint32_t)A.sk[(size_t)rr * N + c];
      if (j < (uint32_t)N) tau[rr * N + j] = sv;
      else tau[rr * N + j - N] = sv ? P.r[rr].q - sv : 0;
    }
  }
  {
    uint32_t v[16];
#pragma unroll
    for (int j = 0; j < 16; j++) v[j] = (uint32_t)A.sk[(size_t)g * N + x + 128 * j];
    ntt_fwd(v, SC + g * NTT_SCRATCH, fwd_tw(P.r[g]), q, x, 1 + g);
#pragma unroll
    for (int j = 0; j < 16; j++)
      shat[g * N + 16 * x + j] = mul_shoup(v[j], P.r[g].ninv_mont, P.r[g].ninv_mont_p, q);
  }
  for (int k = 0; k < ELL; k++) {
    const uint64_t m = (uint64_t)mi * ELL + (uint64_t)k;
    __syncthreads();  // tau and shat complete; the previous row's buffers consumed
    if (tid == 0) {
      uint32_t w[16];
      chacha20_block(key, (1ull << 52) + m, P.one, w);
#pragma unroll
      for (int i = 0; i < 8; i++) seed_w[i] = w[i];
    }
    gaussian8(key, (1ull << 52) + (1ull << 20) + m * (N / 8), P.one, cdt, cdt_len, tid, err);
    __syncthreads();
    const bool ok = expand_seeded_row<2>(P, reinterpret_cast<const uint8_t*>(seed_w), cand, a0, a0 + N, ws, 3, tid);
    if (!ok && tid == 0) A.status[mi] = ERR_EXPAND;
    __syncthreads();
    uint64_t* row_a = A.keys + ((size_t)m * 2 + 0) * 2 * N + (size_t)g * N;
    uint64_t* row_b = A.keys + ((size_t)m * 2 + 1) * 2 * N + (size_t)g * N;
    uint32_t v[16];
#pragma unroll
    for (int j = 0; j < 16; j++) {
      v[j] = a0[g * N + x + 128 * j];
      row_a[x + 128 * j] = v[j];
    }
    ntt_fwd(v, SC + g * NTT_SCRATCH, fwd_tw(P.r[g]), q, x, 1 + g);
#pragma unroll
    for (int j = 0; j < 16; j++) v[j] = redc_lazy((uint64_t)v[j] * shat[g * N + 16 * x + j], q, qinv);
    ntt_inv_noscale(v, SC + g * NTT_SCRATCH, inv_tw(P.r[g]), q, x, 1 + g);
    const uint32_t zp = A.zpow[g][k], zp_p = A.zpow_p[g][k];
#pragma unroll
    for (int j = 0; j < 16; j++) {
      const int c = x + 128 * j;
      uint32_t b = mul_shoup(tau[g * N + c], zp, zp_p, q);  // tau_t(s) z^k
      b = sub_mod(b, canon2(v[j], q), q);                   // - a s
      b = add_mod(b, signed_mod(err[c], q), q);
      row_b[c] = b;
    }
  }
}

// One CTA per vector v: Poly::from_seed_moduli (poly.rs:251-281) of the
// stream's block 2^53 + v, written as [2][N] u64.
__global__ void __launch_bounds__(CT) crs_a_kernel(const __grid_constant__ GaloisGenArgs A, uint64_t* out) {
  extern __shared__ __align__(16) uint32_t smem[];
  uint64_t* cand = reinterpret_cast<uint64_t*>(smem);  // [N]
  uint32_t* a0 = smem + 2 * N;                         // [2][N]
  int* ws = reinterpret_cast<int*>(a0 + 2 * N);        // [20]
  uint32_t* seed_w = reinterpret_cast<uint32_t*>(ws + 20);
  const int tid = threadIdx.x, v = blockIdx.x;
  if (tid == 0) {
    uint32_t key[8], w[16];
#pragma unroll
    for (int i = 0; i < 8; i++) key[i] = A.key[i];
    chacha20_block(key, (1ull << 53) + (uint64_t)v, A.P.one, w);
#pragma unroll
    for (int i = 0; i < 8; i++) seed_w[i] = w[i];
  }
  __syncthreads();
  const bool ok = expand_seeded_row<2>(A.P, reinterpret_cast<const uint8_t*>(seed_w), cand, a0, a0 + N, ws, 3, tid);
  if (!ok && tid == 0) A.status[0] = ERR_EXPAND;
  __syncthreads();
  uint64_t* o = out + (size_t)v * 2 * N;
  for (int c = tid; c < 2 * N; c += CT) o[c] = a0[c];
}

}  // namespace

size_t galois_keys_smem_bytes() {
  return sizeof(uint32_t) * ((size_t)2 * N + 2 * N + 2 * N + 2 * N + N + 2 * NTT_SCRATCH + 2 * MAX_CDT + 20 + 8);
}

cudaError_t launch_ks_matrices(const GaloisGenArgs& a, int nmat, cudaStream_t st) {
  if (nmat <= 0) return cudaSuccess;
  if (nmat > LOGN + 4) return cudaErrorInvalidValue;
  ks_matrices_kernel<<<nmat, CT, galois_keys_smem_bytes(), st>>>(a);
  return cudaGetLastError();
}

size_t crs_a_smem_bytes() { return sizeof(uint32_t) * ((size_t)2 * N + 2 * N + 20 + 8); }

cudaError_t launch_crs_a(const GaloisGenArgs& a, int nvec, uint64_t* out, cudaStream_t st) {
  if (nvec <= 0) return cudaSuccess;
  crs_a_kernel<<<nvec, CT, crs_a_smem_bytes(), st>>>(a, out);
  return cudaGetLastError();
}

size_t client_keys_smem_bytes() {
  return sizeof(uint32_t) * ((size_t)N + N + 2 * N + N + 2 * NTT_SCRATCH + 2 * MAX_CDT);
}

cudaError_t launch_client_keys(const KeyGenArgs& a, int n, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  client_keys_kernel<<<n, CT, client_keys_smem_bytes(), st>>>(a);
  return cudaGetLastError();
}

size_t query_gen_smem_bytes() {
  return sizeof(uint32_t) * ((size_t)2 * N + 2 * N + 2 * N + 2 * N + N + 2 * NTT_SCRATCH + 2 * MAX_CDT + 20 + 8);
}

cudaError_t prepare_client_kernels() {
  cudaError_t e = cudaFuncSetAttribute(query_gen_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)query_gen_smem_bytes());
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(client_keys_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)client_keys_smem_bytes());
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(ks_matrices_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)galois_keys_smem_bytes());
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(crs_a_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)crs_a_smem_bytes());
  return e;
}

cudaError_t launch_query_gen(const QueryGenArgs& a, int n, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  query_gen_kernel<<<n, CT, query_gen_smem_bytes(), st>>>(a);
  return cudaGetLastError();
}

}  // namespace ig
