// ops.cu -- kernel-level operations with the reference's own data semantics:
// batched NttContext::forward / inverse (src/math/ntt.rs:223-325, NTT-domain
// values in Montgomery form with R = 2^64) and the general RLWE x RGSW external
// product (src/rgsw/external_product.rs:88-150).
#include "kernels.h"

namespace ig {

namespace {

// One polynomial (both residues) per CTA; group g transforms residue g.
// Layout: polys[p][r][N] u32.  Forward: coefficients -> reference NTT slots
// (times 2^64).  Inverse: reference NTT slots -> coefficients.
template <bool INVERSE>
__global__ void __launch_bounds__(BLOCK) ntt_ref_kernel(const DevParams P, uint32_t* __restrict__ polys) {
  __shared__ uint32_t SC[2][NTT_SCRATCH];
  const int p = blockIdx.x, tid = threadIdx.x, g = tid >> 7, x = tid & 127;
  const ResidueConsts& C = P.r[g];
  const uint32_t q = C.q;
  uint32_t* a = polys + ((size_t)p * 2 + g) * N;
  uint32_t v[16];
  if (!INVERSE) {
#pragma unroll
    for (int r = 0; r < 16; r++) v[r] = mul_shoup(a[x + 128 * r], C.r64, C.r64_p, q);
    ntt_fwd(v, SC[g], fwd_tw(C), q, x, 1 + g);
#pragma unroll
    for (int r = 0; r < 16; r++) v[r] = canon16(v[r], q);
    uint4* d = reinterpret_cast<uint4*>(a + 16 * x);
#pragma unroll
    for (int r = 0; r < 4; r++) d[r] = make_uint4(v[4 * r], v[4 * r + 1], v[4 * r + 2], v[4 * r + 3]);
  } else {
    const uint4* s = reinterpret_cast<const uint4*>(a + 16 * x);
#pragma unroll
    for (int r = 0; r < 4; r++) {
      uint4 t = s[r];
      v[4 * r] = t.x; v[4 * r + 1] = t.y; v[4 * r + 2] = t.z; v[4 * r + 3] = t.w;
    }
    ntt_inv_noscale(v, SC[g], inv_tw(C), q, x, 1 + g);
#pragma unroll
    for (int r = 0; r < 16; r++) a[x + 128 * r] = mul_shoup(v[r], C.ref_inv_scale, C.ref_inv_scale_p, q);
  }
}

// external_product(rlwe, rgsw): result = sum_i g^-1(a)_i * C[i] + g^-1(b)_i * C[ELL+i].
// ct[p][2 (a,b)][2][N]; rgsw[p][2*ELL rows][2 (a,b)][2][N]; out[p][2][2][N].
__global__ void __launch_bounds__(BLOCK) external_product_kernel(const DevParams P, const uint32_t* __restrict__ ct,
                                                                 const uint32_t* __restrict__ rgsw,
                                                                 uint32_t* __restrict__ out) {
  extern __shared__ __align__(16) uint32_t smem[];
  uint32_t* dig = smem;                   // [2*ELL][N]: digits of a (rows 0..ELL-1), of b (ELL..)
  uint32_t* SC = dig + 2 * ELL * N;       // [2][NTT_SCRATCH]
  const int p = blockIdx.x, tid = threadIdx.x, g = tid >> 7, x = tid & 127;
  const uint32_t* c = ct + (size_t)p * 4 * N;
  for (int j = tid; j < 2 * N; j += BLOCK) {
    const int part = j >> LOGN, jj = j & (N - 1);
    const uint64_t v = crt_compose(P, c[(part * 2 + 0) * N + jj], c[(part * 2 + 1) * N + jj]);
#pragma unroll
    for (int i = 0; i < ELL; i++) dig[(part * ELL + i) * N + jj] = (uint32_t)(v >> (ZBITS * i)) & ((1u << ZBITS) - 1);
  }
  __syncthreads();
  const ResidueConsts& C = P.r[g];
  const uint32_t q = C.q, qinv = C.qinv, q2 = 2 * q;
  uint32_t accA[16], accB[16];
#pragma unroll
  for (int r = 0; r < 16; r++) accA[r] = accB[r] = 0;
  const uint32_t* rows = rgsw + (size_t)p * 2 * ELL * 4 * N;
  for (int d = 0; d < 2 * ELL; d++) {
    uint32_t dh[16], v[16];
#pragma unroll
    for (int r = 0; r < 16; r++) dh[r] = dig[d * N + x + 128 * r];
    ntt_fwd(dh, SC + g * NTT_SCRATCH, fwd_tw(C), q, x, 1 + g);
#pragma unroll
    for (int r = 0; r < 16; r++) dh[r] = canon16(dh[r], q);  // keeps dh * v < 14 q^2 < q 2^32
    // row d: (a, b) of residue g
    for (int part = 0; part < 2; part++) {
      const uint32_t* rp = rows + ((size_t)(d * 2 + part) * 2 + g) * N;
#pragma unroll
      for (int r = 0; r < 16; r++) v[r] = rp[x + 128 * r];
      ntt_fwd(v, SC + g * NTT_SCRATCH, fwd_tw(C), q, x, 1 + g);
#pragma unroll
      for (int r = 0; r < 16; r++) {
        const uint32_t pr = redc_lazy((uint64_t)dh[r] * v[r], q, qinv);
        if (part == 0) accA[r] = acc_2q(accA[r], pr, q2);
        else accB[r] = acc_2q(accB[r], pr, q2);
      }
    }
  }
  uint32_t* o = out + (size_t)p * 4 * N;
#pragma unroll
  for (int r = 0; r < 16; r++) accA[r] = reduce_2q(accA[r], q);
  ntt_inv_noscale(accA, SC + g * NTT_SCRATCH, inv_tw(C), q, x, 1 + g);
#pragma unroll
  for (int r = 0; r < 16; r++) o[(0 * 2 + g) * N + x + 128 * r] = mul_shoup(accA[r], C.ninv_mont, C.ninv_mont_p, q);
#pragma unroll
  for (int r = 0; r < 16; r++) accB[r] = reduce_2q(accB[r], q);
  ntt_inv_noscale(accB, SC + g * NTT_SCRATCH, inv_tw(C), q, x, 1 + g);
#pragma unroll
  for (int r = 0; r < 16; r++) o[(1 * 2 + g) * N + x + 128 * r] = mul_shoup(accB[r], C.ninv_mont, C.ninv_mont_p, q);
}

// Throughput probe of the exact modular multiply the transforms are built
// from (a * w mod q by Shoup's method, lazily reduced to [0, 2q)): every
// thread runs MM_CHAINS independent chains of `iters` dependent multiplies;
// the xor of the chain ends is stored so nothing is dead code.
constexpr int MM_CHAINS = 8;
constexpr int MM_BLOCK = 256;

__global__ void __launch_bounds__(MM_BLOCK) mulmod_rate_kernel(uint32_t q, uint32_t w, uint32_t wp, int iters,
                                                               uint32_t* __restrict__ sink) {
  uint32_t x[MM_CHAINS];
  const uint32_t t = blockIdx.x * MM_BLOCK + threadIdx.x;
#pragma unroll
  for (int c = 0; c < MM_CHAINS; c++) x[c] = (t * 2654435761u + c) % q;
  const uint2 wv = make_uint2(w, wp);
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int c = 0; c < MM_CHAINS; c++) x[c] = mul_shoup_lazy(x[c], wv, q);
  }
  uint32_t acc = 0;
#pragma unroll
  for (int c = 0; c < MM_CHAINS; c++) acc ^= x[c];
  sink[t] = acc;
}

// Integer tensor-core probe.  sm_103a has no tcgen05 INT8 MMA (ptxas
// rejects tcgen05.mma .kind::i8 for this target), so the only INT8 tensor
// instruction is the legacy warp-level mma.sync m16n8k32 s8 x s8 -> s32.
// Every warp loads the same A (16 x 32, row-major) and B (32 x 8,
// column-major) fragments and runs I8_CHAINS independent accumulators
// through `iters` dependent MMAs (D = A B + D).  Warp 0 of block 0 writes its
// accumulators, which must equal iters * A B exactly (|A B| <= 32 * 128^2,
// so iters <= 4096 cannot overflow): the check of the fragment layout and of
// exact INT32 accumulation.  Operations per MMA: 2 * 16 * 8 * 32.
constexpr int I8_CHAINS = 4;

__device__ __forceinline__ uint32_t pack_s8(const int8_t* p, int stride) {
  return (uint32_t)(uint8_t)p[0] | ((uint32_t)(uint8_t)p[stride] << 8) | ((uint32_t)(uint8_t)p[2 * stride] << 16) |
         ((uint32_t)(uint8_t)p[3 * stride] << 24);
}

__global__ void __launch_bounds__(MM_BLOCK) int8_mma_rate_kernel(const int8_t* __restrict__ A,
                                                                 const int8_t* __restrict__ B, int iters,
                                                                 int32_t* __restrict__ out) {
  const int lane = threadIdx.x & 31, grp = lane >> 2, tig = lane & 3;
  // A fragment: rows grp / grp + 8, columns 4 tig + {0..3} and 16 + 4 tig + {0..3}
  const uint32_t a0 = pack_s8(A + grp * 32 + 4 * tig, 1), a1 = pack_s8(A + (grp + 8) * 32 + 4 * tig, 1);
  const uint32_t a2 = pack_s8(A + grp * 32 + 16 + 4 * tig, 1), a3 = pack_s8(A + (grp + 8) * 32 + 16 + 4 * tig, 1);
  // B fragment (B stored row-major 32 x 8 here): rows 4 tig + {0..3} and 16 + 4 tig + {0..3}, column grp
  const uint32_t b0 = pack_s8(B + (4 * tig) * 8 + grp, 8), b1 = pack_s8(B + (16 + 4 * tig) * 8 + grp, 8);
  int32_t d[I8_CHAINS][4] = {};
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int c = 0; c < I8_CHAINS; c++)
      asm volatile(
          "mma.sync.aligned.m16n8k32.row.col.s32.s8.s8.s32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
          "{%0, %1, %2, %3};"
          : "+r"(d[c][0]), "+r"(d[c][1]), "+r"(d[c][2]), "+r"(d[c][3])
          : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
  }
  if (blockIdx.x == 0 && threadIdx.x < 32) {
    // D fragment: d0, d1 at row grp, columns 2 tig + {0, 1}; d2, d3 at row grp + 8
#pragma unroll
    for (int c = 0; c < I8_CHAINS; c++) {
      int32_t* o = out + c * 16 * 8;
      o[grp * 8 + 2 * tig] = d[c][0];
      o[grp * 8 + 2 * tig + 1] = d[c][1];
      o[(grp + 8) * 8 + 2 * tig] = d[c][2];
      o[(grp + 8) * 8 + 2 * tig + 1] = d[c][3];
    }
  } else if (d[0][0] == 0x7fffffff && d[1][1] == 0x7fffffff && d[2][2] == d[3][3]) {
    out[0] = 0;  // never taken for iters <= 4096; keeps the MMAs live
  }
}

// Client-side decrypt + extract_inspiring for one response per CTA
// (src/pir/extract.rs:155-182 with RlweCiphertext::decrypt,
// src/rlwe/enc.rs:90-108, and reconstruct_entry, src/pir/encode_db.rs:186-201).
// Only the first ncols coefficients of a*s + b are needed, so each is a
// direct negacyclic dot product: coeff c = sum_{j<=c} a_j s_{c-j}
// - sum_{j>c} a_j s_{N+c-j}.  Threads: 8 per (column, residue) pair; a pair's
// residues sit 8 lanes apart in one warp.
struct ExtractConsts {
  uint64_t barrett[2];  // floor(2^64 / q_r)
  uint64_t delta, p;
  int ncols, entry_size;
};

__device__ __forceinline__ uint64_t barrett_reduce(uint64_t x, uint64_t m, uint32_t q) {
  uint64_t r = x - __umul64hi(x, m) * q;  // < 2q
  return r >= q ? r - q : r;
}

__global__ void __launch_bounds__(256) extract_kernel(const DevParams P, const ExtractConsts K,
                                                      const uint64_t* __restrict__ sk, const uint64_t* __restrict__ ct,
                                                      uint8_t* __restrict__ entries) {
  const int i = blockIdx.x, t = threadIdx.x;
  const int pr = t >> 3, sub = t & 7, c = pr >> 1, r = pr & 1;
  const uint32_t q = P.r[r].q;
  const uint64_t* a = ct + (size_t)i * 4 * N + (size_t)r * N;
  const uint64_t* b = a + 2 * N;
  const uint64_t* s = sk + (size_t)r * N;
  uint64_t pos = 0, neg = 0;
  if (c < K.ncols) {
    int k = 0;
    for (int j = sub; j < N; j += 8) {
      const uint64_t prod = __ldg(a + j) * (j <= c ? __ldg(s + (c - j)) : __ldg(s + (N + c - j)));
      if (j <= c) pos += prod;
      else neg += prod;
      if (++k == 32) {  // 32 products < 2^56 each fit 64 bits
        pos = barrett_reduce(pos, K.barrett[r], q);
        neg = barrett_reduce(neg, K.barrett[r], q);
        k = 0;
      }
    }
    pos = barrett_reduce(pos, K.barrett[r], q);
    neg = barrett_reduce(neg, K.barrett[r], q);
  }
  uint64_t m = pos >= neg ? pos - neg : pos + q - neg;  // [0, q)
#pragma unroll
  for (int o = 4; o > 0; o >>= 1) m += __shfl_xor_sync(0xffffffffu, m, o);  // < 8q
  m = barrett_reduce(m, K.barrett[r], q);
  if (c < K.ncols) m = barrett_reduce(m + __ldg(b + c), K.barrett[r], q);
  const uint64_t m1 = __shfl_down_sync(0xffffffffu, m, 8);  // residue 1 of this column
  if (sub == 0 && r == 0 && c < K.ncols) {
    const uint64_t v = crt_compose(P, (uint32_t)m, (uint32_t)m1);  // composite coefficient in [0, q)
    const uint64_t val = ((v + K.delta / 2) / K.delta) % K.p;
    uint8_t* e = entries + (size_t)i * K.entry_size;
    if (2 * c < K.entry_size) e[2 * c] = (uint8_t)(val & 0xFF);
    if (2 * c + 1 < K.entry_size) e[2 * c + 1] = (uint8_t)((val >> 8) & 0xFF);
  }
}

}  // namespace

cudaError_t launch_extract(const DevParams& P, uint64_t p, const uint64_t* sk, const uint64_t* ct, int n,
                           int entry_size, uint8_t* entries, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  ExtractConsts K{};
  for (int r = 0; r < 2; r++) K.barrett[r] = (uint64_t)((((unsigned __int128)1) << 64) / P.r[r].q);
  K.delta = P.delta;
  K.p = p;
  K.ncols = (entry_size * 8 + 15) / 16;
  K.entry_size = entry_size;
  extract_kernel<<<n, 256, 0, st>>>(P, K, sk, ct, entries);
  return cudaGetLastError();
}

cudaError_t launch_int8_mma_rate(const int8_t* A, const int8_t* B, int blocks, int iters, int32_t* out,
                                 cudaStream_t st) {
  int8_mma_rate_kernel<<<blocks, MM_BLOCK, 0, st>>>(A, B, iters, out);
  return cudaGetLastError();
}

cudaError_t launch_mulmod_rate(const DevParams& P, int blocks, int iters, uint32_t* sink, cudaStream_t st) {
  if (blocks <= 0 || iters <= 0) return cudaSuccess;
  const uint32_t q = P.r[0].q;
  const uint32_t w = 123456789u % q;
  const uint32_t wp = (uint32_t)(((uint64_t)w << 32) / q);
  mulmod_rate_kernel<<<blocks, MM_BLOCK, 0, st>>>(q, w, wp, iters, sink);
  return cudaGetLastError();
}

cudaError_t launch_ntt_ref(const DevParams& P, uint32_t* polys, int npolys, bool inverse, cudaStream_t st) {
  if (npolys <= 0) return cudaSuccess;
  if (inverse) ntt_ref_kernel<true><<<npolys, BLOCK, 0, st>>>(P, polys);
  else ntt_ref_kernel<false><<<npolys, BLOCK, 0, st>>>(P, polys);
  return cudaGetLastError();
}

constexpr size_t EXT_SMEM = sizeof(uint32_t) * ((size_t)2 * ELL * N + 2 * NTT_SCRATCH);

cudaError_t launch_external_product(const DevParams& P, const uint32_t* ct, const uint32_t* rgsw, uint32_t* out,
                                    int npairs, cudaStream_t st) {
  if (npairs <= 0) return cudaSuccess;
  external_product_kernel<<<npairs, BLOCK, EXT_SMEM, st>>>(P, ct, rgsw, out);
  return cudaGetLastError();
}

cudaError_t prepare_ops_kernels() {
  return cudaFuncSetAttribute(external_product_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)EXT_SMEM);
}

}  // namespace ig
