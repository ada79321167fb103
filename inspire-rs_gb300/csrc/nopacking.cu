// nopacking.cu -- NoPacking Respond: one CTA per query.
//
// respond (src/pir/respond.rs:71-115) and respond_seeded (:408-415): for every
// column c of the named shard, column_ciphertexts[c] =
// external_product(trivial_encrypt(h_c), rgsw) (rgsw/external_product.rs:88-150),
// and the combined ciphertext is their sum (respond.rs:102-109).  As in the
// packed path, only RGSW rows ELL..2ELL-1 contribute (the a part of the
// trivial encryption is zero), so a_c = sum_t D_{c,t} * a_t and
// b_c = sum_t D_{c,t} * b_t with D_{c,t} the base-2^20 digit t of Delta*h_c.
//
// Layout: 768 threads = six groups of 128; group g = 3 r + t owns CRT residue
// r and row/digit t and keeps NTT(a_t), NTT(b_t) of its residue in registers
// (Montgomery form with n^-1 folded) for all columns.  Per column: six digit
// NTTs and products, then groups (r,0)/(r,1) sum the three digits and run the
// inverse NTTs of a_c / b_c.  No global scratch.
#include "expand.cuh"
#include "kernels.h"

namespace ig {

namespace {

template <int MODE_UNUSED, bool SEEDED>
__global__ void __launch_bounds__(RBLOCK, 1) nopacking_kernel(const __grid_constant__ NoPackingArgs A) {
  extern __shared__ __align__(16) uint32_t smem[];
  uint32_t* SC = smem;                        // [RG][NTT_SCRATCH]
  uint32_t* PB = SC + RG * NTT_SCRATCH;       // [2 r][3 t][2 (a,b)][N] products, slot layout (swizzled)
  uint32_t* SUMB = PB + 12 * N;               // [2 r][2 (a,b)][N] running sum over columns (swizzled)
  int* wsb = reinterpret_cast<int*>(SUMB + 4 * N);  // [3][20]
  const DevParams& P = A.P;
  const int ngroups = A.col_groups;
  const int qi = blockIdx.x / ngroups, cg = blockIdx.x - qi * ngroups;
  const int tid = threadIdx.x, g = tid >> 7, x = tid & 127;
  const int r = g / 3, t = g - 3 * r;
  const int gamma = P.gamma;
  const int cper = (gamma + ngroups - 1) / ngroups;
  const int c0 = cg * cper, c1 = min(gamma, c0 + cper);
  const uint32_t shard = A.shard[qi];
  if (shard >= (uint32_t)A.nshards) {
    if (tid == 0 && cg == 0) A.status[qi] = ERR_INDEX;
    return;  // uniform over the CTA
  }
  const uint16_t* H = A.H + (size_t)shard * gamma * N;
  const uint32_t q = P.r[r].q, qinv = P.r[r].qinv;

  // ---- rows ELL..2ELL-1: a_t (expanded or given), b_t ----
  {
    const int st = tid >> 8, lt = tid & 255;
    uint64_t* cand = reinterpret_cast<uint64_t*>(SC) + st * N;  // 3 x 16 KiB within SC
    uint32_t* a0 = PB + st * 2 * N;                              // 3 x 16 KiB within PB
    uint32_t* a1 = a0 + N;
    if (SEEDED) {
      const bool ok = expand_seeded_row<2>(P, A.seeds + ((size_t)qi * ELL + st) * 32, cand, a0, a1, wsb + 20 * st,
                                           7 + st, lt);
      if (lt == 0) wsb[20 * st + 17] = ok;
    } else {
      const uint64_t* ar = A.arows + ((size_t)qi * ELL + st) * 2 * N;
      for (int j = lt; j < 2 * N; j += SUB) a0[j] = (uint32_t)ar[j];
    }
  }
  __syncthreads();
  // the query's status is written once, by one thread
  if (tid == 0 && cg == 0) A.status[qi] = (!SEEDED || (wsb[17] && wsb[37] && wsb[57])) ? 0 : ERR_EXPAND;
  if (!A.out_columns) {
    // Combined ciphertext only.  The NTT is linear mod q_r, so
    // sum_c NTT(D_{c,t}) = NTT(sum_c D_{c,t} mod q_r): one transform of the
    // digit sum per group gives the sum of the column products exactly.
    const ResidueConsts& C = P.r[r];
    uint32_t v[16], w[16];
#pragma unroll
    for (int j = 0; j < 16; j++) v[j] = 0;
    for (int c = 0; c < gamma; c++) {
#pragma unroll
      for (int j = 0; j < 16; j++) {
        const uint64_t xv = P.delta * (uint64_t)__ldg(H + (size_t)c * N + x + 128 * j);
        const uint32_t s = v[j] + ((uint32_t)(xv >> (ZBITS * t)) & ((1u << ZBITS) - 1));
        v[j] = min(s, s - q);  // < q
      }
    }
    ntt_fwd<false>(v, SC + g * NTT_SCRATCH, fwd_tw(C), q, x, 1 + g);
#pragma unroll
    for (int j = 0; j < 16; j++) w[j] = PB[t * 2 * N + r * N + x + 128 * j];
    __syncthreads();  // every group holds its a row: PB (row staging) is reused for products
    const int f = (x >> 1) & 3;
    const uint64_t* brow = A.brows + (((size_t)qi * ELL + t) * 2 + r) * N;
#pragma unroll 1
    for (int ab = 0; ab < 2; ab++) {
      if (ab == 1) {
#pragma unroll
        for (int j = 0; j < 16; j++) w[j] = (uint32_t)__ldg(brow + x + 128 * j);
      }
      ntt_fwd<false>(w, SC + g * NTT_SCRATCH, fwd_tw(C), q, x, 1 + g);
      uint32_t* dst = PB + ((r * 3 + t) * 2 + ab) * N + 16 * x;
#pragma unroll
      for (int r4 = 0; r4 < 4; r4++) {
        uint32_t pr[4];
#pragma unroll
        for (int e = 0; e < 4; e++) {
          const int j = 4 * r4 + e;
          const uint32_t h = mul_shoup(w[j], C.ninv_mont, C.ninv_mont_p, q);
          pr[e] = redc_lazy((uint64_t)v[j] * h, q, qinv);
        }
        *reinterpret_cast<uint4*>(dst + 4 * (r4 ^ f)) = make_uint4(pr[0], pr[1], pr[2], pr[3]);
      }
    }
    __syncthreads();
    if (t < 2) {  // (r,0): a, (r,1): b
      const uint32_t* p0 = PB + ((r * 3 + 0) * 2 + t) * N + 16 * x;
      const uint32_t* p1 = PB + ((r * 3 + 1) * 2 + t) * N + 16 * x;
      const uint32_t* p2 = PB + ((r * 3 + 2) * 2 + t) * N + 16 * x;
#pragma unroll
      for (int r4 = 0; r4 < 4; r4++) {
        const int o = 4 * (r4 ^ f);
        const uint4 a4 = *reinterpret_cast<const uint4*>(p0 + o);
        const uint4 b4 = *reinterpret_cast<const uint4*>(p1 + o);
        const uint4 c4 = *reinterpret_cast<const uint4*>(p2 + o);
        const uint32_t aa[4] = {a4.x, a4.y, a4.z, a4.w}, bb[4] = {b4.x, b4.y, b4.z, b4.w},
                       cc[4] = {c4.x, c4.y, c4.z, c4.w};
#pragma unroll
        for (int e = 0; e < 4; e++) {
          uint32_t sm = aa[e] + bb[e] + cc[e];  // < 6q
          sm = min(sm, sm - 4 * q);
          sm = min(sm, sm - 2 * q);
          v[4 * r4 + e] = min(sm, sm - q);
        }
      }
      ntt_inv_noscale(v, SC + g * NTT_SCRATCH, inv_tw(C), q, x, 1 + g);
      uint64_t* o = A.out + (size_t)qi * 4 * N + (size_t)t * 2 * N + (size_t)r * N;
#pragma unroll
      for (int j = 0; j < 16; j++) o[x + 128 * j] = canon2(v[j], q);
    }
    return;
  }

  // group (r,t): NTT(a_t mod q_r), NTT(b_t mod q_r), kept as x * n^-1 * 2^32
  uint32_t ah[16], bh[16];
  {
    const ResidueConsts& C = P.r[r];
#pragma unroll
    for (int j = 0; j < 16; j++) ah[j] = PB[t * 2 * N + r * N + x + 128 * j];
    ntt_fwd<false>(ah, SC + g * NTT_SCRATCH, fwd_tw(C), q, x, 1 + g);
    const uint64_t* brow = A.brows + (((size_t)qi * ELL + t) * 2 + r) * N;
#pragma unroll
    for (int j = 0; j < 16; j++) bh[j] = (uint32_t)__ldg(brow + x + 128 * j);
    ntt_fwd<false>(bh, SC + g * NTT_SCRATCH, fwd_tw(C), q, x, 1 + g);
#pragma unroll
    for (int j = 0; j < 16; j++) {
      ah[j] = mul_shoup(ah[j], C.ninv_mont, C.ninv_mont_p, q);
      bh[j] = mul_shoup(bh[j], C.ninv_mont, C.ninv_mont_p, q);
    }
  }
  __syncthreads();  // PB (row staging) is reused for products

  // group (r,0): sum_c a_c; group (r,1): sum_c b_c (NTT domain, n^-1 folded)
  uint32_t* sumb = SUMB + (r * 2 + (t < 2 ? t : 0)) * N;
  if (t < 2) {
    const uint32_t zero[16] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    store16(sumb, x, zero);
  }
  uint64_t* outc = A.out_columns ? A.out_columns + (size_t)qi * gamma * 4 * N : nullptr;

  for (int c = c0; c < c1; c++) {
    // digit t of Delta * h_c, NTT mod q_r, products with this group's row
    uint32_t v[16];
#pragma unroll
    for (int j = 0; j < 16; j++) {
      const uint64_t xv = P.delta * (uint64_t)__ldg(H + (size_t)c * N + x + 128 * j);
      v[j] = (uint32_t)(xv >> (ZBITS * t)) & ((1u << ZBITS) - 1);
    }
    ntt_fwd<false>(v, SC + g * NTT_SCRATCH, fwd_tw(P.r[r]), q, x, 1 + g);  // [0, 14q)
    {
      const int f = (x >> 1) & 3;
      uint32_t* da = PB + ((r * 3 + t) * 2 + 0) * N + 16 * x;
      uint32_t* db = PB + ((r * 3 + t) * 2 + 1) * N + 16 * x;
#pragma unroll
      for (int r4 = 0; r4 < 4; r4++) {
        uint32_t pa[4], pb[4];
#pragma unroll
        for (int e = 0; e < 4; e++) {
          const int j = 4 * r4 + e;
          pa[e] = redc_lazy((uint64_t)v[j] * ah[j], q, qinv);
          pb[e] = redc_lazy((uint64_t)v[j] * bh[j], q, qinv);
        }
        *reinterpret_cast<uint4*>(da + 4 * (r4 ^ f)) = make_uint4(pa[0], pa[1], pa[2], pa[3]);
        *reinterpret_cast<uint4*>(db + 4 * (r4 ^ f)) = make_uint4(pb[0], pb[1], pb[2], pb[3]);
      }
    }
    __syncthreads();
    if (t < 2) {  // (r,0): a_c, (r,1): b_c
      const int f = (x >> 1) & 3;
      const uint32_t* p0 = PB + ((r * 3 + 0) * 2 + t) * N + 16 * x;
      const uint32_t* p1 = PB + ((r * 3 + 1) * 2 + t) * N + 16 * x;
      const uint32_t* p2 = PB + ((r * 3 + 2) * 2 + t) * N + 16 * x;
#pragma unroll
      for (int r4 = 0; r4 < 4; r4++) {
        const int o = 4 * (r4 ^ f);
        uint4* sp = reinterpret_cast<uint4*>(sumb + 16 * x + o);
        const uint4 s4 = *sp;
        uint32_t ss[4] = {s4.x, s4.y, s4.z, s4.w};
        const uint4 a4 = *reinterpret_cast<const uint4*>(p0 + o);
        const uint4 b4 = *reinterpret_cast<const uint4*>(p1 + o);
        const uint4 c4 = *reinterpret_cast<const uint4*>(p2 + o);
        const uint32_t aa[4] = {a4.x, a4.y, a4.z, a4.w}, bb[4] = {b4.x, b4.y, b4.z, b4.w},
                       cc[4] = {c4.x, c4.y, c4.z, c4.w};
#pragma unroll
        for (int e = 0; e < 4; e++) {
          const int j = 4 * r4 + e;
          uint32_t sm = aa[e] + bb[e] + cc[e];  // < 6q
          sm = min(sm, sm - 4 * q);
          sm = min(sm, sm - 2 * q);
          sm = min(sm, sm - q);
          v[j] = sm;
          const uint32_t acc = ss[e] + sm;
          ss[e] = min(acc, acc - q);
        }
        *sp = make_uint4(ss[0], ss[1], ss[2], ss[3]);
      }
      if (outc) {
        ntt_inv_noscale(v, SC + g * NTT_SCRATCH, inv_tw(P.r[r]), q, x, 1 + g);
        uint64_t* o = outc + ((size_t)c * 2 + t) * 2 * N + (size_t)r * N;
#pragma unroll
        for (int j = 0; j < 16; j++) o[x + 128 * j] = canon2(v[j], q);
      }
    }
    __syncthreads();
  }
  // combined ciphertext = sum of the column ciphertexts (respond.rs:102-109)
  if (ngroups == 1 && t < 2) {
    uint32_t sv[16];
    load16(sumb, x, sv);
    ntt_inv_noscale(sv, SC + g * NTT_SCRATCH, inv_tw(P.r[r]), q, x, 1 + g);
    uint64_t* o = A.out + (size_t)qi * 4 * N + (size_t)t * 2 * N + (size_t)r * N;
#pragma unroll
    for (int j = 0; j < 16; j++) o[x + 128 * j] = canon2(sv[j], q);
  }
}

// Combined ciphertexts of split queries: out[q] = sum_c columns[q][c] mod q_r
// (respond.rs:102-109), in the coefficient domain (the sum commutes with the
// inverse NTT, so this equals the one-CTA path's bits).
__global__ void column_sum_kernel(const DevParams P, int nq, int gamma, const uint64_t* __restrict__ cols,
                                  uint64_t* __restrict__ out) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;  // over nq * 4N words
  if (i >= (size_t)nq * 4 * N) return;
  const size_t qi = i / (4 * N), w = i - qi * 4 * N;  // w: part (a, b) x residue x coefficient
  const uint32_t q = P.r[(w / N) & 1].q;
  const uint64_t* src = cols + qi * (size_t)gamma * 4 * N + w;
  uint32_t s = 0;
  for (int c = 0; c < gamma; c++) {
    const uint32_t v = s + (uint32_t)src[(size_t)c * 4 * N];
    s = min(v, v - q);
  }
  out[i] = s;
}

}  // namespace

size_t nopacking_smem_bytes() { return sizeof(uint32_t) * ((size_t)RG * NTT_SCRATCH + 16 * N + 64); }

template <bool SEEDED>
static cudaError_t launch_np(const NoPackingArgs& a, cudaStream_t st) {
  nopacking_kernel<0, SEEDED><<<a.nq * a.col_groups, RBLOCK, nopacking_smem_bytes(), st>>>(a);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess && a.col_groups > 1) {
    const size_t words = (size_t)a.nq * 4 * N;
    column_sum_kernel<<<(unsigned)((words + 255) / 256), 256, 0, st>>>(a.P, a.nq, a.P.gamma, a.out_columns, a.out);
    e = cudaGetLastError();
  }
  return e;
}

cudaError_t prepare_nopacking_kernels() {
  const int smem = (int)nopacking_smem_bytes();
  cudaError_t e = cudaFuncSetAttribute(nopacking_kernel<0, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(nopacking_kernel<0, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  return e;
}

cudaError_t launch_nopacking(const NoPackingArgs& a, bool seeded, cudaStream_t st) {
  if (a.nq <= 0) return cudaSuccess;
  if (a.col_groups < 1 || (a.col_groups > 1 && !a.out_columns)) return cudaErrorInvalidValue;
  return seeded ? launch_np<true>(a, st) : launch_np<false>(a, st);
}

}  // namespace ig
