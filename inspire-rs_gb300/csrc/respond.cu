// respond.cu -- fused InsPIRe^2 Respond kernel: one CTA per query.
//
// Computes, for one seeded query against one resident shard, exactly what
// respond_seeded_inspiring / respond_inspiring (src/pir/respond.rs:284-398)
// return: the packed RLWE ciphertext (a_hat, b) of packing_online
// (src/inspiring/inspiring2.rs:1185-1222).  The reference's steps are
// regrouped into an equivalent exact dataflow:
//
//  * expand (rgsw/types.rs:315-318): only RGSW rows ELL..2ELL-1 are needed,
//    because the database ciphertext is (0, Delta*h) (rlwe/enc.rs:174-182) and
//    every digit of its zero a-part is 0 (rgsw/external_product.rs:122-147).
//  * b-part of each column product, coefficient 0 only
//    (rlwe/enc.rs:195-208): b0_c = sum_t sum_i d_{c,t}[i] * b'_t[i] with
//    d = base-2^20 digits of Delta*h and b'_t the negacyclic reversal of row
//    ELL+t's b, accumulated exactly in 64 bits.
//  * a-part + the first stage of packing_offline (inspiring2.rs:948-982): the
//    per-slot 16x16 monomial inner products, the 1/gamma scaling and the 16
//    NTT-domain automorphisms reduce to a length-gamma DFT per NTT slot, which
//    is folded into the resident database ("E", built in setup.cu); per slot
//    only sum_t E[k,t][u] * A_t[u] remains.
//  * the backward recursion (inspiring2.rs:984-1008) and packing_online run
//    interleaved: each T[i][k] NTT is multiplied into R[i] with the CRS key
//    w_all and into the b accumulator with the client key y_all.
//
// Layout: 256 threads = two groups of 128; group g owns CRT residue g for
// every transform.  All intermediate state lives in shared memory and
// registers; the kernel uses no global scratch.
#include "chacha.cuh"
#include "kernels.h"

namespace ig {

namespace {

// Exclusive scan over the 256 threads of the block; ws needs 16 ints.
__device__ __forceinline__ int block_scan_excl(int v, int* ws, int& total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) ws[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    int wv = lane < 8 ? ws[lane] : 0;
#pragma unroll
    for (int o = 1; o < 8; o <<= 1) {
      int t = __shfl_up_sync(0xffffffffu, wv, o);
      if (lane >= o) wv += t;
    }
    if (lane < 8) ws[8 + lane] = wv;
  }
  __syncthreads();
  total = ws[15];
  const int base = warp ? ws[8 + warp - 1] : 0;
  const int r = base + incl - v;
  __syncthreads();
  return r;
}

// Poly::from_seed_moduli (poly.rs:251-281): residue 0 takes the first N
// accepted draws of gen_range(0..q0), residue 1 the next N of gen_range(0..q1).
// NR = 1 stops after residue 0.  Writes a0[N], a1[N]; returns false if the
// iteration bound was hit (never for a working ChaCha stream).
template <int NR>
__device__ bool expand_seeded_row(const DevParams& P, const uint8_t* __restrict__ seed,
                                  uint64_t* cand, uint32_t* a0, uint32_t* a1, int* ws) {
  uint32_t key[8];
#pragma unroll
  for (int i = 0; i < 8; i++)
    key[i] = (uint32_t)seed[4 * i] | ((uint32_t)seed[4 * i + 1] << 8) |
             ((uint32_t)seed[4 * i + 2] << 16) | ((uint32_t)seed[4 * i + 3] << 24);
  const int tid = threadIdx.x;
  int pos0 = 0, pos1 = 0, res = 0;
  uint64_t blk = 0;
  for (int it = 0; it < 64; it++) {
    const int need = res == 0 ? (N - pos0) + (NR == 2 ? N : 0) : (N - pos1);
    const int nblk = min(BLOCK, (need * 9) / 64 + 3);
    if (tid < nblk) {
      uint32_t w[16];
      chacha20_block(key, blk + tid, w);
#pragma unroll
      for (int k = 0; k < 8; k++) cand[8 * tid + k] = (uint64_t)w[2 * k] | ((uint64_t)w[2 * k + 1] << 32);
    }
    blk += nblk;
    __syncthreads();
    int start = 0;
    if (res == 0) {
      uint32_t vals[8];
      unsigned fl = 0;
      int cnt = 0;
      if (tid < nblk) {
#pragma unroll
        for (int k = 0; k < 8; k++)
          if (uniform_accept(cand[8 * tid + k], P.r[0].q, P.r[0].zone, vals[k])) {
            fl |= 1u << k;
            cnt++;
          }
      }
      int total;
      int p = pos0 + block_scan_excl(cnt, ws, total);
#pragma unroll
      for (int k = 0; k < 8; k++)
        if ((fl >> k) & 1u) {
          if (p < N) a0[p] = vals[k];
          if (p == N - 1) ws[16] = 8 * tid + k;
          p++;
        }
      __syncthreads();
      if (pos0 + total >= N) {
        start = ws[16] + 1;
        res = 1;
        pos0 = N;
      } else {
        pos0 += total;
        start = nblk * 8;
      }
      __syncthreads();
      if (NR == 1 && res == 1) return true;
    }
    if (NR == 2 && res == 1) {
      uint32_t vals[8];
      unsigned fl = 0;
      int cnt = 0;
      if (tid < nblk) {
#pragma unroll
        for (int k = 0; k < 8; k++)
          if (8 * tid + k >= start && uniform_accept(cand[8 * tid + k], P.r[1].q, P.r[1].zone, vals[k])) {
            fl |= 1u << k;
            cnt++;
          }
      }
      int total;
      int p = pos1 + block_scan_excl(cnt, ws, total);
#pragma unroll
      for (int k = 0; k < 8; k++)
        if ((fl >> k) & 1u) {
          if (p < N) a1[p] = vals[k];
          p++;
        }
      pos1 += total;
      if (pos1 >= N) return true;
    }
    __syncthreads();
  }
  return false;
}

// b0_c for every column c and residue (see file comment).  bp (6N words) is
// scratch; bpoly[r * 16 + c] receives the result.
__device__ void column_b0(const DevParams& P, const uint16_t* __restrict__ H,
                          const uint64_t* __restrict__ brows, uint32_t* bp, uint64_t* red,
                          uint32_t* bpoly) {
  const int tid = threadIdx.x, gamma = P.gamma;
  for (int idx = tid; idx < ELL * 2 * N; idx += BLOCK) {
    const int i = idx & (N - 1), tr = idx >> LOGN, r = tr & 1;
    const uint64_t* row = brows + (size_t)tr * N;
    uint32_t v = (uint32_t)(i == 0 ? row[0] : row[N - i]);
    if (i != 0 && v != 0) v = P.r[r].q - v;
    bp[idx] = v;
  }
  __syncthreads();
  const int lane = tid & 31, warp = tid >> 5;
  for (int c = 0; c < gamma; c++) {
    uint64_t acc0 = 0, acc1 = 0;
#pragma unroll 4
    for (int v = 0; v < N / BLOCK; v++) {
      const int i = tid + BLOCK * v;
      const uint64_t xv = P.delta * (uint64_t)H[c * N + i];
      const uint32_t d0 = (uint32_t)xv & 0xFFFFFu, d1 = (uint32_t)(xv >> 20) & 0xFFFFFu,
                     d2 = (uint32_t)(xv >> 40);
      acc0 += (uint64_t)d0 * bp[0 * N + i] + (uint64_t)d1 * bp[2 * N + i] + (uint64_t)d2 * bp[4 * N + i];
      acc1 += (uint64_t)d0 * bp[1 * N + i] + (uint64_t)d1 * bp[3 * N + i] + (uint64_t)d2 * bp[5 * N + i];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      acc0 += __shfl_down_sync(0xffffffffu, acc0, o);
      acc1 += __shfl_down_sync(0xffffffffu, acc1, o);
    }
    if (lane == 0) {
      red[(c * 8 + warp) * 2 + 0] = acc0;
      red[(c * 8 + warp) * 2 + 1] = acc1;
    }
  }
  __syncthreads();
  if (tid < 2 * gamma) {
    const int c = tid >> 1, r = tid & 1;
    uint64_t s = 0;
    for (int w = 0; w < 8; w++) s += red[(c * 8 + w) * 2 + r];
    bpoly[r * 16 + c] = (uint32_t)(s % P.r[r].q);
  }
  __syncthreads();
}

// R_i (NTT domain, scaled by n^-1) of packing_offline step 1 for residue g,
// scattered to dst[slot]: source slot u contributes to slot s with
// 2brv(s)+1 = h_i (2brv(u)+1) mod 2n, where h_i = g^-i
// (inspiring2.rs:952-981 with the tables of :208-263).
__device__ __forceinline__ void scatter_r(const DevParams& P, int i, const uint32_t* __restrict__ Eg,
                                          const uint32_t* Ag, int astride, uint32_t* dst, int x,
                                          uint32_t q, uint32_t qinv) {
  const int gamma = P.gamma;
  const uint32_t mi = (uint32_t)(gamma - i) & (uint32_t)(gamma - 1);
  const uint32_t hi = (1u + (uint32_t)(2 * N / gamma) * mi) & (2 * N - 1);
#pragma unroll 4
  for (int v = 0; v < 16; v++) {
    const int u = x + 128 * v;
    const uint32_t e = 2 * brv11(u) + 1;
    const uint32_t k = (e * mi) & (uint32_t)(gamma - 1);
    const uint32_t* ek = Eg + (size_t)k * N + u;
    uint64_t T = (uint64_t)__ldg(ek) * Ag[u] + (uint64_t)__ldg(ek + (size_t)gamma * N) * Ag[astride + u] +
                 (uint64_t)__ldg(ek + (size_t)2 * gamma * N) * Ag[2 * astride + u];
    const uint32_t s = brv11(((hi * e) & (2 * N - 1)) >> 1);
    dst[s] = redc(T, q, qinv);
  }
}

template <int MODE, bool SEEDED>
__global__ void __launch_bounds__(BLOCK, 2) respond_kernel(const RespondArgs A) {
  constexpr int NR = MODE == MODE_COMPAT ? 1 : 2;  // residues needed on the a side
  extern __shared__ __align__(16) uint32_t smem[];
  uint32_t* Ahat = smem;                        // [ELL][NR][N]
  uint32_t* SC = Ahat + ELL * NR * N;           // [2][NTT_SCRATCH]
  uint32_t* RT = SC + 2 * NTT_SCRATCH;          // [3][N]
  uint32_t* misc = RT + 3 * N;
  uint32_t* bpoly = misc;                       // [2][16]
  int* ws = (int*)(misc + 32);                  // [17]
  uint64_t* red = (uint64_t*)(misc + 64);       // [16][8][2]

  const DevParams& P = A.P;
  const int qi = blockIdx.x;
  const int tid = threadIdx.x, g = tid >> 7, x = tid & 127;
  const int gamma = P.gamma;
  const uint32_t shard = A.shard[qi];
  const int32_t cid = A.client[qi];
  if (shard >= (uint32_t)A.nshards || cid < 0 || cid >= A.nclients || A.yhat_table[cid] == nullptr) {
    if (tid == 0) A.status[qi] = ERR_INDEX;
    return;  // uniform over the CTA
  }
  if (tid == 0) A.status[qi] = 0;
  const uint32_t* E = A.E + (size_t)shard * 2 * ELL * gamma * N;
  const uint16_t* H = A.H + (size_t)shard * gamma * N;
  const uint32_t* Y = A.yhat_table[cid];
  const uint32_t q = P.r[g].q, qinv = P.r[g].qinv, q2 = 2 * q;

  column_b0(P, H, A.brows + (size_t)qi * ELL * 2 * N, smem, red, bpoly);

  // ---- rows ELL..2ELL-1: a-polys, forward NTT ----
  for (int t = 0; t < ELL; t++) {
    __syncthreads();
    uint32_t* a0 = SC;
    uint32_t* a1 = SC + NTT_SCRATCH;
    if (SEEDED) {
      bool ok = expand_seeded_row<NR>(P, A.seeds + ((size_t)qi * ELL + t) * 32, (uint64_t*)RT, a0, a1, ws);
      if (!ok && tid == 0) A.status[qi] = ERR_EXPAND;
    } else {
      const uint64_t* ar = A.arows + ((size_t)qi * ELL + t) * 2 * N;
      for (int j = tid; j < NR * N; j += BLOCK) (j < N ? a0 : a1)[j & (N - 1)] = (uint32_t)ar[j];
    }
    __syncthreads();
    if (g < NR) {
      uint32_t v[16];
      const uint32_t* src = g ? a1 : a0;
#pragma unroll
      for (int r = 0; r < 16; r++) v[r] = src[x + 128 * r];
      ntt_fwd(v, SC + g * NTT_SCRATCH, fwd_tw(P.r[g]), q, x, 1 + g);
      uint4* dst = reinterpret_cast<uint4*>(Ahat + (t * NR + g) * N + 16 * x);
#pragma unroll
      for (int r = 0; r < 4; r++) dst[r] = make_uint4(v[4 * r], v[4 * r + 1], v[4 * r + 2], v[4 * r + 3]);
    }
  }
  __syncthreads();

  const bool scat = (MODE == MODE_CRT_FIXED) || g == 0;
  const uint32_t* Eg = E + (size_t)g * ELL * gamma * N;
  const uint32_t* Ag = Ahat + (MODE == MODE_CRT_FIXED ? g : 0) * N;
  uint32_t* dst = RT + (MODE == MODE_CRT_FIXED ? g : 0) * N;

  uint32_t vR[16], acc[16], accb[16];
#pragma unroll
  for (int r = 0; r < 16; r++) accb[r] = 0;

  // R_{gamma-1}
  if (scat) scatter_r(P, gamma - 1, Eg, Ag, NR * N, dst, x, q, qinv);
  __syncthreads();
#pragma unroll
  for (int r = 0; r < 16; r++) {
    const uint32_t w = dst[16 * x + r];
    vR[r] = (MODE == MODE_COMPAT && g == 1) ? compat_residue1_ninv(P, w) : w;
  }

  const uint32_t* Wg = A.what;
  for (int i = gamma - 2; i >= 0; i--) {
    // INTT(R_{i+1}) -> coefficients (values already carry n^-1)
    ntt_inv_noscale(vR, SC + g * NTT_SCRATCH, inv_tw(P.r[g]), q, x, 1 + g);
    __syncthreads();
#pragma unroll
    for (int r = 0; r < 16; r++) RT[g * N + x + 128 * r] = vR[r];
    __syncthreads();
    // gadget_decompose of the composite coefficients (rgsw/external_product.rs:16-37)
#pragma unroll 2
    for (int v = 0; v < N / BLOCK; v++) {
      const int j = tid + BLOCK * v;
      const uint64_t c = crt_compose(P, RT[j], RT[N + j]);
      RT[j] = (uint32_t)c & 0xFFFFFu;
      RT[N + j] = (uint32_t)(c >> 20) & 0xFFFFFu;
      RT[2 * N + j] = (uint32_t)(c >> 40);
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < 16; r++) acc[r] = 0;
    for (int k = 0; k < ELL; k++) {
      uint32_t v[16];
#pragma unroll
      for (int r = 0; r < 16; r++) v[r] = RT[k * N + x + 128 * r];
      ntt_fwd(v, SC + g * NTT_SCRATCH, fwd_tw(P.r[g]), q, x, 1 + g);
      const size_t off = ((size_t)(i * ELL + k) * 2 + g) * N + 16 * x;
      const uint4* w4 = reinterpret_cast<const uint4*>(Wg + off);
      const uint4* y4 = reinterpret_cast<const uint4*>(Y + off);
#pragma unroll
      for (int r4 = 0; r4 < 4; r4++) {
        const uint4 wv = __ldg(w4 + r4), yv = __ldg(y4 + r4);
        const uint32_t ww[4] = {wv.x, wv.y, wv.z, wv.w}, yy[4] = {yv.x, yv.y, yv.z, yv.w};
#pragma unroll
        for (int e = 0; e < 4; e++) {
          const int r = 4 * r4 + e;
          acc[r] = acc_2q(acc[r], redc_lazy((uint64_t)v[r] * ww[e], q, qinv), q2);
          accb[r] = acc_2q(accb[r], redc_lazy((uint64_t)v[r] * yy[e], q, qinv), q2);
        }
      }
    }
    __syncthreads();
    if (scat) scatter_r(P, i, Eg, Ag, NR * N, dst, x, q, qinv);
    __syncthreads();
#pragma unroll
    for (int r = 0; r < 16; r++) {
      const uint32_t w = dst[16 * x + r];
      const uint32_t rh = (MODE == MODE_COMPAT && g == 1) ? compat_residue1_ninv(P, w) : w;
      vR[r] = add_mod(rh, reduce_2q(acc[r], q), q);
    }
  }

  // a_hat = INTT(R_0) (inspiring2.rs:1027-1029)
  uint64_t* out = A.out + (size_t)qi * 4 * N;
  ntt_inv_noscale(vR, SC + g * NTT_SCRATCH, inv_tw(P.r[g]), q, x, 1 + g);
#pragma unroll
  for (int r = 0; r < 16; r++) out[g * N + x + 128 * r] = vR[r];
  // b = b_poly + INTT(sum y_all * bold_t) (inspiring2.rs:1217-1221)
#pragma unroll
  for (int r = 0; r < 16; r++) accb[r] = reduce_2q(accb[r], q);
  ntt_inv_noscale(accb, SC + g * NTT_SCRATCH, inv_tw(P.r[g]), q, x, 1 + g);
  if (x < gamma) accb[0] = add_mod(accb[0], bpoly[g * 16 + x], q);
#pragma unroll
  for (int r = 0; r < 16; r++) out[2 * N + g * N + x + 128 * r] = accb[r];
}

}  // namespace

size_t respond_smem_bytes(int mode) {
  const int nr = mode == MODE_COMPAT ? 1 : 2;
  return sizeof(uint32_t) * ((size_t)ELL * nr * N + 2 * NTT_SCRATCH + 3 * N + 1024);
}

template <int MODE, bool SEEDED>
static cudaError_t launch_one(const RespondArgs& a, cudaStream_t st) {
  const size_t smem = respond_smem_bytes(MODE);
  cudaError_t e = cudaFuncSetAttribute(respond_kernel<MODE, SEEDED>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  respond_kernel<MODE, SEEDED><<<a.nq, BLOCK, smem, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_respond(const RespondArgs& a, bool seeded, cudaStream_t st) {
  if (a.nq <= 0) return cudaSuccess;
  if (a.P.mode == MODE_COMPAT)
    return seeded ? launch_one<MODE_COMPAT, true>(a, st) : launch_one<MODE_COMPAT, false>(a, st);
  return seeded ? launch_one<MODE_CRT_FIXED, true>(a, st) : launch_one<MODE_CRT_FIXED, false>(a, st);
}

}  // namespace ig
