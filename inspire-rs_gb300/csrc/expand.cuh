// expand.cuh -- seeded RGSW-row expansion and the CTA layout shared by the
// per-query kernels (respond.cu, nopacking.cu).
#pragma once
#include "chacha.cuh"
#include "common.cuh"

namespace ig {

constexpr int RG = 6;                 // NTT groups per CTA
constexpr int RBLOCK = RG * NTT_GT;   // 768 threads
constexpr int SUB = 256;              // threads of one expansion sub-block

__device__ __forceinline__ void named_sync(int id, int n) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory");
}
// Arrive at named barrier `id` without waiting (the other participants wait
// in named_sync); orders this thread's earlier shared-memory accesses before
// theirs after the barrier.
__device__ __forceinline__ void named_arrive(int id, int n) {
  asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(n) : "memory");
}

// Exclusive scan over one 256-thread sub-block (lt = thread index in it);
// ws needs 17 ints.
__device__ __forceinline__ int sub_scan_excl(int v, int* ws, int& total, int bar, int lt) {
  const int lane = lt & 31, warp = lt >> 5;
  int incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) ws[warp] = incl;
  named_sync(bar, SUB);
  if (warp == 0) {
    int wv = lane < 8 ? ws[lane] : 0;
#pragma unroll
    for (int o = 1; o < 8; o <<= 1) {
      int t = __shfl_up_sync(0xffffffffu, wv, o);
      if (lane >= o) wv += t;
    }
    if (lane < 8) ws[8 + lane] = wv;
  }
  named_sync(bar, SUB);
  total = ws[15];
  const int base = warp ? ws[8 + warp - 1] : 0;
  const int r = base + incl - v;
  named_sync(bar, SUB);
  return r;
}

// Poly::from_seed_moduli (poly.rs:251-281) by one 256-thread sub-block:
// residue 0 takes the first N accepted draws of gen_range(0..q0), residue 1
// the next N of gen_range(0..q1); NR = 1 stops after residue 0.  Returns false
// if the iteration bound was hit (never for a working ChaCha stream).
template <int NR>
__device__ bool expand_seeded_row(const DevParams& P, const uint8_t* __restrict__ seed, uint64_t* cand,
                                  uint32_t* a0, uint32_t* a1, int* ws, int bar, int lt) {
  uint32_t key[8];
#pragma unroll
  for (int i = 0; i < 8; i++)
    key[i] = (uint32_t)seed[4 * i] | ((uint32_t)seed[4 * i + 1] << 8) | ((uint32_t)seed[4 * i + 2] << 16) |
             ((uint32_t)seed[4 * i + 3] << 24);
  int pos0 = 0, pos1 = 0, res = 0;
  uint64_t blk = 0;
  for (int it = 0; it < 64; it++) {
    const int need = res == 0 ? (N - pos0) + (NR == 2 ? N : 0) : (N - pos1);
    const int nblk = min(SUB, (need * 9) / 64 + 3);
    if (lt < nblk) {
      uint32_t w[16];
      chacha20_block(key, blk + lt, P.one, w);
#pragma unroll
      for (int k = 0; k < 8; k++) cand[k * SUB + lt] = (uint64_t)w[2 * k] | ((uint64_t)w[2 * k + 1] << 32);
    }
    blk += nblk;
    named_sync(bar, SUB);
    int start = 0;
    if (res == 0) {
      uint32_t vals[8];
      unsigned fl = 0;
      int cnt = 0;
      if (lt < nblk) {
#pragma unroll
        for (int k = 0; k < 8; k++)
          if (uniform_accept(cand[k * SUB + lt], P.r[0].q, P.r[0].zone, vals[k])) {
            fl |= 1u << k;
            cnt++;
          }
      }
      int total;
      int p = pos0 + sub_scan_excl(cnt, ws, total, bar, lt);
#pragma unroll
      for (int k = 0; k < 8; k++)
        if ((fl >> k) & 1u) {
          if (p < N) a0[p] = vals[k];
          if (p == N - 1) ws[16] = 8 * lt + k;
          p++;
        }
      named_sync(bar, SUB);
      if (pos0 + total >= N) {
        start = ws[16] + 1;
        res = 1;
        pos0 = N;
      } else {
        pos0 += total;
        start = nblk * 8;
      }
      named_sync(bar, SUB);
      if (NR == 1 && res == 1) return true;
    }
    if (NR == 2 && res == 1) {
      uint32_t vals[8];
      unsigned fl = 0;
      int cnt = 0;
      if (lt < nblk) {
#pragma unroll
        for (int k = 0; k < 8; k++)
          if (8 * lt + k >= start && uniform_accept(cand[k * SUB + lt], P.r[1].q, P.r[1].zone, vals[k])) {
            fl |= 1u << k;
            cnt++;
          }
      }
      int total;
      int p = pos1 + sub_scan_excl(cnt, ws, total, bar, lt);
#pragma unroll
      for (int k = 0; k < 8; k++)
        if ((fl >> k) & 1u) {
          if (p < N) a1[p] = vals[k];
          p++;
        }
      pos1 += total;
      if (pos1 >= N) return true;
    }
    named_sync(bar, SUB);
  }
  return false;
}

// One residue of Poly::from_seed_moduli (poly.rs:251-281) by one 256-thread
// sub-block, for the kernels that expand each residue on its own CTA: the
// first N accepted draws of gen_range(0..q_res) among the stream's 64-bit
// candidates from global index `first` on (candidate 8 b + k is word pair k
// of block b).  Residue 0 starts at 0; residue 1 at the index after residue
// 0's last accepted draw.  Returns the index after the last accepted
// candidate, or -1 if the iteration bound was hit.
//
// Speculative start (spec_blk > 0): the first batch, from block spec_blk on,
// is drawn before `first` is known; then every thread calls get_first(),
// which returns it (at least 8 spec_blk for residue 1, whose position the
// other CTA finds).  Candidates before `first` are skipped, and blocks wholly
// before it are not drawn after the first batch, so the result does not
// depend on the guess.
template <class GetFirst>
__device__ long long expand_residue(const DevParams& P, const uint32_t key[8], int res, uint64_t first,
                                    uint64_t spec_blk, GetFirst&& get_first, uint64_t* cand, uint32_t* dst, int* ws,
                                    int bar, int lt) {
  const uint64_t q = P.r[res].q, zone = P.r[res].zone;
  uint64_t blk = spec_blk ? spec_blk : first / 8;
  int pos = 0;
  for (int it = 0; it < 64; it++) {
    const int nblk = min(SUB, ((N - pos) * 9) / 64 + 3);
    if (lt < nblk) {
      uint32_t w[16];
      chacha20_block(key, blk + lt, P.one, w);
#pragma unroll
      for (int k = 0; k < 8; k++) cand[k * SUB + lt] = (uint64_t)w[2 * k] | ((uint64_t)w[2 * k + 1] << 32);
    }
    const uint64_t gbase = 8 * blk;  // global index of local candidate 0
    blk += nblk;
    named_sync(bar, SUB);
    if (it == 0 && spec_blk) first = get_first();
    uint32_t vals[8];
    unsigned fl = 0;
    int cnt = 0;
    if (lt < nblk) {
#pragma unroll
      for (int k = 0; k < 8; k++)
        if (gbase + 8 * lt + k >= first && uniform_accept(cand[k * SUB + lt], q, zone, vals[k])) {
          fl |= 1u << k;
          cnt++;
        }
    }
    int total;
    int p = pos + sub_scan_excl(cnt, ws, total, bar, lt);
#pragma unroll
    for (int k = 0; k < 8; k++)
      if ((fl >> k) & 1u) {
        if (p < N) dst[p] = vals[k];
        if (p == N - 1) ws[16] = 8 * lt + k;
        p++;
      }
    named_sync(bar, SUB);
    if (pos + total >= N) {
      const long long end = (long long)(gbase + (uint64_t)ws[16] + 1);
      named_sync(bar, SUB);  // ws[16] is read before the next use of ws
      return end;
    }
    pos += total;
    if (blk < first / 8) blk = first / 8;
  }
  return -1;
}

}  // namespace ig
