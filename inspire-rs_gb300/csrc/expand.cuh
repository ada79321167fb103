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

}  // namespace ig
