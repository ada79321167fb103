// chacha.cuh -- ChaCha20 keystream blocks for seeded-polynomial expansion.
//
// Restates the stream that the reference consumes through
// rand_chacha::ChaCha20Rng::from_seed (src/math/poly.rs:278-281): the 32-byte
// seed is the key, the 64-bit block counter (state words 12-13) starts at 0,
// the stream id (words 14-15) is 0, and 64-bit draws take two consecutive
// little-endian keystream words, low word first.  The block function is the
// RFC 8439 one (20 rounds, column then diagonal quarter rounds).
#pragma once
#include <cstdint>

namespace ig {

__device__ __forceinline__ uint32_t rotl32(uint32_t x, int k) { return __funnelshift_l(x, x, k); }

// The quarter round's additions are written as multiply-adds by `one` (a
// runtime 1 the compiler cannot fold), which puts them on the integer
// multiply-add pipe while the xors and rotates use the ALU pipe: the block
// function is otherwise limited by the ALU pipe alone.
#define IG_QR(a, b, c, d)                       \
  a = a * one + b; d ^= a; d = rotl32(d, 16);   \
  c = c * one + d; b ^= c; b = rotl32(b, 12);   \
  a = a * one + b; d ^= a; d = rotl32(d, 8);    \
  c = c * one + d; b ^= c; b = rotl32(b, 7);

// Block `ctr` of the keystream keyed by key[8]; writes 16 words.  `one`
// must be 1.
__device__ __forceinline__ void chacha20_block(const uint32_t key[8], uint64_t ctr, uint32_t one,
                                               uint32_t out[16]) {
  uint32_t x0 = 0x61707865u, x1 = 0x3320646eu, x2 = 0x79622d32u, x3 = 0x6b206574u;
  uint32_t x4 = key[0], x5 = key[1], x6 = key[2], x7 = key[3];
  uint32_t x8 = key[4], x9 = key[5], x10 = key[6], x11 = key[7];
  uint32_t x12 = (uint32_t)ctr, x13 = (uint32_t)(ctr >> 32), x14 = 0, x15 = 0;
  // a loop, not unrolled: the rounds' dependencies leave no cross-round
  // overlap to gain, and the unrolled body (~1000 instructions) measured
  // slower in the kernels that expand once per query (instruction fetch)
#pragma unroll 1
  for (int i = 0; i < 10; i++) {
    IG_QR(x0, x4, x8, x12);
    IG_QR(x1, x5, x9, x13);
    IG_QR(x2, x6, x10, x14);
    IG_QR(x3, x7, x11, x15);
    IG_QR(x0, x5, x10, x15);
    IG_QR(x1, x6, x11, x12);
    IG_QR(x2, x7, x8, x13);
    IG_QR(x3, x4, x9, x14);
  }
  out[0] = x0 + 0x61707865u;
  out[1] = x1 + 0x3320646eu;
  out[2] = x2 + 0x79622d32u;
  out[3] = x3 + 0x6b206574u;
  out[4] = x4 + key[0];
  out[5] = x5 + key[1];
  out[6] = x6 + key[2];
  out[7] = x7 + key[3];
  out[8] = x8 + key[4];
  out[9] = x9 + key[5];
  out[10] = x10 + key[6];
  out[11] = x11 + key[7];
  out[12] = x12 + (uint32_t)ctr;
  out[13] = x13 + (uint32_t)(ctr >> 32);
  out[14] = x14;
  out[15] = x15;
}
#undef IG_QR

// rand 0.8 UniformInt<u64>::sample_single(0, q): draw v, accept when the low
// 64 bits of v*q are <= zone = (q << clz(q)) - 1, value = high 64 bits.
__device__ __forceinline__ bool uniform_accept(uint64_t v, uint64_t q, uint64_t zone,
                                               uint32_t& value) {
  uint64_t lo = v * q;
  value = (uint32_t)__umul64hi(v, q);
  return lo <= zone;
}

}  // namespace ig
