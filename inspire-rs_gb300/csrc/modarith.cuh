// modarith.cuh -- exact 32-bit modular arithmetic for the two 28-bit CRT
// primes of the InsPIRe parameter set (268369921, 249561089).
//
// Values are canonical u32 residues in [0, q).  Products use either Shoup
// multiplication by a precomputed constant (w, w' = floor(w * 2^32 / q)) or
// 32-bit Montgomery reduction (REDC, R = 2^32) of a 64-bit accumulator.  All
// results are exact: the GPU path computes the same integers as the
// reference's u64 / Montgomery-2^64 arithmetic (src/math/ntt.rs:468-479), only
// in a different internal representation.
#pragma once
#include <cstdint>

namespace ig {

// a, b in [0, q): (a + b) mod q
__device__ __forceinline__ uint32_t add_mod(uint32_t a, uint32_t b, uint32_t q) {
  uint32_t s = a + b;
  return min(s, s - q);
}

// a, b in [0, q): (a - b) mod q
__device__ __forceinline__ uint32_t sub_mod(uint32_t a, uint32_t b, uint32_t q) {
  uint32_t d = a - b;
  return min(d, d + q);
}

// a in [0, 2q) -> [0, q)
__device__ __forceinline__ uint32_t reduce_2q(uint32_t a, uint32_t q) { return min(a, a - q); }

// Shoup: a * w mod q for any a < 2^32 and constant w < q < 2^31.
__device__ __forceinline__ uint32_t mul_shoup(uint32_t a, uint32_t w, uint32_t wp, uint32_t q) {
  uint32_t h = __umulhi(a, wp);
  uint32_t r = a * w - h * q;  // in [0, 2q)
  return min(r, r - q);
}

// Montgomery reduction of T < q * 2^32: returns T * 2^-32 mod q in [0, 2q).
__device__ __forceinline__ uint32_t redc_lazy(uint64_t T, uint32_t q, uint32_t qinv) {
  uint32_t m = (uint32_t)T * qinv;             // qinv = -q^-1 mod 2^32
  uint64_t s = T + (uint64_t)m * q;            // low 32 bits are zero
  return (uint32_t)(s >> 32);
}

__device__ __forceinline__ uint32_t redc(uint64_t T, uint32_t q, uint32_t qinv) {
  uint32_t r = redc_lazy(T, q, qinv);
  return min(r, r - q);
}

// a * b * 2^-32 mod q (canonical)
__device__ __forceinline__ uint32_t mont_mul(uint32_t a, uint32_t b, uint32_t q, uint32_t qinv) {
  return redc((uint64_t)a * b, q, qinv);
}

// Lazy accumulate: x, r in [0, 2q) -> x + r in [0, 2q)
__device__ __forceinline__ uint32_t acc_2q(uint32_t x, uint32_t r, uint32_t q2) {
  uint32_t s = x + r;
  return min(s, s - q2);
}

}  // namespace ig
