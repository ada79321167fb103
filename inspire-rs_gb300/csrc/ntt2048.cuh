// ntt2048.cuh -- negacyclic 2048-point NTT / inverse NTT for one CRT residue,
// computed by a "group" of 128 threads (4 warps) with 16 values per thread.
//
// Transform semantics match the reference NttContext (src/math/ntt.rs:269-379):
// forward output slot s holds a(psi^(2*brv(s)+1)), psi being the reference's
// primitive 2n-th root (first g >= 2 with g^((q-1)/2n) of order 2n,
// ntt.rs:525-538); the inverse is its exact inverse.  Values here are plain
// residues (no Montgomery factor); callers fold constant factors (R = 2^64 of
// the reference form, n^-1) into loads or twiddle-free scalings.
//
// Data layout per thread x (0..127) of the group:
//   "coefficient layout" (forward input, inverse output): v[r] = a[x + 128 r]
//   "slot layout" (forward output, inverse input):        v[r] = A[16 x + r]
// Stages 0-3 and 8-10 run in registers; two exchanges through a per-group
// shared-memory scratch of NTT_SCRATCH words re-pair the values for stages
// 4-7 and 8-10.  The two padded index maps keep every exchange free of bank
// conflicts.
#pragma once
#include <cstdint>

#include "modarith.cuh"

namespace ig {

constexpr int NTT_N = 2048;
constexpr int NTT_GT = 128;   // threads per group
constexpr int NTT_SCRATCH = NTT_N + 128;

__device__ __forceinline__ int pad_a(int j) { return j + ((j >> 7) << 3); }
__device__ __forceinline__ int pad_b(int j) { return j + (j >> 4); }

// Barrier over the 128 threads of one group (named barrier `id`, 1..15).
__device__ __forceinline__ void group_sync(int id) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(NTT_GT) : "memory");
}

struct TwiddleRef {
  const uint32_t* __restrict__ w;   // w[k] = psi^(+-brv(k)), k in [1, n)
  const uint32_t* __restrict__ wp;  // Shoup companions floor(w * 2^32 / q)
};

__device__ __forceinline__ void ct_bfly(uint32_t& a, uint32_t& b, uint32_t w, uint32_t wp,
                                        uint32_t q) {
  uint32_t t = mul_shoup(b, w, wp, q);
  uint32_t u = a;
  a = add_mod(u, t, q);
  b = sub_mod(u, t, q);
}

__device__ __forceinline__ void gs_bfly(uint32_t& a, uint32_t& b, uint32_t w, uint32_t wp,
                                        uint32_t q) {
  uint32_t u = a, v = b;
  a = add_mod(u, v, q);
  b = mul_shoup(sub_mod(u, v, q), w, wp, q);
}

// Forward transform (Cooley-Tukey, decimation in time), coefficient layout in,
// slot layout out.  `sc` is this group's scratch; `bar` its barrier id.
__device__ __forceinline__ void ntt_fwd(uint32_t v[16], uint32_t* sc, TwiddleRef tw, uint32_t q,
                                        int x, int bar) {
  // stages 0..3: element r is a[x + 128 r]; pair distance 8 >> s in r
#pragma unroll
  for (int s = 0; s < 4; s++) {
    const int h = 8 >> s;
#pragma unroll
    for (int r = 0; r < 16; r++) {
      if ((r & h) == 0) {
        const int k = (1 << s) + (r >> (4 - s));
        ct_bfly(v[r], v[r + h], __ldg(tw.w + k), __ldg(tw.wp + k), q);
      }
    }
  }
  group_sync(bar);
#pragma unroll
  for (int r = 0; r < 16; r++) sc[pad_a(x + 128 * r)] = v[r];
  group_sync(bar);
  const int b = x >> 3, y = x & 7;
#pragma unroll
  for (int r = 0; r < 16; r++) v[r] = sc[pad_a(128 * b + y + 8 * r)];
  // stages 4..7: element r is a[128 b + y + 8 r]
#pragma unroll
  for (int s = 4; s < 8; s++) {
    const int h = 8 >> (s - 4);
#pragma unroll
    for (int r = 0; r < 16; r++) {
      if ((r & h) == 0) {
        const int k = (1 << s) + (b << (s - 4)) + (r >> (8 - s));
        ct_bfly(v[r], v[r + h], __ldg(tw.w + k), __ldg(tw.wp + k), q);
      }
    }
  }
  group_sync(bar);
#pragma unroll
  for (int r = 0; r < 16; r++) sc[pad_b(128 * b + y + 8 * r)] = v[r];
  group_sync(bar);
#pragma unroll
  for (int r = 0; r < 16; r++) v[r] = sc[pad_b(16 * x + r)];
  // stages 8..10: element r is a[16 x + r]
#pragma unroll
  for (int s = 8; s < 11; s++) {
    const int h = 4 >> (s - 8);
#pragma unroll
    for (int r = 0; r < 16; r++) {
      if ((r & h) == 0) {
        const int k = (1 << s) + (x << (s - 7)) + (r >> (11 - s));
        ct_bfly(v[r], v[r + h], __ldg(tw.w + k), __ldg(tw.wp + k), q);
      }
    }
  }
}

// Inverse transform without the n^-1 factor (Gentleman-Sande, decimation in
// frequency), slot layout in, coefficient layout out.
__device__ __forceinline__ void ntt_inv_noscale(uint32_t v[16], uint32_t* sc, TwiddleRef tw,
                                                uint32_t q, int x, int bar) {
#pragma unroll
  for (int s = 10; s >= 8; s--) {
    const int h = 4 >> (s - 8);
#pragma unroll
    for (int r = 0; r < 16; r++) {
      if ((r & h) == 0) {
        const int k = (1 << s) + (x << (s - 7)) + (r >> (11 - s));
        gs_bfly(v[r], v[r + h], __ldg(tw.w + k), __ldg(tw.wp + k), q);
      }
    }
  }
  const int b = x >> 3, y = x & 7;
  group_sync(bar);
#pragma unroll
  for (int r = 0; r < 16; r++) sc[pad_b(16 * x + r)] = v[r];
  group_sync(bar);
#pragma unroll
  for (int r = 0; r < 16; r++) v[r] = sc[pad_b(128 * b + y + 8 * r)];
#pragma unroll
  for (int s = 7; s >= 4; s--) {
    const int h = 8 >> (s - 4);
#pragma unroll
    for (int r = 0; r < 16; r++) {
      if ((r & h) == 0) {
        const int k = (1 << s) + (b << (s - 4)) + (r >> (8 - s));
        gs_bfly(v[r], v[r + h], __ldg(tw.w + k), __ldg(tw.wp + k), q);
      }
    }
  }
  group_sync(bar);
#pragma unroll
  for (int r = 0; r < 16; r++) sc[pad_a(128 * b + y + 8 * r)] = v[r];
  group_sync(bar);
#pragma unroll
  for (int r = 0; r < 16; r++) v[r] = sc[pad_a(x + 128 * r)];
#pragma unroll
  for (int s = 3; s >= 0; s--) {
    const int h = 8 >> s;
#pragma unroll
    for (int r = 0; r < 16; r++) {
      if ((r & h) == 0) {
        const int k = (1 << s) + (r >> (4 - s));
        gs_bfly(v[r], v[r + h], __ldg(tw.w + k), __ldg(tw.wp + k), q);
      }
    }
  }
}

}  // namespace ig
