// common.cuh -- parameters shared by the InsPIRe GB300 kernels.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "modarith.cuh"
#include "ntt2048.cuh"

namespace ig {

constexpr int N = 2048;        // ring dimension d (params.rs:213-230, secure_128_d2048)
constexpr int LOGN = 11;
constexpr int ELL = 3;         // gadget length (rgsw/types.rs:38-91)
constexpr int ZBITS = 20;      // gadget base 2^20
constexpr int MAX_GAMMA = 16;  // packed columns supported by the fused kernel
constexpr int BLOCK = 256;     // two NTT groups: one per CRT residue

// Automorphism-in-NTT-domain semantics of src/inspiring/inspiring2.rs:279-296.
constexpr int MODE_COMPAT = 0;     // reference behaviour, bit-exact
constexpr int MODE_CRT_FIXED = 1;  // permutation applied to both residues

struct ResidueConsts {
  uint32_t q, qinv;                  // qinv = -q^-1 mod 2^32
  const uint2* fwd;                  // {psi^brv(k), Shoup companion}, k in [1, n)
  const uint2* inv;                  // {psi^-brv(k), Shoup companion}
  const uint32_t* psi_pow;           // psi^e, e in [0, 2n)
  uint32_t r64, r64_p;               // 2^64 mod q: reference Montgomery factor
  uint32_t ref_inv_scale, ref_inv_scale_p;  // n^-1 * 2^-64 mod q
  uint32_t ninv_mont, ninv_mont_p;   // n^-1 * 2^32 mod q
  uint32_t mont, mont_p;             // 2^32 mod q
  uint32_t e_scale, e_scale_p;       // gamma^-1 * n^-1 * 2^96 mod q (database contraction)
  uint32_t d2_nz2, d2_nz2_p;         // n z^-2 mod q  (third gadget digit's transform, z = 2^20)
  uint32_t d2_z2, d2_z2_p;           // z^-2 mod q
  uint32_t d2_z1, d2_z1_p;           // z^-1 mod q
  uint64_t zone;                     // rand 0.8 rejection zone for gen_range(0..q)
};

struct DevParams {
  ResidueConsts r[2];
  uint32_t q0inv_q1, q0inv_q1_p;     // q0^-1 mod q1 (crt.rs:41-50)
  uint32_t conv_a, conv_a_p;         // n * 2^64 mod q0
  uint32_t conv_b, conv_b_p;         // 2^-64 * n^-1 mod q1
  uint32_t conv0_a, conv0_a_p;       // 2^64 mod q0
  uint32_t conv0_b, conv0_b_p;       // 2^-64 mod q1
  uint64_t delta;                    // floor(q / p)
  int gamma;                         // packed columns (num_to_pack)
  int mode;
  uint32_t one;                      // 1 (a value the compiler cannot fold)
};

__device__ __forceinline__ TwiddleRef fwd_tw(const ResidueConsts& c) { return {c.fwd}; }
__device__ __forceinline__ TwiddleRef inv_tw(const ResidueConsts& c) { return {c.inv}; }

__device__ __forceinline__ uint32_t brv11(uint32_t x) { return __brev(x) >> (32 - LOGN); }

// Composite coefficient of (a0 mod q0, a1 mod q1): a0 + q0 * ((a1 - a0) q0^-1 mod q1)
// (crt.rs:41-50); the result is < q0 * q1.
__device__ __forceinline__ uint64_t crt_compose(const DevParams& P, uint32_t a0, uint32_t a1) {
  const uint32_t q0 = P.r[0].q, q1 = P.r[1].q;
  uint32_t a0m = a0 >= q1 ? a0 - q1 : a0;  // q0 < 2 q1
  uint32_t d = sub_mod(a1, a0m, q1);
  uint32_t t = mul_shoup(d, P.q0inv_q1, P.q0inv_q1_p, q1);
  return (uint64_t)a0 + (uint64_t)q0 * t;
}

// Residue 1 rebuilt from a residue-0 NTT value as the reference does in
// apply_automorphism_ntt + Poly::from_coeffs_moduli (inspiring2.rs:279-296,
// poly.rs:127-159): the residue-0 word is the Montgomery form v * 2^64 mod q0,
// reduced mod q1 and read as residue 1's Montgomery form.  `v` and the result
// are plain residues.
__device__ __forceinline__ uint32_t compat_residue1(const DevParams& P, uint32_t v) {
  uint32_t m = mul_shoup(v, P.conv0_a, P.conv0_a_p, P.r[0].q);
  uint32_t g = m >= P.r[1].q ? m - P.r[1].q : m;
  return mul_shoup(g, P.conv0_b, P.conv0_b_p, P.r[1].q);
}

// Same map on values that carry an extra factor n^-1 in both residues.
__device__ __forceinline__ uint32_t compat_residue1_ninv(const DevParams& P, uint32_t v) {
  uint32_t m = mul_shoup(v, P.conv_a, P.conv_a_p, P.r[0].q);
  uint32_t g = m >= P.r[1].q ? m - P.r[1].q : m;
  return mul_shoup(g, P.conv_b, P.conv_b_p, P.r[1].q);
}

// Galois element g^i mod 2n for the InspiRING generator g = 2n/gamma + 1
// (inspiring2.rs:115-127).
__device__ __forceinline__ uint32_t gen_pow(int gamma, int i) {
  const uint32_t g = gamma < N ? (2 * N) / gamma + 1 : 5;
  uint32_t v = 1;
  for (int k = 0; k < i; k++) v = (v * g) & (2 * N - 1);
  return v;
}

}  // namespace ig
