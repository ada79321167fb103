// respond_common.cuh -- device helpers shared by the Respond kernels
// (respond.cu: one CTA per query; respond_pair.cu: a cluster of two CTAs
// per query, one per CRT residue): bulk copies and mbarriers, the scatter of
// the query-only term R_i, and the client key-table runs.
#pragma once
#include "common.cuh"

namespace ig {

// A 64-bit load the compiler may neither hoist nor keep in a register: used
// to re-read a query's database base pointer where it is needed instead of
// holding it through the kernel.
template <class T>
__device__ __forceinline__ T* reload_ptr(T* const* p) {
  uint64_t v;
  asm volatile("ld.global.nc.u64 %0, [%1];" : "=l"(v) : "l"(p));
  return reinterpret_cast<T*>(v);
}

// L2 prefetch of a contiguous device range with bulk (TMA) prefetches.
__device__ __forceinline__ void prefetch_l2(const void* p, size_t bytes) {
  const char* c = static_cast<const char*>(p);
  for (size_t off = 0; off < bytes; off += 65536) {
    const uint32_t sz = (uint32_t)(bytes - off < 65536 ? bytes - off : 65536);
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(c + off), "r"(sz) : "memory");
  }
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// mbarrier with one arrival, visible to the bulk-copy (async) proxy.
__device__ __forceinline__ void mbar_init(uint64_t* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Invalidate an mbarrier before its words are used for anything else.
__device__ __forceinline__ void mbar_inval(uint64_t* bar) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// The single arrival, announcing `bytes` of bulk copies to complete.
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// Bulk copy of `bytes` (a multiple of 16; both addresses 16-byte aligned)
// from global memory -- device or mapped host memory -- into this CTA's shared
// memory, completing on `bar`.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

// Wait, with an iteration bound, for phase `parity` of `bar` to complete;
// false when the bound ran out (at once for limit 0).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t limit) {
  for (uint32_t it = 0; it < limit; it++) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// R_i (NTT domain, scaled by n^-1) of packing_offline step 1 for one residue,
// scattered to dst[slot]: source slot u contributes to slot s with
// 2brv(s)+1 = h_i (2brv(u)+1) mod 2n, where h_i = g^-i
// (inspiring2.rs:952-981 with the tables of :208-263).  Eg is this residue's
// contracted shard [gamma][ELL][N], stored by step (encode_E_kernel): the
// three rows' DFT outputs for slot u of step i sit at [i][t][u], so the loads
// of consecutive slots are contiguous.  Threads p in [0, nthr) handle
// u = p + nthr * v.
// In compat mode `dst1`, if not null, receives residue 1 rebuilt from each
// residue-0 value as the crate's apply_automorphism_ntt does (`dst` may then
// be null: only residue 1 is written).
__device__ __forceinline__ void scatter_r(const DevParams& P, int i, const uint32_t* __restrict__ Eg, const uint32_t* Ag,
                                          int astride, uint32_t* dst, int p, int nthr, uint32_t q, uint32_t qinv,
                                          uint32_t* dst1 = nullptr, int u0 = 0, int u1 = N) {
  const int gamma = P.gamma;
  const uint32_t mi = (uint32_t)(gamma - i) & (uint32_t)(gamma - 1);
  const uint32_t hi = (1u + (uint32_t)(2 * N / gamma) * mi) & (2 * N - 1);
  const uint32_t* Ei = Eg + (size_t)i * ELL * N;
#pragma unroll 4
  for (int u = u0 + p; u < u1; u += nthr) {
    const uint32_t e = 2 * brv11(u) + 1;
    const int us = swz(u);
    const uint64_t T = (uint64_t)__ldg(Ei + u) * Ag[us] + (uint64_t)__ldg(Ei + N + u) * Ag[astride + us] +
                       (uint64_t)__ldg(Ei + 2 * N + u) * Ag[2 * astride + us];
    const uint32_t s = brv11(((hi * e) & (2 * N - 1)) >> 1);
    const uint32_t val = redc(T, q, qinv);
    if (dst) dst[swz(s)] = val;
    if (dst1) dst1[swz(s)] = compat_residue1_ninv(P, val);
  }
}

// y_all[i][k] from NTT(y_body[k]) in registers (gamma = 16).  In the NTT
// domain tau_{g^i} (generate_rotations, inspiring2.rs:1309-1323) is the slot
// permutation s -> u with 2brv(u)+1 = g^i (2brv(s)+1) mod 2n.  With
// g = 2n/16 + 1, g^i = 1 + 256 i mod 2n, so brv(u) = brv(s) + 128 delta mod
// 2n with delta = i (2brv(s)+1) mod 16: only the top four bits of brv(s)
// move, i.e. only the low four bits of s, and delta depends on s only
// through s >> 4.  Each thread's run of slots 16x..16x+15 is therefore a
// rotation by delta of itself, indexed by brv4 of the slot's low bits:
// out[brv4(h)] = in[brv4((h + delta) mod 16)].  Done as a four-stage barrel
// shift of register selects.
__device__ __forceinline__ void rotate_key_run(uint4 (&y)[4], int i, int x) {
  uint32_t z[16];  // z[h] = in[brv4(h)]
#pragma unroll
  for (int h = 0; h < 16; h++) {
    const int j = ((h & 1) << 3) | ((h & 2) << 1) | ((h & 4) >> 1) | ((h & 8) >> 3);
    const uint4& c = y[j >> 2];
    z[h] = (j & 3) == 0 ? c.x : (j & 3) == 1 ? c.y : (j & 3) == 2 ? c.z : c.w;
  }
  const uint32_t delta = ((uint32_t)i * (2u * brv11(16u * (uint32_t)x) + 1u)) & 15u;
#pragma unroll
  for (int b = 0; b < 4; b++) {
    const bool on = (delta >> b) & 1u;
    uint32_t t[16];
#pragma unroll
    for (int h = 0; h < 16; h++) t[h] = on ? z[(h + (1 << b)) & 15] : z[h];
#pragma unroll
    for (int h = 0; h < 16; h++) z[h] = t[h];
  }
  uint32_t o[16];
#pragma unroll
  for (int h = 0; h < 16; h++) {
    const int j = ((h & 1) << 3) | ((h & 2) << 1) | ((h & 4) >> 1) | ((h & 8) >> 3);
    o[j] = z[h];
  }
#pragma unroll
  for (int r4 = 0; r4 < 4; r4++) y[r4] = make_uint4(o[4 * r4], o[4 * r4 + 1], o[4 * r4 + 2], o[4 * r4 + 3]);
}

// Load a 16-slot run of a key slice (uint4 x 4; y: rotated from the body
// table when `ybody`).
__device__ __forceinline__ void key_run(const uint32_t* p, uint4 (&k)[4]) {
  const uint4* k4 = reinterpret_cast<const uint4*>(p);
#pragma unroll
  for (int r4 = 0; r4 < 4; r4++) k[r4] = __ldg(k4 + r4);
}

__device__ __forceinline__ uint32_t u4e(const uint4& v, int e) { return e == 0 ? v.x : e == 1 ? v.y : e == 2 ? v.z : v.w; }

}  // namespace ig
