// ntt2048.cuh -- negacyclic 2048-point NTT / inverse NTT for one CRT residue,
// computed by a "group" of 128 threads (4 warps) with 16 values per thread.
//
// Transform semantics match the reference NttContext (src/math/ntt.rs:269-379):
// forward output slot s holds a(psi^(2*brv(s)+1)), psi being the reference's
// primitive 2n-th root (first g >= 2 with g^((q-1)/2n) of order 2n,
// ntt.rs:525-538); the inverse is its exact inverse.  Values here are plain
// residues (no Montgomery factor); callers fold constant factors (R = 2^64 of
// the reference form, n^-1) into loads or scalings.
//
// Values stay lazily reduced.  The moduli are below 2^28, so 16q < 2^32, and
// Shoup's multiply accepts any 32-bit input and returns [0, 2q).  The forward
// butterflies therefore skip Harvey's per-butterfly reduction: each stage
// grows the bound by 2q, and one conditional subtraction of 8q per value at
// each of the two exchanges keeps it below 16q.  Input [0, 4q) -> 12q after
// stages 0-3 -> 8q -> 16q after stages 4-7 -> 8q -> output [0, 14q).  The
// inverse (Harvey's Gentleman-Sande butterflies) takes [0, 2q) and returns
// [0, 2q).  canon16 / canon4 / canon2 bring values to [0, q).  Twiddles are
// read as {w, floor(w * 2^32 / q)} pairs (one 64-bit load).
//
// Data layout per thread x (0..127) of the group:
//   "coefficient layout" (forward input, inverse output): v[r] = a[x + 128 r]
//   "slot layout" (forward output, inverse input):        v[r] = A[16 x + r]
// Stages 0-3, 4-7 and 8-10 run in registers, each reading its thread's run
// of consecutive twiddle pairs with 128-bit loads; two exchanges through a
// per-group shared-memory scratch of NTT_SCRATCH words re-pair the values
// between the phases.  Both padded index maps keep the exchanges free of bank
// conflicts.
#pragma once
#include <cstdint>

#include "modarith.cuh"

namespace ig {

constexpr int NTT_N = 2048;
constexpr int NTT_GT = 128;  // threads per group
constexpr int NTT_SCRATCH = NTT_N + 128;

__device__ __forceinline__ int pad_a(int j) { return j + ((j >> 7) << 3); }
__device__ __forceinline__ int pad_b(int j) { return j + (j >> 4); }

// Barrier over the 128 threads of one group (named barrier `id`, 1..15).
__device__ __forceinline__ void group_sync(int id) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(NTT_GT) : "memory");
}

struct TwiddleRef {
  const uint2* __restrict__ w;  // w[k] = {psi^(+-brv(k)), floor(w * 2^32 / q)}, k in [1, n)
};

// a * w mod q up to one q: result in [0, 2q) for any a < 2^32.
__device__ __forceinline__ uint32_t mul_shoup_lazy(uint32_t a, uint2 w, uint32_t q) {
  const uint32_t h = __umulhi(a, w.y);
  return a * w.x - h * q;
}

// Cooley-Tukey butterfly without reducing its inputs: both outputs are below
// the inputs' bound plus 2q.
__device__ __forceinline__ void ct_bfly(uint32_t& a, uint32_t& b, uint2 w, uint32_t q, uint32_t q2) {
  const uint32_t x = a;
  const uint32_t t = mul_shoup_lazy(b, w, q);
  a = x + t;
  b = x - t + q2;
}

// Every value below 16q -> below 8q.
__device__ __forceinline__ void reduce_8q(uint32_t v[16], uint32_t q) {
  const uint32_t q8 = 8 * q;
#pragma unroll
  for (int r = 0; r < 16; r++) v[r] = min(v[r], v[r] - q8);
}

// Gentleman-Sande butterfly, inputs and outputs in [0, 2q).
__device__ __forceinline__ void gs_bfly(uint32_t& a, uint32_t& b, uint2 w, uint32_t q, uint32_t q2) {
  const uint32_t u = a, v = b;
  const uint32_t s = u + v;
  a = min(s, s - q2);
  b = mul_shoup_lazy(u - v + q2, w, q);
}

__device__ __forceinline__ uint32_t canon4(uint32_t x, uint32_t q) {
  x = min(x, x - 2 * q);
  return min(x, x - q);
}

// [0, 16q) -> [0, q) (forward transform outputs).
__device__ __forceinline__ uint32_t canon16(uint32_t x, uint32_t q) {
  x = min(x, x - 8 * q);
  x = min(x, x - 4 * q);
  return canon4(x, q);
}

__device__ __forceinline__ uint32_t canon2(uint32_t x, uint32_t q) { return min(x, x - q); }

// Load the CNT contiguous twiddle pairs w[k0 .. k0+CNT) (k0 * 8 bytes is a
// multiple of 16 when CNT >= 2) with 128-bit loads.
template <int CNT>
__device__ __forceinline__ void tw_run(TwiddleRef t, int k0, uint2 (&w)[CNT]) {
  if (CNT == 1) {
    w[0] = __ldg(t.w + k0);
  } else {
    const uint4* p = reinterpret_cast<const uint4*>(t.w + k0);
#pragma unroll
    for (int i = 0; i < CNT / 2; i++) {
      const uint4 v = __ldg(p + i);
      w[2 * i] = make_uint2(v.x, v.y);
      w[2 * i + 1] = make_uint2(v.z, v.w);
    }
  }
}

// One register stage.  Element r pairs with r + H when (r & H) == 0 and uses
// twiddle run[r >> SH].
template <int H, int SH, int CNT, bool FWD>
__device__ __forceinline__ void reg_stage(uint32_t v[16], const uint2 (&run)[CNT], uint32_t q, uint32_t q2) {
#pragma unroll
  for (int r = 0; r < 16; r++) {
    if ((r & H) == 0) {
      if (FWD) ct_bfly(v[r], v[r + H], run[r >> SH], q, q2);
      else gs_bfly(v[r], v[r + H], run[r >> SH], q, q2);
    }
  }
}

// Stage S of a register phase: element r uses twiddle (1 << S) + first +
// (r >> SHIFT), i.e. a run of 16 >> SHIFT consecutive pairs per thread.
template <int S, int SHIFT, bool FWD>
__device__ __forceinline__ void stage(uint32_t v[16], TwiddleRef tw, int first, uint32_t q, uint32_t q2) {
  constexpr int CNT = 16 >> SHIFT;
  constexpr int H = (S < 4) ? (8 >> S) : (S < 8 ? (8 >> (S - 4)) : (4 >> (S - 8)));
  uint2 run[CNT];
  tw_run<CNT>(tw, (1 << S) + first, run);
  reg_stage<H, SHIFT, CNT, FWD>(v, run, q, q2);
}

// ---- exchanges within aligned 8-lane groups, by warp shuffles ----
// A thread's register index R and its lane index within the 8-lane group
// each carry some bits of the element index.  swap_lane_reg<J, K> exchanges
// lane bit J with register bit K: the value at (lane bit l, register bit s)
// moves to (lane bit s, register bit l), so values with l == s stay and the
// others trade places with the partner lane (lane ^ 2^J) at R ^ 2^K.  Three
// such swaps transpose an 8-lane group's values without shared memory or a
// barrier (the 8 lanes of a group are one warp's).
template <int NV, int J, int K>
__device__ __forceinline__ void swap_lane_reg(uint32_t* v, bool l) {
  constexpr int m = 1 << K;
#pragma unroll
  for (int R = 0; R < NV; R++) {
    if (R & m) continue;
    const uint32_t send = l ? v[R] : v[R | m];
    const uint32_t recv = __shfl_xor_sync(0xffffffffu, send, 1 << J);
    if (l) v[R] = recv;
    else v[R | m] = recv;
  }
}

// 128-thread transforms, between the layouts "element r is a[128 b + y + 8 r]"
// and "element r is a[16 x + r]" (x = 8 b + y, y = x & 7; the 8 lanes of b
// hold the same 128 elements).  Element e = y + 8 r of the block has lane
// bits (e0, e1, e2) and register bits (e3, e4, e5, e6); the target has lane
// bits (e4, e5, e6) and register bits (e0, e1, e2, e3).  Swapping lane bit j
// with register bit j + 1 (j = 0, 1, 2) leaves register bits (e3, e0, e1,
// e2), a static renaming of the registers.
__device__ __forceinline__ void xpose_16(uint32_t* v, int y) {
  swap_lane_reg<16, 0, 1>(v, y & 1);
  swap_lane_reg<16, 1, 2>(v, (y >> 1) & 1);
  swap_lane_reg<16, 2, 3>(v, (y >> 2) & 1);
  uint32_t w[16];
#pragma unroll
  for (int r = 0; r < 16; r++) w[r] = v[((r >> 3) & 1) | ((r & 7) << 1)];
#pragma unroll
  for (int r = 0; r < 16; r++) v[r] = w[r];
}

// Forward transform (Cooley-Tukey, decimation in time), coefficient layout in
// ([0, 4q)), slot layout out ([0, 14q)).  `sc` is this group's scratch; `bar`
// its barrier id.  SHFL: the second exchange by warp shuffles (xpose_16)
// instead of shared memory and two barriers.  Measured on GB300 in one A/B
// comparison: the batched transform 4 % faster, the Respond kernels
// unchanged, the NoPacking and tree kernels 2-4 % slower (about their
// run-to-run spread); those keep the shared-memory form.  The same 8-lane
// shuffle transpose in the 256-thread inverse made the two-CTA Respond
// kernel 15 % slower, so the inverse transforms keep shared memory.
template <bool SHFL = true>
__device__ __forceinline__ void ntt_fwd(uint32_t v[16], uint32_t* sc, TwiddleRef tw, uint32_t q, int x, int bar) {
  const uint32_t q2 = 2 * q;
  // stages 0..3: element r is a[x + 128 r]; twiddle (1 << s) + (r >> (4 - s))
  stage<0, 4, true>(v, tw, 0, q, q2);
  stage<1, 3, true>(v, tw, 0, q, q2);
  stage<2, 2, true>(v, tw, 0, q, q2);
  stage<3, 1, true>(v, tw, 0, q, q2);
  reduce_8q(v, q);  // < 12q -> < 8q
  group_sync(bar);
#pragma unroll
  for (int r = 0; r < 16; r++) sc[pad_a(x + 128 * r)] = v[r];
  group_sync(bar);
  const int b = x >> 3, y = x & 7;
#pragma unroll
  for (int r = 0; r < 16; r++) v[r] = sc[pad_a(128 * b + y + 8 * r)];
  // stages 4..7: element r is a[128 b + y + 8 r]; twiddle (1 << s) + (b << (s - 4)) + (r >> (8 - s))
  stage<4, 4, true>(v, tw, b, q, q2);
  stage<5, 3, true>(v, tw, b << 1, q, q2);
  stage<6, 2, true>(v, tw, b << 2, q, q2);
  stage<7, 1, true>(v, tw, b << 3, q, q2);
  reduce_8q(v, q);  // < 16q -> < 8q
  if (SHFL) {
    xpose_16(v, y);  // within the 8 lanes of b: no shared memory, no barrier
  } else {
    group_sync(bar);
#pragma unroll
    for (int r = 0; r < 16; r++) sc[pad_b(128 * b + y + 8 * r)] = v[r];
    group_sync(bar);
#pragma unroll
    for (int r = 0; r < 16; r++) v[r] = sc[pad_b(16 * x + r)];
  }
  // stages 8..10: element r is a[16 x + r]; twiddle (1 << s) + (x << (s - 7)) + (r >> (11 - s))
  stage<8, 3, true>(v, tw, x << 1, q, q2);
  stage<9, 2, true>(v, tw, x << 2, q, q2);
  stage<10, 1, true>(v, tw, x << 3, q, q2);
}

// Inverse transform without the n^-1 factor (Gentleman-Sande, decimation in
// frequency), slot layout in ([0, 2q)), coefficient layout out ([0, 2q)).
__device__ __forceinline__ void ntt_inv_noscale(uint32_t v[16], uint32_t* sc, TwiddleRef tw, uint32_t q, int x,
                                                int bar) {
  const uint32_t q2 = 2 * q;
  stage<10, 1, false>(v, tw, x << 3, q, q2);
  stage<9, 2, false>(v, tw, x << 2, q, q2);
  stage<8, 3, false>(v, tw, x << 1, q, q2);
  const int b = x >> 3, y = x & 7;
  group_sync(bar);
#pragma unroll
  for (int r = 0; r < 16; r++) sc[pad_b(16 * x + r)] = v[r];
  group_sync(bar);
#pragma unroll
  for (int r = 0; r < 16; r++) v[r] = sc[pad_b(128 * b + y + 8 * r)];
  stage<7, 1, false>(v, tw, b << 3, q, q2);
  stage<6, 2, false>(v, tw, b << 2, q, q2);
  stage<5, 3, false>(v, tw, b << 1, q, q2);
  stage<4, 4, false>(v, tw, b, q, q2);
  group_sync(bar);
#pragma unroll
  for (int r = 0; r < 16; r++) sc[pad_a(128 * b + y + 8 * r)] = v[r];
  group_sync(bar);
#pragma unroll
  for (int r = 0; r < 16; r++) v[r] = sc[pad_a(x + 128 * r)];
  stage<3, 1, false>(v, tw, 0, q, q2);
  stage<2, 2, false>(v, tw, 0, q, q2);
  stage<1, 3, false>(v, tw, 0, q, q2);
  stage<0, 4, false>(v, tw, 0, q, q2);
}

// ---- Inverse transform on a 256-thread team, 8 values per thread ----
// Used where one residue's inverse NTT is on the critical path and two
// groups are free to run it: half the dependent butterflies per thread of
// the 128-thread transform, one more exchange.  Slot layout in (thread t
// holds A[8t + r]), coefficient layout out (v[r] = a[t + 256 r]), values in
// [0, 2q) both ways, no n^-1 factor.  Register phases run stages 10-8, 7-5,
// 4-2 and 1-0; three exchanges through `sc` (2048 words) re-pair the values:
//   after stage 8:  idx = (t & 7) + 8 r + 64 (t >> 3)
//   after stage 5:  idx = (t & 63) + 64 r + 512 (t >> 6)
//   after stage 2:  idx = t + 256 r
// stored at idx ^ ((idx >> 3) & 31) (first two exchanges) and
// idx ^ ((idx >> 10) & 15) (third); both maps are permutations of [0, 2048)
// and keep every 32-bit access of a warp on 32 distinct banks.  Stage s pairs
// j with j + 1024 / 2^s and uses twiddle 2^s + (j >> (11 - s)), as the
// 128-thread transform does.

// Barrier over the 256 threads of a team (named barrier `id`).
__device__ __forceinline__ void team_sync(int id) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(2 * NTT_GT) : "memory");
}

__device__ __forceinline__ int x12(int i) { return i ^ ((i >> 3) & 31); }
__device__ __forceinline__ int x3(int i) { return i ^ ((i >> 10) & 15); }

// One GS stage over the 8 registers: element r pairs with r + H when
// (r & H) == 0, twiddle run[r >> SH].
template <int H, int SH, int CNT>
__device__ __forceinline__ void inv8_stage(uint32_t v[8], const uint2 (&run)[CNT], uint32_t q, uint32_t q2) {
#pragma unroll
  for (int r = 0; r < 8; r++)
    if ((r & H) == 0) gs_bfly(v[r], v[r + H], run[r >> SH], q, q2);
}

__device__ __forceinline__ void ntt_inv_noscale8(uint32_t v[8], uint32_t* sc, TwiddleRef tw, uint32_t q, int t,
                                                 int bar) {
  const uint32_t q2 = 2 * q;
  {
    uint2 r4[4], r2[2], r1[1];
    tw_run<4>(tw, 1024 + 4 * t, r4);
    inv8_stage<1, 1, 4>(v, r4, q, q2);
    tw_run<2>(tw, 512 + 2 * t, r2);
    inv8_stage<2, 2, 2>(v, r2, q, q2);
    tw_run<1>(tw, 256 + t, r1);
    inv8_stage<4, 3, 1>(v, r1, q, q2);
  }
  team_sync(bar);
#pragma unroll
  for (int r = 0; r < 8; r++) sc[x12(8 * t + r)] = v[r];
  team_sync(bar);
  const int b3 = t >> 3, b6 = t >> 6;
#pragma unroll
  for (int r = 0; r < 8; r++) v[r] = sc[x12((t & 7) + (r << 3) + (b3 << 6))];
  {
    uint2 r4[4], r2[2], r1[1];
    tw_run<4>(tw, 128 + 4 * b3, r4);
    inv8_stage<1, 1, 4>(v, r4, q, q2);
    tw_run<2>(tw, 64 + 2 * b3, r2);
    inv8_stage<2, 2, 2>(v, r2, q, q2);
    tw_run<1>(tw, 32 + b3, r1);
    inv8_stage<4, 3, 1>(v, r1, q, q2);
  }
  team_sync(bar);
#pragma unroll
  for (int r = 0; r < 8; r++) sc[x12((t & 7) + (r << 3) + (b3 << 6))] = v[r];
  team_sync(bar);
#pragma unroll
  for (int r = 0; r < 8; r++) v[r] = sc[x12((t & 63) + (r << 6) + (b6 << 9))];
  {
    uint2 r4[4], r2[2], r1[1];
    tw_run<4>(tw, 16 + 4 * b6, r4);
    inv8_stage<1, 1, 4>(v, r4, q, q2);
    tw_run<2>(tw, 8 + 2 * b6, r2);
    inv8_stage<2, 2, 2>(v, r2, q, q2);
    tw_run<1>(tw, 4 + b6, r1);
    inv8_stage<4, 3, 1>(v, r1, q, q2);
  }
  team_sync(bar);
#pragma unroll
  for (int r = 0; r < 8; r++) sc[x3((t & 63) + (r << 6) + (b6 << 9))] = v[r];
  team_sync(bar);
#pragma unroll
  for (int r = 0; r < 8; r++) v[r] = sc[x3(t + 256 * r)];
  {
    uint2 r2[2], r1[1];
    tw_run<2>(tw, 2, r2);
    inv8_stage<2, 2, 2>(v, r2, q, q2);
    tw_run<1>(tw, 1, r1);
    inv8_stage<4, 3, 1>(v, r1, q, q2);
  }
}

// Slot-layout arrays in shared memory are stored with this XOR swizzle, which
// moves 4-word chunks inside each 16-word block so that the 128-bit accesses
// of load16/store16 (thread x: words 16x..16x+15) hit eight distinct bank
// groups per quarter warp, while single-word accesses of 32 consecutive slots
// stay conflict-free.
__device__ __forceinline__ int swz(int s) { return s ^ (((s >> 5) & 3) << 2); }

__device__ __forceinline__ void load16(const uint32_t* base, int x, uint32_t v[16]) {
  const int f = (x >> 1) & 3;
#pragma unroll
  for (int r4 = 0; r4 < 4; r4++) {
    const uint4 t = *reinterpret_cast<const uint4*>(base + 16 * x + 4 * (r4 ^ f));
    v[4 * r4] = t.x;
    v[4 * r4 + 1] = t.y;
    v[4 * r4 + 2] = t.z;
    v[4 * r4 + 3] = t.w;
  }
}

__device__ __forceinline__ void store16(uint32_t* base, int x, const uint32_t v[16]) {
  const int f = (x >> 1) & 3;
#pragma unroll
  for (int r4 = 0; r4 < 4; r4++)
    *reinterpret_cast<uint4*>(base + 16 * x + 4 * (r4 ^ f)) = make_uint4(v[4 * r4], v[4 * r4 + 1], v[4 * r4 + 2], v[4 * r4 + 3]);
}

}  // namespace ig
