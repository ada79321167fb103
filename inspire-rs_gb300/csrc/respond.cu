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
// Layout: 768 threads = six groups of 128, group g = 3 r + k owns CRT residue
// r and gadget digit k.  Per recursion step, groups (r,0) run the inverse NTT
// while groups (r,1),(r,2) scatter the query-only term R_i; then the three
// digit NTTs of each residue run concurrently.  All intermediate state lives
// in shared memory and registers, and no global scratch is used: device-row
// launches take the b side from bside_kernel, which parks it in the last
// 128 bytes of each query's response slot.
#include "expand.cuh"
#include "kernels.h"
#include "respond_common.cuh"

namespace ig {

namespace {

// b0_c for every column c and residue (see file comment).  rows holds the
// query's rows ELL..2ELL-1 (b polys, u64; device memory or staged in shared
// memory); bp (6N words) is scratch; bpoly[r * 16 + c] receives the result.
// Warp c handles column c:
// lane l takes the coefficient pairs i = 2 (l + 32 m) + {0, 1}, reading the
// raw column as u32 pairs and the staged rows as 64-bit words, so every
// shared-memory read of a warp covers 256 contiguous bytes (no bank
// conflicts).  Each lane issues its column loads 16 at a time, so the column
// costs two memory latencies.
template <int NT>
__device__ void column_b0(const DevParams& P, const uint16_t* __restrict__ H, const uint64_t* rows, uint32_t* bp,
                          uint32_t* bpoly) {
  const int tid = threadIdx.x, gamma = P.gamma;
  const int lane = tid & 31, c = tid >> 5;
#pragma unroll 8
  for (int idx = tid; idx < ELL * 2 * N; idx += NT) {
    const int i = idx & (N - 1), tr = idx >> LOGN, r = tr & 1;
    uint32_t v = (uint32_t)rows[(size_t)tr * N + (i == 0 ? 0 : N - i)];
    if (i != 0 && v != 0) v = P.r[r].q - v;
    bp[idx] = v;
  }
  __syncthreads();
  if (c < gamma) {
    const uint32_t* h2 = reinterpret_cast<const uint32_t*>(H + (size_t)c * N);
    const uint2* b2 = reinterpret_cast<const uint2*>(bp);
    uint64_t acc0 = 0, acc1 = 0;
#pragma unroll 1
    for (int m0 = 0; m0 < N / 64; m0 += 16) {
      uint32_t hw[16];
#pragma unroll
      for (int m = 0; m < 16; m++) hw[m] = __ldg(h2 + lane + 32 * (m0 + m));
#pragma unroll
      for (int m = 0; m < 16; m++) {
        const int j = lane + 32 * (m0 + m);  // pair index: coefficients 2j, 2j + 1
        const uint2 b00 = b2[0 * (N / 2) + j], b01 = b2[1 * (N / 2) + j];  // digit 0: residue 0, 1
        const uint2 b10 = b2[2 * (N / 2) + j], b11 = b2[3 * (N / 2) + j];  // digit 1
        const uint2 b20 = b2[4 * (N / 2) + j], b21 = b2[5 * (N / 2) + j];  // digit 2
#pragma unroll
        for (int e = 0; e < 2; e++) {
          const uint64_t xv = P.delta * (uint64_t)((hw[m] >> (16 * e)) & 0xFFFFu);
          const uint32_t d0 = (uint32_t)xv & 0xFFFFFu, d1 = (uint32_t)(xv >> 20) & 0xFFFFFu,
                         d2 = (uint32_t)(xv >> 40);
          acc0 += (uint64_t)d0 * (e ? b00.y : b00.x) + (uint64_t)d1 * (e ? b10.y : b10.x) +
                  (uint64_t)d2 * (e ? b20.y : b20.x);
          acc1 += (uint64_t)d0 * (e ? b01.y : b01.x) + (uint64_t)d1 * (e ? b11.y : b11.x) +
                  (uint64_t)d2 * (e ? b21.y : b21.x);
        }
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      acc0 += __shfl_down_sync(0xffffffffu, acc0, o);
      acc1 += __shfl_down_sync(0xffffffffu, acc1, o);
    }
    if (lane == 0) {
      bpoly[c] = (uint32_t)(acc0 % P.r[0].q);
      bpoly[16 + c] = (uint32_t)(acc1 % P.r[1].q);
    }
  }
  __syncthreads();
}

// Device-row launches compute the b side in a launch of their own
// (bside_kernel, 512 threads and 48 KiB of shared memory per query, so many
// queries' loads are in flight per SM) and park each query's 32 b0 values in
// the last 128 bytes of its response, which the Respond kernel reads at its
// start and overwrites with the response at its end.
constexpr int BSIDE_THREADS = 512;
__device__ __forceinline__ uint32_t* b_parking(uint64_t* out, int qi) {
  return reinterpret_cast<uint32_t*>(out + (size_t)qi * 4 * N + 4 * N - 16);
}

__global__ void __launch_bounds__(BSIDE_THREADS) bside_kernel(const __grid_constant__ RespondArgs A) {
  extern __shared__ __align__(16) uint32_t sm[];  // [ELL][2][N] staged rows, then bpoly[32]
  const int qi = blockIdx.x;
  const uint32_t shard = A.shard[qi];
  if (shard >= (uint32_t)A.nshards) return;  // the Respond kernel reports it
  uint32_t* bpoly = sm + ELL * 2 * N;
  if (threadIdx.x < 32) bpoly[threadIdx.x] = 0;  // columns past gamma
  column_b0<BSIDE_THREADS>(A.P, A.H + (size_t)shard * A.P.gamma * N, A.brows + (size_t)qi * ELL * 2 * N, sm, bpoly);
  if (threadIdx.x < 32) b_parking(A.out, qi)[threadIdx.x] = bpoly[threadIdx.x];
}

// Shared-memory layout in u32 words (NR = residues of the a side).  With the
// 1 KiB every CTA reserves, the device-row variant (163 KiB) fills the SM's
// 164 KiB configuration and the serving variant (195 KiB) its 196 KiB one,
// so the SM keeps 92 or 60 KiB of L1, which holds the transforms' twiddle
// tables.  Each residue's b accumulator is the scratch of its group (r,2),
// which runs no transform during the recursion (words [0, N)); words
// N..N+15 of it keep the residue's b side (bpoly) until the outputs.
template <int NR, bool QDB>
struct Smem {
  static constexpr int AHAT = 0;                    // [ELL][NR][N] row transforms
  static constexpr int SC = AHAT + ELL * NR * N;    // [RG][NTT_SCRATCH] per-group exchange scratch
  static constexpr int T = SC + RG * NTT_SCRATCH;   // [2][N] R_{i+1} (slots) -> its inverse (coefficients) -> digits d0, d1
  static constexpr int PB1 = T + 2 * N;             // [2][N] NTT(d1) w'[i][1]
  static constexpr int SCAT = PB1 + 2 * N;          // [2 steps][2][N] query-only term of R_i (slots), then partial R_i
  // T..T+6N also hold the unseeded rows' a parts and SCAT+2N.. the
  // expansion's workspace ws[3][20] (device rows).  The serving variant
  // stages the query's raw b rows (u64, 12N words) from T on until the b
  // side, and keeps ws[3][20], the staged seeds (96 B) and the rows'
  // mbarrier in MISC, the words of SC past the expansion's candidates (6N
  // words), until the row transforms reuse them
  static constexpr int MISC = QDB ? SC + 6 * N : SCAT + 4 * N;
  static constexpr int TOTAL = QDB ? T + 12 * N : SCAT + 4 * N;
  static_assert(!QDB || MISC + 128 <= SC + 5 * NTT_SCRATCH + N, "MISC stays clear of the b side's words");
};

// Slots of the next step's query-only term computed by group (r,2) in [A];
// the rest follow in [C].
constexpr int SCATTER_SPLIT = N / 8;

// One query (index qi) by the whole CTA; every return is uniform over the CTA.
//
// The recursion step of packing_offline (inspiring2.rs:984-1008) with
// packing_online interleaved needs, per residue, sum_k NTT(d_k) w[i][k] for
// R_i and sum_k NTT(d_k) y[i][k] for b, over the three gadget digits d_k of
// INTT(R_{i+1}).  The key tables here have the third digit folded in
// (fold_third_digit_kernel, setup.cu): with keys k' the sums are
// k'0 NTT(d0) + k'1 NTT(d1) + k'2 R_{i+1}, so d2 is never formed and only two
// digit transforms run per residue and step.  Per step i (gamma-2 .. 0),
// residue r's three groups:
//  [A] (r,0)+(r,1) as one 256-thread team: inverse NTT of R_{i+1} (T[r]),
//      written back to T[r] once (r,2) has read it (named barrier 9 + r);
//      (r,2): SCAT[r] += R_{i+1} w'2 and the b accumulator += R_{i+1} y'2,
//      then the first part of the next step's query-only term R_{i-1}
//      (into the other SCAT buffer);
//  [B] all threads: CRT compose + digits d0, d1 into T;
//  [C] (r,0): NTT(d0); SCAT[r] += NTT(d0) w'0 (in place), the b
//      accumulator += NTT(d0) y'0;
//      (r,1): NTT(d1); PB1 = NTT(d1) w'1, NTT(d1) y'1 kept in registers;
//      (r,2): the rest of R_{i-1};
//  [D] (r,0): R_i = SCAT[r] + PB1 -> T[r] (slots) for the next step;
//      (r,1): the b accumulator += NTT(d1) y'1.
template <int MODE, bool SEEDED, bool QDB>
__device__ __forceinline__ void respond_one(const RespondArgs& A, const int qi) {
  constexpr int NR = MODE == MODE_COMPAT ? 1 : 2;
  using L = Smem<NR, QDB>;
  extern __shared__ __align__(16) uint32_t smem[];
  uint32_t* Ahat = smem + L::AHAT;
  uint32_t* SC = smem + L::SC;
  uint32_t* T = smem + L::T;
  uint32_t* PB1 = smem + L::PB1;
  uint32_t* SCAT = smem + L::SCAT;
  uint32_t* bpoly = QDB ? SC + 5 * NTT_SCRATCH + N : nullptr;  // serving: the b side, both residues, until the recursion
  int* wsb = reinterpret_cast<int*>(QDB ? smem + L::MISC + 32 : SCAT + 2 * N);

  const DevParams& P = A.P;
  const int tid = threadIdx.x, g = tid >> 7, x = tid & 127;
  const int r = g / 3, kd = g - 3 * r;  // residue, role of this group
  const int gamma = P.gamma;
  // QDB (serving loop): this query's fields come from its descriptor in
  // device memory, its rows and response from / to pinned host memory;
  // otherwise from the launch's arrays.  Descriptor fields are re-read where
  // used (reload_*) rather than held in registers.
  const QueryDesc* D = QDB ? A.qdesc + qi : nullptr;
  const uint32_t shard = QDB ? D->shard : A.shard[qi];
  const int32_t cid = QDB ? D->client : A.client[qi];
  const uint32_t* Ebase = QDB ? D->db.E : A.E;
  const uint16_t* Hbase = QDB ? D->db.H : A.H;
  const int nshards = QDB ? D->db.nshards : A.nshards;
  auto status_ptr = [&]() -> int32_t* {
    return QDB ? reload_ptr(&D->status) : A.status + qi;
  };
  if (shard >= (uint32_t)nshards || cid < 0 || cid >= A.nclients || A.yhat_table[cid] == nullptr) {
    if (tid == 0) *status_ptr() = ERR_INDEX;
    return;  // uniform over the CTA
  }
  const uint32_t* E = Ebase + (size_t)shard * 2 * ELL * gamma * N;
  const uint16_t* H = Hbase + (size_t)shard * gamma * N;
  // The client's key table: a body table (tag bit 0 set: NTT(y_body[k]),
  // ELL polys, 48 KiB) whose rotations are formed in registers, or the full
  // table of (gamma-1)*ELL rotated polys (explicit y_all).
  const uintptr_t ytag = reinterpret_cast<uintptr_t>(A.yhat_table[cid]);
  const bool ybody = (ytag & 1) != 0;
  const uint32_t* Y = reinterpret_cast<const uint32_t*>(ytag & ~(uintptr_t)1);
  const ResidueConsts& C = P.r[r];
  const uint32_t q = C.q, qinv = C.qinv, q2 = 2 * q;
  const uint64_t* brows = QDB ? D->brows : A.brows + (size_t)qi * ELL * 2 * N;

  // Serving loop (rows in host memory): the query's b rows (96 KiB) are
  // bulk-copied (TMA) into shared memory (T..T+12N) while the rows are
  // expanded, so the host link's latency stays off the critical path, and the
  // b side follows the row NTTs.  Rows in device memory: bside_kernel has
  // already computed the b side and parked it in the response slot; the
  // contracted shard and client keys are streamed into L2 from the start.
  uint64_t* raw = reinterpret_cast<uint64_t*>(T);                      // 16-byte aligned
  uint64_t* rbar = reinterpret_cast<uint64_t*>(smem + L::MISC + 120);  // the rows' mbarrier
  if (QDB && tid == 0) {
    mbar_init(rbar);
    wsb[18] = 0;  // set when the rows do not arrive
  }
  if (QDB && tid == 0) prefetch_l2(H, sizeof(uint16_t) * (size_t)gamma * N);
  // the seeds, inline in the query's descriptor: staged into shared memory
  // (ordered before the expansion by the barrier below)
  uint8_t* seed_sm = reinterpret_cast<uint8_t*>(smem + L::MISC + 96);
  if (QDB && tid < ELL * 32) seed_sm[tid] = D->seeds[tid];
  if (tid == 0) {
    // the contracted shard's blocks of the first three steps (the rest are
    // prefetched two steps ahead of their use in the recursion)
    const int i0 = gamma >= 3 ? gamma - 3 : 0;
    for (int rr = 0; rr < NR; rr++)
      prefetch_l2(E + ((size_t)rr * gamma + i0) * ELL * N, sizeof(uint32_t) * (size_t)(gamma - i0) * ELL * N);
    if (gamma > 1) prefetch_l2(Y, sizeof(uint32_t) * (size_t)(ybody ? 1 : gamma - 1) * ELL * 2 * N);
  }
  if (QDB) {
    __syncthreads();  // the mbarrier is initialised, the seeds staged
    if (tid == 0) {
      mbar_expect_tx(rbar, (uint32_t)(sizeof(uint64_t) * ELL * 2 * N));
#pragma unroll
      for (int p = 0; p < 2 * ELL; p++) bulk_g2s(raw + (size_t)p * N, brows + (size_t)p * N, sizeof(uint64_t) * N, rbar);
    }
  }

  // ---- rows ELL..2ELL-1: expand (one sub-block per row), forward NTT ----
  {
    const int t = tid >> 8, lt = tid & 255;
    uint64_t* cand = reinterpret_cast<uint64_t*>(SC) + t * N;  // 3 x 16 KiB within SC
    // serving loop: in place of the row's transforms (T..T+12N hold the
    // staged rows); otherwise within T..PB1
    uint32_t* a0 = QDB ? Ahat + t * NR * N : T + t * 2 * N;
    uint32_t* a1 = a0 + N;
    if (SEEDED) {
      const uint8_t* seed = QDB ? seed_sm + 32 * t : A.seeds + ((size_t)qi * ELL + t) * 32;
      const bool ok = expand_seeded_row<NR>(P, seed, cand, a0, a1, wsb + 20 * t, 7 + t, lt);
      if (lt == 0) wsb[20 * t + 17] = ok;
    } else {
      const uint64_t* ar = A.arows + ((size_t)qi * ELL + t) * 2 * N;
      for (int j = lt; j < NR * N; j += SUB) a0[j] = (uint32_t)ar[j];  // a1 follows a0
    }
  }
  if (QDB) {
    // rows that do not arrive within A.stage_wait_iters end the query with
    // a status, after a second bounded wait for the copies still in flight
    const bool arrived = mbar_wait(rbar, 0, A.stage_wait_iters);
    if (!arrived) wsb[18] = 1;
  }
  __syncthreads();
  const bool exp_ok = !SEEDED || (wsb[17] && wsb[37] && wsb[57]);
  if (QDB && wsb[18]) {
    // The CTA must not exit while its bulk copies can still write into its
    // shared memory (the next CTA on this SM would own it).  If even the
    // drain wait runs out, ERR_STAGE_LOST tells the host to drop every
    // result of this launch.
    const int lost = __syncthreads_or(!mbar_wait(rbar, 0, STAGE_DRAIN_ITERS));
    if (tid == 0) *status_ptr() = lost ? ERR_STAGE_LOST : ERR_STAGE;
    return;  // uniform over the CTA
  }
  if (QDB) {
    // the row transforms reuse the words of the workspace, seeds and mbarrier
    if (tid == 0) mbar_inval(rbar);
    __syncthreads();
  }
  // the query's status is written once, by one thread
  if (tid == 0) *status_ptr() = exp_ok ? 0 : ERR_EXPAND;
  if (r < NR) {  // group (r, t=kd) transforms row kd, residue r
    uint32_t v[16];
    const uint32_t* src = QDB ? Ahat + (kd * NR + r) * N : T + kd * 2 * N + r * N;
#pragma unroll
    for (int j = 0; j < 16; j++) v[j] = src[x + 128 * j];
    ntt_fwd(v, SC + g * NTT_SCRATCH, fwd_tw(C), q, x, 1 + g);
#pragma unroll
    for (int j = 0; j < 16; j++) v[j] = canon16(v[j], q);
    store16(Ahat + (kd * NR + r) * N, x, v);
  }
  __syncthreads();

  // ---- serving loop: b part of the column products (bp in SC, rows staged) ----
  if (QDB) column_b0<RBLOCK>(P, H, raw, SC, bpoly);

  // Eg: the scatter's residue of the contracted shard; with per-query
  // databases it is re-derived at each use from the query's view
  const uint32_t* Eg_fixed = QDB ? nullptr : E;
  auto Eg_at = [&](int sres) -> const uint32_t* {
    if (!QDB) return Eg_fixed + (size_t)sres * ELL * gamma * N;
    const uint32_t sh = *reinterpret_cast<const volatile uint32_t*>(&D->shard);
    return reload_ptr(&D->db.E) + ((size_t)sh * 2 * ELL + (size_t)sres * ELL) * gamma * N;
  };

  // ---- R_{gamma-1} into T, R_{gamma-2} into SCAT[(gamma-2) & 1], by all
  //      groups (fixed: each residue's 384 threads; compat: residue 0 by all) ----
  {
    const int sres = MODE == MODE_CRT_FIXED ? r : 0;
    const int sp = MODE == MODE_CRT_FIXED ? kd * NTT_GT + x : tid;
    const int snthr = MODE == MODE_CRT_FIXED ? 3 * NTT_GT : RBLOCK;
    const uint32_t sq = P.r[sres].q, sqinv = P.r[sres].qinv;
    const uint32_t* Ag = Ahat + sres * N;
    scatter_r(P, gamma - 1, Eg_at(sres), Ag, NR * N, T + sres * N, sp, snthr, sq, sqinv,
              MODE == MODE_COMPAT ? T + N : nullptr);
    if (gamma > 1) {
      uint32_t* sc2 = SCAT + ((gamma - 2) & 1) * 2 * N;
      scatter_r(P, gamma - 2, Eg_at(sres), Ag, NR * N, sc2 + sres * N, sp, snthr, sq, sqinv,
                MODE == MODE_COMPAT ? sc2 + N : nullptr);
    }
    for (int j = tid; j < 2 * N; j += RBLOCK) SC[(3 * (j >> LOGN) + 2) * NTT_SCRATCH + (j & (N - 1))] = 0;
    // the b side (serving: computed above; device rows: parked by
    // bside_kernel), residue r's beside its accumulator
    if (tid < 32) {
      const uint32_t bv = QDB ? bpoly[tid] : b_parking(A.out, qi)[tid];
      __syncwarp();
      SC[(3 * (tid >> 4) + 2) * NTT_SCRATCH + N + (tid & 15)] = bv;
    }
  }
  __syncthreads();

  const int team_t = tid - 384 * r;  // thread of residue r's (r,0)+(r,1) team, valid for kd < 2
  uint32_t* team_sc = SC + 3 * r * NTT_SCRATCH;  // the team's exchange scratch (two groups' worth)
  // the next step's query-only term by the (r,2) groups, in two parts ([A] and [C])
  auto scatter_next = [&](int i, int u0, int u1) {
    const int sres = MODE == MODE_CRT_FIXED ? r : 0;
    const int sp = MODE == MODE_CRT_FIXED ? x : r * NTT_GT + x;
    const int snthr = MODE == MODE_CRT_FIXED ? NTT_GT : 2 * NTT_GT;
    uint32_t* sc2 = SCAT + ((i - 1) & 1) * 2 * N;
    scatter_r(P, i - 1, Eg_at(sres), Ahat + sres * N, NR * N, sc2 + sres * N, sp, snthr, P.r[sres].q, P.r[sres].qinv,
              MODE == MODE_COMPAT ? sc2 + N : nullptr, u0, u1);
  };
  const int f = (x >> 1) & 3;  // chunk swizzle of this thread's 16-slot run (store16 / load16)
  for (int i = gamma - 2; i >= 0; i--) {
    const size_t yoff = ybody ? (size_t)i * ELL * 2 * N : 0;  // body tables: the key slices of i = 0, rotated
    if (tid == 0 && i >= 2)  // the block the next step's scatter reads (R_{i-2})
      for (int rr = 0; rr < NR; rr++) prefetch_l2(Eg_at(rr) + (size_t)(i - 2) * ELL * N, sizeof(uint32_t) * ELL * N);
    // [A] inverse NTT of R_{i+1} by residue r's team; the products of
    //     R_{i+1} with the third key slices by group (r,2)
    if (kd < 2) {
      uint32_t v[8];
      const int s0 = 8 * team_t;
      const uint4 lo = *reinterpret_cast<const uint4*>(T + r * N + swz(s0));
      const uint4 hi = *reinterpret_cast<const uint4*>(T + r * N + swz(s0 + 4));
      v[0] = lo.x; v[1] = lo.y; v[2] = lo.z; v[3] = lo.w;
      v[4] = hi.x; v[5] = hi.y; v[6] = hi.z; v[7] = hi.w;
      ntt_inv_noscale8(v, team_sc, inv_tw(C), q, team_t, 7 + r);
      named_sync(9 + r, 3 * NTT_GT);  // group (r,2) has read R_{i+1}
#pragma unroll
      for (int j = 0; j < 8; j++) T[r * N + team_t + 256 * j] = canon2(v[j], q);
    } else {
      uint32_t rs[16];
      load16(T + r * N, x, rs);
      named_arrive(9 + r, 3 * NTT_GT);
      const size_t off2 = ((size_t)(i * ELL + 2) * 2 + r) * N + 16 * x;
      uint4 wv[4], yv[4];
      key_run(A.what + off2, wv);
      key_run(Y + off2 - yoff, yv);
      if (ybody) rotate_key_run(yv, i, x);
      uint32_t* accb = SC + g * NTT_SCRATCH;  // the residue's b accumulator
      uint32_t* part = SCAT + (i & 1) * 2 * N + r * N;
#pragma unroll
      for (int r4 = 0; r4 < 4; r4++) {
        const int o = 16 * x + 4 * (r4 ^ f);
        uint4* ap = reinterpret_cast<uint4*>(accb + o);
        uint4* hp = reinterpret_cast<uint4*>(part + o);
        const uint4 a4 = *ap, h4 = *hp;
        uint32_t ab[4], pr[4];
#pragma unroll
        for (int e = 0; e < 4; e++) {
          const int j = 4 * r4 + e;
          ab[e] = acc_2q(u4e(a4, e), redc_lazy((uint64_t)rs[j] * u4e(yv[r4], e), q, qinv), q2);
          pr[e] = u4e(h4, e) + redc_lazy((uint64_t)rs[j] * u4e(wv[r4], e), q, qinv);  // [0, 3q)
        }
        *ap = make_uint4(ab[0], ab[1], ab[2], ab[3]);
        *hp = make_uint4(pr[0], pr[1], pr[2], pr[3]);
      }
      if (i >= 1) scatter_next(i, 0, SCATTER_SPLIT);
    }
    __syncthreads();
    // [B] gadget_decompose of the composite coefficients (rgsw/external_product.rs:16-37):
    //     digits 0 and 1 (the third is folded into the keys)
    for (int j = tid; j < N; j += RBLOCK) {
      const uint64_t c = crt_compose(P, T[j], T[N + j]);
      T[j] = (uint32_t)c & 0xFFFFFu;
      T[N + j] = (uint32_t)(c >> 20) & 0xFFFFFu;
    }
    __syncthreads();
    // [C]
    uint32_t* accb = SC + (3 * r + 2) * NTT_SCRATCH;  // the residue's b accumulator
    uint32_t py[16];  // group (r,1): NTT(d1) y'1, added to the b accumulator in [D]
    if (kd < 2) {
      const size_t off = ((size_t)(i * ELL + kd) * 2 + r) * N + 16 * x;
      uint4 wv[4], yv[4];
      key_run(A.what + off, wv);  // this step's key slices, fetched before the transform
      key_run(Y + off - yoff, yv);
      uint32_t v[16];
#pragma unroll
      for (int j = 0; j < 16; j++) v[j] = T[kd * N + x + 128 * j];
      ntt_fwd(v, SC + g * NTT_SCRATCH, fwd_tw(C), q, x, 1 + g);  // slots 16x.., [0, 14q)
      if (ybody) rotate_key_run(yv, i, x);
      // group (r,0): the b accumulator and the partial R_i in place of the
      // query-only term; group (r,1): PB1
      uint32_t* pdst = kd == 0 ? SCAT + (i & 1) * 2 * N + r * N : PB1 + r * N;
#pragma unroll
      for (int r4 = 0; r4 < 4; r4++) {
        const int o = 16 * x + 4 * (r4 ^ f);
        uint4* hp = reinterpret_cast<uint4*>(pdst + o);
        const uint4 h4 = kd == 0 ? *hp : make_uint4(0, 0, 0, 0);
        uint32_t pr[4];
#pragma unroll
        for (int e = 0; e < 4; e++)
          pr[e] = redc_lazy((uint64_t)v[4 * r4 + e] * u4e(wv[r4], e), q, qinv) + u4e(h4, e);  // [0, 5q)
        *hp = make_uint4(pr[0], pr[1], pr[2], pr[3]);
#pragma unroll
        for (int e = 0; e < 4; e++) py[4 * r4 + e] = redc_lazy((uint64_t)v[4 * r4 + e] * u4e(yv[r4], e), q, qinv);
        if (kd == 0) {
          uint4* ap = reinterpret_cast<uint4*>(accb + o);
          const uint4 a4 = *ap;
          *ap = make_uint4(acc_2q(a4.x, py[4 * r4], q2), acc_2q(a4.y, py[4 * r4 + 1], q2),
                           acc_2q(a4.z, py[4 * r4 + 2], q2), acc_2q(a4.w, py[4 * r4 + 3], q2));
        }
      }
    } else if (i >= 1) {
      scatter_next(i, SCATTER_SPLIT, N);
    }
    __syncthreads();
    // [D] R_i (group (r,0)); b += NTT(d1) y'1 (group (r,1))
    if (kd == 1) {
#pragma unroll
      for (int r4 = 0; r4 < 4; r4++) {
        uint4* ap = reinterpret_cast<uint4*>(accb + 16 * x + 4 * (r4 ^ f));
        const uint4 a4 = *ap;
        *ap = make_uint4(acc_2q(a4.x, py[4 * r4], q2), acc_2q(a4.y, py[4 * r4 + 1], q2),
                         acc_2q(a4.z, py[4 * r4 + 2], q2), acc_2q(a4.w, py[4 * r4 + 3], q2));
      }
    } else if (kd == 0) {
#pragma unroll
      for (int r4 = 0; r4 < 4; r4++) {
        const int o = r * N + 16 * x + 4 * (r4 ^ f);
        const uint4 pa = *reinterpret_cast<const uint4*>(SCAT + (i & 1) * 2 * N + o);
        const uint4 p1 = *reinterpret_cast<const uint4*>(PB1 + o);
        uint32_t outv[4];
#pragma unroll
        for (int e = 0; e < 4; e++) {
          uint32_t sum = u4e(pa, e) + u4e(p1, e);  // < 7q < 2^31
          sum = min(sum, sum - 4 * q);
          sum = min(sum, sum - 2 * q);
          outv[e] = min(sum, sum - q);
        }
        *reinterpret_cast<uint4*>(T + o) = make_uint4(outv[0], outv[1], outv[2], outv[3]);  // R_i for the next step
      }
    }
    __syncthreads();
  }

  // ---- outputs: a_hat = INTT(R_0) (inspiring2.rs:1027-1029) by each
  //      residue's team, b = b_poly + INTT(sum y_all * bold_t)
  //      (inspiring2.rs:1217-1221) by group (r,2) ----
  uint64_t* out = QDB ? reload_ptr(&D->out) : A.out + (size_t)qi * 4 * N;
  if (kd < 2) {
    uint32_t v[8];
    const int s0 = 8 * team_t;
    const uint4 lo = *reinterpret_cast<const uint4*>(T + r * N + swz(s0));
    const uint4 hi = *reinterpret_cast<const uint4*>(T + r * N + swz(s0 + 4));
    v[0] = lo.x; v[1] = lo.y; v[2] = lo.z; v[3] = lo.w;
    v[4] = hi.x; v[5] = hi.y; v[6] = hi.z; v[7] = hi.w;
    ntt_inv_noscale8(v, team_sc, inv_tw(C), q, team_t, 7 + r);
#pragma unroll
    for (int j = 0; j < 8; j++) out[r * N + team_t + 256 * j] = canon2(v[j], q);
  } else {
    uint32_t b0[16];
    load16(SC + g * NTT_SCRATCH, x, b0);  // the b accumulator, [0, 2q)
    const uint32_t bp = x < gamma ? SC[g * NTT_SCRATCH + N + x] : 0;
    ntt_inv_noscale(b0, SC + g * NTT_SCRATCH, inv_tw(C), q, x, 1 + g);  // first exchange after a group barrier
#pragma unroll
    for (int j = 0; j < 16; j++) b0[j] = canon2(b0[j], q);
    if (x < gamma) b0[0] = add_mod(b0[0], bp, q);
#pragma unroll
    for (int j = 0; j < 16; j++) out[2 * N + r * N + x + 128 * j] = b0[j];
  }
}

// One query per CTA.
template <int MODE, bool SEEDED, bool QDB>
__global__ void __launch_bounds__(RBLOCK, 1) respond_kernel(const __grid_constant__ RespondArgs A) {
  respond_one<MODE, SEEDED, QDB>(A, blockIdx.x);
}

// Capped grid (device-resident rows): CTA b answers queries b, b + gridDim.x,
// ... in turn, so a grid of one CTA per SM keeps every SM busy to the end of
// a large batch.
template <int MODE, bool SEEDED>
__global__ void __launch_bounds__(RBLOCK, 1) respond_kernel_loop(const __grid_constant__ RespondArgs A) {
  for (int qi = blockIdx.x; qi < A.nq; qi += gridDim.x) {
    if (qi != (int)blockIdx.x) __syncthreads();  // the previous query's shared memory is no longer read
    respond_one<MODE, SEEDED, false>(A, qi);
  }
}

}  // namespace

size_t respond_smem_bytes(int mode, bool qdb) {
  const int words = mode == MODE_COMPAT ? (qdb ? Smem<1, true>::TOTAL : Smem<1, false>::TOTAL)
                                        : (qdb ? Smem<2, true>::TOTAL : Smem<2, false>::TOTAL);
  return sizeof(uint32_t) * words;
}

template <int MODE, bool SEEDED, bool QDB>
static cudaError_t set_smem_attr() {
  cudaError_t e = cudaFuncSetAttribute(respond_kernel<MODE, SEEDED, QDB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)respond_smem_bytes(MODE, QDB));
  if (e == cudaSuccess && !QDB)
    e = cudaFuncSetAttribute(respond_kernel_loop<MODE, SEEDED>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)respond_smem_bytes(MODE, false));
  return e;
}

// Launches issue no configuration call (so they can be captured in a CUDA
// graph): the shared-memory attribute of every variant is set once per
// device by prepare_respond_kernels.
size_t bside_smem_bytes() { return sizeof(uint32_t) * ((size_t)ELL * 2 * N + 32); }

template <int MODE, bool SEEDED, bool QDB>
static cudaError_t launch_one(const RespondArgs& a, int ctas, cudaStream_t st) {
  if (!QDB) {
    bside_kernel<<<a.nq, BSIDE_THREADS, bside_smem_bytes(), st>>>(a);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  if (!QDB && ctas < a.nq)
    respond_kernel_loop<MODE, SEEDED><<<ctas, RBLOCK, respond_smem_bytes(MODE, false), st>>>(a);
  else
    respond_kernel<MODE, SEEDED, QDB><<<a.nq, RBLOCK, respond_smem_bytes(MODE, QDB), st>>>(a);
  return cudaGetLastError();
}

cudaError_t prepare_respond_kernels() {
  const cudaError_t es[] = {
      set_smem_attr<MODE_COMPAT, false, false>(),    set_smem_attr<MODE_COMPAT, true, false>(),
      set_smem_attr<MODE_COMPAT, false, true>(),     set_smem_attr<MODE_COMPAT, true, true>(),
      set_smem_attr<MODE_CRT_FIXED, false, false>(), set_smem_attr<MODE_CRT_FIXED, true, false>(),
      set_smem_attr<MODE_CRT_FIXED, false, true>(),  set_smem_attr<MODE_CRT_FIXED, true, true>()};
  for (cudaError_t e : es)
    if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(bside_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bside_smem_bytes());
}

template <int MODE>
static cudaError_t launch_mode(const RespondArgs& a, bool seeded, int ctas, cudaStream_t st) {
  if (a.qdesc) return seeded ? launch_one<MODE, true, true>(a, ctas, st) : launch_one<MODE, false, true>(a, ctas, st);
  return seeded ? launch_one<MODE, true, false>(a, ctas, st) : launch_one<MODE, false, false>(a, ctas, st);
}

cudaError_t launch_respond(const RespondArgs& a, bool seeded, cudaStream_t st, int max_ctas, int pair_max) {
  if (a.nq <= 0) return cudaSuccess;
  if (max_ctas <= 0 && a.nq <= pair_max) return launch_respond_pair(a, seeded, st);
  const int ctas = (max_ctas > 0 && max_ctas < a.nq) ? max_ctas : a.nq;
  return a.P.mode == MODE_COMPAT ? launch_mode<MODE_COMPAT>(a, seeded, ctas, st)
                                 : launch_mode<MODE_CRT_FIXED>(a, seeded, ctas, st);
}

}  // namespace ig
