// respond_pair.cu -- the Respond kernel for small batches: a cluster of two
// CTAs per query, CTA r computing CRT residue r.
//
// It returns exactly what respond.cu's one-CTA kernel returns (the packed
// ciphertext of respond_seeded_inspiring / respond_inspiring,
// src/pir/respond.rs:284-398, through packing_online,
// src/inspiring/inspiring2.rs:1185-1222), from the same regrouped dataflow;
// only the placement differs.  Of the recursion step (inspiring2.rs:984-1008)
// only the gadget decomposition needs both residues: it reads the composite
// coefficient of INTT(R_{i+1}).  Everything else -- the row transforms, the
// query-only terms R_i, the digit transforms and key products, the b side --
// is per residue.  So each CTA runs one residue's chain on its own SM and
// the two exchange the 2048 coefficients of INTT(R_{i+1}) once per step
// through distributed shared memory.  A lone query then uses two SMs, and
// each step's transforms share their SM with half the work of the one-CTA
// kernel; large batches keep the one-CTA kernel, which needs fewer SMs per
// query.
//
// Per CTA (768 threads, six groups of 128), per step i (gamma-2 .. 0),
// p = i & 1:
//  [A] groups 0-1 (a 256-thread team): INTT(R_{i+1}) -> TC[p][r] here and in
//      the peer CTA; groups 2-5: first half of the query-only term R_{i-1};
//      cluster barrier (the peer's residue has arrived);
//  [B] all: digits d0, d1 of the composite coefficients, in place in TC[p];
//  [C] group 0: NTT(d0); partial R_i = query-only term + NTT(d0) w'0,
//      b += NTT(d0) y'0; group 1: NTT(d1); PB1 = NTT(d1) w'1, b += NTT(d1)
//      y'1; group 2: PB2 = R_{i+1} w'[i][2]; group 3: b += R_{i+1} y'[i][2];
//      then (groups 0-3 meet) group 0 sums R_i = partial + PB1 + PB2 into
//      RN; groups 4-5: second half of R_{i-1}, and the b side (coefficient 0
//      of the column products) of one column, two in the last step.
// TC is double-buffered by step parity: the peer writes TC[p] again only in
// step i - 2, after the cluster barrier of step i - 1, which this CTA reaches
// only after its last read of TC[p].  The only other remote writes are the
// expansion hand-off (residue 1's stream position) and the status flags, each
// followed by a cluster barrier; after the last step's barrier nothing
// touches the peer's shared memory, so either CTA may exit.
#include "expand.cuh"
#include "kernels.h"
#include "respond_common.cuh"

namespace ig {

namespace {

__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}

// Address of this CTA's shared variable `p` in CTA `rank` of the cluster.
__device__ __forceinline__ uint32_t peer_smem(const void* p, uint32_t rank) {
  uint32_t a;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(a) : "r"(smem_u32(p)), "r"(rank));
  return a;
}

__device__ __forceinline__ void st_peer(uint32_t addr, uint32_t v) {
  asm volatile("st.shared::cluster.u32 [%0], %1;" ::"r"(addr), "r"(v) : "memory");
}

__device__ __forceinline__ void cluster_arrive_relaxed() {
  asm volatile("barrier.cluster.arrive.relaxed;" ::: "memory");
}
__device__ __forceinline__ void cluster_wait() { asm volatile("barrier.cluster.wait.acquire;" ::: "memory"); }

// Every thread of both CTAs: this CTA's earlier writes (local and remote)
// are visible to the peer and the peer's to this CTA afterwards.
__device__ __forceinline__ void cluster_sync_all() {
  asm volatile("barrier.cluster.arrive.release;\n\tbarrier.cluster.wait.acquire;" ::: "memory");
}

// Shared-memory layout in u32 words.
struct PairSmem {
  static constexpr int AH = 0;                       // [ELL][N] row transforms (this CTA's a-side residue)
  static constexpr int SC = AH + ELL * N;            // [3][NTT_SCRATCH] exchange scratch (groups 0-2)
  static constexpr int W = SC + 3 * NTT_SCRATCH;     // working region
  static constexpr int TC = W;                       // [2 parity][2 residues][N] INTT(R_{i+1}) -> digits d0, d1
  static constexpr int RN = TC + 4 * N;              // [N] R_{i+1} (slots) -> R_i
  static constexpr int PB1 = RN + N;                 // [N] NTT(d1) w'1
  static constexpr int PB2 = PB1 + N;                // [N] R_{i+1} w'2
  static constexpr int SCAT = PB2 + N;               // [2 parity][N] query-only term of R_i, then partial R_i
  static constexpr int ACC = SCAT + 2 * N;           // [3][N] b accumulators (one per digit product)
  // until the row transforms: this residue's b rows (u64 [ELL][N]) at W and
  // the expansion's candidates (u64 [3][8 * SUB]) after them
  static constexpr int ROWS = W;
  static constexpr int CAND = W + 2 * ELL * N;
  static constexpr int BP = ACC + 3 * N;             // [ELL][N] negacyclic reversal of the b rows (b side)
  static constexpr int MISC = BP + ELL * N;
  // MISC words: [0, 32) b0 sums per column (u64); [32, 92) scan scratch of
  // the three sub-blocks (20 each, [17] = expansion ok); [96, 120) staged
  // seeds; [120, 123) residue 1's stream positions; [124, 126) flags by CTA
  // rank; [126, 128) drain results by rank; [128] rows-missing flag;
  // [132, 134) the rows' mbarrier
  static constexpr int TOTAL = MISC + 160;
};
static_assert(PairSmem::CAND + 2 * 3 * 8 * SUB <= PairSmem::BP, "candidates fit the working region");
static_assert(PairSmem::W % 4 == 0 && PairSmem::CAND % 4 == 0 && PairSmem::BP % 4 == 0 && PairSmem::MISC % 4 == 0,
              "16-byte alignment");

// The b side of the column products, coefficient 0 only (rlwe/enc.rs:195-208;
// see respond.cu): b0_c = sum_t sum_i d_{c,t}[i] b'_t[i], d the base-2^20
// digits of Delta * h_c and b'_t the negacyclic reversal of row ELL+t's b
// (BP).  Spread over the recursion steps: thread t of 512 adds coefficient
// pairs t and t + 512 of one column (its two words of the raw column in h0,
// h1) and each warp adds its sum to the column's 64-bit total (< 2^61).
__device__ __forceinline__ void column_b0_part(const DevParams& P, uint32_t h0, uint32_t h1, const uint32_t* BP,
                                               int t, unsigned long long* total) {
  const uint2* b2 = reinterpret_cast<const uint2*>(BP);
  uint64_t acc = 0;
#pragma unroll
  for (int jj = 0; jj < 2; jj++) {
    const int j = t + 512 * jj;  // coefficients 2j, 2j + 1
    const uint32_t hw = jj ? h1 : h0;
    const uint2 b0 = b2[j], b1 = b2[N / 2 + j], bb2 = b2[N + j];
#pragma unroll
    for (int e = 0; e < 2; e++) {
      const uint64_t xv = P.delta * (uint64_t)((hw >> (16 * e)) & 0xFFFFu);
      const uint32_t d0 = (uint32_t)xv & 0xFFFFFu, d1 = (uint32_t)(xv >> 20) & 0xFFFFFu, d2 = (uint32_t)(xv >> 40);
      acc += (uint64_t)d0 * (e ? b0.y : b0.x) + (uint64_t)d1 * (e ? b1.y : b1.x) + (uint64_t)d2 * (e ? bb2.y : bb2.x);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((t & 31) == 0) atomicAdd(total, (unsigned long long)acc);
}

template <int MODE, bool SEEDED, bool QDB>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(RBLOCK, 1)
    respond_pair_kernel(const __grid_constant__ RespondArgs A) {
  using L = PairSmem;
  extern __shared__ __align__(16) uint32_t smem[];
  const uint32_t r = cluster_rank(), peer = r ^ 1u;  // this CTA's residue
  const int qi = blockIdx.x >> 1;
  const DevParams& P = A.P;
  const int tid = threadIdx.x, g = tid >> 7, x = tid & 127;
  const int gamma = P.gamma;
  int* misc = reinterpret_cast<int*>(smem + L::MISC);
  unsigned long long* b0sum = reinterpret_cast<unsigned long long*>(smem + L::MISC);

  const QueryDesc* D = QDB ? A.qdesc + qi : nullptr;
  const uint32_t shard = QDB ? D->shard : A.shard[qi];
  const int32_t cid = QDB ? D->client : A.client[qi];
  const int nshards = QDB ? D->db.nshards : A.nshards;
  auto status_ptr = [&]() -> int32_t* { return QDB ? reload_ptr(&D->status) : A.status + qi; };
  // both CTAs read the same fields: every return here is uniform over the cluster
  if (shard >= (uint32_t)nshards || cid < 0 || cid >= A.nclients || A.yhat_table[cid] == nullptr) {
    if (r == 0 && tid == 0) *status_ptr() = ERR_INDEX;
    return;
  }
  // the peer's shared memory may be written only once it has started
  cluster_arrive_relaxed();

  // residue of the a side and the query-only terms: this CTA's, or residue 0
  // for both CTAs in compat mode (residue 1 is then rebuilt from it)
  const int sres = MODE == MODE_CRT_FIXED ? (int)r : 0;
  const bool conv1 = MODE == MODE_COMPAT && r == 1;
  const uint16_t* H = (QDB ? D->db.H : A.H) + (size_t)shard * gamma * N;
  const uintptr_t ytag = reinterpret_cast<uintptr_t>(A.yhat_table[cid]);
  const bool ybody = (ytag & 1) != 0;
  const uint32_t* Y = reinterpret_cast<const uint32_t*>(ytag & ~(uintptr_t)1);
  const ResidueConsts& C = P.r[r];
  const uint32_t q = C.q, qinv = C.qinv, q2 = 2 * q;
  const uint64_t* brows = QDB ? D->brows : A.brows + (size_t)qi * ELL * 2 * N;
  auto Eg_at = [&]() -> const uint32_t* {
    if (!QDB) return A.E + ((size_t)shard * 2 * ELL + (size_t)sres * ELL) * gamma * N;
    const uint32_t sh = *reinterpret_cast<const volatile uint32_t*>(&D->shard);
    return reload_ptr(&D->db.E) + ((size_t)sh * 2 * ELL + (size_t)sres * ELL) * gamma * N;
  };

  uint32_t* AH = smem + L::AH;
  uint32_t* SC = smem + L::SC;
  uint32_t* RN = smem + L::RN;
  uint32_t* PB1 = smem + L::PB1;
  uint32_t* PB2 = smem + L::PB2;
  uint32_t* SCAT = smem + L::SCAT;
  uint32_t* ACC = smem + L::ACC;
  uint64_t* rows = reinterpret_cast<uint64_t*>(smem + L::ROWS);
  uint32_t* BP = smem + L::BP;
  uint64_t* rbar = reinterpret_cast<uint64_t*>(smem + L::MISC + 132);
  uint8_t* seed_sm = reinterpret_cast<uint8_t*>(smem + L::MISC + 96);
  if (tid == 0) {
    mbar_init(rbar);
    misc[128] = 0;
    prefetch_l2(H, sizeof(uint16_t) * (size_t)gamma * N);
    // the contracted shard's blocks of the first three steps (the rest are
    // prefetched two steps ahead of their use in the recursion)
    const int i0 = gamma >= 3 ? gamma - 3 : 0;
    prefetch_l2(Eg_at() + (size_t)i0 * ELL * N, sizeof(uint32_t) * (size_t)(gamma - i0) * ELL * N);
    if (gamma > 1) prefetch_l2(Y, sizeof(uint32_t) * (size_t)(ybody ? 1 : gamma - 1) * ELL * 2 * N);
  }
  if (tid < MAX_GAMMA) b0sum[tid] = 0;
  if (QDB && tid < ELL * 32) seed_sm[tid] = D->seeds[tid];
  __syncthreads();  // the mbarrier is initialised, the seeds staged
  if (tid == 0) {
    // this residue's b rows (48 KiB) while the rows are expanded
    mbar_expect_tx(rbar, (uint32_t)(sizeof(uint64_t) * ELL * N));
#pragma unroll
    for (int t = 0; t < ELL; t++)
      bulk_g2s(rows + (size_t)t * N, brows + (size_t)(2 * t + r) * N, sizeof(uint64_t) * N, rbar);
  }

  // ---- rows ELL..2ELL-1, residue sres: expand (one sub-block per row) ----
  bool started = false;  // the start barrier has been waited for
  {
    const int t = tid >> 8, lt = tid & 255;
    uint64_t* cand = reinterpret_cast<uint64_t*>(smem + L::CAND) + (size_t)t * 8 * SUB;
    uint32_t* dst = AH + t * N;
    int* ws = misc + 32 + 20 * t;
    if (SEEDED) {
      const uint8_t* seed = QDB ? seed_sm + 32 * t : A.seeds + ((size_t)qi * ELL + t) * 32;
      uint32_t key[8];
#pragma unroll
      for (int k = 0; k < 8; k++)
        key[k] = (uint32_t)seed[4 * k] | ((uint32_t)seed[4 * k + 1] << 8) | ((uint32_t)seed[4 * k + 2] << 16) |
                 ((uint32_t)seed[4 * k + 3] << 24);
      long long end;
      if (MODE == MODE_CRT_FIXED && r == 1) {
        // residue 1 starts after residue 0's last accepted draw, which CTA 0
        // finds: the first N candidates after residue 0's minimum are drawn
        // meanwhile, and its position arrives through the hand-off barrier
        end = expand_residue(
            P, key, 1, 0, (uint64_t)N / 8,
            [&]() -> uint64_t {
              cluster_wait();
              cluster_sync_all();
              return (uint32_t)misc[120 + t];
            },
            cand, dst, ws, 5 + t, lt);
        started = true;
      } else {
        end = expand_residue(P, key, sres, 0, 0, []() -> uint64_t { return 0; }, cand, dst, ws, 5 + t, lt);
        if (MODE == MODE_CRT_FIXED) {
          cluster_wait();
          started = true;
          if (lt == 0) st_peer(peer_smem(misc + 120 + t, peer), end < 0 ? 0xFFFFFFFFu : (uint32_t)end);
          cluster_sync_all();
        }
      }
      if (lt == 0) ws[17] = end >= 0;
    } else {
      const uint64_t* ar = A.arows + ((size_t)qi * ELL + t) * 2 * N + (size_t)sres * N;
      for (int j = lt; j < N; j += SUB) dst[j] = (uint32_t)ar[j];
    }
  }
  if (!started) cluster_wait();

  // ---- the rows' arrival and the expansion, agreed over the cluster ----
  if (!mbar_wait(rbar, 0, QDB ? A.stage_wait_iters : STAGE_WAIT_ITERS_DEFAULT)) misc[128] = 1;
  __syncthreads();
  if (tid == 0) {
    const int fl = (misc[128] ? 1 : 0) | ((SEEDED && !(misc[32 + 17] && misc[52 + 17] && misc[72 + 17])) ? 2 : 0);
    misc[124 + r] = fl;
    st_peer(peer_smem(misc + 124 + r, peer), (uint32_t)fl);
  }
  cluster_sync_all();
  const int flags = misc[124] | misc[125];
  if (flags & 1) {
    // As in the one-CTA kernel: no CTA exits while its own bulk copies can
    // still land; the drain results are agreed before the status is written.
    const int lost = __syncthreads_or(!mbar_wait(rbar, 0, STAGE_DRAIN_ITERS));
    if (tid == 0) {
      misc[126 + r] = lost;
      st_peer(peer_smem(misc + 126 + r, peer), (uint32_t)lost);
    }
    cluster_sync_all();
    if (r == 0 && tid == 0) *status_ptr() = (misc[126] | misc[127]) ? ERR_STAGE_LOST : ERR_STAGE;
    return;  // uniform over the cluster
  }
  if (r == 0 && tid == 0) *status_ptr() = (flags & 2) ? ERR_EXPAND : 0;

  // ---- row transforms (groups 0-2, one row each); groups 3-5: the b rows'
  //      negacyclic reversal for the b side ----
  if (g < ELL) {
    const ResidueConsts& Cs = P.r[sres];
    uint32_t v[16];
#pragma unroll
    for (int j = 0; j < 16; j++) v[j] = AH[g * N + x + 128 * j];
    ntt_fwd(v, SC + g * NTT_SCRATCH, fwd_tw(Cs), Cs.q, x, 2 + g);
#pragma unroll
    for (int j = 0; j < 16; j++) v[j] = canon16(v[j], Cs.q);
    store16(AH + g * N, x, v);
  } else {
#pragma unroll 4
    for (int idx = tid - ELL * NTT_GT; idx < ELL * N; idx += ELL * NTT_GT) {
      const int i = idx & (N - 1), t = idx >> LOGN;
      uint32_t v = (uint32_t)rows[(size_t)t * N + (i == 0 ? 0 : N - i)];
      if (i != 0 && v != 0) v = q - v;
      BP[idx] = v;
    }
  }
  __syncthreads();

  // ---- R_{gamma-1} into RN, R_{gamma-2} into SCAT[(gamma-2) & 1]; b accumulators zeroed ----
  const uint32_t sq = P.r[sres].q, sqinv = P.r[sres].qinv;
  scatter_r(P, gamma - 1, Eg_at(), AH, N, conv1 ? nullptr : RN, tid, RBLOCK, sq, sqinv, conv1 ? RN : nullptr);
  if (gamma > 1) {
    uint32_t* s2 = SCAT + ((gamma - 2) & 1) * N;
    scatter_r(P, gamma - 2, Eg_at(), AH, N, conv1 ? nullptr : s2, tid, RBLOCK, sq, sqinv, conv1 ? s2 : nullptr);
  }
  for (int j = tid; j < 3 * N; j += RBLOCK) ACC[j] = 0;
  if (gamma == 1 && tid >= 2 * NTT_GT) {  // no recursion step: the one column's b side here
    const uint32_t* h2 = reinterpret_cast<const uint32_t*>(H);
    const int t = tid - 2 * NTT_GT;
    column_b0_part(P, __ldg(h2 + t), __ldg(h2 + t + 512), BP, t, b0sum);
  }
  __syncthreads();

  // the next step's query-only term R_{i-1}, slots [u0, u1) by threads p of nthr
  auto scatter_next = [&](int i, int p, int nthr, int u0, int u1) {
    uint32_t* s2 = SCAT + ((i - 1) & 1) * N;
    scatter_r(P, i - 1, Eg_at(), AH, N, conv1 ? nullptr : s2, p, nthr, sq, sqinv, conv1 ? s2 : nullptr, u0, u1);
  };
  const uint32_t tc_peer = peer_smem(smem + L::TC, peer);
  const int f = (x >> 1) & 3;  // chunk swizzle of this thread's 16-slot run (store16 / load16)
  for (int i = gamma - 2; i >= 0; i--) {
    const int p = i & 1;
    uint32_t* TC = smem + L::TC + p * 2 * N;
    const size_t yoff = ybody ? (size_t)i * ELL * 2 * N : 0;  // body tables: the key slices of i = 0, rotated
    if (tid == 0 && i >= 2) prefetch_l2(Eg_at() + (size_t)(i - 2) * ELL * N, sizeof(uint32_t) * ELL * N);
    // [A]
    if (tid < 2 * NTT_GT) {
      uint32_t v[8];
      const int s0 = 8 * tid;
      const uint4 lo = *reinterpret_cast<const uint4*>(RN + swz(s0));
      const uint4 hi = *reinterpret_cast<const uint4*>(RN + swz(s0 + 4));
      v[0] = lo.x; v[1] = lo.y; v[2] = lo.z; v[3] = lo.w;
      v[4] = hi.x; v[5] = hi.y; v[6] = hi.z; v[7] = hi.w;
      ntt_inv_noscale8(v, SC, inv_tw(C), q, tid, 1);
      const uint32_t rbase = tc_peer + 4u * (uint32_t)(p * 2 * N + r * N + tid);
#pragma unroll
      for (int j = 0; j < 8; j++) {
        const uint32_t c = canon2(v[j], q);
        TC[r * N + tid + 256 * j] = c;
        st_peer(rbase + 4u * 256u * (uint32_t)j, c);
      }
    } else if (i >= 1) {
      scatter_next(i, tid - 2 * NTT_GT, 4 * NTT_GT, 0, N / 2);  // groups 2-5
    }
    cluster_sync_all();
    // [B] gadget_decompose of the composite coefficients (rgsw/external_product.rs:16-37):
    //     digits 0 and 1 (the third is folded into the keys)
    for (int j = tid; j < N; j += RBLOCK) {
      const uint64_t c = crt_compose(P, TC[j], TC[N + j]);
      TC[j] = (uint32_t)c & 0xFFFFFu;
      TC[N + j] = (uint32_t)(c >> 20) & 0xFFFFFu;
    }
    __syncthreads();
    // [C]
    if (g < 2) {
      const int kd = g;
      const size_t off = ((size_t)(i * ELL + kd) * 2 + r) * N + 16 * x;
      uint4 wv[4], yv[4];
      key_run(A.what + off, wv);  // this step's key slices, fetched before the transform
      key_run(Y + off - yoff, yv);
      uint32_t v[16];
#pragma unroll
      for (int j = 0; j < 16; j++) v[j] = TC[kd * N + x + 128 * j];
      ntt_fwd(v, SC + kd * NTT_SCRATCH, fwd_tw(C), q, x, 2 + kd);  // slots 16x.., [0, 14q)
      if (ybody) rotate_key_run(yv, i, x);
      uint32_t* accb = ACC + kd * N;
      uint32_t* pdst = kd == 0 ? SCAT + p * N : PB1;
#pragma unroll
      for (int r4 = 0; r4 < 4; r4++) {
        const int o = 16 * x + 4 * (r4 ^ f);
        uint4* ap = reinterpret_cast<uint4*>(accb + o);
        const uint4 a4 = *ap;
        uint4* hp = reinterpret_cast<uint4*>(pdst + o);
        const uint4 h4 = kd == 0 ? *hp : make_uint4(0, 0, 0, 0);
        uint32_t ab[4], pr[4];
#pragma unroll
        for (int e = 0; e < 4; e++) {
          const int j = 4 * r4 + e;
          ab[e] = acc_2q(u4e(a4, e), redc_lazy((uint64_t)v[j] * u4e(yv[r4], e), q, qinv), q2);
          pr[e] = redc_lazy((uint64_t)v[j] * u4e(wv[r4], e), q, qinv) + u4e(h4, e);  // [0, 3q)
        }
        *ap = make_uint4(ab[0], ab[1], ab[2], ab[3]);
        *hp = make_uint4(pr[0], pr[1], pr[2], pr[3]);
      }
      named_sync(8, 4 * NTT_GT);  // PB1, PB2, the partial R_i are complete; R_{i+1} no longer read
      if (kd == 0) {
#pragma unroll
        for (int r4 = 0; r4 < 4; r4++) {
          const int o = 16 * x + 4 * (r4 ^ f);
          const uint4 pa = *reinterpret_cast<const uint4*>(SCAT + p * N + o);
          const uint4 p1 = *reinterpret_cast<const uint4*>(PB1 + o);
          const uint4 p2 = *reinterpret_cast<const uint4*>(PB2 + o);
          uint32_t outv[4];
#pragma unroll
          for (int e = 0; e < 4; e++) {
            uint32_t sum = u4e(pa, e) + u4e(p1, e) + u4e(p2, e);  // < 7q < 2^31
            sum = min(sum, sum - 4 * q);
            sum = min(sum, sum - 2 * q);
            outv[e] = min(sum, sum - q);
          }
          *reinterpret_cast<uint4*>(RN + o) = make_uint4(outv[0], outv[1], outv[2], outv[3]);  // R_i
        }
      }
    } else if (g == 2) {
      // PB2 = R_{i+1} w'2
      uint4 wv[4];
      key_run(A.what + ((size_t)(i * ELL + 2) * 2 + r) * N + 16 * x, wv);
      uint32_t rs[16], pr[16];
      load16(RN, x, rs);
#pragma unroll
      for (int j = 0; j < 16; j++) pr[j] = redc_lazy((uint64_t)rs[j] * u4e(wv[j >> 2], j & 3), q, qinv);
      store16(PB2, x, pr);
      named_sync(8, 4 * NTT_GT);
    } else if (g == 3) {
      // b += R_{i+1} y'2
      uint4 k2[4];
      key_run(Y + ((size_t)(i * ELL + 2) * 2 + r) * N + 16 * x - yoff, k2);
      if (ybody) rotate_key_run(k2, i, x);
      uint32_t* accb = ACC + 2 * N;
#pragma unroll
      for (int r4 = 0; r4 < 4; r4++) {
        const int o = 16 * x + 4 * (r4 ^ f);
        const uint4 rr = *reinterpret_cast<const uint4*>(RN + o);
        uint4* ap = reinterpret_cast<uint4*>(accb + o);
        const uint4 a4 = *ap;
        uint32_t ab[4];
#pragma unroll
        for (int e = 0; e < 4; e++)
          ab[e] = acc_2q(u4e(a4, e), redc_lazy((uint64_t)u4e(rr, e) * u4e(k2[r4], e), q, qinv), q2);
        *ap = make_uint4(ab[0], ab[1], ab[2], ab[3]);
      }
      named_sync(8, 4 * NTT_GT);
    } else {
      // groups 4-5: the second half of R_{i-1}, and the b side of this
      // step's columns (step gamma-2-i takes column gamma-2-i; the last step
      // also column gamma-1)
      const int t = tid - 4 * NTT_GT;
      const int c0 = gamma - 2 - i;
      const bool two = i == 0;
      const uint32_t* h0 = reinterpret_cast<const uint32_t*>(H + (size_t)c0 * N);
      const uint32_t* h1 = reinterpret_cast<const uint32_t*>(H + (size_t)(gamma - 1) * N);
      const uint32_t w0 = __ldg(h0 + t), w1 = __ldg(h0 + t + 512), w2 = __ldg(h0 + t + 256),
                     w3 = __ldg(h0 + t + 768);
      uint32_t w4 = 0, w5 = 0, w6 = 0, w7 = 0;
      if (two) {
        w4 = __ldg(h1 + t);
        w5 = __ldg(h1 + t + 512);
        w6 = __ldg(h1 + t + 256);
        w7 = __ldg(h1 + t + 768);
      }
      if (i >= 1) scatter_next(i, t, 2 * NTT_GT, N / 2, N);
      column_b0_part(P, w0, w1, BP, t, b0sum + c0);
      column_b0_part(P, w2, w3, BP, t + 256, b0sum + c0);
      if (two) {
        column_b0_part(P, w4, w5, BP, t, b0sum + gamma - 1);
        column_b0_part(P, w6, w7, BP, t + 256, b0sum + gamma - 1);
      }
    }
    __syncthreads();
  }

  // ---- outputs: a_hat = INTT(R_0) (inspiring2.rs:1027-1029) by groups 0-1,
  //      b = b_poly + INTT(sum y_all * bold_t) (inspiring2.rs:1217-1221) by
  //      groups 2-3, this residue's halves of the response ----
  uint64_t* out = QDB ? reload_ptr(&D->out) : A.out + (size_t)qi * 4 * N;
  if (tid < 4 * NTT_GT) {
    const bool bside = tid >= 2 * NTT_GT;
    const int t = tid & (2 * NTT_GT - 1);
    const int s0 = 8 * t;
    uint32_t v[8];
    if (!bside) {
      const uint4 lo = *reinterpret_cast<const uint4*>(RN + swz(s0));
      const uint4 hi = *reinterpret_cast<const uint4*>(RN + swz(s0 + 4));
      v[0] = lo.x; v[1] = lo.y; v[2] = lo.z; v[3] = lo.w;
      v[4] = hi.x; v[5] = hi.y; v[6] = hi.z; v[7] = hi.w;
    } else {
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const int o = swz(s0 + 4 * h);
        const uint4 a0 = *reinterpret_cast<const uint4*>(ACC + o);
        const uint4 a1 = *reinterpret_cast<const uint4*>(ACC + N + o);
        const uint4 a2 = *reinterpret_cast<const uint4*>(ACC + 2 * N + o);
#pragma unroll
        for (int e = 0; e < 4; e++) v[4 * h + e] = acc_2q(acc_2q(u4e(a0, e), u4e(a1, e), q2), u4e(a2, e), q2);
      }
    }
    ntt_inv_noscale8(v, SC + (bside ? NTT_SCRATCH : 0), inv_tw(C), q, t, bside ? 9 : 1);
    uint64_t* o = out + (bside ? 2 * N : 0) + (size_t)r * N;
#pragma unroll
    for (int j = 0; j < 8; j++) {
      const int c = t + 256 * j;
      uint32_t val = canon2(v[j], q);
      if (bside && c < gamma) val = add_mod(val, (uint32_t)(b0sum[c] % q), q);
      o[c] = val;
    }
  }
}

template <int MODE, bool SEEDED, bool QDB>
static cudaError_t set_pair_smem_attr() {
  return cudaFuncSetAttribute(respond_pair_kernel<MODE, SEEDED, QDB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)(sizeof(uint32_t) * PairSmem::TOTAL));
}

template <int MODE>
static cudaError_t launch_pair_mode(const RespondArgs& a, bool seeded, cudaStream_t st) {
  const size_t smem = sizeof(uint32_t) * PairSmem::TOTAL;
  const int ctas = 2 * a.nq;
  if (a.qdesc) {
    if (seeded) respond_pair_kernel<MODE, true, true><<<ctas, RBLOCK, smem, st>>>(a);
    else respond_pair_kernel<MODE, false, true><<<ctas, RBLOCK, smem, st>>>(a);
  } else {
    if (seeded) respond_pair_kernel<MODE, true, false><<<ctas, RBLOCK, smem, st>>>(a);
    else respond_pair_kernel<MODE, false, false><<<ctas, RBLOCK, smem, st>>>(a);
  }
  return cudaGetLastError();
}

}  // namespace

size_t respond_pair_smem_bytes() { return sizeof(uint32_t) * PairSmem::TOTAL; }

cudaError_t prepare_respond_pair_kernels() {
  const cudaError_t es[] = {
      set_pair_smem_attr<MODE_COMPAT, false, false>(),    set_pair_smem_attr<MODE_COMPAT, true, false>(),
      set_pair_smem_attr<MODE_COMPAT, false, true>(),     set_pair_smem_attr<MODE_COMPAT, true, true>(),
      set_pair_smem_attr<MODE_CRT_FIXED, false, false>(), set_pair_smem_attr<MODE_CRT_FIXED, true, false>(),
      set_pair_smem_attr<MODE_CRT_FIXED, false, true>(),  set_pair_smem_attr<MODE_CRT_FIXED, true, true>()};
  for (cudaError_t e : es)
    if (e != cudaSuccess) return e;
  return cudaSuccess;
}

cudaError_t launch_respond_pair(const RespondArgs& a, bool seeded, cudaStream_t st) {
  if (a.nq <= 0) return cudaSuccess;
  return a.P.mode == MODE_COMPAT ? launch_pair_mode<MODE_COMPAT>(a, seeded, st)
                                 : launch_pair_mode<MODE_CRT_FIXED>(a, seeded, st);
}

}  // namespace ig
