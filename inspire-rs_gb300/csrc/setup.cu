// setup.cu -- setup-time GPU kernels: resident database, CRS key table and
// per-client key tables.  All outputs stay in HBM for the lifetime of their
// handles; Respond then reads them without further preprocessing.
#include <algorithm>

#include "kernels.h"

namespace ig {

namespace {

// encode_database (src/pir/encode_db.rs:106-181): shard s holds entries
// [s*N, s*N + N); column c, coefficient i = little-endian u16 of bytes
// (2c, 2c+1) of that entry (a lone trailing byte is the value itself).
__global__ void columns_from_raw_kernel(const uint8_t* __restrict__ raw, uint64_t n_entries,
                                        int entry_size, int gamma, int nshards,
                                        uint16_t* __restrict__ H) {
  const uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const uint64_t total = (uint64_t)nshards * N;
  if (idx >= total) return;
  const uint64_t s = idx >> LOGN, i = idx & (N - 1);
  const uint64_t e = idx;  // global entry index = s * N + i
  for (int c = 0; c < gamma; c++) {
    uint16_t v = 0;
    if (e < n_entries) {
      const uint8_t* ent = raw + e * (uint64_t)entry_size;
      const int bo = 2 * c;
      if (bo + 1 < entry_size) v = (uint16_t)(ent[bo] | (ent[bo + 1] << 8));
      else if (bo < entry_size) v = ent[bo];
    }
    H[(s * gamma + c) * N + i] = v;
  }
}

// E[s][r][t][k][u] = K * sum_j zeta^(k j) * omega_u^j * NTT(d_t(Delta h_j))[u]
// with omega_u = psi^(2brv(u)+1), zeta = psi^(2n/gamma), K = gamma^-1 n^-1
// 2^32 (Montgomery form, n^-1 pre-applied for the unscaled inverse NTTs of
// the Respond kernel).  Grid: (shard, residue, digit t).
__global__ void __launch_bounds__(BLOCK) encode_E_kernel(const DevParams P, const uint16_t* __restrict__ H,
                                                         uint32_t* __restrict__ E) {
  extern __shared__ __align__(16) uint32_t smem[];
  const int gamma = P.gamma;
  uint32_t* Dh = smem;                  // [gamma][N]
  uint32_t* SC = Dh + gamma * N;        // [2][NTT_SCRATCH]
  uint32_t* zp = SC + 2 * NTT_SCRATCH;  // [gamma] powers of zeta
  const int s = blockIdx.x, r = blockIdx.y, t = blockIdx.z;
  const int tid = threadIdx.x, g = tid >> 7, x = tid & 127;
  const ResidueConsts& C = P.r[r];
  const uint32_t q = C.q, qinv = C.qinv;
  if (tid < gamma) zp[tid] = C.psi_pow[((2 * N / gamma) * tid) & (2 * N - 1)];
  for (int j = g; j < gamma; j += 2) {
    const uint16_t* h = H + ((size_t)s * gamma + j) * N;
    uint32_t v[16];
#pragma unroll
    for (int rr = 0; rr < 16; rr++) {
      const uint64_t xv = P.delta * (uint64_t)h[x + 128 * rr];
      v[rr] = (uint32_t)(xv >> (ZBITS * t)) & ((1u << ZBITS) - 1);  // digit t < 2^20 < q
    }
    ntt_fwd(v, SC + g * NTT_SCRATCH, fwd_tw(C), q, x, 1 + g);
#pragma unroll
    for (int rr = 0; rr < 16; rr++) v[rr] = canon16(v[rr], q);
    uint4* dst = reinterpret_cast<uint4*>(Dh + j * N + 16 * x);
#pragma unroll
    for (int rr = 0; rr < 4; rr++) dst[rr] = make_uint4(v[4 * rr], v[4 * rr + 1], v[4 * rr + 2], v[4 * rr + 3]);
  }
  __syncthreads();
  // Stored by recursion step: the scatter of R_i reads, at source slot u, the
  // DFT output k = (2brv(u)+1) m_i mod gamma with m_i = (gamma - i) mod gamma
  // (scatter_r), so entry [i][t][u] holds output k of (t, u) and a warp's
  // loads at consecutive slots are contiguous.  For odd 2brv(u)+1 the map
  // i -> k is a bijection: the table is a permutation of the outputs.
  uint32_t* Eo = E + (((size_t)s * 2 + r) * gamma * ELL + t) * N;
  for (int v = 0; v < N / BLOCK; v++) {
    const int u = tid + BLOCK * v;
    const uint32_t e = 2 * brv11(u) + 1;
    uint32_t c[MAX_GAMMA];
#pragma unroll
    for (int j = 0; j < MAX_GAMMA; j++)
      if (j < gamma) c[j] = mont_mul(Dh[j * N + u], __ldg(C.psi_pow + ((e * j) & (2 * N - 1))), q, qinv);
    for (int i = 0; i < gamma; i++) {
      const int k = (int)((e * ((uint32_t)(gamma - i) & (uint32_t)(gamma - 1))) & (uint32_t)(gamma - 1));
      uint64_t T = 0;
#pragma unroll
      for (int j = 0; j < MAX_GAMMA; j++)
        if (j < gamma) T += (uint64_t)zp[(k * j) & (gamma - 1)] * c[j];
      // the two REDCs divided by 2^64; e_scale = gamma^-1 n^-1 2^96 leaves
      // the factor 2^32 gamma^-1 n^-1
      Eo[(size_t)i * ELL * N + u] = mul_shoup(redc(T, q, qinv), C.e_scale, C.e_scale_p, q);
    }
  }
}

// OfflinePackingKeys::generate (inspiring2.rs:448-506): w_all_ntt[i][k] =
// NTT-domain automorphism tau_{g^i} of NTT(w_mask[k]) for i < gamma-1, with the
// reference's residue-1 behaviour in compat mode.  Stored times n^-1 2^32.
__global__ void __launch_bounds__(BLOCK) crs_what_kernel(const DevParams P, const uint32_t* __restrict__ wmask,
                                                         uint32_t* __restrict__ what) {
  __shared__ __align__(16) uint32_t W[2][N];
  __shared__ uint32_t SC[2][NTT_SCRATCH];
  const int k = blockIdx.x, tid = threadIdx.x, g = tid >> 7, x = tid & 127;
  const int gamma = P.gamma;
  {
    const ResidueConsts& C = P.r[g];
    uint32_t v[16];
#pragma unroll
    for (int rr = 0; rr < 16; rr++) v[rr] = wmask[((size_t)k * 2 + g) * N + x + 128 * rr];
    ntt_fwd(v, SC[g], fwd_tw(C), C.q, x, 1 + g);
#pragma unroll
    for (int rr = 0; rr < 16; rr++) W[g][16 * x + rr] = canon16(v[rr], C.q);
  }
  __syncthreads();
  for (int i = 0; i + 1 < gamma; i++) {
    const uint32_t tg = gen_pow(gamma, i);
    for (int v = 0; v < N / BLOCK; v++) {
      const int s = tid + BLOCK * v;
      const uint32_t es = 2 * brv11(s) + 1;
      const int u = brv11(((tg * es) & (2 * N - 1)) >> 1);  // table_{g^i}[s]
      uint32_t v0 = W[0][u];
      uint32_t v1 = P.mode == MODE_COMPAT ? compat_residue1(P, v0) : W[1][u];
      v0 = mul_shoup(v0, P.r[0].ninv_mont, P.r[0].ninv_mont_p, P.r[0].q);
      v1 = mul_shoup(v1, P.r[1].ninv_mont, P.r[1].ninv_mont_p, P.r[1].q);
      what[(((size_t)i * ELL + k) * 2 + 0) * N + s] = v0;
      what[(((size_t)i * ELL + k) * 2 + 1) * N + s] = v1;
    }
  }
}

// Client key table from y_body: generate_rotations (inspiring2.rs:1309-1323)
// followed by the forward NTT of packing_online (:1199-1213).  tau in the
// coefficient domain is the slot permutation in the NTT domain on both
// residues.  Stored times n^-1 2^32.  The first nrot rotations are written
// (nrot = 1: the body table NTT(y_body[k]), rotated by the Respond kernel).
__global__ void __launch_bounds__(BLOCK) client_ybody_kernel(const DevParams P, const uint64_t* __restrict__ yb,
                                                             uint32_t* __restrict__ yhat, int nrot) {
  __shared__ __align__(16) uint32_t W[2][N];
  __shared__ uint32_t SC[2][NTT_SCRATCH];
  const int k = blockIdx.x, tid = threadIdx.x, g = tid >> 7, x = tid & 127;
  const int gamma = P.gamma;
  const ResidueConsts& C = P.r[g];
  {
    uint32_t v[16];
#pragma unroll
    for (int rr = 0; rr < 16; rr++) v[rr] = (uint32_t)yb[((size_t)k * 2 + g) * N + x + 128 * rr];
    ntt_fwd(v, SC[g], fwd_tw(C), C.q, x, 1 + g);
#pragma unroll
    for (int rr = 0; rr < 16; rr++) W[g][16 * x + rr] = mul_shoup(v[rr], C.ninv_mont, C.ninv_mont_p, C.q);
  }
  __syncthreads();
  for (int i = 0; i + 1 < gamma && i < nrot; i++) {
    const uint32_t tg = gen_pow(gamma, i);
    for (int v = 0; v < N / BLOCK; v++) {
      const int s = tid + BLOCK * v;
      const uint32_t es = 2 * brv11(s) + 1;
      const int u = brv11(((tg * es) & (2 * N - 1)) >> 1);
      yhat[(((size_t)i * ELL + k) * 2 + 0) * N + s] = W[0][u];
      yhat[(((size_t)i * ELL + k) * 2 + 1) * N + s] = W[1][u];
    }
  }
}

// Client key table from an explicit y_all ((gamma-1)*ELL coefficient polys).
__global__ void __launch_bounds__(BLOCK) client_yall_kernel(const DevParams P, const uint64_t* __restrict__ ya,
                                                            uint32_t* __restrict__ yhat) {
  __shared__ uint32_t SC[2][NTT_SCRATCH];
  const int p = blockIdx.x, tid = threadIdx.x, g = tid >> 7, x = tid & 127;
  const ResidueConsts& C = P.r[g];
  uint32_t v[16];
#pragma unroll
  for (int rr = 0; rr < 16; rr++) v[rr] = (uint32_t)ya[((size_t)p * 2 + g) * N + x + 128 * rr];
  ntt_fwd(v, SC[g], fwd_tw(C), C.q, x, 1 + g);
#pragma unroll
  for (int rr = 0; rr < 16; rr++)
    yhat[((size_t)p * 2 + g) * N + 16 * x + rr] = mul_shoup(v[rr], C.ninv_mont, C.ninv_mont_p, C.q);
}

// Key tables with the third gadget digit folded in.  In the NTT domain of
// residue r, the digits of the composite coefficient c = INTT(R) satisfy
// NTT(d0) + z NTT(d1) + z^2 NTT(d2) = R (mod q_r), so for any key triple
// (k0, k1, k2):  k0 NTT(d0) + k1 NTT(d1) + k2 NTT(d2)
//   = (k0 - z^-2 k2) NTT(d0) + (k1 - z^-1 k2) NTT(d1) + (z^-2 k2) R.
// With R kept as n^-1 R (the Respond kernel's R_{i+1}), the third key is
// n z^-2 k2.  `tbl` holds ngroups triples [g][k<3][2][N] (any constant
// scaling, applied alike to the three keys), rewritten in place.
__global__ void __launch_bounds__(BLOCK) fold_third_digit_kernel(const DevParams P, uint32_t* __restrict__ tbl,
                                                                 int ngroups) {
  const size_t per = (size_t)2 * N;
  const size_t total = (size_t)ngroups * per;
  for (size_t idx = (size_t)blockIdx.x * BLOCK + threadIdx.x; idx < total; idx += (size_t)gridDim.x * BLOCK) {
    const size_t g = idx / per, rs = idx - g * per;
    const int r = (int)(rs >> LOGN);
    const ResidueConsts& C = P.r[r];
    uint32_t* t = tbl + g * 3 * per + rs;
    const uint32_t k0 = t[0], k1 = t[per], k2 = t[2 * per];
    t[0] = sub_mod(k0, mul_shoup(k2, C.d2_z2, C.d2_z2_p, C.q), C.q);
    t[per] = sub_mod(k1, mul_shoup(k2, C.d2_z1, C.d2_z1_p, C.q), C.q);
    t[2 * per] = mul_shoup(k2, C.d2_nz2, C.d2_nz2_p, C.q);
  }
}

}  // namespace

cudaError_t launch_fold_third_digit(const DevParams& P, uint32_t* tbl, int ngroups, cudaStream_t st) {
  if (ngroups <= 0) return cudaSuccess;
  const size_t total = (size_t)ngroups * 2 * N;
  const unsigned blocks = (unsigned)std::min<size_t>((total + BLOCK - 1) / BLOCK, 4096);
  fold_third_digit_kernel<<<blocks, BLOCK, 0, st>>>(P, tbl, ngroups);
  return cudaGetLastError();
}

cudaError_t launch_columns_from_raw(const uint8_t* raw, uint64_t n_entries, int entry_size, int gamma,
                                    int nshards, uint16_t* H, cudaStream_t st) {
  const uint64_t total = (uint64_t)nshards * N;
  const unsigned blocks = (unsigned)((total + 255) / 256);
  if (blocks) columns_from_raw_kernel<<<blocks, 256, 0, st>>>(raw, n_entries, entry_size, gamma, nshards, H);
  return cudaGetLastError();
}

cudaError_t prepare_setup_kernels() {
  const size_t smem = sizeof(uint32_t) * ((size_t)MAX_GAMMA * N + 2 * NTT_SCRATCH + MAX_GAMMA);
  return cudaFuncSetAttribute(encode_E_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

cudaError_t launch_encode_E(const DevParams& P, const uint16_t* H, int nshards, uint32_t* E, cudaStream_t st) {
  if (nshards <= 0) return cudaSuccess;
  const size_t smem = sizeof(uint32_t) * ((size_t)P.gamma * N + 2 * NTT_SCRATCH + MAX_GAMMA);
  // grid.x is limited to 2^31-1 shards; y = residue, z = digit
  encode_E_kernel<<<dim3(nshards, 2, ELL), BLOCK, smem, st>>>(P, H, E);
  return cudaGetLastError();
}

cudaError_t launch_crs_what(const DevParams& P, const uint32_t* wmask, uint32_t* what, cudaStream_t st) {
  if (P.gamma < 2) return cudaSuccess;
  crs_what_kernel<<<ELL, BLOCK, 0, st>>>(P, wmask, what);
  return cudaGetLastError();
}

cudaError_t launch_client_from_ybody(const DevParams& P, const uint64_t* ybody, uint32_t* yhat, int nrot,
                                     cudaStream_t st) {
  if (P.gamma < 2) return cudaSuccess;
  client_ybody_kernel<<<ELL, BLOCK, 0, st>>>(P, ybody, yhat, nrot);
  return cudaGetLastError();
}

cudaError_t launch_client_from_yall(const DevParams& P, const uint64_t* yall, uint32_t* yhat, cudaStream_t st) {
  if (P.gamma < 2) return cudaSuccess;
  client_yall_kernel<<<(P.gamma - 1) * ELL, BLOCK, 0, st>>>(P, yall, yhat);
  return cudaGetLastError();
}

}  // namespace ig
