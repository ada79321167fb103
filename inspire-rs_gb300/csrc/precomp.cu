// precomp.cu -- setup's InspiRING offline precomputation on the GPU:
// packing_offline (src/inspiring/inspiring2.rs:926-1041) over the first gamma
// crs_a_vectors, which setup stores as ServerCrs.inspiring_precomp
// (src/pir/setup.rs:194-224): a_hat (coefficient form) and bold_t, the
// gadget digits T[i][k] of every recursion step (coefficient form).
//
// Three launches on the context's stream:
//  1. one CTA per a-poly: forward NTT of both residues (plain residues);
//  2. one CTA per i < gamma: R_i = tau_{g^i}(gamma^-1 sum_j X^{j h_i} a_j)
//     in the NTT domain, h_i = g^((n - i) mod n) (inspiring2.rs:948-982):
//     the monomial X^e is psi^(e (2brv(u)+1)) at slot u, and tau_{g^i} is the
//     slot permutation of the closed-form table (inspiring2.rs:208-263); in
//     compat mode residue 1 is rebuilt from residue 0 as the crate's
//     apply_automorphism_ntt does (inspiring2.rs:279-296).  Stored times n^-1
//     (the inverse transforms below then need no scaling);
//  3. one CTA of two NTT groups (one per residue) runs the backward recursion
//     (inspiring2.rs:984-1008): T[i] = G^-1(INTT(R[i+1])), written out as
//     bold_t[i], and R[i] += sum_k NTT(T[i][k]) * w_all_ntt[i][k] with the
//     context's rotated w_mask table (the same table the Respond kernel
//     uses); finally a_hat = INTT(R[0]).
// R lives in a device scratch buffer of gamma polys (u32); this is a
// setup-time call, not a hot path.
#include <vector>

#include "host.h"

namespace ig {
namespace {

struct PrecompArgs {
  DevParams P;
  const uint64_t* a;     // [gamma][2][N] a-polys, coefficient form
  uint32_t* ahat;        // [gamma][2][N] NTT(a_j), plain residues
  uint32_t* R;           // [gamma][2][N] R_i times n^-1
  const uint32_t* what;  // [(gamma-1)][ELL][2][N] w_all_ntt times n^-1 2^32
  uint64_t* a_hat;       // [2][N] output
  uint64_t* bold_t;      // [(gamma-1)][ELL][2][N] output
  uint32_t gpow[MAX_GAMMA];  // g^i mod 2n
  uint32_t hinv[MAX_GAMMA];  // g^((n - i) mod n) mod 2n
  uint32_t scale[2];         // gamma^-1 n^-1 mod q_r
};

__global__ void __launch_bounds__(BLOCK) precomp_ntt_kernel(const __grid_constant__ PrecompArgs A) {
  __shared__ uint32_t SC[2][NTT_SCRATCH];
  const int j = blockIdx.x, tid = threadIdx.x, g = tid >> 7, x = tid & 127;
  const ResidueConsts& C = A.P.r[g];
  uint32_t v[16];
#pragma unroll
  for (int rr = 0; rr < 16; rr++) v[rr] = (uint32_t)A.a[((size_t)j * 2 + g) * N + x + 128 * rr];
  ntt_fwd(v, SC[g], fwd_tw(C), C.q, x, 1 + g);
#pragma unroll
  for (int rr = 0; rr < 16; rr++) A.ahat[((size_t)j * 2 + g) * N + 16 * x + rr] = canon16(v[rr], C.q);
}

// Pre-permutation value of R_i at slot u for residue r, times n^-1.
__device__ __forceinline__ uint32_t r_slot(const PrecompArgs& A, int i, int r, uint32_t u) {
  const ResidueConsts& C = A.P.r[r];
  const uint32_t e = 2 * brv11(u) + 1;
  uint64_t acc = 0;  // gamma products < 2^56 each
  for (int j = 0; j < A.P.gamma; j++) {
    const uint32_t idx = ((uint32_t)j * A.hinv[i]) & (2 * N - 1);
    acc += (uint64_t)__ldg(C.psi_pow + ((idx * e) & (2 * N - 1))) * A.ahat[((size_t)j * 2 + r) * N + u];
  }
  return (uint32_t)((acc % C.q) * A.scale[r] % C.q);
}

__global__ void __launch_bounds__(BLOCK) precomp_r_kernel(const __grid_constant__ PrecompArgs A) {
  const int i = blockIdx.x;
  for (int s = threadIdx.x; s < N; s += BLOCK) {
    const uint32_t es = 2 * brv11(s) + 1;
    const uint32_t u = brv11(((A.gpow[i] * es) & (2 * N - 1)) >> 1);  // table_{g^i}[s]
    const uint32_t v0 = r_slot(A, i, 0, u);
    const uint32_t v1 = A.P.mode == MODE_COMPAT ? compat_residue1_ninv(A.P, v0) : r_slot(A, i, 1, u);
    A.R[((size_t)i * 2 + 0) * N + s] = v0;
    A.R[((size_t)i * 2 + 1) * N + s] = v1;
  }
}

__global__ void __launch_bounds__(BLOCK) precomp_recursion_kernel(const __grid_constant__ PrecompArgs A) {
  __shared__ uint32_t SC[2][NTT_SCRATCH];
  __shared__ uint32_t Cf[2][N];  // INTT(R[i+1]) per residue
  const int tid = threadIdx.x, r = tid >> 7, x = tid & 127;
  const ResidueConsts& C = A.P.r[r];
  const uint32_t q = C.q, qinv = C.qinv;
  const int gamma = A.P.gamma;
  for (int i = gamma - 2; i >= 0; i--) {
    uint32_t v[16];
    uint32_t* Ri1 = A.R + ((size_t)(i + 1) * 2 + r) * N;
#pragma unroll
    for (int j = 0; j < 16; j++) v[j] = Ri1[16 * x + j];
    ntt_inv_noscale(v, SC[r], inv_tw(C), q, x, 1 + r);
#pragma unroll
    for (int j = 0; j < 16; j++) Cf[r][x + 128 * j] = canon2(v[j], q);
    __syncthreads();
    // gadget_decompose of the composite coefficients (rgsw/external_product.rs:16-37)
    for (int c = tid; c < N; c += BLOCK) {
      const uint64_t comp = crt_compose(A.P, Cf[0][c], Cf[1][c]);
      const uint32_t d[ELL] = {(uint32_t)comp & 0xFFFFFu, (uint32_t)(comp >> 20) & 0xFFFFFu, (uint32_t)(comp >> 40)};
#pragma unroll
      for (int k = 0; k < ELL; k++) {
        uint64_t* bt = A.bold_t + (((size_t)i * ELL + k) * 2) * N;
        bt[c] = d[k];      // each digit is below both moduli: equal residues
        bt[N + c] = d[k];
      }
    }
    __syncthreads();  // the digits in bold_t are visible to the whole CTA
    // R[i] += sum_k NTT(T[i][k]) * w_all_ntt[i][k]
    uint32_t* Ri = A.R + ((size_t)i * 2 + r) * N;
    uint32_t acc[16];
#pragma unroll
    for (int j = 0; j < 16; j++) acc[j] = Ri[16 * x + j];
    for (int k = 0; k < ELL; k++) {
      const uint64_t* bt = A.bold_t + (((size_t)i * ELL + k) * 2) * N;
#pragma unroll
      for (int j = 0; j < 16; j++) v[j] = (uint32_t)bt[x + 128 * j];
      ntt_fwd(v, SC[r], fwd_tw(C), q, x, 1 + r);  // slot layout, [0, 14q)
      const uint32_t* w = A.what + (((size_t)i * ELL + k) * 2 + r) * N + 16 * x;
#pragma unroll
      for (int j = 0; j < 16; j++) acc[j] = add_mod(acc[j], redc((uint64_t)v[j] * __ldg(w + j), q, qinv), q);
    }
#pragma unroll
    for (int j = 0; j < 16; j++) Ri[16 * x + j] = acc[j];
    __syncthreads();
  }
  // a_hat = INTT(R[0]) (inspiring2.rs:1027-1029)
  uint32_t v[16];
#pragma unroll
  for (int j = 0; j < 16; j++) v[j] = A.R[(size_t)r * N + 16 * x + j];
  ntt_inv_noscale(v, SC[r], inv_tw(C), q, x, 1 + r);
#pragma unroll
  for (int j = 0; j < 16; j++) A.a_hat[(size_t)r * N + x + 128 * j] = canon2(v[j], q);
}

uint64_t powmod(uint64_t b, uint64_t e, uint64_t m) {
  unsigned __int128 r = 1, x = b % m;
  while (e) {
    if (e & 1) r = r * x % m;
    x = x * x % m;
    e >>= 1;
  }
  return (uint64_t)r;
}

}  // namespace
}  // namespace ig

using namespace ighost;

extern "C" int inspire_inspiring_precomp(inspire_ctx* c, const uint64_t* a_polys, uint64_t* a_hat, uint64_t* bold_t) {
  if (!c || !a_polys || !a_hat) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null argument");
  std::lock_guard<std::mutex> lk(c->mu);
  if (!c->has_crs) return fail(INSPIRE_ERR_NO_CRS, "no CRS loaded (inspire_crs_load)");
  const int gamma = c->gamma;
  if (gamma > 1 && !bold_t) return fail(INSPIRE_ERR_INVALID_ARGUMENT, "null bold_t");
  if (int rc = set_device(c)) return rc;
  const size_t pw = poly_words();
  DevMem d_a(c->ledger), d_ahat(c->ledger), d_R(c->ledger), d_out(c->ledger);
  CUDA_TRY(d_a.ensure(sizeof(uint64_t) * gamma * pw));
  CUDA_TRY(d_ahat.ensure(sizeof(uint32_t) * gamma * pw));
  CUDA_TRY(d_R.ensure(sizeof(uint32_t) * gamma * pw));
  const size_t nbt = (size_t)std::max(0, gamma - 1) * ELL * pw;
  CUDA_TRY(d_out.ensure(sizeof(uint64_t) * (pw + std::max<size_t>(nbt, 1))));
  CUDA_TRY(cudaMemcpyAsync(d_a.p, a_polys, sizeof(uint64_t) * gamma * pw, cudaMemcpyHostToDevice, c->stream));
  PrecompArgs A{};
  A.P = c->P;
  A.a = d_a.as<uint64_t>();
  A.ahat = d_ahat.as<uint32_t>();
  A.R = d_R.as<uint32_t>();
  A.what = c->what.as<uint32_t>();
  A.a_hat = d_out.as<uint64_t>();
  A.bold_t = A.a_hat + pw;
  const uint32_t n2 = 2 * N;
  const uint32_t g = gamma < N ? (2 * N) / gamma + 1 : 5;  // PackParams generator (inspiring2.rs:115-127)
  for (int i = 0; i < gamma; i++) {
    A.gpow[i] = (uint32_t)powmod(g, (uint64_t)i, n2);
    A.hinv[i] = (uint32_t)powmod(g, (uint64_t)((N - i) % N), n2);
  }
  for (int r = 0; r < 2; r++) {
    const uint64_t q = c->params.crt_moduli[r];
    const uint64_t inv = powmod((uint64_t)gamma * N % q, q - 2, q);  // q prime
    A.scale[r] = (uint32_t)inv;
  }
  precomp_ntt_kernel<<<gamma, BLOCK, 0, c->stream>>>(A);
  CUDA_TRY(cudaGetLastError());
  precomp_r_kernel<<<gamma, BLOCK, 0, c->stream>>>(A);
  CUDA_TRY(cudaGetLastError());
  precomp_recursion_kernel<<<1, BLOCK, 0, c->stream>>>(A);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaMemcpyAsync(a_hat, A.a_hat, sizeof(uint64_t) * pw, cudaMemcpyDeviceToHost, c->stream));
  if (nbt) CUDA_TRY(cudaMemcpyAsync(bold_t, A.bold_t, sizeof(uint64_t) * nbt, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  return INSPIRE_OK;
}
