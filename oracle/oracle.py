"""ctypes binding of the CPU oracle (test infrastructure only).

The oracle is a plain-C restatement of the reference crate
igor53627/inspire-rs v0.1.2 for the InsPIRe Respond path (see
inspire_oracle.h for what it follows and how it is pinned).  Only tests/,
__graft_entry__.smoke() and bench.py (cpu_baseline and the reference arm) may
import this module; the product library never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libinspire_oracle.so")

MODE_COMPAT = 0
MODE_CRT_FIXED = 1

U64P = np.ctypeslib.ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS")
I32P = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
U32P = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
U8P = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")

_lib = None


def build() -> str:
    """Compile the oracle with its Makefile (gcc, OpenMP)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        build()
    L = C.CDLL(LIB_PATH)
    vp = C.c_void_p
    sig = {
        "io_ctx_new": (vp, [C.c_int, C.c_int, U64P, C.c_uint64, C.c_double, C.c_uint64, C.c_int]),
        "io_ctx_free": (None, [vp]),
        "io_ctx_q": (C.c_uint64, [vp]),
        "io_ctx_delta": (C.c_uint64, [vp]),
        "io_ctx_psi": (C.c_uint64, [vp, C.c_int]),
        "io_ctx_twiddles": (None, [vp, C.c_int, U64P, U64P]),
        "io_ntt_forward": (None, [vp, U64P, C.c_int]),
        "io_ntt_inverse": (None, [vp, U64P, C.c_int]),
        "io_poly_mul": (None, [vp, U64P, U64P, U64P]),
        "io_poly_coeff": (C.c_uint64, [vp, U64P, C.c_int]),
        "io_poly_from_composite": (None, [vp, U64P, U64P]),
        "io_gadget_decompose": (None, [vp, U64P, U64P]),
        "io_gadget_reconstruct": (None, [vp, U64P, U64P]),
        "io_external_product": (None, [vp, U64P, U64P, U64P]),
        "io_automorphism": (None, [vp, U64P, C.c_int, U64P]),
        "io_chacha20_block": (None, [U32P, U32P, U32P]),
        "io_rng_from_seed": (vp, [U8P]),
        "io_rng_seed_from_u64": (vp, [C.c_uint64]),
        "io_rng_free": (None, [vp]),
        "io_rng_next_u32": (C.c_uint32, [vp]),
        "io_rng_next_u64": (C.c_uint64, [vp]),
        "io_rng_gen_range_u64": (C.c_uint64, [vp, C.c_uint64, C.c_uint64]),
        "io_poly_from_seed": (None, [vp, U8P, U64P]),
        "io_mask_from_seed": (None, [vp, U8P, C.c_int, U64P]),
        "io_automorph_table_closed": (None, [C.c_int, C.c_int, I32P]),
        "io_automorph_table_brute": (None, [vp, C.c_int, vp, I32P]),
        "io_pack_new": (vp, [vp, C.c_int, U8P, C.c_int, C.c_int, C.c_uint64]),
        "io_pack_free": (None, [vp]),
        "io_pack_generator": (C.c_int, [vp]),
        "io_pack_gen_pows": (None, [vp, I32P]),
        "io_pack_mod_inv_gamma": (C.c_uint64, [vp]),
        "io_pack_w_all_ntt": (None, [vp, U64P]),
        "io_packing_offline": (None, [vp, U64P, U64P, U64P]),
        "io_generate_rotations": (None, [vp, U64P, U64P]),
        "io_packing_online": (None, [vp, U64P, U64P, U64P, U64P, U64P]),
        "io_respond_inspiring": (C.c_int, [vp, vp, C.c_int, U8P, U64P, C.c_int, U64P, vp, vp, U64P, C.c_int]),
        "io_expand_rgsw": (None, [vp, U8P, U64P, U64P]),
        "io_respond_nopacking": (C.c_int, [vp, U64P, C.c_int, U64P, U64P, vp, C.c_int]),
        "io_num_columns": (C.c_int, [C.c_int]),
        "io_encode_shard": (None, [vp, U8P, C.c_uint64, C.c_int, C.c_uint32, U64P]),
        "io_inverse_monomial": (None, [vp, C.c_int, U64P]),
        "io_sampler_new": (vp, [C.c_double, C.c_uint64]),
        "io_sampler_free": (None, [vp]),
        "io_sampler_sample": (C.c_int64, [vp]),
        "io_sk_generate": (None, [vp, vp, U64P]),
        "io_rlwe_encrypt": (None, [vp, vp, vp, U64P, U64P, U64P]),
        "io_rgsw_encrypt": (None, [vp, vp, vp, U64P, U64P, U64P]),
        "io_query_seeded": (None, [vp, vp, vp, U64P, C.c_int, U8P, U64P]),
        "io_client_packing_keys": (None, [vp, vp, U64P, U64P, U64P]),
        "io_decrypt": (None, [vp, U64P, U64P, U64P]),
        "io_extract_inspiring": (None, [vp, U64P, U64P, C.c_int, U8P]),
        "io_automorphism_ks_matrix": (None, [vp, vp, vp, U64P, C.c_int, U64P]),
        "io_galois_keys": (None, [vp, vp, vp, U64P, U64P]),
        "io_pack_lwes": (C.c_int, [vp, U64P, U64P, C.c_int, U64P, C.c_int, U64P, U64P]),
        "io_respond_one_packing": (C.c_int, [vp, U64P, C.c_int, U64P, U64P, C.c_int, U64P, U64P, C.c_int]),
        "io_extract_packed": (None, [vp, U64P, U64P, C.c_int, U8P]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def _ptr(a):
    """Raw pointer of an optional uint64 array (for nullable arguments)."""
    if a is None:
        return None
    assert a.dtype == np.uint64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.c_void_p)


CRT_MODULI = (268369921, 249561089)
SINGLE_Q = 1152921504606830593


class Ctx:
    """InspireParams + NttContext (params.rs:135-298)."""

    def __init__(self, n=2048, moduli=CRT_MODULI, p=1 << 16, sigma=6.4,
                 gadget_base=1 << 20, gadget_len=3):
        self.L = lib()
        self.n = n
        self.moduli = tuple(int(m) for m in moduli)
        self.crt = len(self.moduli)
        self.p = p
        self.sigma = sigma
        self.zbase = gadget_base
        self.ell = gadget_len
        self.h = self.L.io_ctx_new(n, self.crt, np.array(self.moduli, dtype=np.uint64), p, sigma,
                                   gadget_base, gadget_len)
        if not self.h:
            raise ValueError("invalid oracle parameters")
        self.q = self.L.io_ctx_q(self.h)
        self.delta = self.L.io_ctx_delta(self.h)
        self.plen = n * self.crt

    def __del__(self):
        if getattr(self, "h", None):
            self.L.io_ctx_free(self.h)
            self.h = None

    def zeros(self, k=None):
        shape = (self.plen,) if k is None else (k, self.plen)
        return np.zeros(shape, dtype=np.uint64)

    # ---- transforms / arithmetic ----
    def ntt_forward(self, polys):
        a = np.ascontiguousarray(polys, dtype=np.uint64).copy()
        self.L.io_ntt_forward(self.h, a, a.size // self.plen)
        return a

    def ntt_inverse(self, polys):
        a = np.ascontiguousarray(polys, dtype=np.uint64).copy()
        self.L.io_ntt_inverse(self.h, a, a.size // self.plen)
        return a

    def poly_mul(self, a, b):
        out = self.zeros()
        self.L.io_poly_mul(self.h, np.ascontiguousarray(a, np.uint64), np.ascontiguousarray(b, np.uint64), out)
        return out

    def coeff(self, poly, i):
        return self.L.io_poly_coeff(self.h, np.ascontiguousarray(poly, np.uint64), i)

    def from_composite(self, coeffs):
        out = self.zeros()
        self.L.io_poly_from_composite(self.h, np.ascontiguousarray(coeffs, np.uint64), out)
        return out

    def composite(self, poly):
        poly = np.asarray(poly, dtype=np.uint64)
        if self.crt == 1:
            return [int(x) for x in poly]
        q0, q1 = self.moduli
        inv = pow(q0, -1, q1)
        a0 = poly[: self.n].astype(object)
        a1 = poly[self.n:].astype(object)
        return [int((x + q0 * (((y - x) * inv) % q1)) % self.q) for x, y in zip(a0, a1)]

    def gadget_decompose(self, poly):
        out = self.zeros(self.ell)
        self.L.io_gadget_decompose(self.h, np.ascontiguousarray(poly, np.uint64), out)
        return out

    def gadget_reconstruct(self, digits):
        out = self.zeros()
        self.L.io_gadget_reconstruct(self.h, np.ascontiguousarray(digits, np.uint64), out)
        return out

    def external_product(self, ct, rgsw):
        out = self.zeros(2)
        self.L.io_external_product(self.h, np.ascontiguousarray(ct, np.uint64),
                                   np.ascontiguousarray(rgsw, np.uint64), out)
        return out

    def automorphism(self, poly, t):
        out = self.zeros()
        self.L.io_automorphism(self.h, np.ascontiguousarray(poly, np.uint64), t, out)
        return out

    def poly_from_seed(self, seed):
        out = self.zeros()
        self.L.io_poly_from_seed(self.h, np.frombuffer(bytes(seed), dtype=np.uint8).copy(), out)
        return out

    def mask_from_seed(self, seed, count):
        out = self.zeros(count)
        self.L.io_mask_from_seed(self.h, np.frombuffer(bytes(seed), dtype=np.uint8).copy(), count, out)
        return out

    def expand_rgsw(self, seeds, b_rows):
        out = self.zeros(4 * self.ell)
        self.L.io_expand_rgsw(self.h, np.ascontiguousarray(seeds, np.uint8).reshape(-1),
                              np.ascontiguousarray(b_rows, np.uint64), out)
        return out

    def encode_shard(self, db: np.ndarray, entry_size: int, shard_id: int):
        ncols = self.L.io_num_columns(entry_size)
        out = self.zeros(ncols)
        self.L.io_encode_shard(self.h, np.ascontiguousarray(db, np.uint8), db.size, entry_size, shard_id, out)
        return out

    def inverse_monomial(self, k):
        out = self.zeros()
        self.L.io_inverse_monomial(self.h, k, out)
        return out

    # ---- respond ----
    def respond_inspiring(self, shard, rgsw, w_seed, *, mode=MODE_CRT_FIXED, pack=None,
                          y_body=None, y_all=None, nthreads=0):
        gamma = shard.shape[0]
        out = self.zeros(2)
        yb = None if y_body is None else np.ascontiguousarray(y_body, np.uint64)
        ya = None if y_all is None else np.ascontiguousarray(y_all, np.uint64)
        rc = self.L.io_respond_inspiring(self.h, pack.h if pack is not None else None, mode,
                                         np.frombuffer(bytes(w_seed), dtype=np.uint8).copy(),
                                         np.ascontiguousarray(shard, np.uint64), gamma,
                                         np.ascontiguousarray(rgsw, np.uint64), _ptr(yb), _ptr(ya),
                                         out, nthreads)
        if rc < 0:
            raise ValueError("InspiRING packing keys invalid: y_all and y_body are both empty")
        return out

    def respond_nopacking(self, shard, rgsw, nthreads=0, with_columns=False):
        ncols = shard.shape[0]
        out = self.zeros(2)
        cols = self.zeros(2 * ncols) if with_columns else None
        self.L.io_respond_nopacking(self.h, np.ascontiguousarray(shard, np.uint64), ncols,
                                    np.ascontiguousarray(rgsw, np.uint64), out, _ptr(cols), nthreads)
        return (out, cols.reshape(ncols, 2, self.plen)) if with_columns else out

    def pack_lwes(self, leaf_a, bvals, keys, mode=MODE_CRT_FIXED):
        """pack_lwes on prepped LWEs (leaf a polys, composite b values);
        returns (a, b) with b of 2*plen words in compat mode with two moduli."""
        la = np.ascontiguousarray(leaf_a, np.uint64).reshape(-1, self.plen)
        bv = np.ascontiguousarray(bvals, np.uint64)
        out_a = self.zeros()
        out_b = self.zeros(2)
        w = self.L.io_pack_lwes(self.h, la, bv, la.shape[0], np.ascontiguousarray(keys, np.uint64), mode, out_a,
                                out_b.reshape(-1))
        return out_a, out_b.reshape(-1)[:max(w, self.plen)]

    def respond_one_packing(self, shard, rgsw, keys, mode=MODE_CRT_FIXED, nthreads=0):
        """respond_one_packing (respond.rs:213-268): (a, b) of the packed
        ciphertext, b of 2*plen words in compat mode with two moduli."""
        ncols = shard.shape[0]
        out_a = self.zeros()
        out_b = self.zeros(2)
        w = self.L.io_respond_one_packing(self.h, np.ascontiguousarray(shard, np.uint64), ncols,
                                          np.ascontiguousarray(rgsw, np.uint64), np.ascontiguousarray(keys, np.uint64),
                                          mode, out_a, out_b.reshape(-1), nthreads)
        return out_a, out_b.reshape(-1)[:max(w, self.plen)]

    def extract_packed(self, sk, ct, entry_size):
        out = np.zeros(entry_size, dtype=np.uint8)
        self.L.io_extract_packed(self.h, np.ascontiguousarray(sk, np.uint64), np.ascontiguousarray(ct, np.uint64),
                                 entry_size, out)
        return out

    # ---- client ----
    def decrypt(self, sk, ct):
        out = np.zeros(self.n, dtype=np.uint64)
        self.L.io_decrypt(self.h, np.ascontiguousarray(sk, np.uint64), np.ascontiguousarray(ct, np.uint64), out)
        return out

    def extract_inspiring(self, sk, ct, entry_size):
        out = np.zeros(entry_size, dtype=np.uint8)
        self.L.io_extract_inspiring(self.h, np.ascontiguousarray(sk, np.uint64),
                                    np.ascontiguousarray(ct, np.uint64), entry_size, out)
        return out


class Rng:
    """ChaCha20Rng restatement (rand_chacha 0.3)."""

    def __init__(self, seed=None, u64=None):
        self.L = lib()
        if seed is not None:
            self.h = self.L.io_rng_from_seed(np.frombuffer(bytes(seed), dtype=np.uint8).copy())
        else:
            self.h = self.L.io_rng_seed_from_u64(u64 or 0)

    def __del__(self):
        if getattr(self, "h", None):
            self.L.io_rng_free(self.h)
            self.h = None

    def next_u32(self):
        return self.L.io_rng_next_u32(self.h)

    def next_u64(self):
        return self.L.io_rng_next_u64(self.h)

    def gen_range(self, lo, hi):
        return self.L.io_rng_gen_range_u64(self.h, lo, hi)


class Sampler:
    """GaussianSampler restatement (math/gaussian.rs)."""

    def __init__(self, sigma=6.4, seed=0):
        self.L = lib()
        self.h = self.L.io_sampler_new(sigma, seed)

    def __del__(self):
        if getattr(self, "h", None):
            self.L.io_sampler_free(self.h)
            self.h = None

    def sample(self):
        return self.L.io_sampler_sample(self.h)


class Pack:
    """PackParams + OfflinePackingKeys (inspiring2.rs:107-506)."""

    def __init__(self, ctx: Ctx, gamma: int, w_seed: bytes, mode=MODE_CRT_FIXED, brute=False, rng_seed=0x5EED):
        self.ctx = ctx
        self.L = ctx.L
        self.gamma = gamma
        self.mode = mode
        self.h = self.L.io_pack_new(ctx.h, gamma, np.frombuffer(bytes(w_seed), dtype=np.uint8).copy(), mode,
                                    1 if brute else 0, rng_seed)

    def __del__(self):
        if getattr(self, "h", None):
            self.L.io_pack_free(self.h)
            self.h = None

    @property
    def generator(self):
        return self.L.io_pack_generator(self.h)

    def gen_pows(self):
        out = np.zeros(self.ctx.n, dtype=np.int32)
        self.L.io_pack_gen_pows(self.h, out)
        return out

    @property
    def mod_inv_gamma(self):
        return self.L.io_pack_mod_inv_gamma(self.h)

    def w_all_ntt(self):
        out = self.ctx.zeros((self.gamma - 1) * self.ctx.ell)
        self.L.io_pack_w_all_ntt(self.h, out)
        return out

    def packing_offline(self, a_ct):
        a_hat = self.ctx.zeros()
        bold_t = self.ctx.zeros(max(1, (self.gamma - 1) * self.ctx.ell))
        self.L.io_packing_offline(self.h, np.ascontiguousarray(a_ct, np.uint64), a_hat, bold_t)
        return a_hat, bold_t[: (self.gamma - 1) * self.ctx.ell]

    def generate_rotations(self, y_body):
        out = self.ctx.zeros(max(1, (self.gamma - 1) * self.ctx.ell))
        self.L.io_generate_rotations(self.h, np.ascontiguousarray(y_body, np.uint64), out)
        return out[: (self.gamma - 1) * self.ctx.ell]

    def client_packing_keys(self, sampler: Sampler, sk):
        y_body = self.ctx.zeros(self.ctx.ell)
        y_all = self.ctx.zeros(max(1, (self.gamma - 1) * self.ctx.ell))
        self.L.io_client_packing_keys(self.h, sampler.h, np.ascontiguousarray(sk, np.uint64), y_body, y_all)
        return y_body, y_all[: (self.gamma - 1) * self.ctx.ell]


class Client:
    """Client side of the protocol (query.rs, extract.rs), for fixtures."""

    def __init__(self, ctx: Ctx, seed=0, rng_seed=1):
        self.ctx = ctx
        self.L = ctx.L
        self.sampler = Sampler(ctx.sigma, seed)
        self.rng = Rng(u64=rng_seed)
        self.sk = ctx.zeros()
        self.L.io_sk_generate(ctx.h, self.sampler.h, self.sk)

    def rlwe_encrypt(self, msg):
        ct = self.ctx.zeros(2)
        self.L.io_rlwe_encrypt(self.ctx.h, self.sampler.h, self.rng.h, self.sk,
                               np.ascontiguousarray(msg, np.uint64), ct)
        return ct

    def rgsw_encrypt(self, msg):
        out = self.ctx.zeros(4 * self.ctx.ell)
        self.L.io_rgsw_encrypt(self.ctx.h, self.sampler.h, self.rng.h, self.sk,
                               np.ascontiguousarray(msg, np.uint64), out)
        return out

    def query_seeded(self, local_idx):
        seeds = np.zeros((2 * self.ctx.ell, 32), dtype=np.uint8)
        b_rows = self.ctx.zeros(2 * self.ctx.ell)
        self.L.io_query_seeded(self.ctx.h, self.sampler.h, self.rng.h, self.sk, local_idx,
                               seeds.reshape(-1), b_rows)
        return seeds, b_rows

    def packing_keys(self, pack: Pack):
        return pack.client_packing_keys(self.sampler, self.sk)

    def decrypt(self, ct):
        return self.ctx.decrypt(self.sk, ct)

    def extract_inspiring(self, ct, entry_size):
        return self.ctx.extract_inspiring(self.sk, ct, entry_size)

    def galois_keys(self):
        """The tree-packing key-switching matrices of setup (setup.rs:164-173):
        log2(d) matrices of gadget_len rows (a, b), shape (log2 d, 2*ell, plen)."""
        ld = int(self.ctx.n).bit_length() - 1
        out = self.ctx.zeros(ld * 2 * self.ctx.ell)
        self.L.io_galois_keys(self.ctx.h, self.sampler.h, self.rng.h, self.sk, out)
        return out.reshape(ld, 2 * self.ctx.ell, self.ctx.plen)

    def extract_packed(self, ct, entry_size):
        return self.ctx.extract_packed(self.sk, ct, entry_size)


def chacha20_block(key_words, ctr_nonce):
    out = np.zeros(16, dtype=np.uint32)
    lib().io_chacha20_block(np.asarray(key_words, dtype=np.uint32), np.asarray(ctr_nonce, dtype=np.uint32), out)
    return out


def automorph_table_closed(n, t):
    out = np.zeros(n, dtype=np.int32)
    lib().io_automorph_table_closed(n, t, out)
    return out


def automorph_table_brute(ctx: Ctx, t, rng: Rng):
    out = np.zeros(ctx.n, dtype=np.int32)
    lib().io_automorph_table_brute(ctx.h, t, rng.h, out)
    return out
