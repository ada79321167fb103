"""Restatement of the device-side client's randomness (test helper): the
discrete Gaussian of the crate's sigma with tail cut ceil(6 sigma)
(math/gaussian.rs:31-38, 88-104) drawn by inverse cumulative table from
ChaCha20 keystream blocks, 8 samples per block."""
import math

import numpy as np

N = 2048
SIGMA = 6.4
Q = (268369921, 249561089)


def cdt_table(sigma):
    """Cumulative |e| table of the discrete Gaussian on [-T, T], T = ceil(6 sigma)
    (math/gaussian.rs:31-38, 88-104): cdt[j] = floor(2^63 P(|e| <= j)), j < T."""
    T = math.ceil(sigma * 6.0)
    s2 = 2.0 * sigma * sigma
    total = sum(math.exp(-x * x / s2) for x in range(-T, T + 1))
    cum, out = 0.0, []
    for j in range(T):
        cum += (2.0 if j else 1.0) * math.exp(-j * j / s2) / total
        out.append(int(math.ldexp(min(cum, 1.0), 63)))
    return np.array(out, dtype=np.uint64), T


def gaussian_blocks(key, blk0, n=N):
    """n discrete Gaussian samples, 8 per keystream block blk0, blk0 + 1, ..."""
    from oracle import oracle as O

    cdt, T = cdt_table(SIGMA)
    words = []
    for t in range(n // 8):
        c = blk0 + t
        words.append(O.chacha20_block(key, [c & 0xFFFFFFFF, c >> 32, 0, 0]))
    w64 = np.concatenate(words).astype(np.uint64)
    u = w64[0::2] | (w64[1::2] << np.uint64(32))
    mag = u & np.uint64((1 << 63) - 1)
    j = np.minimum(np.searchsorted(cdt, mag, side="right"), T).astype(np.int64)
    neg = (u >> np.uint64(63)).astype(bool) & (j != 0)
    return np.where(neg, -j, j)


def residues(e):
    """Signed coefficients -> residue-major u64 poly."""
    return np.concatenate([(e % Q[0]), (e % Q[1])]).astype(np.uint64)
