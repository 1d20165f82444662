"""Philox4x32-10 in numpy (oracle; TEST INFRASTRUCTURE ONLY).

Restates the published counter-based generator of Salmon, Moraes, Dror &
Shaw, "Parallel random numbers: as easy as 1, 2, 3" (SC'11): ten rounds of
two 32x32->64 multiplies with the round keys bumped by the Weyl constants.
It reproduces, word for word, the device generator that drives the GPU
sampler, so an oracle run fed with these words walks exactly the same
chain.  Counter layout (shared with the device): (index, iter_lo, purpose,
iter_hi), key = (seed_lo, seed_hi).
"""
from __future__ import annotations

import numpy as np

M0, M1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
W0, W1 = np.uint64(0x9E3779B9), np.uint64(0xBB67AE85)
MASK = np.uint64(0xFFFFFFFF)

STRETCH0 = 1
SWAP_PERM = 3
SWAP_ACC = 4


def philox4x32_10(c0, c1, c2, c3, k0, k1):
    """Vectorised over broadcastable uint32 counters; returns 4 uint32 arrays."""
    x = [np.asarray(v, dtype=np.uint64) & MASK for v in (c0, c1, c2, c3)]
    x = np.broadcast_arrays(*x)
    x = [v.copy() for v in x]
    k0 = np.uint64(k0) & MASK
    k1 = np.uint64(k1) & MASK
    for _ in range(10):
        p0 = M0 * x[0]
        p1 = M1 * x[2]
        hi0, lo0 = p0 >> np.uint64(32), p0 & MASK
        hi1, lo1 = p1 >> np.uint64(32), p1 & MASK
        x = [(hi1 ^ x[1] ^ k0) & MASK, lo1, (hi0 ^ x[3] ^ k1) & MASK, lo0]
        k0 = (k0 + W0) & MASK
        k1 = (k1 + W1) & MASK
    return [v.astype(np.uint32) for v in x]


def draw(seed, index, it, purpose):
    seed = int(seed) & ((1 << 64) - 1)
    it = np.asarray(it, dtype=np.uint64)
    return philox4x32_10(index, it & MASK, purpose, it >> np.uint64(32),
                         seed & 0xFFFFFFFF, seed >> 32)


def u53(a, b):
    """Uniform in [0,1) from the top 27 + 26 bits of two words."""
    k = ((np.asarray(a, dtype=np.uint64) >> np.uint64(5)) << np.uint64(26)) | \
        (np.asarray(b, dtype=np.uint64) >> np.uint64(6))
    return k.astype(np.float64) * (1.0 / 9007199254740992.0)


def u32u(a):
    return (np.asarray(a, dtype=np.float64) + 0.5) * (1.0 / 4294967296.0)


def mulhi(a, n):
    """floor(a * n / 2^32) for uint32 a."""
    return ((np.asarray(a, dtype=np.uint64) * np.uint64(n)) >> np.uint64(32)).astype(np.int64)
