"""The swap kernel's chain order equals the sequential pair order.

The reference's temperature swaps visit the pairs (i, i-1) from the hottest
down, each over all walkers at once (oracle/pt.py, swap_and_adapt).  The
device kernel instead lets each thread follow one chain of positions
x -> perm_i(x) = (m_i x + b_i) mod W through all pairs (no barrier between
pairs).  This restates both orders in numpy on random ladders, logL and
permutations and checks that the final slot tables and the per-pair
acceptance counts agree exactly.
"""
import numpy as np
import pytest

from oracle.pt import perm_units


def _sequential(members, logl, betas, perms, logu):
    T, W = members.shape
    mem = members.copy()
    counts = np.zeros(T, dtype=np.int64)
    for i in range(T - 1, 0, -1):
        m, b = perms[i]
        j = np.arange(W)
        jp = (m * j + b) % W
        sa, sb = mem[i, j].copy(), mem[i - 1, jp].copy()
        acc = logu[i, j] < (betas[i - 1] - betas[i]) * (logl[sa] - logl[sb])
        mem[i, j[acc]] = sb[acc]
        mem[i - 1, jp[acc]] = sa[acc]
        counts[i] = acc.sum()
    return mem, counts


def _chains(members, logl, betas, perms, logu):
    T, W = members.shape
    mem = members.copy()
    ll = logl[mem]                         # logL by position, swapped with the slots
    counts = np.zeros(T, dtype=np.int64)
    for j in range(W):                     # one thread per chain, in any order
        x = j
        for i in range(T - 1, 0, -1):
            m, b = perms[i]
            jp = (m * x + b) % W
            if logu[i, x] < (betas[i - 1] - betas[i]) * (ll[i, x] - ll[i - 1, jp]):
                mem[i, x], mem[i - 1, jp] = mem[i - 1, jp], mem[i, x]
                ll[i, x], ll[i - 1, jp] = ll[i - 1, jp], ll[i, x]
                counts[i] += 1
            x = jp
    return mem, counts


@pytest.mark.parametrize('T,W,seed', [(2, 8, 0), (3, 16, 1), (10, 64, 2), (7, 30, 3), (32, 20, 4)])
def test_chain_order_equals_sequential_pairs(T, W, seed):
    rng = np.random.default_rng(seed)
    members = rng.permutation(T * W).reshape(T, W)
    logl = rng.normal(scale=30.0, size=T * W) - 500.0
    betas = np.concatenate([[1.0], np.sort(rng.uniform(0.01, 0.99, T - 1))[::-1]])
    units = perm_units(W)
    perms = {i: (int(units[rng.integers(len(units))]), int(rng.integers(W))) for i in range(1, T)}
    logu = np.log(rng.uniform(size=(T, W)))
    a, ca = _sequential(members, logl, betas, perms, logu)
    b, cb = _chains(members, logl, betas, perms, logu)
    np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(ca, cb)
    assert ca[1:].sum() > 0
