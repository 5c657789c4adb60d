"""CPU restatement of the incremental sort's merge (engine_impl.cuh: warp_lower_bound, k_inc_merge), checked
against numpy on seeded inputs and edge cases.

The merge takes the stayers (storage indices whose key did not change, in storage order, so their keys ascend)
and the movers (keys sorted stably, with their storage indices). Tile j of 1024 stayers owns the movers from the
lower bound of its first stayer key to the lower bound of the next tile's first stayer key; a stayer goes to its
stayer rank plus the movers below its key, a mover to its mover rank plus the stayers at or below its key. The
result must be the keys in ascending order with, among equal keys, the stayers first (in storage order) and then
the movers (in their sorted order): a permutation of every storage index. The GPU form is checked against the
full radix sort on the device by the GPU sort tests; this pins the index arithmetic itself, including the warp's
32-probe lower bound.
"""
import bisect

import numpy as np
import pytest

TILE = 1024


def warp_lower_bound(v, lo, hi, key):
    """The 32-lane search: each step probes 32 evenly spaced points and keeps the sub-range holding the answer."""
    while hi - lo > 32:
        step = (hi - lo + 31) // 32
        c = sum(1 for lane in range(32) if lo + lane * step < hi and v[lo + lane * step] < key)
        nlo = lo if c == 0 else lo + (c - 1) * step + 1
        nhi = hi if c == 32 else min(lo + c * step, hi)
        lo, hi = nlo, nhi
    return lo + sum(1 for lane in range(32) if lo + lane < hi and v[lo + lane] < key)


def inc_merge(keys, stay, mkeys, mvals):
    n = len(stay) + len(mkeys)
    S, M = len(stay), len(mkeys)
    out_k = np.full(n, -1, dtype=np.int64)
    out_v = np.full(n, -1, dtype=np.int64)
    tiles = max(1, (S + TILE - 1) // TILE)
    for j in range(tiles):
        a0 = j * TILE
        if a0 >= S and j > 0:
            continue
        na = max(0, min(TILE, S - a0))
        sk = [int(keys[stay[a0 + t]]) for t in range(na)]
        lo = 0 if j == 0 else warp_lower_bound(mkeys, 0, M, keys[stay[a0]])
        hi = M if a0 + TILE >= S else warp_lower_bound(mkeys, 0, M, keys[stay[a0 + TILE]])
        hi = max(hi, lo)
        for t in range(na):
            pos = a0 + t + bisect.bisect_left(mkeys, sk[t], lo, hi)
            assert 0 <= pos < n
            out_k[pos], out_v[pos] = sk[t], stay[a0 + t]
        for m in range(lo, hi):
            pos = m + a0 + bisect.bisect_right(sk, int(mkeys[m]))
            assert 0 <= pos < n
            out_k[pos], out_v[pos] = mkeys[m], mvals[m]
    return out_k, out_v


def make_case(rng, n, move_frac, key_range, dup_heavy=False):
    """Old sorted keys (storage order), then new keys: stayers keep theirs, movers get random ones."""
    hi = 8 if dup_heavy else key_range
    old = np.sort(rng.integers(0, hi, n))
    new = old.copy()
    movers = rng.random(n) < move_frac
    new[movers] = rng.integers(0, hi, movers.sum())
    stay_mask = new == old  # the partition's test: the key at that slot did not change
    stay = np.nonzero(stay_mask)[0]
    move = np.nonzero(~stay_mask)[0]
    order = np.argsort(new[move], kind="stable")
    return new, stay, new[move][order], move[order]


def expected(new, stay, mvals):
    """Key order with stayers before movers among equal keys, each group in its own order."""
    items = [(int(new[i]), 0, r, int(i)) for r, i in enumerate(stay)] + [(int(new[i]), 1, r, int(i)) for r, i in enumerate(mvals)]
    items.sort()
    return np.array([k for k, _, _, _ in items]), np.array([i for _, _, _, i in items])


@pytest.mark.parametrize("n,move_frac,key_range,dup", [
    (5000, 0.02, 1 << 20, False),  # the slab's regime: a few percent movers, spread keys
    (3000, 0.5, 1 << 12, False),  # many movers
    (2500, 0.1, 8, True),  # heavy duplicates: ties between stayers and movers
    (1, 1.0, 4, False),  # one particle, moved
    (2048, 0.0, 1 << 10, False),  # nobody moved: exactly two full tiles of stayers
    (1500, 1.0, 1 << 16, False),  # everybody moved: tile 0 alone places all movers
])
def test_merge_matches_reference_order(n, move_frac, key_range, dup):
    rng = np.random.default_rng(n + int(move_frac * 100))
    new, stay, mkeys, mvals = make_case(rng, n, move_frac, key_range, dup)
    out_k, out_v = inc_merge(new, stay, mkeys, mvals)
    ek, ev = expected(new, stay, mvals)
    assert (out_v >= 0).all() and sorted(out_v.tolist()) == list(range(n))  # a permutation of every slot
    assert (np.diff(out_k) >= 0).all()
    np.testing.assert_array_equal(out_k, ek)
    np.testing.assert_array_equal(out_v, ev)


def test_warp_lower_bound_equals_bisect():
    rng = np.random.default_rng(11)
    for size in (0, 1, 31, 32, 33, 1000, 40000):
        v = np.sort(rng.integers(0, 500, size)).tolist()
        for key in list(rng.integers(-5, 505, 40)) + ([v[0], v[-1]] if v else []):
            lo = int(rng.integers(0, size + 1))
            hi = int(rng.integers(lo, size + 1))
            assert warp_lower_bound(v, lo, hi, key) == bisect.bisect_left(v, key, lo, hi)
