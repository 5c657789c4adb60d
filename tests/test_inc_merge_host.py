"""CPU restatement of the hand-written incremental sort (engine_impl.cuh: k_sort_tiles, k_sort_bucket, k_sort_merge
and the head placement of k_heads_activate) and of the group-head pass (k_group_heads), checked against numpy's
stable sort on seeded inputs and edge cases.

Storage index i holds the key the particle was sorted by in the previous substep (kold, ascending) and its new
key (knew). Stayers (knew == kold) are already in key order. Storage is cut into tiles of T indices; B[j] is the
smallest stayer key in tiles >= j, and a mover with key k joins bucket b(k) = the largest j with B[j] <= k (0 if
none). Tile j's output starts after all stayers of lower tiles and movers of lower buckets; inside it a stayer
goes to its rank among the tile's stayers plus the bucket's movers with a smaller key, a mover to its rank in the
bucket (ordered by key, then storage index) plus the tile's stayers with a key not above it. The result must be
the order (key, stayers first, storage index) whatever order the movers were listed in. The GPU form is checked
against the full radix sort on the device by the GPU sort tests; this pins the index arithmetic.
"""
import bisect

import numpy as np
import pytest

NOKEY = 0xFFFFFFFF


def incremental_sort(knew, kold, T, mover_order_seed=0, maxm=None):
    n = len(knew)
    stay = knew == kold
    tiles = max(1, -(-n // T))
    t_stay = [int(stay[j * T:(j + 1) * T].sum()) for j in range(tiles)]
    t_first = []
    for j in range(tiles):
        idx = np.nonzero(stay[j * T:(j + 1) * T])[0]
        t_first.append(int(knew[j * T + idx[0]]) if len(idx) else NOKEY)
    stay_off = np.concatenate([[0], np.cumsum(t_stay)[:-1]]).astype(np.int64)
    # B[q]: the first stayer key at or after tile q (k_sort_bucket walks past tiles without a stayer); it equals the
    # suffix minimum of the tiles' first stayer keys because the stayers keep their sorted order
    B = []
    for q in range(tiles):
        r = q
        while t_first[r] == NOKEY and r + 1 < tiles:
            r += 1
        B.append(t_first[r])
    assert B == [int(v) for v in np.minimum.accumulate(np.array(t_first[::-1], dtype=np.uint64))[::-1]]
    movers = list(np.nonzero(~stay)[0])
    np.random.default_rng(mover_order_seed).shuffle(movers)  # the device's list order is arbitrary
    bucket = {}
    for i in movers:
        k = int(knew[i])
        b = max(0, bisect.bisect_right(B, k) - 1)
        bucket.setdefault(b, []).append((k, int(i)))
    bcnt = [len(bucket.get(j, [])) for j in range(tiles)]
    boff = np.concatenate([[0], np.cumsum(bcnt)[:-1]]).astype(np.int64)
    out_k = np.full(n, -1, np.int64)
    out_i = np.full(n, -1, np.int64)
    # the key before each tile's output (k_sort_merge): the largest of the lower tiles' last stayer keys and the lower
    # buckets' largest mover keys (None when nothing comes before)
    t_last = []
    for j in range(tiles):
        idx = np.nonzero(stay[j * T:(j + 1) * T])[0]
        t_last.append(int(knew[j * T + idx[-1]]) if len(idx) else NOKEY)
    preds = []
    for j in range(tiles):
        below = [v for v in t_last[:j] if v != NOKEY] + [max(k for k, _ in bucket[q]) for q in range(j) if bucket.get(q)]
        preds.append(max(below) if below else None)
    for j in range(tiles):
        S = [(int(knew[i]), i) for i in range(j * T, min(n, (j + 1) * T)) if stay[i]]
        Mv = sorted(bucket.get(j, []))
        if maxm is not None and len(Mv) > maxm:
            return None  # the device raises FLAG_SORT: the substep is repeated with a full sort
        sk, mk = [k for k, _ in S], [k for k, _ in Mv]
        base = stay_off[j] + boff[j]
        for t, (k, i) in enumerate(S):
            p = base + t + bisect.bisect_left(mk, k)
            assert out_k[p] == -1
            out_k[p], out_i[p] = k, i
        for r, (k, i) in enumerate(Mv):
            p = base + r + bisect.bisect_right(sk, k)
            assert out_k[p] == -1
            out_k[p], out_i[p] = k, i
    for j in range(tiles):  # the predecessor rule names the key the output actually holds before each tile
        base = stay_off[j] + boff[j]
        if base < n and (t_stay[j] or bcnt[j]):
            assert preds[j] == (None if base == 0 else int(out_k[base - 1])), j
    return out_k, out_i


def reference_order(knew, kold):
    """(key, stayers first, storage index)"""
    n = len(knew)
    cls = (knew != kold).astype(np.int64)
    order = np.lexsort((np.arange(n), cls, knew.astype(np.int64)))
    return knew[order].astype(np.int64), order


def group_heads(sorted_keys, group_of, T):
    """k_group_heads: per tile the head flags, compacted at the tile's prefix of head counts."""
    n = len(sorted_keys)
    g = group_of(sorted_keys)
    head = np.ones(n, bool)
    head[1:] = g[1:] != g[:-1]
    tiles = max(1, -(-n // T))
    counts = [int(head[j * T:(j + 1) * T].sum()) for j in range(tiles)]
    prefix = np.concatenate([[0], np.cumsum(counts)[:-1]])
    out = np.full(int(sum(counts)), -1, np.int64)
    for j in np.random.default_rng(3).permutation(tiles):  # tiles finish in any order; positions do not depend on it
        loc = np.nonzero(head[j * T:(j + 1) * T])[0]
        out[prefix[j]:prefix[j] + len(loc)] = j * T + loc
    return out


def scene(seed, n, move_frac, key_bits=20, spread=8):
    rng = np.random.default_rng(seed)
    kold = np.sort(rng.integers(0, 1 << key_bits, n)).astype(np.uint64)
    knew = kold.copy()
    m = rng.random(n) < move_frac
    knew[m] = np.clip(kold[m].astype(np.int64) + rng.integers(-spread * 64, spread * 64 + 1, m.sum()), 0, (1 << 31) - 1).astype(np.uint64)
    return knew, kold


@pytest.mark.parametrize("seed,n,frac,T", [(1, 10000, 0.02, 2048), (2, 4097, 0.5, 2048), (3, 3000, 1.0, 64), (4, 2000, 0.0, 64),
                                           (5, 777, 0.05, 16), (6, 50000, 0.01, 2048), (7, 5000, 0.3, 16)])
def test_incremental_sort_equals_stable_order(seed, n, frac, T):
    knew, kold = scene(seed, n, frac)
    got = incremental_sort(knew, kold, T, mover_order_seed=seed)
    want_k, want_i = reference_order(knew, kold)
    assert np.array_equal(got[0], want_k)
    assert np.array_equal(got[1], want_i)
    assert np.all(np.diff(got[0]) >= 0)


def test_movers_outside_the_stayers_key_range_and_equal_keys_across_tiles():
    T = 8
    kold = np.array([5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 7, 7, 9, 9, 9, 9, 9, 9, 9, 9, 20, 20], dtype=np.uint64)
    knew = kold.copy()
    knew[[0, 3, 11, 21]] = [1, 30, 5, 9]  # below every stayer, above every stayer, onto a key spanning two tiles
    knew[13] = 9  # unchanged (still a stayer)
    got = incremental_sort(knew, kold, T)
    want_k, want_i = reference_order(knew, kold)
    assert np.array_equal(got[0], want_k) and np.array_equal(got[1], want_i)


def test_tiles_without_stayers_in_the_middle():
    T = 16
    kold = np.arange(80, dtype=np.uint64) * 3
    knew = kold.copy()
    knew[16:48] = kold[16:48] + 1  # tiles 1 and 2 keep no stayer
    got = incremental_sort(knew, kold, T, mover_order_seed=9)
    want_k, want_i = reference_order(knew, kold)
    assert np.array_equal(got[0], want_k) and np.array_equal(got[1], want_i)


def test_a_bucket_beyond_the_merge_capacity_is_reported():
    knew, kold = scene(11, 4000, 1.0, key_bits=6)  # every particle moves into a few keys
    assert incremental_sort(knew, kold, 2048, maxm=1024) is None


def test_order_independent_of_the_movers_list_order():
    knew, kold = scene(12, 9000, 0.1)
    a = incremental_sort(knew, kold, 512, mover_order_seed=1)
    b = incremental_sort(knew, kold, 512, mover_order_seed=2)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


@pytest.mark.parametrize("T", [16, 2048])
def test_group_heads_compaction(T):
    rng = np.random.default_rng(5)
    keys = np.sort(rng.integers(0, 1 << 16, 9000))
    group_of = lambda k: k >> 6  # noqa: E731 (page = key without the 6 cell bits)
    got = group_heads(keys, group_of, T)
    g = group_of(keys)
    want = np.nonzero(np.concatenate([[True], g[1:] != g[:-1]]))[0]
    assert np.array_equal(got, want)
