"""CPU check of the shared-memory node tiles that P2G and the implicit damage solve accumulate into
(engine_impl.cuh: OffsetTiles, add_to_offset_tile, flush_offset_tiles and their *_cg forms).

A CTA has one thread per (cell, stencil x-offset ii): thread t has ii = t // nodes and cell c = t % nodes, the
cell's coordinates taken from c as the block layout's element index (x-major, z fastest). Each thread adds its
9 nodes (cx + ii, cy + jj, cz + kk) into tile ii at (cx, cy + jj, cz + kk), one (jj, kk) step at a time, with a
plain read-modify-write. That is race-free only if, within a step, the lanes of a warp touch distinct entries
and no two warps touch the same tile; the flush must read every tile entry once and give the same node sums
as one direct accumulation. Both block layouts are checked: 4x4x4 (FP32) and 2x4x4 (FP64).
"""
import numpy as np
import pytest

LAYOUTS = {"f32": (4, 4, 4), "f64": (2, 4, 4)}


def threads(sx, sy, sz):
    nodes = sx * sy * sz
    ybits, zbits = sy.bit_length() - 1, sz.bit_length() - 1
    out = []
    for t in range(3 * nodes):
        ii, c = divmod(t, nodes)
        out.append((t, ii, c >> (zbits + ybits), (c >> zbits) & (sy - 1), c & (sz - 1)))
    return out


@pytest.mark.parametrize("name", sorted(LAYOUTS))
def test_warps_touch_disjoint_tile_entries(name):
    sx, sy, sz = LAYOUTS[name]
    th = threads(sx, sy, sz)
    assert len(th) % 32 == 0  # whole warps: every lane reaches each __syncwarp
    warps = [th[w:w + 32] for w in range(0, len(th), 32)]
    for warp in warps:
        assert len({ii for _, ii, _, _, _ in warp}) == 1  # one stencil offset per warp
        for jj in range(3):
            for kk in range(3):
                entries = [(cx, cy + jj, cz + kk) for _, _, cx, cy, cz in warp]
                assert len(set(entries)) == 32  # one step: distinct entries within the warp
    by_offset = {}
    for warp in warps:
        by_offset.setdefault(warp[0][1], []).append({cx for _, _, cx, _, _ in warp})
    for ii, xsets in by_offset.items():
        seen = set()
        for xs in xsets:
            assert not (xs & seen)  # warps of one offset cover disjoint x: no two warps share an entry
            seen |= xs


@pytest.mark.parametrize("name", sorted(LAYOUTS))
def test_flush_reads_each_entry_once_and_matches_direct_sums(name):
    sx, sy, sz = LAYOUTS[name]
    TX, TY, TZ = sx + 2, sy + 2, sz + 2
    rng = np.random.default_rng(7)
    th = threads(sx, sy, sz)
    contrib = {(t, jj, kk): rng.standard_normal() for t, *_ in th for jj in range(3) for kk in range(3)}
    direct = np.zeros((TX, TY, TZ))
    tiles = np.zeros((3, sx, TY, TZ))
    for t, ii, cx, cy, cz in th:
        for jj in range(3):
            for kk in range(3):
                v = contrib[(t, jj, kk)]
                direct[cx + ii, cy + jj, cz + kk] += v
                tiles[ii, cx, cy + jj, cz + kk] += v
    reads = np.zeros_like(tiles, dtype=int)
    flushed = np.zeros((TX, TY, TZ))
    # P2G's flush: z columns split at the block boundary (sz + 2 nodes: sz, then 2), offsets summed per column
    for X in range(TX):
        for Y in range(TY):
            for z0, n in ((0, sz), (sz, 2)):
                for ii in range(3):
                    xl = X - ii
                    if 0 <= xl < sx:
                        flushed[X, Y, z0:z0 + n] += tiles[ii, xl, Y, z0:z0 + n]
                        reads[ii, xl, Y, z0:z0 + n] += 1
    assert (reads == 1).all()
    np.testing.assert_allclose(flushed, direct, rtol=1e-12, atol=1e-12)
    # the implicit solve's flush walks the nodes one by one: the same sums
    per_node = np.zeros_like(direct)
    for X in range(TX):
        for ii in range(3):
            if 0 <= X - ii < sx:
                per_node[X] += tiles[ii, X - ii]
    np.testing.assert_allclose(per_node, direct, rtol=1e-12, atol=1e-12)


def test_tile_footprint_keeps_three_fused_ctas_per_sm():
    # FP32 fused P2G: payload 26 fields x (512 + 64) words, three per-offset tiles of 6 fields, the chunk's cell
    # table; three CTAs (plus 1 KB reserved each) must fit the 228 KB of shared memory an SM has
    sx, sy, sz = LAYOUTS["f32"]
    tile_bytes = 4 * 3 * 6 * sx * (sy + 2) * (sz + 2)
    payload = 4 * 26 * (512 + 512 // 8)
    static_other = 512 + 2 * 2 * 64 + 64  # cellof, cfirst/clast, scalars (approx.)
    assert 3 * (payload + tile_bytes + static_other + 1024) <= 228 * 1024
