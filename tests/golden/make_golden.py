"""Generate the binning golden fixtures from the reference's own SPGrid code.

Runs ``oracle/_ref/spgrid_ref`` (built by ``make -C oracle ref`` from the reference tree's
Lib/SPGrid/Core sources) on seeded particle positions and stores inputs and outputs as
``tests/golden/binning_<case>.npz``. The fixtures pin, bit for bit:

* SPGrid Linear_Offset / Packed_Add / LinearToCoord for the float (4x4x4) and double (2x4x4) layouts
  (Lib/SPGrid/Core/SPGrid_Mask.h:150-245),
* the 64-bit particle sort keys, the sorted order, the particle groups and their block offsets
  (Lib/MPM/MpmSimulationBase.cpp:1531-1573),
* the active-page set produced by pollute with the reference's SPGrid_Page_Map, in first-touch order
  (Lib/MPM/MpmGrid.h:153-193, Lib/SPGrid/Core/SPGrid_Page_Map.h:61-70).

Run from the repository root:  python tests/golden/make_golden.py
"""
import os
import struct
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF_BIN = os.path.join(ROOT, "oracle", "_ref", "spgrid_ref")


def lattice(rng, lo_cell, ncell, dx, ppc_side=2, jitter=True):
    """Particles on a ppc_side^3 sub-lattice per cell, optionally jittered within each sub-cell."""
    pts = []
    sub = dx / ppc_side
    for i in range(ncell[0]):
        for j in range(ncell[1]):
            for k in range(ncell[2]):
                for a in range(ppc_side):
                    for b in range(ppc_side):
                        for c in range(ppc_side):
                            u = rng.random(3) if jitter else np.full(3, 0.5)
                            cell = np.array([lo_cell[0] + i, lo_cell[1] + j, lo_cell[2] + k], dtype=np.float64)
                            pts.append(cell * dx + (np.array([a, b, c]) + u) * sub)
    return np.array(pts)


def cases(rng):
    out = {}
    dx = 1.0 / 64
    # a jittered cube (shuffled so the input order is not spatial)
    x = lattice(rng, (20, 30, 21), (6, 5, 7), dx)
    rng.shuffle(x)
    out["jitter"] = (dx, x)
    # edges: x*inv_dx - 0.5 exactly integer, block-boundary cells, duplicate positions, tiny offsets
    e = []
    for i in range(40, 49):
        for j in range(60, 63):
            e.append([(i + 0.5) * dx, (j + 0.5) * dx, (i % 5 + 30.5) * dx])
            e.append([(i + 0.5) * dx - 1e-9, (j + 0.5) * dx + 1e-9, 31.0 * dx])
            e.append([i * dx, j * dx, (i + j) % 9 * dx + 32 * dx])
    e += [[0.7, 0.7, 0.7]] * 5
    e = np.array(e)
    rng.shuffle(e)
    out["edges"] = (dx, e)
    # wide: large coordinates to exercise high page bits (cells up to ~4000)
    dxw = 1.0 / 2048
    w = rng.random((3000, 3)) * np.array([1.9, 1.2, 1.95]) + 0.01
    out["wide"] = (dxw, w)
    # a cell size whose reciprocal is not exact in binary (1/100, 1/75): x * (1/dx) rounds in T, so positions on
    # and next to cell faces and centres land on either side of the floor depending on the T-precision product
    for name, dxo in (("odd100", 1.0 / 100), ("odd75", 1.0 / 75)):
        o = []
        for i in range(30, 42):
            for j in range(33, 36):
                for f in (0.0, 0.5):
                    for eps in (-2e-9, 0.0, 2e-9):
                        o.append([(i + f) * dxo + eps, (j + f) * dxo - eps, (i + j + f) * dxo * 0.5 + eps])
        o += list(rng.random((400, 3)) * 0.2 + 0.3)
        o = np.array(o)
        rng.shuffle(o)
        out[name] = (dxo, o)
    return out


def run_ref(precision, dx, x):
    n = x.shape[0]
    with tempfile.TemporaryDirectory() as td:
        fin, fout = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        with open(fin, "wb") as f:
            f.write(struct.pack("<qd", n, dx))
            f.write(np.ascontiguousarray(x, dtype="<f8").tobytes())
        subprocess.check_call([REF_BIN, str(precision), fin, fout])
        buf = open(fout, "rb").read()
    pos = 0

    def take(dtype, count):
        nonlocal pos
        a = np.frombuffer(buf, dtype=dtype, count=count, offset=pos)
        pos += a.nbytes
        return a.copy()

    r = {}
    r["masks"] = take("<u8", 3)
    r["bits"] = take("<i4", 5)
    r["base"] = take("<i4", 3 * n).reshape(n, 3)
    r["offset"] = take("<u8", n)
    r["key"] = take("<u8", n)
    r["sorted"] = take("<u8", n)
    r["order"] = take("<i4", n)
    ng = int(take("<i8", 1)[0])
    r["group_first"] = take("<i4", ng)
    r["group_last"] = take("<i4", ng)
    r["block_offset"] = take("<u8", ng)
    npg = int(take("<i8", 1)[0])
    r["pages"] = take("<u8", npg)
    r["coord_back"] = take("<i4", 3 * n).reshape(n, 3)
    r["packed_add"] = take("<u8", 4 * n).reshape(n, 4)
    assert pos == len(buf), (pos, len(buf))
    return r


def main():
    if not os.path.exists(REF_BIN):
        sys.exit("build the reference-linked generator first: make -C oracle ref")
    rng = np.random.default_rng(20200713)
    for name, (dx, x) in cases(rng).items():
        for precision, tag in ((4, "f32"), (8, "f64")):
            xx = x.astype(np.float32).astype(np.float64) if precision == 4 else x
            r = run_ref(precision, dx, xx)
            path = os.path.join(HERE, f"binning_{name}_{tag}.npz")
            np.savez_compressed(path, dx=np.float64(dx), x=xx, precision=np.int32(precision), **r)
            print(f"{path}: n={len(xx)} groups={len(r['group_first'])} pages={len(r['pages'])}")


if __name__ == "__main__":
    main()
