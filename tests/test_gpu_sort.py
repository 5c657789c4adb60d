"""GPU: the incremental sort (stayers already in order, movers sorted and merged) against the full radix sort
and the oracle. The merge orders items by (key, storage index), which is the stable sort's order, so the two
sorts give the same particle order; results differ only by the order of atomic grid sums between runs."""
import os

import numpy as np
import pytest

import ziran2020_gb300 as zr
import scenes

pytestmark = pytest.mark.gpu


def run(desc, prec, steps, sort=None):
    old = os.environ.get("ZR_SORT")
    if sort:
        os.environ["ZR_SORT"] = sort
    try:
        s = scenes.gpu_scene(desc, prec)  # the engine reads ZR_SORT when the scene is first stepped
        s.set_autotune(0)
        s.step(steps)
    finally:
        if sort:
            if old is None:
                del os.environ["ZR_SORT"]
            else:
                os.environ["ZR_SORT"] = old
    return s


def test_incremental_sort_matches_full_sort():
    d = scenes.aniso_slab(size=(0.1, 0.05, 0.1), sigma_c=(20.0, 2.0), pull=1.0)
    inc = run(d, zr.F64, 30)
    full = run(d, zr.F64, 30, sort="full")
    for f, tol in (("x", 1e-12), ("v", 1e-9), ("F", 1e-9), ("d", 1e-9)):
        assert np.abs(inc.get(f) - full.get(f)).max() <= tol, f


@pytest.mark.parametrize("prec", [zr.F64, zr.F32])
def test_many_movers_grow_the_buffer_and_match_the_oracle(prec):
    """40 m/s at dt = 1e-4 and dx = 1/64 moves every particle 0.26 cell per substep: about a quarter of them
    change cell each substep, more than the first mover buffer (1/16 of the particles) holds. The substep is
    repeated with a larger buffer; the result still matches the FP64 oracle."""
    d = scenes.elastic_box(size=0.25, v0=(0.0, -40.0, 0.0), gravity=(0.0, 0.0, 0.0), ground=-1.0, center=(0.5, 0.7, 0.5))
    assert len(d["m"]) == 32768  # the first mover buffer holds 4096
    s = run(d, prec, 12)
    o = scenes.oracle_scene(d, 8)
    o.step(12)
    e = scenes.errors(scenes.gpu_state(s), o.state())
    assert e["x"][0] < (1e-12 if prec == zr.F64 else 1e-5), e
    assert d["x"][:, 1].min() - o.state()["x"][:, 1].min() > 0.04  # the cube moved ~5 cm


def test_mover_overflow_after_a_slow_phase_matches_full_sort():
    """A slow phase lets the mover buffer shrink and fills every sort buffer with real indices; then the velocity
    jumps (a state write that keeps the sort base) so the next substeps have far more movers than the buffer
    holds. They are repeated with a larger buffer; the run equals the same run with the full sort."""
    d = scenes.elastic_box(size=0.25, v0=(0.0, -0.5, 0.0), gravity=(0.0, 0.0, 0.0), ground=-1.0, center=(0.5, 0.7, 0.5))
    out = []
    for sort in (None, "full"):
        old = os.environ.get("ZR_SORT")
        if sort:
            os.environ["ZR_SORT"] = sort
        try:
            s = scenes.gpu_scene(d, zr.F64)
            s.set_autotune(0)
            s.step(40)
            v = s.get("v")
            v[:, 1] = -40.0
            s.set("v", v)
            s.step(10)
            out.append({f: s.get(f) for f in ("x", "v", "F")})
        finally:
            if sort:
                if old is None:
                    del os.environ["ZR_SORT"]
                else:
                    os.environ["ZR_SORT"] = old
    for f, tol in (("x", 1e-12), ("v", 1e-9), ("F", 1e-9)):
        assert np.abs(out[0][f] - out[1][f]).max() <= tol, f
