"""GPU: snapshots and the reference driver's frames with CFL restarts (SimulationBase.h:149-187, 275-354;
MpmSimulationBase.cpp:1060-1114, 1480-1510). A state image restores the scene bit for bit; stepping on from
it repeats the original run (the order of atomic sums is the only difference); frames land on their
boundaries exactly; a substep that breaks the CFL bound restarts its frame with dt halved, and the result
equals a run started with the halved dt."""
import numpy as np
import pytest

import ziran2020_gb300 as zr
import scenes

pytestmark = pytest.mark.gpu

FIELDS = ("x", "v", "C", "F", "d")
# replay tolerances, relative to max(1, |field|): the order of atomic sums differs between runs; C = B 4/dx^2
# carries the grid velocities' rounding times ~4/dx
TOL = {zr.F64: {"x": 1e-12, "v": 1e-11, "C": 1e-9, "F": 1e-11, "d": 1e-10},
       zr.F32: {"x": 1e-6, "v": 1e-5, "C": 1e-4, "F": 1e-5, "d": 1e-4}}


def state(s):
    return {f: s.get(f) for f in FIELDS}


@pytest.mark.parametrize("prec", [zr.F64, zr.F32])
def test_snapshot_restores_exactly_and_replays(prec):
    tol = TOL[prec]
    d = scenes.aniso_slab(size=(0.08, 0.04, 0.08), sigma_c=(20.0, 2.0), pull=1.0)
    s = scenes.gpu_scene(d, prec)
    s.set_autotune(0)
    s.step(5)
    t5, saved = s.time, state(s)
    image = s.save_state()
    assert len(image) == 48 + len(d["m"]) * 29 * (8 if prec == zr.F64 else 4)  # x v C F d m V0 sigma_c, D~ history
    s.step(10)
    first = state(s)
    s.load_state(image)
    assert s.time == t5
    for f in FIELDS:
        assert np.array_equal(s.get(f), saved[f]), f
    s.step(10)
    for f in FIELDS:
        assert np.abs(s.get(f) - first[f]).max() <= tol[f] * max(1.0, np.abs(first[f]).max()), f


def test_state_file_into_a_fresh_scene_and_rejections(tmp_path):
    d = scenes.elastic_box(size=0.0625)
    a = scenes.gpu_scene(d, zr.F64)
    a.step(7)
    path = str(tmp_path / "frame7.zrstate")
    a.write_state(path)
    b = scenes.gpu_scene(d, zr.F64)  # built the same way, then read, as the reference's restart does
    b.read_state(path)
    assert b.time == a.time
    for f in FIELDS:
        assert np.array_equal(b.get(f), a.get(f)), f
    image = a.save_state()
    c32 = scenes.gpu_scene(d, zr.F32)
    with pytest.raises(zr.ZrError) as ei:
        c32.load_state(image)
    assert ei.value.code == zr.ZR_ERR_ARG  # other precision
    with pytest.raises(zr.ZrError):
        b.load_state(image[: len(image) // 2])  # truncated
    with pytest.raises(zr.ZrError):
        b.load_state(b"NOTSTATE" + image[8:])
    other = scenes.gpu_scene(scenes.elastic_box(size=0.125), zr.F64)
    with pytest.raises(zr.ZrError):
        other.load_state(image)  # different particle count


def test_frames_hit_boundaries_and_cfl_restart_halves_dt():
    # v = 30 m/s at dt = 1e-3 moves 3 cells (dx = 1/64): the first substep breaks the bound; dt = 5e-4 moves
    # 0.96 cell and passes after one restart
    d = scenes.elastic_box(size=0.0625, v0=(0.0, -30.0, 0.0), dt=1e-3, gravity=(0.0, 0.0, 0.0), ground=-1.0, center=(0.5, 0.8, 0.5))
    frame_dt = 1.0 / 240
    s = scenes.gpu_scene(d, zr.F64)
    restarts = s.advance_frames(2, frame_dt, min_dt=1e-5)
    assert restarts == 1
    assert abs(s.time - 2 * frame_dt) < 1e-15
    ref = scenes.gpu_scene(dict(d, dt=5e-4), zr.F64)
    assert ref.advance_frames(2, frame_dt, min_dt=1e-5) == 0
    assert abs(ref.time - s.time) < 1e-15
    for f in FIELDS:
        assert np.abs(s.get(f) - ref.get(f)).max() <= TOL[zr.F64][f] * max(1.0, np.abs(ref.get(f)).max()), f


def test_cfl_derived_dt_needs_no_restart():
    d = scenes.elastic_box(size=0.0625, v0=(0.0, -30.0, 0.0), dt=1e-3, gravity=(0.0, 0.0, 0.0), ground=-1.0, center=(0.5, 0.8, 0.5))
    s = scenes.gpu_scene(d, zr.F32)
    assert s.advance_frames(3, 1.0 / 240, min_dt=1e-5, cfl_dt=True) == 0
    assert abs(s.time - 3.0 / 240) < 1e-6
