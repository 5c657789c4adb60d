"""GPU: collision objects other than sticky plates, against the FP64 oracle (AnalyticCollisionObject,
CollisionObject.cpp:67-105 multiObjectCollision, :342-406 detectAndResolveCollision; HalfSpace,
AnalyticLevelSet.cpp:318-334).

An elastic box (corotated) whose lower nodes start inside the objects: a tilted SLIP plane with friction; a
SEPARATE floor with friction, the box moving sideways and down; a corner of three walls (SLIP, moving
SEPARATE, SLIP) followed by a STICKY plane that every corner node is also inside, which the loop must skip
once three slip normals are in the basis. FP64: positions within 1e-12 of the oracle, v and F within 1e-9;
FP32: positions within 1e-5 of the unit domain."""
import numpy as np
import pytest

import ziran2020_gb300 as zr
import scenes

pytestmark = pytest.mark.gpu

CASES = {
    "tilted_slip_friction": [dict(origin=(0.5, 0.475, 0.5), normal=(0.25, 1.0, 0.1), type=zr.SLIP, friction=0.3, velocity=(0, 0, 0))],
    "separate_floor_friction": [dict(origin=(0.0, 0.472, 0.0), normal=(0.0, 1.0, 0.0), type=zr.SEPARATE, friction=0.5, velocity=(0, 0, 0))],
    "corner_then_sticky": [dict(origin=(0.0, 0.475, 0.0), normal=(0.0, 1.0, 0.0), type=zr.SLIP, friction=0.2, velocity=(0, 0, 0)),
                           dict(origin=(0.475, 0.0, 0.0), normal=(1.0, 0.0, 0.15), type=zr.SEPARATE, friction=0.1, velocity=(0.2, 0, 0)),
                           dict(origin=(0.0, 0.0, 0.478), normal=(0.1, 0.0, 1.0), type=zr.SLIP, friction=0.0, velocity=(0, 0, 0)),
                           dict(origin=(0.0, 0.49, 0.0), normal=(0.0, 1.0, 0.0), type=zr.STICKY, friction=0.0, velocity=(0, 0, 0))],
}


def box(case):
    d = scenes.elastic_box(size=0.0625, seed=3, center=(0.5, 0.5, 0.5), v0=(0.8, -1.0, 0.3) if case != "corner_then_sticky" else (-0.6, -1.0, -0.5))
    d["objects"] = CASES[case]
    return d


@pytest.mark.parametrize("case", sorted(CASES))
def test_collision_objects_match_oracle(case):
    d = box(case)
    o = scenes.oracle_scene(d, 8)
    o.step(40)
    r = o.state()
    free = scenes.elastic_box(size=0.0625, seed=3, center=(0.5, 0.5, 0.5), v0=d["v"][0])
    free["objects"] = []
    of = scenes.oracle_scene(free, 8)
    of.step(40)
    assert np.abs(of.state()["v"] - r["v"]).max() > 0.1  # the objects changed the motion
    for prec, xtol, vtol in ((zr.F64, 1e-12, 1e-9), (zr.F32, 1e-5, 1e-3)):
        s = scenes.gpu_scene(d, prec)
        s.step(40)
        e = scenes.errors(scenes.gpu_state(s), r)
        assert e["x"][0] <= xtol, (case, prec, e)
        assert e["v"][0] <= vtol, (case, prec, e)
        if prec == zr.F64:
            assert e["F"][0] <= 1e-9, (case, e)
