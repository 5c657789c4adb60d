"""GPU: the continuous-batching request loop. Each request's result equals the same scene run alone
(differences come only from the order of atomic grid sums: FP32 positions within 1e-5 m, FP64 within
1e-11 m), the memory budget bounds the resident set, and oversized requests are refused."""
import numpy as np
import pytest

import ziran2020_gb300 as zr
from ziran2020_gb300 import workloads

pytestmark = pytest.mark.gpu


def small_requests(seed, count):
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        n = int(rng.integers(3000, 20000))
        r = workloads.elastic_family(rng, n) if k % 2 == 0 else workloads.slab_family(rng, n)
        out.append((r, int(rng.integers(15, 45))))
    return out


def run_alone(prec, r, substeps):
    s = zr.Scene(prec)
    s.from_recipe(r)
    s.step(substeps)
    return s.get("x"), s.get("d")


@pytest.mark.parametrize("prec,tol", [(zr.F32, 1e-5), (zr.F64, 1e-11)])
def test_each_result_is_the_same_alone_and_in_the_mix(prec, tol):
    reqs = small_requests(3, 7)
    sv = zr.Server(prec, budget_bytes=2e9, tick_substeps=8, max_scenes=16)
    ids = []
    # staggered arrivals: two requests first, the others while those run
    for k, (r, steps) in enumerate(reqs):
        ids.append(sv.submit(r, steps))
        if k >= 1:
            sv.tick()
    for _ in range(200):
        running, queued, _ = sv.tick()
        if running == 0 and queued == 0:
            break
    for rid, (r, steps) in zip(ids, reqs):
        info = sv.request(rid)
        assert info["state"] == zr.Server.DONE and info["latency_s"] > 0
        x_alone, d_alone = run_alone(prec, r, steps)
        x_mix = sv.result(rid, "x")
        assert np.abs(x_mix - x_alone).max() <= tol, (rid, np.abs(x_mix - x_alone).max())
        assert np.abs(sv.result(rid, "d") - d_alone).max() <= (1e-4 if prec == zr.F32 else 1e-10)


def test_budget_bounds_the_resident_set_and_refuses_oversized_requests():
    rng = np.random.default_rng(5)
    reqs = [(workloads.elastic_family(rng, 8000), 12) for _ in range(6)]  # equal sizes: the bound is exact
    n = zr.recipe_count(reqs[0][0])
    per_scene = n * (2 * (30 * 4 + 4) + 28 + 27 * 4 * 9 / 8 + 24) + 8 * (n / 256 + 64) * (10 * 64 * 4 + 64)  # the server's estimate
    sv = zr.Server(zr.F32, budget_bytes=2.5 * per_scene, tick_substeps=5, max_scenes=64)
    for r, steps in reqs:
        sv.submit(r, steps)
    peak = 0
    for _ in range(400):
        running, queued, _ = sv.tick()
        peak = max(peak, running)
        if running == 0 and queued == 0:
            break
    assert peak == 2
    big = zr.recipe(zr.RECIPE_ELASTIC_BOX, size=(0.5, 0.5, 0.5))
    with pytest.raises(zr.ZrError) as ei:
        sv.submit(big, 10)
    assert ei.value.code == zr.ZR_ERR_BUDGET
