"""GPU: launch schedules and the autotuner. Every compiled schedule (P2G chunk and staging buffers, P2G CTAs
per SM, G2P threads per CTA) gives the oracle's result (FP64: positions within 1e-12 m, as the order of sums is the
only difference); the autotuner's trial substeps leave the state and the scene clock untouched, and the
tuned run equals a run with a fixed schedule within the same rounding bound."""
import itertools

import numpy as np
import pytest

import ziran2020_gb300 as zr
import scenes

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [zr.F64, zr.F32])
def test_every_schedule_matches_the_oracle(prec):
    d = scenes.aniso_slab(size=(0.1, 0.05, 0.1), sigma_c=(20.0, 2.0), pull=1.0)
    o = scenes.oracle_scene(d, 8)
    o.step(12)
    r = o.state()
    big = 512 if prec == zr.F32 else 256
    # split form: (particles per staged chunk, staging buffers); fused form: one kernel, chunk = a block;
    # warp-specialised fused form: half a block per chunk, two buffers
    variants = ((0, big, 1), (0, big, 2), (0, big // 2, 2), (1, big, 0), (2, big, 0), (3, big // 2, 2))
    xtol = 1e-12 if prec == zr.F64 else 2e-6
    # G2P: threads per CTA, register budget (+1) and the halo staged by bulk copies (+2)
    for (fused, chunk, nbuf), ctas, (nt, tight) in itertools.product(variants, (1, 2), ((64, 0), (128, 0), (256, 0), (64, 1), (128, 1), (64, 2),
                                                                                        (256, 3))):
        s = scenes.gpu_scene(d, prec)
        s.set_schedule(chunk, nbuf, ctas, nt, fused=fused, g2p_tight=tight)
        s.step(12)
        sc = s.schedule()
        assert (sc["fused"], sc["chunk"], sc["buffers"], sc["g2p_threads"], sc["tuned"]) == (fused, chunk, nbuf, nt, False)
        e = scenes.errors(scenes.gpu_state(s), r)
        assert e["x"][0] < xtol, (fused, chunk, nbuf, ctas, nt, e)
        assert e["d"][0] < (1e-9 if prec == zr.F64 else 1e-3), (fused, chunk, nbuf, ctas, nt, e)


def test_autotuner_trials_leave_the_state_untouched():
    d = scenes.elastic_box(size=0.125)
    fixed = scenes.gpu_scene(d, zr.F64)
    fixed.set_autotune(0)
    tuned = scenes.gpu_scene(d, zr.F64)
    tuned.set_autotune(2)
    fixed.step(10)
    tuned.step(10)
    sc = tuned.schedule()
    assert sc["tuned"] and (sc["chunk"], sc["buffers"]) in ((256, 1), (256, 2), (128, 2), (256, 0)) and sc["g2p_threads"] in (64, 128, 256)
    assert not fixed.schedule()["tuned"]
    assert abs(tuned.time - 10 * d["dt"]) < 1e-15 and abs(fixed.time - tuned.time) < 1e-15
    e = scenes.errors(scenes.gpu_state(tuned), scenes.gpu_state(fixed))
    assert e["x"][0] < 1e-12 and e["v"][0] < 1e-9, e


def test_batch_is_tuned_once_and_cached():
    from ziran2020_gb300 import workloads

    rs = workloads.batch_recipes(seed=4, count=6, n_min=2000, n_max=20000)
    b1 = zr.Batch(zr.F32)
    for r in rs:
        b1.add_recipe(r)
    b1.step(3)
    s1 = b1.schedule()
    assert s1["tuned"]
    b2 = zr.Batch(zr.F32)
    for r in rs:
        b2.add_recipe(r)
    b2.step(3)
    assert b2.schedule() == s1  # same workload class: the cached choice
