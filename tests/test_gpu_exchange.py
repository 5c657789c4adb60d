"""GPU: zr_scene_exchange_state (download the state, upload another, in one call) equals zr_scene_get_state followed
by zr_scene_set_state, bit for bit, with pinned host buffers (one kernel, both link directions at once), with
pageable ones (one direction after the other) and with one of each; overlapping buffers are refused."""
import numpy as np
import pytest

import ziran2020_gb300 as zr
import scenes

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _buf(n, dtype, pinned):
    if pinned:
        t = torch.zeros((n, 25), dtype=torch.float32 if dtype == np.float32 else torch.float64).pin_memory()
        return t.numpy()
    return np.zeros((n, 25), dtype)


@pytest.mark.parametrize("prec", [zr.F32, zr.F64])
@pytest.mark.parametrize("pin_in,pin_out", [(True, True), (False, False), (True, False)])
def test_exchange_equals_get_then_set(prec, pin_in, pin_out):
    dtype = np.float32 if prec == zr.F32 else np.float64
    d = scenes.aniso_slab(size=(0.1, 0.05, 0.1), sigma_c=(20.0, 2.0), pull=1.0)
    s1 = scenes.gpu_scene(d, prec)
    s2 = scenes.gpu_scene(d, prec)
    s1.step(3)
    s2.step(7)
    n = s1.count
    x1 = s1.get_state(np.zeros((n, 25), dtype))
    x2 = s2.get_state(np.zeros((n, 25), dtype))
    assert not np.array_equal(x1, x2)
    a = _buf(n, dtype, pin_in)
    a[:] = x1
    out = _buf(n, dtype, pin_out)
    s2.exchange_state(a, out)
    assert np.array_equal(out, x2)  # the state from before the call
    back = s2.get_state(np.zeros((n, 25), dtype))
    assert np.array_equal(back, x1)  # the uploaded state
    # the keys were rebuilt from the new positions: both scenes continue alike (the order of the atomic sums only)
    s1.step(4)
    s2.step(4)
    tol = 1e-12 if prec == zr.F64 else 1e-5
    assert np.abs(s1.get("x") - s2.get("x")).max() < tol
    assert np.abs(s1.get("d") - s2.get("d")).max() < (1e-10 if prec == zr.F64 else 1e-4)


def test_exchange_refuses_overlapping_buffers():
    d = scenes.elastic_box(size=0.0625)
    s = scenes.gpu_scene(d, zr.F32)
    a = _buf(s.count, np.float32, True)
    s.get_state(a)
    with pytest.raises(Exception):
        s.exchange_state(a, a)
    with pytest.raises(ValueError):
        s.exchange_state(a, np.zeros((s.count, 25), np.float64))


@pytest.mark.parametrize("prec", [zr.F32, zr.F64])
@pytest.mark.parametrize("pinned", [True, False])
def test_step_stream_equals_set_step_get(prec, pinned):
    """Four jobs with different input states: each result equals zr_scene_set_state, one substep and
    zr_scene_get_state run one after the other (up to the order of the atomic grid sums)."""
    dtype = np.float32 if prec == zr.F32 else np.float64
    d = scenes.aniso_slab(size=(0.1, 0.05, 0.1), sigma_c=(20.0, 2.0), pull=1.0)
    src = scenes.gpu_scene(d, prec)
    n = src.count
    states = []
    for k in range(4):
        src.step(2)
        states.append(src.get_state(np.zeros((n, 25), dtype)))
    ins = [_buf(n, dtype, pinned) for _ in range(4)]
    outs = [_buf(n, dtype, pinned) for _ in range(4)]
    for a, st in zip(ins, states):
        a[:] = st
    s = scenes.gpu_scene(d, prec)
    s.step_stream(ins, outs)
    assert s.stream_reruns == 0  # every job after the first ran on the pipelined path
    ref = scenes.gpu_scene(d, prec)
    tol = 1e-12 if prec == zr.F64 else 1e-5
    for a, o in zip(ins, outs):
        ref.set_state(a)
        ref.step(1)
        want = ref.get_state(np.zeros((n, 25), dtype))
        assert np.abs(o[:, :3] - want[:, :3]).max() < tol  # positions
        assert np.abs(o - want).max() < (1e-9 if prec == zr.F64 else 2e-3)  # every field (F, C carry the sum order more)
    # the scene holds the last job's result
    assert np.abs(s.get_state(np.zeros((n, 25), dtype)) - outs[-1]).max() == 0


def test_step_stream_stops_at_a_failing_job():
    """A job whose input leaves the domain fails; the earlier results are written, the error is reported and the
    scene holds the failing job's input."""
    d = scenes.elastic_box(size=0.0625)
    s = scenes.gpu_scene(d, zr.F32)
    n = s.count
    good = s.get_state(np.zeros((n, 25), np.float32))
    bad = good.copy()
    bad[:, 0] += 2.0  # positions past the domain
    ins = [_buf(n, np.float32, True) for _ in range(3)]
    outs = [_buf(n, np.float32, True) for _ in range(3)]
    ins[0][:] = good
    ins[1][:] = bad
    ins[2][:] = good
    with pytest.raises(Exception):
        s.step_stream(ins, outs)
    assert np.abs(outs[0][:, :3] - good[:, :3]).max() < 1e-2  # the first job ran
    assert 0 < np.abs(outs[0] - good).max()
    assert np.array_equal(s.get_state(np.zeros((n, 25), np.float32)), bad)


@pytest.mark.parametrize("bad_job", [2, 5])
def test_step_stream_recovers_the_jobs_after_a_failure_inside_the_pipeline(bad_job):
    """Jobs after the first run without a host check between them; a job whose substep aborts (a particle pushed
    more than a cell in one substep) makes the later ones run again the safe way. Every job before the failing one
    matches the one-by-one result, and the failure is reported."""
    d = scenes.elastic_box(size=0.0625)
    s = scenes.gpu_scene(d, zr.F64)
    n = s.count
    good = s.get_state(np.zeros((n, 25)))
    ref = scenes.gpu_scene(d, zr.F64)
    want = []
    for k in range(6):
        ref.set_state(good)
        ref.step(1)
        want.append(ref.get_state(np.zeros((n, 25))))
    fast = good.copy()
    fast[:, 4] = -300.0  # v_y: 3e-2 per substep, more than a cell of 1/64
    ins = [_buf(n, np.float64, True) for _ in range(6)]
    outs = [_buf(n, np.float64, True) for _ in range(6)]
    for k in range(6):
        ins[k][:] = fast if k == bad_job else good
    with pytest.raises(Exception):
        s.step_stream(ins, outs)
    assert s.stream_reruns == 6 - bad_job  # the failing job and the ones after it ran again the safe way
    for k in range(bad_job):
        assert np.abs(outs[k] - want[k]).max() < 1e-9, k


def test_step_stream_refuses_an_output_that_is_a_later_input():
    d = scenes.elastic_box(size=0.0625)
    s = scenes.gpu_scene(d, zr.F32)
    a = _buf(s.count, np.float32, True)
    b = _buf(s.count, np.float32, True)
    s.get_state(a)
    b[:] = a
    with pytest.raises(Exception):
        s.step_stream([a, b], [b, a])  # job 0 would write the input of job 1
    s.step_stream([a, b], [a, b])  # in place is fine
