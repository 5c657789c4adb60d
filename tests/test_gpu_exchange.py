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
