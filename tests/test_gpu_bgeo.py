"""GPU: a scene's frame file (zr_scene_write_bgeo) holds its particles in the caller's order: positions, velocity,
damage and the current fibre director a_1 = R e1 (R from F's polar decomposition), as float32, read back with
the independent reader in tests/bgeo_format.py."""
import numpy as np
import pytest

import ziran2020_gb300 as zr
import scenes
from bgeo_format import read_bgeo

pytestmark = pytest.mark.gpu


def polar_R(F):
    U, _, Vt = np.linalg.svd(F)
    R = U @ Vt
    if np.linalg.det(R) < 0:
        U[:, -1] *= -1
        R = U @ Vt
    return R


def test_scene_frame_file(tmp_path):
    d = scenes.aniso_slab(size=(0.1, 0.05, 0.1), sigma_c=(20.0, 2.0), pull=1.0)
    s = scenes.gpu_scene(d, zr.F64)
    s.step(20)
    p = tmp_path / "anisoFrax_000.bgeo"
    s.write_bgeo(str(p), v=True, d=True, a1=True)
    g = read_bgeo(str(p))
    f32 = lambda a: a.astype(np.float32).astype(np.float64)  # noqa: E731
    assert np.array_equal(g["P"], f32(s.get("x")))
    assert np.array_equal(g["v"], f32(s.get("v")))
    assert np.array_equal(g["d"], f32(s.get("d")))
    F = s.get("F").reshape(-1, 3, 3)
    want = np.stack([polar_R(f)[:, 0] for f in F])
    assert np.abs(g["a_1"] - want).max() < 1e-6
    assert g["d"].max() > 0  # the frame carries grown damage
    q = tmp_path / "partio_000.bgeo"
    s.write_bgeo(str(q))  # positions only, as writePartio
    assert set(read_bgeo(str(q))) == {"P", "w"}
