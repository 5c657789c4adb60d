"""CPU: the .bgeo frame writer (zr_write_bgeo) round-trips through an independent reader of the format
(tests/bgeo_format.py): header counts, attribute names and sizes, float32 values, w = 1, end bytes."""
import numpy as np

import ziran2020_gb300 as zr
from bgeo_format import read_bgeo


def test_bgeo_round_trip(tmp_path):
    rng = np.random.default_rng(4)
    n = 1000
    x = rng.random((n, 3))
    a1 = rng.normal(size=(n, 3))
    d = rng.random(n)
    p = tmp_path / "frame.bgeo"
    zr.write_bgeo(str(p), x, {"a_1": a1, "d": d})
    g = read_bgeo(str(p))
    assert np.array_equal(g["P"], x.astype(np.float32).astype(np.float64))
    assert np.array_equal(g["a_1"], a1.astype(np.float32).astype(np.float64))
    assert np.array_equal(g["d"], d.astype(np.float32).astype(np.float64))
    assert np.all(g["w"] == 1.0)


def test_bgeo_positions_only_and_empty(tmp_path):
    p = tmp_path / "pos.bgeo"
    zr.write_bgeo(str(p), np.array([[0.1, 0.2, 0.3]]))
    g = read_bgeo(str(p))
    assert set(g) == {"P", "w"} and g["P"].shape == (1, 3)
    q = tmp_path / "empty.bgeo"
    zr.write_bgeo(str(q), np.zeros((0, 3)))
    assert read_bgeo(str(q))["P"].shape == (0, 3)
    assert (tmp_path / "empty.bgeo").read_bytes()[:5] == b"BgeoV"
