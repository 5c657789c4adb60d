"""GPU: the FP64 polar decomposition that takes over from the Newton iteration for inverted or badly
conditioned F (the reference decomposes every F with its implicit-QR SVD and sign convention,
ImplicitQRSVD.h:518-558, for the corotated stress, CorotatedElasticity.cpp:56-76).

A corotated box in which some particles start inverted (det F < 0) and some nearly flat (det F > 0,
Frobenius condition number above 1e3): the GPU must count FP64 fallbacks in both precisions, keep every
value finite, and match the FP64 oracle (FP64 path: positions within 1e-12, v and F within 1e-9; FP32:
positions within 1e-5 of the unit domain, F within 1e-3)."""
import numpy as np
import pytest

import ziran2020_gb300 as zr
import scenes

pytestmark = pytest.mark.gpu


def rotation(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def degenerate_box():
    d = scenes.elastic_box(size=0.0625, seed=5, v0=(0.0, -0.5, 0.0))
    rng = np.random.default_rng(2024)
    n = len(d["m"])
    F = d["F"].reshape(n, 3, 3).copy()
    inv = rng.choice(n, n // 50, replace=False)
    rest = np.setdiff1d(np.arange(n), inv)
    flat = rng.choice(rest, n // 50, replace=False)
    for p in inv:  # inverted: one negative stretch, distinct singular values
        F[p] = rotation(rng) @ np.diag([1.08, 0.93, -0.35]) @ rotation(rng).T
    for p in flat:  # nearly flat: condition number ~ 3e3
        F[p] = rotation(rng) @ np.diag([1.02, 0.97, 5e-4]) @ rotation(rng).T
    d["F"] = F.reshape(n, 9)
    return d, inv, flat


def test_fp64_polar_fallback_matches_oracle():
    d, inv, flat = degenerate_box()
    o = scenes.oracle_scene(d, 8)
    o.step(5)
    r = o.state()
    for prec, xtol, vtol, ftol in ((zr.F64, 1e-12, 1e-9, 1e-9), (zr.F32, 1e-5, 1e-3, 1e-3)):
        s = scenes.gpu_scene(d, prec)
        s.step(5)
        g = scenes.gpu_state(s)
        for k in ("x", "v", "C", "F"):
            assert np.isfinite(g[k]).all(), (prec, k)
        st = s.stats()
        # every inverted particle takes the FP64 path in every substep; FP32 also sends the nearly flat ones
        assert st["fallbacks"] >= 5 * len(inv), (prec, st["fallbacks"])
        if prec == zr.F32:
            assert st["fallbacks"] >= 5 * (len(inv) + len(flat)), st["fallbacks"]
        e = scenes.errors(g, r)
        print(f"precision {prec}: fallbacks {st['fallbacks']}, errors vs the FP64 oracle {e}")
        assert e["x"][0] <= xtol, (prec, e)
        assert e["v"][0] <= vtol, (prec, e)
        assert e["F"][0] <= ftol, (prec, e)
