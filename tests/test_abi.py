"""CPU: the C-ABI library builds, loads and exports every entry point include/ziran_gb300.h declares;
host-only helpers behave. No device compute runs here."""
import ctypes
import os
import re

import numpy as np

import ziran2020_gb300 as zr

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if h.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", h)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names |= set(re.findall(r"\b(zr_[a-z0-9_]+)\s*\(", txt))
    return names


def test_library_exports_every_declared_symbol():
    L = zr.load_library()
    names = declared_symbols()
    assert len(names) > 30
    missing = [n for n in sorted(names) if not hasattr(L, n)]
    assert not missing, missing


def test_library_is_in_tree_and_static_cudart():
    p = zr.library_path()
    assert p.startswith(os.path.join(ROOT, "ziran2020_gb300"))
    assert os.path.exists(p)


def test_recipe_counts():
    assert zr.recipe_count(zr.recipe(zr.RECIPE_ELASTIC_BOX)) == 32768
    assert zr.recipe_count(zr.recipe(zr.RECIPE_ANISO_SLAB)) == 425984
    assert zr.recipe_count(zr.recipe(zr.RECIPE_ANISO_SLAB, dx=1 / 256, l0=0.5 / 256)) == 3407872


def test_recipe_is_seeded_and_fibres_follow_vmf():
    r = zr.recipe(zr.RECIPE_ANISO_SLAB, size=(0.1, 0.05, 0.1))
    a, b = zr.recipe_generate(r), zr.recipe_generate(r)
    assert np.array_equal(a["x"], b["x"]) and np.array_equal(a["F"], b["F"])
    F = a["F"].reshape(-1, 3, 3)
    assert np.abs(np.einsum("nij,nkj->nik", F, F) - np.eye(3)).max() < 1e-12
    assert np.abs(np.linalg.det(F) - 1).max() < 1e-12
    # vMF(kappa=20) about +x: mean cosine = coth(20) - 1/20
    assert abs(F[:, 0, 0].mean() - (1 / np.tanh(20) - 1 / 20)) < 0.01
    assert abs(a["sigma_c"].mean() - 400) < 5 and abs(a["sigma_c"].std() - 40) < 5


def test_rotated_F_rule():
    F = zr.rotated_F([0, 0, 1.0])  # director along z: second column is e1 (MpmParticleHandleBase.cpp:242-244)
    np.testing.assert_allclose(F[:, 0], [0, 0, 1])
    np.testing.assert_allclose(F[:, 1], [1, 0, 0])
    F = zr.rotated_F([1.0, 0, 0])
    np.testing.assert_allclose(F, np.eye(3), atol=1e-15)


def test_nhb_sigma_crit_matches_formula():
    E, nu, p = 5e4, 0.25, 0.05
    lam = E * nu / ((1 + nu) * (1 - 2 * nu))
    mu = E / (2 * (1 + nu))
    kappa = 0.666666 * mu + lam
    J = (1 + p) ** 3
    assert abs(zr.nhb_sigma_crit(E, nu, p) - kappa / 2 * ((J * J - 1) / 2 - np.log(J))) < 1e-9


def test_errors_without_device_are_reported_not_raised_in_c():
    s = zr.Scene(zr.F32)
    s.set_params(1 / 64, 1e-4)
    with np.testing.assert_raises(zr.ZrError):
        s.set_params(-1, 1e-4)
