"""CPU: a frozen record of the oracle's per-particle physics on edge-case deformation gradients
(tests/golden/physics_edge_cases.npz, written by tests/golden/make_physics_golden.py) pins three things at once:
the oracle still computes exactly what it computed when the record was made (bit for bit, FP64 and FP32); the GPU's
physics routines compiled as host code (physics.cuh through tests/cpu_physics) agree with it (polar rotation of
Ziran's sign convention, Kirchhoff stress of each model with and without degradation, the anisotropic damage
drive); and numpy formulas written from the reference's equations agree with it (corotated and Borden stress).
Edge cases: rotations, repeated and all-equal singular values, inverted F, nearly singular F, large shear."""
import ctypes as C
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
import make_physics_golden as mg  # noqa: E402

GOLD = os.path.join(ROOT, "tests", "golden", "physics_edge_cases.npz")


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(GOLD))


@pytest.fixture(scope="module")
def shim(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("shim") / "libphysics_shim.so")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", os.path.join(ROOT, "tests", "cpu_physics", "physics_shim.cpp"), "-o", so])
    L = C.CDLL(so)
    pd = C.POINTER(C.c_double)
    L.shim_polar.argtypes = [C.c_int, pd, pd]
    L.shim_tau2.restype = C.c_double
    L.shim_tau2.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, pd, C.c_double, C.c_int, pd]
    L.shim_drive.restype = C.c_double
    L.shim_drive.argtypes = [C.c_int, C.c_int] + [C.c_double] * 6 + [pd]
    return L


def p(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def same(a, b):
    return np.array_equal(np.nan_to_num(a, nan=1.2345e300), np.nan_to_num(b, nan=1.2345e300))


def test_oracle_reproduces_the_record(gold):
    now = mg.compute(gold["F"])
    for k, v in gold.items():
        assert same(np.asarray(now[k]), v), k


@pytest.mark.parametrize("prec,tag,tol", [(8, "f64", 1e-12), (4, "f32", 2e-5)])
def test_gpu_polar_rotation_matches_the_record(shim, gold, prec, tag, tol):
    for i, f in enumerate(gold["F"]):
        U, V = gold[f"U_{tag}"][i].reshape(3, 3), gold[f"V_{tag}"][i].reshape(3, 3)
        R = np.zeros(9)
        shim.shim_polar(prec, p(np.ascontiguousarray(f)), p(R))
        assert np.abs(R.reshape(3, 3) - U @ V.T).max() < tol, (i, R.reshape(3, 3), U @ V.T)


@pytest.mark.parametrize("prec,tag,tol", [(8, "f64", 1e-11), (4, "f32", 5e-5)])
def test_gpu_stress_matches_the_record(shim, gold, prec, tag, tol):
    E, nu = float(gold["E"]), float(gold["nu"])
    for k, (model, g, kx, eff) in enumerate(gold["tau_cases"]):
        for i, f in enumerate(gold["F"]):
            want = gold[f"tau_{tag}"][k, i]
            got = np.zeros(9)
            shim.shim_tau2(prec, int(model), E, nu, kx, 0.0, p(np.ascontiguousarray(f)), g, int(eff), p(got))
            if np.isnan(want).any():  # Borden's J^(-2/3) of an inverted F is NaN in the reference too
                assert np.isnan(got).any(), (k, i)
                continue
            scale = max(E, np.abs(want).max())  # rounding of F - R enters as 2 mu |dR|: relative to the modulus
            assert np.abs(got - want).max() <= tol * scale, (k, i, got, want)


@pytest.mark.parametrize("prec,tag,tol", [(8, "f64", 1e-9), (4, "f32", 2e-3)])
def test_gpu_damage_drive_matches_the_record(shim, gold, prec, tag, tol):
    E, nu = float(gold["E"]), float(gold["nu"])
    for k, (model, kx, alpha) in enumerate(gold["drive_cases"]):
        for i, f in enumerate(gold["F"]):
            want = gold[f"drive_{tag}"][k, i]
            if np.isnan(want):
                continue
            got = shim.shim_drive(prec, int(model), E, nu, kx, alpha, 1.0, 50.0, p(np.ascontiguousarray(f)))
            assert abs(got - want) <= tol * max(1.0, abs(want)), (k, i, got, want)


def test_reference_formulas_match_the_record(gold):
    """Corotated: P = 2 mu (F - R) + lambda (J - 1) J F^-T, tau = P F^T (CorotatedElasticity.cpp:56-76); Borden:
    tau = g mu J^(-2/3) dev(F F^T) + J kappa/2 (J - 1/J) I, the volumetric part degraded only for J >= 1, kappa =
    0.666666 mu + lambda (NeoHookeanBorden.cpp:16-108). R from the record's SVD."""
    E, nu = float(gold["E"]), float(gold["nu"])
    lam, mu = E * nu / ((1 + nu) * (1 - 2 * nu)), E / (2 * (1 + nu))
    kappa = 0.666666 * mu + lam
    for k, (model, g, kx, eff) in enumerate(gold["tau_cases"]):
        if model == 2:
            continue
        gg = 1.0 if eff else g
        for i, f in enumerate(gold["F"]):
            F = f.reshape(3, 3)
            J = np.linalg.det(F)
            if model == 0:
                R = gold["U_f64"][i].reshape(3, 3) @ gold["V_f64"][i].reshape(3, 3).T
                if abs(J) < 1e-3:
                    continue  # F^-T of a nearly singular F: the formula's own rounding dominates
                want = (2 * mu * (F - R) + lam * (J - 1) * J * np.linalg.inv(F).T) @ F.T
            else:
                if J <= 0:
                    continue
                B = F @ F.T
                dev = mu * J ** (-2 / 3) * (B - np.trace(B) / 3 * np.eye(3))
                vol = J * kappa / 2 * (J - 1 / J) * np.eye(3)
                want = gg * (dev + vol) if J >= 1 else gg * dev + vol
            got = gold["tau_f64"][k, i].reshape(3, 3)
            assert np.abs(got - want).max() <= 1e-9 * max(1.0, np.abs(want).max()), (k, i)
