"""CPU: the GPU physics routines (physics.cuh compiled as host C++ through tests/cpu_physics) against the
oracle's restatement and numpy: polar decomposition incl. inverted and singular F (FP64 SVD fallback),
the tensile stress split, both constitutive models, the damage update and the SPGrid key."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

import pyoracle as po

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpu_physics", "physics_shim.cpp")


@pytest.fixture(scope="module")
def shim(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("shim") / "libphysics_shim.so")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", SRC, "-o", so])
    L = C.CDLL(so)
    pd = C.POINTER(C.c_double)
    L.shim_polar.argtypes = [C.c_int, pd, pd]
    L.shim_svd_jacobi.argtypes = [pd, pd, pd, pd]
    L.shim_tension.argtypes = [C.c_int, pd, pd]
    L.shim_tau.argtypes = [C.c_int, C.c_double, C.c_double, pd, C.c_double, pd]
    L.shim_damage.restype = C.c_double
    L.shim_damage.argtypes = [C.c_double] * 7 + [pd] + [C.c_double] * 4
    L.shim_key.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_uint, C.POINTER(C.c_ulonglong)]
    L.shim_tau2.restype = C.c_double
    L.shim_tau2.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, pd, C.c_double, C.c_int, pd]
    L.shim_qr.argtypes = [pd, pd, pd]
    L.shim_damage2.restype = C.c_double
    L.shim_damage2.argtypes = [C.c_int] + [C.c_double] * 7 + [pd] + [C.c_double] * 4
    L.shim_collide.argtypes = [C.c_int, C.c_int, pd, C.c_double, pd, pd]
    return L


def p(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def oracle_R(prec, F):
    U, s, V = po.svd3(prec, F)
    return U @ V.T


def test_polar_matches_oracle_svd(shim):
    rng = np.random.default_rng(1)
    fallbacks = 0
    for t in range(400):
        if t % 4 == 0:
            F = np.eye(3) + 0.02 * rng.normal(size=(3, 3))  # small strain
        elif t % 4 == 1:
            F = rng.normal(size=(3, 3))  # generic, often inverted
        elif t % 4 == 2:
            Q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
            F = Q * np.array([1.0, 1.0, 1.0])  # a pure rotation / reflection: degenerate singular values
        else:
            F = np.diag([1.5, 0.7, 1e-9]) @ np.linalg.qr(rng.normal(size=(3, 3)))[0]  # nearly singular
        F = np.ascontiguousarray(F)
        R = np.zeros(9)
        fallbacks += shim.shim_polar(8, p(F), p(R))
        R = R.reshape(3, 3)
        assert abs(np.linalg.det(R) - 1) < 1e-9 and np.abs(R @ R.T - np.eye(3)).max() < 1e-9
        s = np.linalg.svd(F, compute_uv=False)
        if s[1] + s[2] > 1e-6:  # the polar rotation is unique: it must equal the reference's U V^T
            assert np.abs(R - oracle_R(8, F)).max() < 1e-8 / (s[1] + s[2]), t
    assert fallbacks > 50  # the inverted and singular cases took the FP64 SVD path


def test_polar_fp32_accuracy(shim):
    rng = np.random.default_rng(2)
    for t in range(200):
        F = np.ascontiguousarray(np.eye(3) + 0.3 * rng.normal(size=(3, 3)))
        R = np.zeros(9)
        shim.shim_polar(4, p(F), p(R))
        assert np.abs(R.reshape(3, 3) - oracle_R(8, F)).max() < 2e-5


def test_svd_jacobi_sign_convention(shim):
    rng = np.random.default_rng(3)
    for t in range(200):
        A = np.ascontiguousarray(rng.normal(size=(3, 3)))
        U, s, V = np.zeros(9), np.zeros(3), np.zeros(9)
        shim.shim_svd_jacobi(p(A), p(U), p(s), p(V))
        U, V = U.reshape(3, 3), V.reshape(3, 3)
        assert np.abs(U @ np.diag(s) @ V.T - A).max() < 1e-12
        assert abs(np.linalg.det(U) - 1) < 1e-12 and abs(np.linalg.det(V) - 1) < 1e-12
        assert s[0] >= s[1] >= abs(s[2]) and s[1] >= 0
        assert np.sign(s[2]) == np.sign(np.linalg.det(A)) or abs(s[2]) < 1e-12


def test_tension_part(shim):
    rng = np.random.default_rng(4)
    for t in range(500):
        Q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        lam = rng.normal(size=3) * 100
        if t % 5 == 0:
            lam[1] = lam[0]  # repeated eigenvalue
        if t % 7 == 0:
            lam[:] = lam[0]  # multiple of the identity
        S = np.ascontiguousarray(Q @ np.diag(lam) @ Q.T)
        want = Q @ np.diag(np.maximum(lam, 0)) @ Q.T
        got = np.zeros(9)
        shim.shim_tension(8, p(S), p(got))
        assert np.abs(got.reshape(3, 3) - want).max() < 1e-9 * max(1, np.abs(lam).max()), t
        shim.shim_tension(4, p(S), p(got))
        assert np.abs(got.reshape(3, 3) - want).max() < 2e-4 * max(1, np.abs(lam).max()), t


def tau_reference(model, E, nu, F, g):
    lam = E * nu / ((1 + nu) * (1 - 2 * nu))
    mu = E / (2 * (1 + nu))
    J = np.linalg.det(F)
    if model == 0:
        R = oracle_R(8, F)
        P = 2 * mu * (F - R) + lam * (J - 1) * J * np.linalg.inv(F).T
        return P @ F.T
    kappa = 0.666666 * mu + lam
    B = F @ F.T
    dev = mu * J ** (-2 / 3) * (B - np.trace(B) / 3 * np.eye(3))
    vol = J * kappa / 2 * (J - 1 / J) * np.eye(3)
    return g * (dev + vol) if J >= 1 else g * dev + vol


@pytest.mark.parametrize("model", [0, 1])
def test_stress_models(shim, model):
    rng = np.random.default_rng(5)
    for t in range(100):
        F = np.ascontiguousarray(np.eye(3) + 0.2 * rng.normal(size=(3, 3)))
        if np.linalg.det(F) <= 0.1:
            continue
        g = rng.uniform(0.01, 1)
        tau = np.zeros(9)
        shim.shim_tau(model, 5e4, 0.25, p(F), g, p(tau))
        want = tau_reference(model, 5e4, 0.25, F, g)
        assert np.abs(tau.reshape(3, 3) - want).max() < 1e-8 * 5e4


def test_damage_update_matches_reference_formula(shim):
    rng = np.random.default_rng(6)
    E, nu, alpha, l0, eta, zeta, k = 5e4, 0.25, -1.0, 0.002, 0.1, 1.0, 0.01
    for t in range(200):
        F = np.ascontiguousarray(np.eye(3) + 0.05 * rng.normal(size=(3, 3)))
        d, lap, sc, dt = rng.uniform(0, 0.5), rng.normal() * 100, rng.uniform(50, 500), 5e-5
        got = shim.shim_damage(E, nu, alpha, l0, eta, zeta, k, p(F), d, lap, sc, dt)
        # AnisoFractureSimulation.h:219-281 with numpy's symmetric eigen-decomposition
        J = np.linalg.det(F)
        S = tau_reference(1, E, nu, F, 1.0) / J
        w, Q = np.linalg.eigh((S + S.T) / 2)
        sp = Q @ np.diag(np.maximum(w, 0)) @ Q.T
        a = oracle_R(8, F)[:, 0]
        A = np.eye(3) + alpha * np.outer(a, a)
        phi = np.sum((A @ sp) * (sp @ A)) / sc ** 2
        dtil = zeta * max(phi - 1, 0)
        want = min(d + dt / eta * max((1 - d) * dtil - (d - l0 * l0 * lap), 0), 1)
        assert abs(got - want) < 1e-10, t


def test_gpu_key_function_matches_oracle_layout(shim):
    rng = np.random.default_rng(7)
    for prec in (4, 8):
        for t in range(300):
            i, j, k = (int(v) for v in rng.integers(0, 4000, 3))
            key = C.c_ulonglong()
            idx = int(rng.integers(0, 1 << 20))
            shim.shim_key(prec, i, j, k, idx, C.byref(key))
            bb = 6 if prec == 4 else 5
            data_bits = 6 if prec == 4 else 7
            want = ((po.linear_offset(prec, i, j, k) >> data_bits) << (32 - bb)) + idx
            assert key.value == want


# ---------------------------------------------------------------- QR-stable Neo-Hookean (QRStableNeoHookean.h)
E_, NU_ = 5e4, 0.25
LAM_, MU_ = E_ * NU_ / ((1 + NU_) * (1 - 2 * NU_)), E_ / (2 * (1 + NU_))


def qrnh_psi(F, g=1.0, kx=0.0, ky=0.0):
    """The model's energy from the R of F = QR (QRStableNeoHookean.h:124-151); |r| makes it independent of
    the sign convention of the factorisation, except J = det F."""
    R = np.abs(np.linalg.qr(F)[1])
    J = np.linalg.det(F)
    vol = 0.5 * LAM_ * (J - 1) ** 2 * (g if J >= 1 else 1.0)
    dev = g * (MU_ / 2 * (np.sum(np.triu(R) ** 2) - 3) - MU_ * (J - 1))
    fib = kx * MU_ / 2 * (R[0, 0] - 1) ** 2 + ky * MU_ / 2 * (np.sqrt(R[0, 1] ** 2 + R[1, 1] ** 2) - 1) ** 2
    return vol + dev + fib


def random_F(rng, spread=0.15):
    while True:
        F = np.eye(3) + spread * rng.normal(size=(3, 3))
        if np.linalg.det(F) > 0.3:
            return F


def test_givens_qr_convention(shim):
    rng = np.random.default_rng(11)
    for t in range(200):
        F = np.ascontiguousarray(rng.normal(size=(3, 3)))
        Q, R = np.zeros(9), np.zeros(9)
        shim.shim_qr(p(F), p(Q), p(R))
        Q, R = Q.reshape(3, 3), R.reshape(3, 3)
        assert np.abs(Q @ R - F).max() < 1e-12 and np.abs(Q.T @ Q - np.eye(3)).max() < 1e-12
        assert abs(np.linalg.det(Q) - 1) < 1e-12 and np.abs(np.tril(R, -1)).max() < 1e-12
        assert R[0, 0] >= 0 and R[1, 1] >= 0 and np.sign(R[2, 2]) == np.sign(np.linalg.det(F))


@pytest.mark.parametrize("g,kx,ky", [(1.0, 0.0, 0.0), (0.3, 0.0, 0.0), (1.0, 10.0, 0.0), (0.5, 4.0, 2.0)])
def test_qrnh_stress_is_the_energy_gradient_and_matches_the_oracle(shim, g, kx, ky):
    rng = np.random.default_rng(12)
    for t in range(40):
        F = np.ascontiguousarray(random_F(rng))
        got = np.zeros(9)
        J = shim.shim_tau2(8, 2, E_, NU_, kx, ky, p(F), g, 0, p(got))
        got = got.reshape(3, 3)
        ref, Jr = po.tau(8, 2, E_, NU_, F, g=g, kx_scale=kx, ky_scale=ky)
        assert abs(J - np.linalg.det(F)) < 1e-12 and abs(Jr - J) < 1e-12
        assert np.abs(got - ref).max() < 1e-9 * np.abs(ref).max(), t  # tau = Q A Q^T here, P F^T in the oracle
        # P = dpsi/dF by central differences, tau = P F^T
        h, P = 1e-6, np.zeros((3, 3))
        for a in range(3):
            for b in range(3):
                Fp, Fm = F.copy(), F.copy()
                Fp[a, b] += h
                Fm[a, b] -= h
                P[a, b] = (qrnh_psi(Fp, g, kx, ky) - qrnh_psi(Fm, g, kx, ky)) / (2 * h)
        assert np.abs(P @ F.T - ref).max() < 1e-5 * max(1.0, np.abs(ref).max()), t
        got32 = np.zeros(9)
        shim.shim_tau2(4, 2, E_, NU_, kx, ky, p(F), g, 0, p(got32))
        assert np.abs(got32.reshape(3, 3) - ref).max() < 2e-5 * np.abs(ref).max()


def test_qrnh_effective_stress_and_sigma_crit(shim):
    import ziran2020_gb300 as zr

    rng = np.random.default_rng(13)
    for t in range(20):
        F = np.ascontiguousarray(random_F(rng))
        eff = np.zeros(9)
        shim.shim_tau2(8, 2, E_, NU_, 10.0, 3.0, p(F), 0.2, 1, p(eff))
        iso = np.zeros(9)
        shim.shim_tau2(8, 2, E_, NU_, 0.0, 0.0, p(F), 1.0, 0, p(iso))
        assert np.abs(eff - iso).max() < 1e-9 * np.abs(iso).max()  # undegraded, fibres off
    for pc in (0.05, 0.2):
        assert abs(zr.qrnh_sigma_crit(E_, NU_, pc) - qrnh_psi((1 + pc) * np.eye(3))) < 1e-9 * qrnh_psi((1 + pc) * np.eye(3))


def test_qrnh_damage_update_matches_reference_formula(shim):
    rng = np.random.default_rng(14)
    alpha, l0, eta, zeta, k = -1.0, 0.002, 0.1, 1.0, 0.01
    for t in range(100):
        F = np.ascontiguousarray(np.eye(3) + 0.05 * rng.normal(size=(3, 3)))
        d, lap, sc, dt = rng.uniform(0, 0.5), rng.normal() * 100, rng.uniform(50, 500), 5e-5
        got = shim.shim_damage2(2, E_, NU_, alpha, l0, eta, zeta, k, p(F), d, lap, sc, dt)
        tau, J = po.tau(8, 2, E_, NU_, F, effective=True)
        S = tau / J
        w, Q = np.linalg.eigh((S + S.T) / 2)
        sp = Q @ np.diag(np.maximum(w, 0)) @ Q.T
        a = oracle_R(8, F)[:, 0]
        A = np.eye(3) + alpha * np.outer(a, a)
        phi = np.sum((A @ sp) * (sp @ A)) / sc ** 2
        want = min(d + dt / eta * max((1 - d) * zeta * max(phi - 1, 0) - (d - l0 * l0 * lap), 0), 1)
        assert abs(got - want) < 1e-10, t


@pytest.mark.parametrize("alpha", [-1.0, -0.5, 0.5, 2.0])
def test_borden_drive_in_the_material_frame_equals_the_rotated_director_form(shim, alpha):
    """The Borden drive is evaluated on F^T F with A = diag(1 + alpha, 1, 1), without the polar rotation; the
    reference rotates the director, a = R e1 with F = R S (AnisoFractureSimulation.h:224-270, :365-391), and builds
    sigma+ from F F^T. Large rotations and stretches up to 1.6, critical stresses that put phi between 0.5 and 20:
    the two forms agree to rounding (FP64) and to FP32 rounding of the stress (FP32)."""
    shim.shim_drive.restype = C.c_double
    shim.shim_drive.argtypes = [C.c_int, C.c_int] + [C.c_double] * 6 + [C.POINTER(C.c_double)]
    rng = np.random.default_rng(33)
    E, nu, zeta = 5e4, 0.25, 1.0
    nonzero = 0
    for t in range(200):
        q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        if np.linalg.det(q) < 0:
            q[:, 0] = -q[:, 0]
        w, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        S = w @ np.diag(rng.uniform(0.7, 1.6, 3)) @ w.T
        F = np.ascontiguousarray(q @ S)
        J = np.linalg.det(F)
        sig = tau_reference(1, E, nu, F, 1.0) / J
        ev, Q = np.linalg.eigh((sig + sig.T) / 2)
        sp = Q @ np.diag(np.maximum(ev, 0)) @ Q.T
        a = oracle_R(8, F)[:, 0]
        A = np.eye(3) + alpha * np.outer(a, a)
        c = np.sum((A @ sp) * (sp @ A))
        if c <= 0:
            continue
        sc = np.sqrt(c / rng.uniform(0.5, 20.0))
        want = zeta * max(c / sc ** 2 - 1, 0)
        nonzero += want > 0
        got = shim.shim_drive(8, 1, E, nu, 0.0, alpha, zeta, sc, p(F))
        assert abs(got - want) <= 1e-11 * max(1.0, want), (t, got, want)
        got32 = shim.shim_drive(4, 1, E, nu, 0.0, alpha, zeta, sc, p(F))
        assert abs(got32 - want) <= 2e-4 * max(1.0, c / sc ** 2), (t, got32, want)
    assert nonzero > 100


@pytest.mark.parametrize("alpha", [-1.0, 0.5, 2.0])
def test_damage_drive_zero_bound_changes_nothing(shim, alpha):
    """The drive skips the tensile split and the polar decomposition when max(1, (1+alpha)^2) |sigma|_F^2 is at
    most 0.999 sigma_c^2 (then phi <= 1 exactly). Critical stresses straddling that bound within +-10% give the
    reference formula's damage either way."""
    rng = np.random.default_rng(21)
    E, nu, l0, eta, zeta, k = 5e4, 0.25, 0.002, 0.1, 1.0, 0.01
    skipped = computed = 0
    for t in range(300):
        F = np.ascontiguousarray(np.eye(3) + 0.01 * rng.normal(size=(3, 3)))
        J = np.linalg.det(F)
        S = tau_reference(1, E, nu, F, 1.0) / J
        bound = max(1.0, (1 + alpha) ** 2) * np.sum(S * S)
        sc = np.sqrt(bound / 0.999) * rng.uniform(0.9, 1.1)
        d, lap, dt = rng.uniform(0, 0.5), rng.normal() * 100, 5e-5
        got = shim.shim_damage(E, nu, alpha, l0, eta, zeta, k, p(F), d, lap, sc, dt)
        w, Q = np.linalg.eigh((S + S.T) / 2)
        sp = Q @ np.diag(np.maximum(w, 0)) @ Q.T
        a = oracle_R(8, F)[:, 0]
        A = np.eye(3) + alpha * np.outer(a, a)
        phi = np.sum((A @ sp) * (sp @ A)) / sc ** 2
        want = min(d + dt / eta * max((1 - d) * zeta * max(phi - 1, 0) - (d - l0 * l0 * lap), 0), 1)
        assert abs(got - want) < 1e-10, (t, phi)
        if bound <= 0.999 * sc * sc:
            skipped += 1
            assert phi <= 1.0
        else:
            computed += 1
    assert skipped > 50 and computed > 50


def _objects(rows):
    """collision objects as the 11-double rows of shim_collide / orc_collide"""
    return np.ascontiguousarray([list(o) + list(n) + list(v) + [fr, ty] for o, n, v, fr, ty in rows], dtype=np.float64)


def _collide(fn, prec, objs, t, x, v):
    out = np.array(v, dtype=np.float64)
    fn(prec, len(objs), p(objs), t, p(np.asarray(x, dtype=np.float64)), p(out))
    return out


def _oracle_collide(prec, n, objs, t, x, v):
    lib = po.lib()
    lib.orc_collide.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_double), C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    out = np.array(v, dtype=np.float64)
    lib.orc_collide(prec, n, p(objs), t, p(np.asarray(x, dtype=np.float64)), p(out))
    return out


@pytest.mark.parametrize("prec", [4, 8])
def test_collide_matches_oracle_multi_object(shim, prec):
    """collide (CollisionObject.cpp:67-105, :342-406) against the oracle on random nodes and velocities through
    a corner of three SLIP/SEPARATE walls with friction, moving objects, and a STICKY plane listed last: where
    a node lies inside the three walls the basis is complete after them and the STICKY plane is never applied
    (the loop ends after dim slip normals); elsewhere it applies when the node is inside it."""
    rng = np.random.default_rng(7)
    rows = [((0.0, 0.2, 0.0), (0.1, 1.0, 0.05), (0.0, 0.0, 0.0), 0.4, 2),  # tilted floor, SLIP with friction
            ((0.3, 0.0, 0.0), (1.0, 0.0, 0.2), (0.05, 0.0, 0.0), 0.0, 3),  # moving wall, SEPARATE
            ((0.0, 0.0, 0.3), (0.0, 0.3, 1.0), (0.0, 0.0, 0.0), 0.2, 3),  # SEPARATE with friction
            ((0.0, 0.25, 0.0), (0.0, 1.0, 0.0), (0.0, 0.0, 0.0), 0.0, 1)]  # STICKY plane after the walls
    objs = _objects(rows)
    stopped = applied_sticky = 0
    for _ in range(4000):
        x = rng.uniform(0.1, 0.4, 3)
        v = rng.normal(0, 1, 3)
        t = float(rng.uniform(0, 0.5))
        g = _collide(shim.shim_collide, prec, objs, t, x, v)
        o = _oracle_collide(prec, len(rows), objs, t, x, v)
        tol = 1e-5 if prec == 4 else 1e-12
        assert np.abs(g - o).max() <= tol * max(1.0, np.abs(o).max()), (x, v, g, o)
        inside = [np.dot(np.array(n) / np.linalg.norm(n), x - np.array(vel) * t - np.array(org)) <= 0 for org, n, vel, _, _ in rows]
        if all(inside[:3]) and inside[3]:
            stopped += 1
            assert not np.allclose(g, 0.0)  # the STICKY plane did not apply
        elif inside[3] and not any(inside[:3]):
            applied_sticky += 1
            assert np.allclose(g, 0.0)
    assert stopped > 20 and applied_sticky > 20  # both cases were exercised


def test_collide_parallel_normals_add_nothing_to_the_basis(shim):
    """Two SLIP planes with the same normal count once: after them two more SLIP planes with independent
    normals still apply, and a STICKY plane after those does not (three basis vectors)."""
    rows = [((0.0, 0.5, 0.0), (0.0, 1.0, 0.0), (0.0, 0.0, 0.0), 0.0, 2),
            ((0.0, 0.6, 0.0), (0.0, 1.0, 0.0), (0.0, 0.0, 0.0), 0.0, 2),
            ((0.5, 0.0, 0.0), (1.0, 0.0, 0.0), (0.0, 0.0, 0.0), 0.0, 2),
            ((0.0, 0.0, 0.5), (0.0, 0.0, 1.0), (0.0, 0.0, 0.0), 0.0, 2),
            ((1.0, 1.0, 1.0), (1.0, 1.0, 1.0), (0.3, 0.0, 0.0), 0.0, 1)]
    objs = _objects(rows)
    x, v = (0.2, 0.2, 0.2), (-1.0, -2.0, -3.0)
    for prec in (4, 8):
        g = _collide(shim.shim_collide, prec, objs, 0.0, x, v)
        o = _oracle_collide(prec, len(rows), objs, 0.0, x, v)
        assert np.array_equal(g, o)
        assert np.array_equal(g, np.zeros(3))  # three orthogonal SLIP walls remove every component; STICKY skipped
    rows[3] = ((0.0, 0.0, -5.0), (0.0, 0.0, 1.0), (0.0, 0.0, 0.0), 0.0, 2)  # the z wall no longer contains x
    objs = _objects(rows)
    g = _collide(shim.shim_collide, 8, objs, 0.0, x, v)
    assert np.allclose(g, (0.3, 0.0, 0.0))  # two basis vectors only: the moving STICKY plane applies


def test_fully_damaged_particle_stays_at_one(shim):
    """d = 1: the update d + dt/eta <(1 - d) D~ - (d - l0^2 lap)> is at least 1 and capped at 1 (AnisoFractureSimulation.h:
    276-281), so the drive is not evaluated; the result equals the formula's for any F and Laplacian."""
    rng = np.random.default_rng(11)
    E, nu, alpha, l0, eta, zeta, k = 5e4, 0.25, -1.0, 0.002, 0.1, 1.0, 0.01
    for _ in range(50):
        F = np.ascontiguousarray(np.eye(3) + 0.3 * rng.normal(size=(3, 3)))
        lap = rng.normal() * 1e6
        assert shim.shim_damage(E, nu, alpha, l0, eta, zeta, k, p(F), 1.0, lap, 10.0, 5e-5) == 1.0
