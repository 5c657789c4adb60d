"""Writes tests/golden/physics_edge_cases.npz: the oracle's per-particle physics on edge-case deformation gradients,
in FP64 and FP32 (the oracle is the CPU restatement of the reference in oracle/mpm_oracle.cpp; test infrastructure).

Edge cases, as the reference meets them: identity and rotations; uniaxial stretch and compression; repeated and
all-equal singular values; inverted F (det < 0, Ziran's sign convention puts the minus on the smallest singular value,
ImplicitQRSVD.h:518-533); nearly singular F; large shear; small random perturbations. Per F and precision: the
implicit-QR SVD (U, sigma, V; ImplicitQRSVD.h:354-558), the Kirchhoff stress of each constitutive model with and
without degradation (CorotatedElasticity.cpp:56-76, NeoHookeanBorden.cpp:16-108, QRStableNeoHookean.h:35-213), and
the anisotropic damage drive (AnisoFractureSimulation.h:224-270).

Run: python tests/golden/make_physics_golden.py   (rebuilds the oracle if needed)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "oracle"))
import ctypes as C  # noqa: E402

import pyoracle as po  # noqa: E402

E, NU = 5e4, 0.25
TAU_CASES = [  # (model, g, kx_scale, effective)
    (0, 1.0, 0.0, 0), (1, 1.0, 0.0, 0), (1, 0.3, 0.0, 0), (1, 0.3, 0.0, 1), (2, 1.0, 0.0, 0), (2, 0.3, 10.0, 0), (2, 0.3, 10.0, 1)]
DRIVE_CASES = [(1, 0.0, -1.0), (1, 0.0, 0.0), (2, 10.0, -1.0)]  # (model, kx_scale, alpha); zeta = 1, sigma_c = 50


def rot(q):
    q = np.asarray(q, dtype=np.float64)
    w, x, y, z = q / np.linalg.norm(q)
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def edge_cases():
    Ra, Rb = rot([0.9, 0.2, -0.3, 0.1]), rot([0.3, -0.7, 0.5, 0.4])
    c, s = np.cos(np.pi / 6), np.sin(np.pi / 6)
    Fs = [np.eye(3), np.array([[c, -s, 0], [s, c, 0], [0, 0, 1.0]]), Ra, np.diag([1.5, 1.0, 1.0]), np.diag([0.5, 1.0, 1.0]),
          Ra @ np.diag([1.2, 1.2, 0.8]) @ Rb.T, 1.1 * np.eye(3), Ra @ np.diag([1.1, 0.9, -0.3]) @ Rb.T, np.diag([1.0, 1.0, 1e-4]),
          np.diag([1.0, 1e-3, 1e-3]), np.array([[1.0, 2.0, 0], [0, 1.0, 0], [0, 0, 1.0]]), Rb @ np.diag([2.0, 0.7, 0.7]),
          Ra @ (1.3 * np.eye(3)), np.diag([1.02, 0.97, -0.05]) @ Rb.T]
    rng = np.random.default_rng(2020)
    Fs += [np.eye(3) + 0.1 * rng.normal(size=(3, 3)) for _ in range(4)]
    return np.stack([np.ascontiguousarray(f, dtype=np.float64).reshape(9) for f in Fs])


def compute(F):
    L = po.lib()
    L.orc_damage_drive.restype = C.c_double
    L.orc_damage_drive.argtypes = [C.c_int, C.c_int] + [C.c_double] * 6 + [C.POINTER(C.c_double)]
    out = {"F": F, "E": np.array(E), "nu": np.array(NU), "tau_cases": np.array(TAU_CASES, dtype=np.float64),
           "drive_cases": np.array(DRIVE_CASES, dtype=np.float64)}
    for prec, tag in ((8, "f64"), (4, "f32")):
        U = np.zeros((len(F), 9)); S = np.zeros((len(F), 3)); V = np.zeros((len(F), 9))
        for i, f in enumerate(F):
            u, sg, v = po.svd3(prec, f.reshape(3, 3))
            U[i], S[i], V[i] = u.reshape(9), sg, v.reshape(9)
        out[f"U_{tag}"], out[f"sigma_{tag}"], out[f"V_{tag}"] = U, S, V
        tau = np.zeros((len(TAU_CASES), len(F), 9))
        for k, (model, g, kx, eff) in enumerate(TAU_CASES):
            for i, f in enumerate(F):
                tau[k, i] = po.tau(prec, model, E, NU, f.reshape(3, 3), g=g, effective=bool(eff), kx_scale=kx)[0].reshape(9)
        out[f"tau_{tag}"] = tau
        drv = np.full((len(DRIVE_CASES), len(F)), np.nan)
        for k, (model, kx, alpha) in enumerate(DRIVE_CASES):
            for i, f in enumerate(F):
                if np.linalg.det(f.reshape(3, 3)) > 0.05:
                    fp = np.ascontiguousarray(f)
                    drv[k, i] = L.orc_damage_drive(prec, int(model), E, NU, kx, alpha, 1.0, 50.0, fp.ctypes.data_as(C.POINTER(C.c_double)))
        out[f"drive_{tag}"] = drv
    return out


if __name__ == "__main__":
    np.savez_compressed(os.path.join(HERE, "physics_edge_cases.npz"), **compute(edge_cases()))
    print("wrote", os.path.join(HERE, "physics_edge_cases.npz"))
