"""GPU: the CUDA substep against the CPU oracle on the same seeded inputs, through the C ABI.

Tolerances (stated per test): the FP64 GPU path differs from the FP64 oracle only by the order of
floating-point sums (atomic scatter vs the reference's colour-ordered scatter), so it agrees to ~1e-12
relative; the FP32 path is held to 1e-4 domain-relative position error (the path's stated FP32 bound)."""
import numpy as np
import pytest

import ziran2020_gb300 as zr
import scenes

pytestmark = pytest.mark.gpu


def run_pair(desc, gpu_prec, steps, oracle_prec=8):
    s = scenes.gpu_scene(desc, gpu_prec)
    o = scenes.oracle_scene(desc, oracle_prec)
    s.step(steps)
    o.step(steps)
    return s, o, scenes.gpu_state(s), o.state()


@pytest.mark.parametrize("steps", [1, 20])
def test_elastic_box_fp64_matches_oracle(steps):
    d = scenes.elastic_box(size=0.125)
    s, o, g, r = run_pair(d, zr.F64, steps)
    e = scenes.errors(g, r)
    assert e["x"][0] < 1e-12, e  # metres in a unit domain
    assert e["v"][0] < 1e-9, e
    assert e["F"][0] < 1e-9, e
    assert e["C"][0] < 1e-6, e
    assert abs(s.time - o.time()) < 1e-15


def test_elastic_box_fp32_within_1e4_of_fp64_oracle():
    d = scenes.elastic_box(size=0.125)
    s, o, g, r = run_pair(d, zr.F32, 100)
    e = scenes.errors(g, r)
    assert e["x"][0] < 1e-4, e  # domain-relative position error bound
    assert e["F"][0] < 1e-3, e


def test_elastic_cube_200_substeps_against_fp64_oracle():
    """The plain FP64 scene the position bound is stated on: a 0.25 m corotated cube at dx = 1/64
    (32,768 particles, E = 1e4, nu = 0.3, rho = 1000, v0 = (0, -1, 0), gravity, sticky ground at y = 0.05,
    dt = 1e-4), 200 substeps. FP32: max position error <= 1e-4 of the unit domain; FP64: <= 1e-11."""
    d = scenes.elastic_box(size=0.25)
    assert len(d["m"]) == 32768
    o = scenes.oracle_scene(d, 8)
    o.step(200)
    r = o.state()
    for prec, xtol, ftol in ((zr.F32, 1e-4, 1e-3), (zr.F64, 1e-11, 1e-8)):
        s = scenes.gpu_scene(d, prec)
        s.step(200)
        e = scenes.errors(scenes.gpu_state(s), r)
        assert e["x"][0] <= xtol, (prec, e)
        assert e["F"][0] <= ftol, (prec, e)
    assert d["x"][:, 1].min() - r["x"][:, 1].min() > 0.015  # the cube fell ~2 cm (1 m/s for 0.02 s plus gravity)


@pytest.mark.parametrize("steps", [1, 30])
def test_aniso_slab_fp64_matches_oracle(steps):
    d = scenes.aniso_slab(size=(0.1, 0.05, 0.1), sigma_c=(20.0, 2.0), pull=1.0)
    s, o, g, r = run_pair(d, zr.F64, steps)
    e = scenes.errors(g, r)
    assert e["x"][0] < 1e-12, e
    assert e["v"][0] < 1e-9, e
    assert e["F"][0] < 1e-9, e
    assert e["d"][0] < 1e-9, e
    if steps > 1:
        assert r["d"].max() > 0  # damage actually grew, so the comparison covers the damage path


@pytest.mark.parametrize("alpha,sigma_c", [(-0.5, 400.0), (0.5, 800.0), (2.0, 800.0)])
def test_aniso_slab_structural_weights_match_oracle(alpha, sigma_c):
    """The damage drive for structural-tensor weights other than the demos' -1 (which removes the stress along the
    fibre): the GPU evaluates the Borden drive in the material frame with A = diag(1 + alpha, 1, 1), the oracle as
    the reference does, with the director rotated by the polar rotation of F (AnisoFractureSimulation.h:224-270,
    :365-391). 30 substeps of a damaging slab, the critical stress set so that damage grows without saturating
    (the oracle's largest damage 0.33 to 0.86): FP64 within 1e-12 (positions) and 1e-9 (damage; measured 3e-14),
    FP32 within 1e-5 and 2e-4 (measured 7.5e-7 and 5.4e-5)."""
    d = scenes.aniso_slab(size=(0.1, 0.05, 0.1), sigma_c=(sigma_c, 0.1 * sigma_c), pull=1.0, alpha=alpha)
    o = scenes.oracle_scene(d, 8)
    o.step(30)
    r = o.state()
    assert 0.1 < r["d"].max() < 1  # damage grew and did not saturate
    for prec, xtol, dtol in ((zr.F64, 1e-12, 1e-9), (zr.F32, 1e-5, 2e-4)):
        s = scenes.gpu_scene(d, prec)
        s.step(30)
        e = scenes.errors(scenes.gpu_state(s), r)
        print(f"slab, alpha {alpha}, precision {prec}: {e}")
        assert e["x"][0] < xtol, (prec, e)
        assert e["d"][0] < dtol, (prec, e)


@pytest.mark.parametrize("fiber", [0.0, 10.0])
def test_qr_stable_slab_matches_oracle(fiber):
    """QR-stable Neo-Hookean (the AnisoMPM demos' model, fibre stiffness kx = fiber mu as in
    examples/tubepull.h:104-107) with anisotropic damage: FP64 within 1e-12 of the FP64 oracle after 30
    substeps, FP32 within 1e-5 after 30; damage within 1e-9 (FP64) and 3e-4 (FP32, about 3x the measured 9e-5)."""
    d = scenes.aniso_slab(size=(0.1, 0.05, 0.1), sigma_c=(20.0, 2.0), pull=1.0, model=zr.QR_STABLE_NEOHOOKEAN, fiber=fiber)
    o = scenes.oracle_scene(d, 8)
    o.step(30)
    r = o.state()
    assert r["d"].max() > 0  # damage grew
    for prec, xtol in ((zr.F64, 1e-12), (zr.F32, 1e-5)):
        s = scenes.gpu_scene(d, prec)
        s.step(30)
        e = scenes.errors(scenes.gpu_state(s), r)
        print(f"QR-stable slab, fibre {fiber}, precision {prec}: {e}")
        assert e["x"][0] < xtol, (prec, e)
        assert e["d"][0] < (1e-9 if prec == zr.F64 else 3e-4), (prec, e)


def test_aniso_slab_fp32_close_to_fp64_oracle():
    """FP32 after 60 substeps of a damaging slab: positions within 1e-5; damage max within 1e-3 and RMS within 5e-5
    (about 3x the measured 3.4e-4 and 1.7e-5: the damage threshold phi > 1 amplifies FP32 rounding)."""
    d = scenes.aniso_slab(size=(0.1, 0.05, 0.1), sigma_c=(20.0, 2.0), pull=1.0)
    s, o, g, r = run_pair(d, zr.F32, 60)
    e = scenes.errors(g, r)
    print(f"slab FP32 after 60 substeps: {e}")
    assert e["x"][0] < 1e-5, e
    assert e["d"][0] < 1e-3, e
    assert e["d"][1] < 5e-5, e


def test_conservation_fp64_reductions():
    d = scenes.elastic_box(size=0.125)
    s = scenes.gpu_scene(d, zr.F64)
    r0 = s.reductions()
    s.step(10)
    r1 = s.reductions()
    assert abs(r1[0] - r0[0]) == 0  # particle mass
    assert abs(r1[6] - r0[0]) < 1e-12 * r0[0]  # grid mass of the last P2G equals particle mass (partition of unity)
    np.testing.assert_allclose(r1[1:4], r0[1:4] + r0[0] * np.array(d["gravity"]) * 10 * d["dt"], rtol=0, atol=1e-11)


def test_set_get_state_roundtrip_and_rekey():
    d = scenes.elastic_box(size=0.0625)
    s = scenes.gpu_scene(d, zr.F64)
    s.step(3)
    st = np.zeros((s.count, 25))
    s.get_state(st)
    s2 = scenes.gpu_scene(d, zr.F64)
    s2.step(1)
    s2.set_state(st)
    st2 = np.zeros_like(st)
    s2.get_state(st2)
    assert np.array_equal(st, st2)
    s.step(2)
    s2.step(2)
    assert np.abs(s.get("x") - s2.get("x")).max() < 1e-12


def test_cfl_violation_reports_and_keeps_state():
    d = scenes.elastic_box(size=0.0625, v0=(0.0, -300.0, 0.0))  # moves 3e-2 per substep > dx = 1/64
    s = scenes.gpu_scene(d, zr.F64)
    x0 = s.get("x")
    with pytest.raises(zr.ZrError) as ei:
        s.step(5)
    assert ei.value.code == zr.ZR_ERR_CFL
    assert s.last_done == 0
    assert np.array_equal(s.get("x"), x0)  # state left at the start of the failing substep
    s.set_dt(1e-5)
    s.step(1)  # smaller dt passes (the reference's restart with a halved max_dt)


def test_out_of_domain_reported():
    d = scenes.elastic_box(size=0.0625, v0=(0.0, -1.0, 0.0), center=(0.5, 0.5, 0.5))
    d["x"][:, 0] += 0.5  # pushes the cube past x = 1 + 4 dx
    s = scenes.gpu_scene(d, zr.F32)
    with pytest.raises(zr.ZrError) as ei:
        s.step(1)
    assert ei.value.code == zr.ZR_ERR_OUT_OF_DOMAIN
