"""GPU against the FP64 oracle on degenerate layouts: a single particle, small clusters that each occupy their own
SPGrid block (every active block is one cluster's, with no shared neighbours), particles exactly on cell faces and
corners, and a batch that mixes a one-particle scene with full ones. Same inputs on both sides;
FP64 within 1e-12 (positions) and 1e-9 (velocities, F), the order of the atomic sums being the only difference."""
import numpy as np
import pytest

import ziran2020_gb300 as zr
import scenes

pytestmark = pytest.mark.gpu


def custom(x, v, dx=1 / 64, dt=1e-4, gravity=(0.0, -9.8, 0.0), E=1e4, nu=0.3, rho=1000.0, model=zr.COROTATED, objects=()):
    x = np.asarray(x, dtype=np.float64)
    n = len(x)
    vol = dx ** 3 / 8
    return {"dx": dx, "dt": dt, "gravity": gravity, "apic": 1.0, "cfl": 0.6, "domain": int(round(1 / dx)) + 4, "x": x,
            "v": np.asarray(v, dtype=np.float64), "m": np.full(n, rho * vol), "V0": np.full(n, vol),
            "F": np.tile(np.eye(3).reshape(1, 9), (n, 1)), "materials": [dict(model=model, E=E, nu=nu)], "damage": None,
            "objects": list(objects)}


def run_both(desc, prec, steps):
    s = scenes.gpu_scene(desc, prec)
    o = scenes.oracle_scene(desc, 8)
    s.step(steps)
    o.step(steps)
    return scenes.errors(scenes.gpu_state(s), o.state())


@pytest.mark.parametrize("prec", [zr.F64, zr.F32])
def test_single_particle(prec):
    d = custom([[0.5, 0.6, 0.5]], [[0.3, -1.0, 0.2]])
    e = run_both(d, prec, 25)
    assert e["x"][0] < (1e-12 if prec == zr.F64 else 1e-6), e
    assert e["v"][0] < (1e-9 if prec == zr.F64 else 1e-4), e


@pytest.mark.parametrize("prec", [zr.F64, zr.F32])
def test_isolated_particles_each_in_its_own_block(prec):
    """27 clusters of 8 particles, 24 cells apart (6 blocks in FP32, where blocks are 4 cells wide; 6-12 in FP64,
    2x4x4): every group is one cluster and the blocks it activates belong to it alone; the lowest layer starts inside
    a sticky floor that moves up."""
    rng = np.random.default_rng(3)
    dx = 1 / 64
    pts = [[(8 + 24 * i + 0.37) * dx, (10 + 24 * j + 0.61) * dx, (8 + 24 * k + 0.13) * dx] for i in range(3) for j in range(3) for k in range(3)]
    x = np.array([p for p in pts for _ in range(8)]) + rng.uniform(-0.3, 0.3, (8 * len(pts), 3)) * dx
    v = rng.uniform(-1.0, 1.0, x.shape)
    floor = dict(origin=(0, 11 * dx, 0), normal=(0, 1, 0), type=zr.STICKY, friction=0.0, velocity=(0, 0.2, 0))
    d = custom(x, v, dx=dx, objects=[floor])
    e = run_both(d, prec, 20)
    assert e["x"][0] < (1e-12 if prec == zr.F64 else 1e-6), e
    assert e["v"][0] < (1e-9 if prec == zr.F64 else 1e-4), e
    assert e["F"][0] < (1e-9 if prec == zr.F64 else 1e-4), e


@pytest.mark.parametrize("prec", [zr.F64, zr.F32])
def test_particles_on_cell_faces_and_corners(prec):
    """Positions exactly on grid nodes and cell faces (x = k dx and (k + 1/2) dx), where the base node's floor and the
    weights' breakpoints sit; a stiff cube pushed sideways so particles cross those faces in the first substeps."""
    dx = 1 / 64
    g = np.arange(28, 36) * dx
    h = (np.arange(28, 36) + 0.5) * dx
    x = np.array([[a, b, c] for a in g for b in h for c in g] + [[a, b, c] for a in h for b in g for c in h])
    v = np.tile([[2.0, -0.5, 1.0]], (len(x), 1))
    d = custom(x, v, dx=dx, E=5e4, gravity=(0.0, 0.0, 0.0))
    e = run_both(d, prec, 15)
    assert e["x"][0] < (1e-12 if prec == zr.F64 else 1e-6), e
    assert e["v"][0] < (1e-9 if prec == zr.F64 else 1e-4), e


@pytest.mark.parametrize("prec", [zr.F64, zr.F32])
def test_batch_with_a_one_particle_scene(prec):
    """A one-particle scene batched between two full ones: every slot equals its scene run alone (the order of the
    grid sums aside), and the lone particle's group sits among the full groups of the other scenes."""
    descs = [scenes.elastic_box(size=0.0625, seed=1, center=(0.4, 0.5, 0.5)),
             custom([[0.52, 0.55, 0.48]], [[0.1, -0.5, 0.3]]),
             scenes.aniso_slab(size=(0.08, 0.04, 0.08), sigma_c=(20.0, 2.0), pull=1.0)]
    b = zr.Batch(prec)
    singles = []
    for d in descs:
        sc = scenes.gpu_scene(d, prec)
        b.add_scene(sc)
        singles.append(sc)
    b.commit()
    b.step(20)
    tol = 1e-11 if prec == zr.F64 else 1e-5
    for k, sc in enumerate(singles):
        sc.step(20)
        for f in ("x", "v", "F"):
            a, c = b.get(k, f), sc.get(f)
            assert np.abs(a - c).max() <= tol * max(1.0, np.abs(c).max()), (k, f, np.abs(a - c).max())


@pytest.mark.parametrize("prec", [zr.F64, zr.F32])
def test_two_materials_collide(prec):
    """Two cubes of different models in one scene (a fixed-corotated one, and a Neo-Hookean (Borden) one with
    anisotropic damage and a low critical stress) driven into each other: the kernels for mixed models (material
    per particle) against the oracle with the same per-particle materials; damage grows where they meet."""
    dx, dt = 1 / 64, 1e-4
    rng = np.random.default_rng(9)

    def cube(c0, n=4):
        cells = [(c0[0] + i, c0[1] + j, c0[2] + k) for i in range(n) for j in range(n) for k in range(n)]
        x = [[(c[a] + (((s >> (2 - a)) & 1) + 0.5) * 0.5) * dx for a in range(3)] for c in cells for s in range(8)]
        return np.asarray(x) + rng.uniform(-0.1, 0.1, (len(x), 3)) * dx

    xa, xb = cube((26, 30, 30)), cube((32, 31, 30))
    na, nb = len(xa), len(xb)
    vol = dx ** 3 / 8
    va, vb = np.tile([[4.0, 0.0, 0.3]], (na, 1)), np.tile([[-4.0, 0.2, 0.0]], (nb, 1))
    eye = np.tile(np.eye(3).reshape(1, 9), (na + nb, 1))
    m = np.full(na + nb, 1000.0 * vol)
    sc_b = rng.normal(30.0, 3.0, nb)
    dmg = dict(alpha=-1.0, l0=0.5 * dx, eta=0.1, zeta=1.0, residual=0.01)

    s = zr.Scene(prec)
    s.set_params(dx, dt, (0.0, 0.0, 0.0), 1.0, 0.6, int(round(1 / dx)) + 4)
    fa = s.add_particles(xa, m[:na], np.full(na, vol), v=va, F=eye[:na])
    s.add_corotated(fa, na, 1e4, 0.3)
    fb = s.add_particles(xb, m[na:], np.full(nb, vol), v=vb, F=eye[na:])
    s.add_neohookean_borden(fb, nb, 3e4, 0.25)
    s.add_aniso_damage(fb, nb, dmg["alpha"], dmg["l0"], dmg["eta"], dmg["zeta"], dmg["residual"], sc_b)

    import pyoracle as po

    o = po.OracleScene(8, dx, dt, (0.0, 0.0, 0.0), 1.0, 0.6)
    o.add_material(zr.COROTATED, 1e4, 0.3)
    o.add_material(zr.NEOHOOKEAN_BORDEN, 3e4, 0.25, True, dmg["alpha"], dmg["l0"], dmg["eta"], dmg["zeta"], dmg["residual"])
    o.set_particles(np.vstack([xa, xb]), np.vstack([va, vb]), m, np.full(na + nb, vol), F=eye,
                    sigma_c=np.concatenate([np.full(na, 1e30), sc_b]), material=np.r_[np.zeros(na, np.int32), np.ones(nb, np.int32)])
    s.step(60)
    o.step(60)
    e = scenes.errors(scenes.gpu_state(s), o.state())
    assert e["x"][0] < (1e-12 if prec == zr.F64 else 1e-5), e
    assert e["v"][0] < (1e-9 if prec == zr.F64 else 1e-3), e
    assert e["d"][0] < (1e-9 if prec == zr.F64 else 1e-3), e
    assert o.state()["d"][na:].max() > 0.01  # the cubes met and the damageable one took damage
