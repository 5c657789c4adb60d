"""Shared scene descriptions for the tests: one description builds both the GPU scene (through the
C ABI) and the CPU oracle with identical inputs."""
import numpy as np

import ziran2020_gb300 as zr
import pyoracle as po


def elastic_box(size=0.125, dx=1 / 64, seed=7, E=1e4, nu=0.3, rho=1000.0, v0=(0.0, -1.0, 0.0), dt=1e-4, center=(0.5, 0.6, 0.5),
                gravity=(0.0, -9.8, 0.0), ground=0.05, apic=1.0):
    r = zr.recipe(zr.RECIPE_ELASTIC_BOX, dx=dx, seed=seed, size=(size, size, size), center=center, velocity=v0, E=E, nu=nu, rho=rho, dt=dt,
                  gravity=gravity, ground_y=ground, apic_rpic_ratio=apic)
    g = zr.recipe_generate(r)
    return {"dx": dx, "dt": dt, "gravity": gravity, "apic": apic, "cfl": 0.6, "domain": int(round(1 / dx)) + 4, **g,
            "materials": [dict(model=zr.COROTATED, E=E, nu=nu)], "damage": None,
            "objects": [dict(origin=(0, ground, 0), normal=(0, 1, 0), type=zr.STICKY, friction=0.0, velocity=(0, 0, 0))]}


def aniso_slab(size=(0.1, 0.05, 0.1), dx=1 / 128, seed=11, sigma_c=(400.0, 40.0), pull=0.5, dt=5e-5, E=5e4, nu=0.25, rho=800.0, apic=0.0,
               grip=2, model=None, fiber=0.0, implicit=False, alpha=-1.0):
    """model: zr.NEOHOOKEAN_BORDEN (default) or zr.QR_STABLE_NEOHOOKEAN with fibre stiffness kx = fiber mu;
    implicit: the implicit damage solve instead of the explicit update; alpha: the structural tensor's weight
    (A = I + alpha a a^T; -1, the demos' value, removes the stress along the fibre)."""
    model = zr.NEOHOOKEAN_BORDEN if model is None else model
    r = zr.recipe(zr.RECIPE_ANISO_SLAB, dx=dx, seed=seed, size=size, l0=0.5 * dx, sigma_c_mean=sigma_c[0], sigma_c_std=sigma_c[1],
                  pull_speed=pull, dt=dt, E=E, nu=nu, rho=rho, apic_rpic_ratio=apic, grip_cells=grip)
    g = zr.recipe_generate(r)
    nc = [max(1, int(round(s / dx))) for s in size]
    lo = [int(round((0.5 - 0.5 * n * dx) / dx)) for n in nc]
    x_lo, x_hi = lo[0] * dx, (lo[0] + nc[0]) * dx
    return {"dx": dx, "dt": dt, "gravity": (0.0, 0.0, 0.0), "apic": apic, "cfl": 0.6, "domain": int(round(1 / dx)) + 4, **g,
            "materials": [dict(model=model, E=E, nu=nu, kx=fiber)],
            "damage": dict(alpha=alpha, l0=0.5 * dx, eta=0.1, zeta=1.0, residual=0.01), "implicit": implicit,
            "objects": [dict(origin=(x_lo + grip * dx, 0, 0), normal=(1, 0, 0), type=zr.STICKY, friction=0.0, velocity=(-pull, 0, 0)),
                        dict(origin=(x_hi - grip * dx, 0, 0), normal=(-1, 0, 0), type=zr.STICKY, friction=0.0, velocity=(pull, 0, 0))]}


def gpu_scene(desc, precision):
    s = zr.Scene(precision)
    s.set_params(desc["dx"], desc["dt"], desc["gravity"], desc["apic"], desc["cfl"], desc["domain"])
    first = s.add_particles(desc["x"], desc["m"], desc["V0"], v=desc["v"], F=desc["F"])
    n = len(desc["m"])
    mat = desc["materials"][0]
    if mat["model"] == zr.COROTATED:
        s.add_corotated(first, n, mat["E"], mat["nu"])
    elif mat["model"] == zr.QR_STABLE_NEOHOOKEAN:
        s.add_qr_stable_neohookean(first, n, mat["E"], mat["nu"], mat.get("kx", 0.0))
    else:
        s.add_neohookean_borden(first, n, mat["E"], mat["nu"])
    if desc["damage"]:
        dm = desc["damage"]
        s.add_aniso_damage(first, n, dm["alpha"], dm["l0"], dm["eta"], dm["zeta"], dm["residual"], desc["sigma_c"])
    for o in desc["objects"]:
        s.add_halfspace(o["origin"], o["normal"], o["type"], o["friction"], o["velocity"])
    if desc.get("implicit"):
        s.set_implicit_damage(True)
    return s


def oracle_scene(desc, precision):
    o = po.OracleScene(precision, desc["dx"], desc["dt"], desc["gravity"], desc["apic"], desc["cfl"])
    mat = desc["materials"][0]
    if desc["damage"]:
        dm = desc["damage"]
        o.add_material(mat["model"], mat["E"], mat["nu"], True, dm["alpha"], dm["l0"], dm["eta"], dm["zeta"], dm["residual"],
                       kx_scale=mat.get("kx", 0.0))
    else:
        o.add_material(mat["model"], mat["E"], mat["nu"], kx_scale=mat.get("kx", 0.0))
    for ob in desc["objects"]:
        o.add_halfspace(ob["origin"], ob["normal"], ob["type"], ob["friction"], ob["velocity"])
    o.set_particles(desc["x"], desc["v"], desc["m"], desc["V0"], F=desc["F"], sigma_c=desc["sigma_c"] if desc["damage"] else None)
    if desc.get("implicit"):
        o.set_implicit_damage(True)
    return o


def gpu_state(s):
    return {"x": s.get("x"), "v": s.get("v"), "C": s.get("C"), "F": s.get("F"), "d": s.get("d")}


def errors(a, b, scale=None):
    """max and RMS of |a-b| per field; scale divides (domain-relative positions)."""
    out = {}
    for k in ("x", "v", "C", "F", "d"):
        e = np.abs(np.asarray(a[k], dtype=np.float64) - np.asarray(b[k], dtype=np.float64))
        if scale and k in scale:
            e = e / scale[k]
        out[k] = (float(e.max()) if e.size else 0.0, float(np.sqrt(np.mean(e * e))) if e.size else 0.0)
    return out
