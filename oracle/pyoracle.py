"""TEST INFRASTRUCTURE — ctypes front end of the CPU oracle (oracle/mpm_oracle.cpp).

Only the tests, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import this module, and only
as the checker or the timed CPU baseline. It builds ``oracle/_build/liboracle.so`` with ``make`` on
first use.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

_lib = None


def build(force=False):
    src = os.path.join(HERE, "mpm_oracle.cpp")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.check_call(["make", "-s", "-C", HERE, "all"])
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        vp, d, i32, i64, u64 = C.c_void_p, C.c_double, C.c_int, C.c_int64, C.c_uint64
        P = C.POINTER
        L.orc_create.restype = vp
        L.orc_create.argtypes = [i32, d, d, P(d), d, d]
        L.orc_destroy.argtypes = [vp]
        L.orc_add_material.restype = i32
        L.orc_add_material.argtypes = [vp, i32, d, d, i32, d, d, d, d, d, d, d]
        L.orc_set_implicit.argtypes = [vp, i32]
        L.orc_cg_iterations.restype = i32
        L.orc_cg_iterations.argtypes = [vp]
        L.orc_tau.restype = d
        L.orc_tau.argtypes = [i32, i32, d, d, d, d, d, i32, P(d), P(d)]
        L.orc_add_halfspace.argtypes = [vp, P(d), P(d), i32, d, P(d)]
        L.orc_set_particles.argtypes = [vp, i64] + [P(d)] * 8 + [P(C.c_int32)]
        L.orc_step.restype = i32
        L.orc_step.argtypes = [vp, i32]
        L.orc_get_state.argtypes = [vp] + [P(d)] * 5
        L.orc_time.restype = d
        L.orc_time.argtypes = [vp]
        L.orc_bin.restype = i64
        L.orc_bin.argtypes = [vp, P(u64), P(C.c_int32), P(C.c_int32), P(C.c_int32), P(u64), P(u64), P(i64)]
        L.orc_linear_offset.restype = u64
        L.orc_linear_offset.argtypes = [i32, i32, i32, i32]
        L.orc_packed_add.restype = u64
        L.orc_packed_add.argtypes = [i32, u64, u64]
        L.orc_masks.argtypes = [i32, P(u64)]
        L.orc_svd3.argtypes = [i32, P(d), P(d), P(d), P(d)]
        L.orc_reductions.argtypes = [vp, P(d)]
        L.orc_num_threads.restype = i32
        L.orc_seeded_inputs.restype = i64
        L.orc_seeded_inputs.argtypes = [i32, i32, u64, d, P(d), P(d), P(d), d, d, d, d] + [P(d)] * 6 + [P(i64)]
        _lib = L
    return _lib


def _p(a, ct=C.c_double):
    return None if a is None else a.ctypes.data_as(C.POINTER(ct))


def _f64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


class OracleScene:
    """One scene of the oracle. precision 4 = float, 8 = double. Arrays are float64 at the interface."""

    def __init__(self, precision, dx, dt, gravity=(0.0, 0.0, 0.0), apic_ratio=1.0, cfl=0.6):
        self.L = lib()
        g = np.asarray(gravity, dtype=np.float64)
        self.h = self.L.orc_create(precision, dx, dt, _p(g), apic_ratio, cfl)
        self.precision = precision
        self.n = 0

    def close(self):
        if self.h:
            self.L.orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_material(self, model, E, nu, damage=False, alpha=0.0, l0=0.0, eta=1.0, zeta=1.0, residual=0.0, kx_scale=0.0, ky_scale=0.0):
        return self.L.orc_add_material(self.h, model, E, nu, int(damage), alpha, l0, eta, zeta, residual, kx_scale, ky_scale)

    def set_implicit_damage(self, on=True):
        self.L.orc_set_implicit(self.h, int(on))

    def cg_iterations(self):
        return self.L.orc_cg_iterations(self.h)

    def add_halfspace(self, origin, normal, type_, friction=0.0, velocity=(0.0, 0.0, 0.0)):
        o, n, v = (np.asarray(a, dtype=np.float64) for a in (origin, normal, velocity))
        self.L.orc_add_halfspace(self.h, _p(o), _p(n), type_, friction, _p(v))

    def set_particles(self, x, v, m, V0, F=None, C_=None, d=None, sigma_c=None, material=None):
        x, v, m, V0, F, C_, d, sigma_c = (_f64(a) for a in (x, v, m, V0, F, C_, d, sigma_c))
        mat = None if material is None else np.ascontiguousarray(material, dtype=np.int32)
        self.n = x.shape[0]
        self._keep = (x, v, m, V0, F, C_, d, sigma_c, mat)
        self.L.orc_set_particles(self.h, self.n, _p(x), _p(v), _p(m), _p(V0), _p(F), _p(C_), _p(d), _p(sigma_c), _p(mat, C.c_int32))

    def step(self, n=1):
        return self.L.orc_step(self.h, n)

    def state(self):
        n = self.n
        x, v, Cm, F, d = (np.zeros((n, 3)), np.zeros((n, 3)), np.zeros((n, 9)), np.zeros((n, 9)), np.zeros(n))
        self.L.orc_get_state(self.h, _p(x), _p(v), _p(Cm), _p(F), _p(d))
        return {"x": x, "v": v, "C": Cm, "F": F, "d": d}

    def time(self):
        return self.L.orc_time(self.h)

    def bin(self):
        n = self.n
        sorter = np.zeros(n, np.uint64)
        order = np.zeros(n, np.int32)
        gf = np.zeros(n, np.int32)
        gl = np.zeros(n, np.int32)
        bo = np.zeros(n, np.uint64)
        pages = np.zeros(8 * n, np.uint64)
        npg = C.c_int64(0)
        ng = self.L.orc_bin(self.h, _p(sorter, C.c_uint64), _p(order, C.c_int32), _p(gf, C.c_int32), _p(gl, C.c_int32),
                            _p(bo, C.c_uint64), _p(pages, C.c_uint64), C.byref(npg))
        return {"sorted": sorter, "order": order, "group_first": gf[:ng], "group_last": gl[:ng],
                "block_offset": bo[:ng], "pages": pages[:npg.value]}

    def reductions(self):
        out = np.zeros(6)
        self.L.orc_reductions(self.h, _p(out))
        return out


def linear_offset(precision, i, j, k):
    return int(lib().orc_linear_offset(precision, i, j, k))


def packed_add(precision, a, b):
    return int(lib().orc_packed_add(precision, a, b))


def masks(precision):
    out = np.zeros(6, np.uint64)
    lib().orc_masks(precision, _p(out, C.c_uint64))
    return out


def svd3(precision, A):
    A = np.ascontiguousarray(A, dtype=np.float64).reshape(9)
    U, s, V = np.zeros(9), np.zeros(3), np.zeros(9)
    lib().orc_svd3(precision, _p(A), _p(U), _p(s), _p(V))
    return U.reshape(3, 3), s, V.reshape(3, 3)


def tau(precision, model, E, nu, F, g=1.0, effective=False, kx_scale=0.0, ky_scale=0.0):
    """Kirchhoff stress of one constitutive model at F (3x3); returns (tau, J)."""
    F = np.ascontiguousarray(F, dtype=np.float64).reshape(9)
    out = np.zeros(9)
    J = lib().orc_tau(precision, model, E, nu, kx_scale, ky_scale, g, int(effective), _p(F), _p(out))
    return out.reshape(3, 3), J


def num_threads():
    return int(lib().orc_num_threads())


# Scene families of the benchmarks (the library's recipe defaults, restated): kind 0 = elastic box, kind 1 =
# AnisoMPM fibre slab. Values: MpmSimulationBase.cpp:39-48 (cfl 0.6), examples/vonMisesTear.h:28 (RPIC for the
# AnisoMPM demos), anisofractureBatch3D.py:144-147 (eta 0.1, zeta 1, residual 0.01).
RECIPE_DEFAULTS = {
    0: dict(dx=1 / 64, dt=1e-4, size=(0.25, 0.25, 0.25), center=(0.5, 0.6, 0.5), velocity=(0.0, -1.0, 0.0), gravity=(0.0, -9.8, 0.0),
            E=1e4, nu=0.3, rho=1000.0, apic=1.0, ground_y=0.05),
    1: dict(dx=1 / 128, dt=5e-5, size=(0.5, 0.1, 0.5), center=(0.5, 0.5, 0.5), velocity=(0.0, 0.0, 0.0), gravity=(0.0, 0.0, 0.0),
            E=5e4, nu=0.25, rho=800.0, apic=0.0, kappa=20.0, alpha=-1.0, l0=None, eta=0.1, zeta=1.0, residual=0.01,
            sigma_c=(400.0, 40.0), pull=0.5, grip=2, model=1, fiber=0.0),
}


def seeded_inputs(kind, seed=12345, ppc_side=2, **over):
    """Particles of a recipe scene from the oracle's own generator: dict of x, v, m, V0, F, sigma_c (float64)
    plus the scene parameters used."""
    p = dict(RECIPE_DEFAULTS[kind])
    p.update(over)
    size, center, vel = (np.asarray(p[k], dtype=np.float64) for k in ("size", "center", "velocity"))
    sc = p.get("sigma_c", (1.0, 0.0))
    L = lib()
    args = [kind, ppc_side, seed, p["dx"], _p(size), _p(center), _p(vel), p["rho"], p.get("kappa", 0.0), sc[0], sc[1]]
    n = L.orc_seeded_inputs(*args, None, None, None, None, None, None, None)
    if n <= 0:
        raise ValueError("empty recipe")
    out = {"x": np.zeros((n, 3)), "v": np.zeros((n, 3)), "m": np.zeros(n), "V0": np.zeros(n), "F": np.zeros((n, 9)), "sigma_c": np.zeros(n)}
    lo = np.zeros(3, np.int64)
    L.orc_seeded_inputs(*args, *(_p(out[k]) for k in ("x", "v", "m", "V0", "F", "sigma_c")), _p(lo, C.c_int64))
    nc = [max(1, int(round(s_ / p["dx"]))) for s_ in size]
    p["lo_cell"], p["cells"] = lo.tolist(), nc
    return out, p


def recipe_scene(kind, precision=8, seed=12345, inputs=None, **over):
    """An OracleScene of a recipe family with inputs from seeded_inputs: the elastic box (corotated, sticky ground)
    or the fibre slab (Neo-Hookean Borden or QR-stable with anisotropic damage, ends pulled apart by sticky
    plates grip cells wide). inputs: particle arrays (x, v, m, V0, F, sigma_c) to use instead of the generated
    ones (the same scene fed with another generator's particles). Returns (scene, particle count)."""
    inp, p = seeded_inputs(kind, seed=seed, **over)
    if inputs is not None:
        if len(inputs["m"]) != len(inp["m"]):
            raise ValueError("inputs of another particle count")
        inp = {k: np.asarray(inputs[k], dtype=np.float64).reshape(inp[k].shape) for k in inp}
    dx = p["dx"]
    o = OracleScene(precision, dx, p["dt"], p["gravity"], p["apic"], 0.6)
    if kind == 0:
        o.add_material(0, p["E"], p["nu"])
        o.add_halfspace((0.0, p["ground_y"], 0.0), (0.0, 1.0, 0.0), 1, 0.0)
        o.set_particles(inp["x"], inp["v"], inp["m"], inp["V0"], F=inp["F"])
    else:
        l0 = p["l0"] if p.get("l0") is not None else 0.5 * dx
        o.add_material(p["model"], p["E"], p["nu"], True, p["alpha"], l0, p["eta"], p["zeta"], p["residual"], kx_scale=p["fiber"])
        x_lo, x_hi = p["lo_cell"][0] * dx, (p["lo_cell"][0] + p["cells"][0]) * dx
        o.add_halfspace((x_lo + p["grip"] * dx, 0.0, 0.0), (1.0, 0.0, 0.0), 1, 0.0, (-p["pull"], 0.0, 0.0))
        o.add_halfspace((x_hi - p["grip"] * dx, 0.0, 0.0), (-1.0, 0.0, 0.0), 1, 0.0, (p["pull"], 0.0, 0.0))
        o.set_particles(inp["x"], inp["v"], inp["m"], inp["V0"], F=inp["F"], sigma_c=inp["sigma_c"])
        if p.get("implicit"):
            o.set_implicit_damage(True)
    return o, len(inp["m"])
