"""Python front end of the GB300 explicit-MPM library (ctypes over the C ABI in include/ziran_gb300.h).

The compute path is the in-tree CUDA library ``libziran_gb300.so``; there is no CPU fallback. Importing
the package builds the library when it is missing or stale (nvcc required) and raises if it cannot be
loaded. Names follow Ziran's MPM API: a :class:`Scene` is one ``MpmSimulationBase<T,3>`` /
``AnisoFractureSimulation``, a :class:`Batch` advances many scenes in one launch per kernel.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

HERE = os.path.dirname(os.path.abspath(__file__))

ZR_OK = 0
ZR_ERR_ARG, ZR_ERR_CUDA, ZR_ERR_CFL, ZR_ERR_NONFINITE, ZR_ERR_OUT_OF_DOMAIN = 1, 2, 3, 4, 5
ZR_ERR_BUDGET, ZR_ERR_TIMEOUT, ZR_ERR_CAPACITY, ZR_ERR_STATE = 6, 7, 8, 9
ERROR_NAMES = {1: "ARG", 2: "CUDA", 3: "CFL", 4: "NONFINITE", 5: "OUT_OF_DOMAIN", 6: "BUDGET", 7: "TIMEOUT", 8: "CAPACITY", 9: "STATE"}
F32, F64 = 4, 8
COROTATED, NEOHOOKEAN_BORDEN, QR_STABLE_NEOHOOKEAN = 0, 1, 2
STICKY, SLIP, SEPARATE = 1, 2, 3
FIELD = {"x": (0, 3), "v": (1, 3), "C": (2, 9), "F": (3, 9), "d": (4, 1), "m": (5, 1), "V0": (6, 1), "sigma_c": (7, 1), "dtilde_max": (8, 1)}
RECIPE_ELASTIC_BOX, RECIPE_ANISO_SLAB = 0, 1
BGEO_V, BGEO_D, BGEO_A1 = 1, 2, 4


class ZrError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"ZR_ERR_{ERROR_NAMES.get(code, code)}: {msg}")
        self.code = code


class SimParams(C.Structure):
    _fields_ = [("dx", C.c_double), ("dt", C.c_double), ("gravity", C.c_double * 3), ("apic_rpic_ratio", C.c_double),
                ("cfl", C.c_double), ("domain_cells", C.c_int32), ("reserved", C.c_int32)]


class Recipe(C.Structure):
    _fields_ = [("kind", C.c_int32), ("ppc_side", C.c_int32), ("seed", C.c_uint64), ("dx", C.c_double), ("dt", C.c_double),
                ("size", C.c_double * 3), ("center", C.c_double * 3), ("velocity", C.c_double * 3), ("gravity", C.c_double * 3),
                ("E", C.c_double), ("nu", C.c_double), ("rho", C.c_double), ("apic_rpic_ratio", C.c_double), ("ground_y", C.c_double),
                ("kappa_vmf", C.c_double), ("alpha", C.c_double), ("l0", C.c_double), ("eta", C.c_double), ("zeta", C.c_double),
                ("residual", C.c_double), ("sigma_c_mean", C.c_double), ("sigma_c_std", C.c_double), ("pull_speed", C.c_double),
                ("grip_cells", C.c_double), ("domain_cells", C.c_int32), ("model", C.c_int32), ("fiber_stiffness", C.c_double),
                ("implicit_damage", C.c_int32), ("reserved2", C.c_int32)]


_lib = None


def library_path():
    return _build.LIB


def load_library(build_if_needed=True):
    """Load libziran_gb300.so (building it in-tree first when needed). Raises when it cannot be loaded."""
    global _lib
    if _lib is not None:
        return _lib
    if build_if_needed:
        _build.build()
    if not os.path.exists(_build.LIB):
        raise RuntimeError("libziran_gb300.so is missing: run `python -m ziran2020_gb300.build`")
    L = C.CDLL(_build.LIB)
    P, vp, i32, i64, d = C.POINTER, C.c_void_p, C.c_int, C.c_int64, C.c_double
    pd = P(d)
    sig = {
        "zr_scene_create": (i32, [i32, P(vp)]),
        "zr_scene_destroy": (i32, [vp]),
        "zr_scene_set_params": (i32, [vp, P(SimParams)]),
        "zr_scene_add_particles": (i32, [vp, i64, pd, pd, pd, pd, pd, P(i64)]),
        "zr_scene_add_corotated": (i32, [vp, i64, i64, d, d]),
        "zr_scene_add_neohookean_borden": (i32, [vp, i64, i64, d, d]),
        "zr_scene_add_aniso_damage": (i32, [vp, i64, i64, d, d, d, d, d, pd]),
        "zr_scene_add_halfspace": (i32, [vp, pd, pd, i32, d, pd]),
        "zr_scene_step": (i32, [vp, i32, P(i32)]),
        "zr_scene_get_field": (i32, [vp, i32, vp, i32]),
        "zr_scene_set_field": (i32, [vp, i32, vp, i32]),
        "zr_scene_get_state": (i32, [vp, vp, i32]),
        "zr_scene_set_state": (i32, [vp, vp, i32]),
        "zr_scene_exchange_state": (i32, [vp, vp, vp, i32]),
        "zr_scene_step_stream": (i32, [vp, i32, vp, vp, i32]),
        "zr_scene_stream_reruns": (i32, [vp, P(i64)]),
        "zr_scene_reductions": (i32, [vp, pd]),
        "zr_scene_set_dt": (i32, [vp, d]),
        "zr_scene_set_implicit_damage": (i32, [vp, i32]),
        "zr_scene_cg_iterations": (i32, [vp, P(i32)]),
        "zr_scene_time": (d, [vp]),
        "zr_scene_count": (i64, [vp]),
        "zr_scene_last_error": (C.c_char_p, [vp]),
        "zr_scene_last_step_ms": (d, [vp]),
        "zr_scene_last_grid": (i32, [vp, P(i64), P(i64)]),
        "zr_batch_last_step_ms": (d, [vp]),
        "zr_scene_binning": (i32, [vp, P(C.c_uint64), P(C.c_int32), P(C.c_int32), P(i64), P(C.c_uint64), P(i64)]),
        "zr_scene_set_timing": (i32, [vp, i32]),
        "zr_scene_get_timing": (i32, [vp, pd, P(i64)]),
        "zr_scene_set_autotune": (i32, [vp, i32]),
        "zr_scene_state_bytes": (i64, [vp]),
        "zr_scene_save_state": (i32, [vp, vp, i64]),
        "zr_scene_load_state": (i32, [vp, vp, i64]),
        "zr_scene_write_state_file": (i32, [vp, C.c_char_p]),
        "zr_scene_read_state_file": (i32, [vp, C.c_char_p]),
        "zr_scene_write_bgeo": (i32, [vp, C.c_char_p, i32]),
        "zr_write_bgeo": (i32, [C.c_char_p, i64, pd, i32, P(C.c_char_p), P(C.c_int32), P(pd)]),
        "zr_scene_advance_frames": (i32, [vp, i32, d, d, i32, P(i32)]),
        "zr_scene_set_schedule": (i32, [vp, P(i32)]),
        "zr_scene_get_schedule": (i32, [vp, P(i32)]),
        "zr_scene_stats": (i32, [vp, P(i64), P(i64), P(i64)]),
        "zr_recipe_default": (i32, [i32, P(Recipe)]),
        "zr_recipe_count": (i64, [P(Recipe)]),
        "zr_recipe_generate": (i32, [P(Recipe), pd, pd, pd, pd, pd, pd]),
        "zr_scene_from_recipe": (i32, [vp, P(Recipe)]),
        "zr_rotated_F": (None, [pd, pd]),
        "zr_nhb_sigma_crit": (d, [d, d, d]),
        "zr_qrnh_sigma_crit": (d, [d, d, d]),
        "zr_scene_add_qr_stable_neohookean": (i32, [vp, i64, i64, d, d, d, d]),
        "zr_batch_create": (i32, [i32, P(vp)]),
        "zr_batch_destroy": (i32, [vp]),
        "zr_batch_add_scene": (i32, [vp, vp, P(i32)]),
        "zr_batch_add_recipe": (i32, [vp, P(Recipe), P(i32)]),
        "zr_batch_commit": (i32, [vp]),
        "zr_batch_step": (i32, [vp, i32, P(i32)]),
        "zr_batch_get_field": (i32, [vp, i32, i32, vp, i32]),
        "zr_batch_reductions": (i32, [vp, i32, pd]),
        "zr_batch_count": (i64, [vp, i32]),
        "zr_batch_set_timing": (i32, [vp, i32]),
        "zr_batch_get_timing": (i32, [vp, pd, P(i64)]),
        "zr_batch_set_autotune": (i32, [vp, i32]),
        "zr_batch_get_schedule": (i32, [vp, P(i32)]),
        "zr_batch_stats": (i32, [vp, P(i64), P(i64), P(i64)]),
        "zr_batch_last_error": (C.c_char_p, [vp]),
        "zr_version": (C.c_char_p, []),
        "zr_server_create": (i32, [i32, d, i32, i32, P(vp)]),
        "zr_server_destroy": (i32, [vp]),
        "zr_server_submit_recipe": (i32, [vp, P(Recipe), i32, P(i64)]),
        "zr_server_submit_scene": (i32, [vp, vp, i32, P(i64)]),
        "zr_server_tick": (i32, [vp, P(i32), P(i32), P(i32)]),
        "zr_server_request": (i32, [vp, i64, P(i32), P(d), P(i64), P(i32)]),
        "zr_server_result": (i32, [vp, i64, i32, vp, i32]),
        "zr_server_release": (i32, [vp, i64]),
        "zr_server_stats": (i32, [vp, P(d), P(d), P(i64)]),
        "zr_server_last_error": (C.c_char_p, [vp]),
        "zr_bin_device_noalloc": (i32, [i32, i64, vp, d, C.c_int32, vp, vp, vp, P(i64), vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def _dp(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


def _f64(a, shape_last=None):
    if a is None:
        return None
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a


def recipe(kind, **kw):
    """Default recipe of `kind` with fields overridden by keyword (vectors as 3-sequences)."""
    L = load_library()
    r = Recipe()
    rc = L.zr_recipe_default(kind, C.byref(r))
    if rc:
        raise ZrError(rc, "unknown recipe kind")
    for k, v in kw.items():
        if k in ("size", "center", "velocity", "gravity"):
            getattr(r, k)[:] = [float(t) for t in v]
        else:
            setattr(r, k, v)
    return r


def recipe_count(r):
    return int(load_library().zr_recipe_count(C.byref(r)))


def recipe_generate(r):
    """Particles of a recipe as float64 arrays: x (n,3), v (n,3), m, V0, F (n,9), sigma_c."""
    n = recipe_count(r)
    x, v, F = np.zeros((n, 3)), np.zeros((n, 3)), np.zeros((n, 9))
    m, V0, sc = np.zeros(n), np.zeros(n), np.zeros(n)
    rc = load_library().zr_recipe_generate(C.byref(r), _dp(x), _dp(v), _dp(m), _dp(V0), _dp(F), _dp(sc))
    if rc:
        raise ZrError(rc, "recipe generation failed")
    return {"x": x, "v": v, "m": m, "V0": V0, "F": F, "sigma_c": sc}


def rotated_F(a0):
    a = np.ascontiguousarray(a0, dtype=np.float64)
    F = np.zeros(9)
    load_library().zr_rotated_F(_dp(a), _dp(F))
    return F.reshape(3, 3)


def nhb_sigma_crit(E, nu, percentage):
    return float(load_library().zr_nhb_sigma_crit(E, nu, percentage))


def qrnh_sigma_crit(E, nu, percentage):
    return float(load_library().zr_qrnh_sigma_crit(E, nu, percentage))


class Scene:
    """One explicit-MPM simulation on the GPU (MpmSimulationBase<T,3> with the AnisoMPM damage override)."""

    def __init__(self, precision=F32):
        self.L = load_library()
        self.h = C.c_void_p()
        self._check(self.L.zr_scene_create(precision, C.byref(self.h)))
        self.precision = precision

    def _check(self, rc):
        if rc:
            msg = self.L.zr_scene_last_error(self.h).decode() if getattr(self, "h", None) else ""
            raise ZrError(rc, msg)
        return rc

    def close(self):
        if self.h:
            self.L.zr_scene_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, dx, dt, gravity=(0.0, 0.0, 0.0), apic_rpic_ratio=1.0, cfl=0.6, domain_cells=0):
        p = SimParams(dx, dt, (C.c_double * 3)(*gravity), apic_rpic_ratio, cfl, domain_cells, 0)
        self._check(self.L.zr_scene_set_params(self.h, C.byref(p)))

    def add_particles(self, x, m, V0, v=None, F=None):
        x, m, V0, v, F = _f64(x), _f64(m), _f64(V0), _f64(v), _f64(F)
        first = C.c_int64()
        self._check(self.L.zr_scene_add_particles(self.h, x.shape[0], _dp(x), _dp(v), _dp(m), _dp(V0), _dp(F), C.byref(first)))
        return first.value

    def add_corotated(self, first, count, E, nu):
        self._check(self.L.zr_scene_add_corotated(self.h, first, count, E, nu))

    def add_neohookean_borden(self, first, count, E, nu):
        self._check(self.L.zr_scene_add_neohookean_borden(self.h, first, count, E, nu))

    def add_qr_stable_neohookean(self, first, count, E, nu, fiber_x=0.0, fiber_y=0.0):
        self._check(self.L.zr_scene_add_qr_stable_neohookean(self.h, first, count, E, nu, fiber_x, fiber_y))

    def add_aniso_damage(self, first, count, alpha, l0, eta, zeta, residual, sigma_crit):
        sc = _f64(sigma_crit)
        self._check(self.L.zr_scene_add_aniso_damage(self.h, first, count, alpha, l0, eta, zeta, residual, _dp(sc)))

    def add_halfspace(self, origin, normal, type_=STICKY, friction=0.0, velocity=(0.0, 0.0, 0.0)):
        o, n, v = (np.ascontiguousarray(a, dtype=np.float64) for a in (origin, normal, velocity))
        self._check(self.L.zr_scene_add_halfspace(self.h, _dp(o), _dp(n), type_, friction, _dp(v)))

    def from_recipe(self, r):
        self._check(self.L.zr_scene_from_recipe(self.h, C.byref(r)))

    def step(self, n=1):
        done = C.c_int()
        rc = self.L.zr_scene_step(self.h, n, C.byref(done))
        self.last_done = done.value
        self._check(rc)
        return done.value

    def get(self, name, dtype=np.float64):
        fid, nc = FIELD[name]
        n = self.count
        out = np.zeros((n, nc) if nc > 1 else n, dtype=dtype)
        self._check(self.L.zr_scene_get_field(self.h, fid, out.ctypes.data_as(C.c_void_p), F64 if dtype == np.float64 else F32))
        return out

    def set(self, name, values):
        fid, nc = FIELD[name]
        a = np.ascontiguousarray(values)
        dt = F32 if a.dtype == np.float32 else F64
        if dt == F64:
            a = a.astype(np.float64, copy=False)
        self._check(self.L.zr_scene_set_field(self.h, fid, a.ctypes.data_as(C.c_void_p), dt))

    def get_state(self, out):
        dt = F32 if out.dtype == np.float32 else F64
        self._check(self.L.zr_scene_get_state(self.h, out.ctypes.data_as(C.c_void_p), dt))
        return out

    def set_state(self, a):
        dt = F32 if a.dtype == np.float32 else F64
        self._check(self.L.zr_scene_set_state(self.h, a.ctypes.data_as(C.c_void_p), dt))

    def exchange_state(self, a, out):
        """Download the state into out and upload a as the new state, in one call (a and out of one dtype, not
        overlapping; with both in pinned memory the two directions of the host link run at once)."""
        if a.dtype != out.dtype:
            raise ValueError("exchange_state: input and output buffers must have the same dtype")
        for b in (a, out):
            if b.size != self.count * 25 or not b.flags.c_contiguous:
                raise ValueError("exchange_state: buffers of count x 25 contiguous values expected")
        dt = F32 if a.dtype == np.float32 else F64
        self._check(self.L.zr_scene_exchange_state(self.h, a.ctypes.data_as(C.c_void_p), out.ctypes.data_as(C.c_void_p), dt))
        return out

    def step_stream(self, inputs, outputs):
        """len(inputs) independent jobs: job i sets the state from inputs[i], advances one substep and writes the result
        to outputs[i] (count x 25 arrays of one dtype); copies of the next inputs and the last results overlap the
        computation (pinned arrays give the overlap)."""
        n = len(inputs)
        if len(outputs) != n:
            raise ValueError("step_stream: as many outputs as inputs")
        if n == 0:
            return outputs
        dtype = inputs[0].dtype
        for b in list(inputs) + list(outputs):
            if b.dtype != dtype or b.size != self.count * 25 or not b.flags.c_contiguous:
                raise ValueError("step_stream: buffers of count x 25 contiguous values of one dtype expected")
        pin = (C.c_void_p * n)(*[b.ctypes.data for b in inputs])
        pout = (C.c_void_p * n)(*[b.ctypes.data for b in outputs])
        self._check(self.L.zr_scene_step_stream(self.h, n, C.cast(pin, C.c_void_p), C.cast(pout, C.c_void_p), F32 if dtype == np.float32 else F64))
        return outputs

    @property
    def stream_reruns(self):
        """Jobs of step_stream calls run again the safe way after an aborted job (cumulative)."""
        v = C.c_int64()
        self._check(self.L.zr_scene_stream_reruns(self.h, C.byref(v)))
        return v.value

    def reductions(self):
        out = np.zeros(7)
        self._check(self.L.zr_scene_reductions(self.h, _dp(out)))
        return out

    def set_dt(self, dt):
        self._check(self.L.zr_scene_set_dt(self.h, dt))

    def set_implicit_damage(self, on=True):
        """Solve the damage implicitly (AnisoFractureSimulation.h:437-626) instead of the explicit update;
        before the first substep."""
        self._check(self.L.zr_scene_set_implicit_damage(self.h, 1 if on else 0))

    @property
    def cg_iterations(self):
        """Conjugate-gradient iterations of the last substep's implicit damage solve."""
        it = C.c_int(0)
        self._check(self.L.zr_scene_cg_iterations(self.h, C.byref(it)))
        return it.value

    @property
    def last_step_ms(self):
        return float(self.L.zr_scene_last_step_ms(self.h))

    def last_grid(self):
        g, b = C.c_int64(), C.c_int64()
        self._check(self.L.zr_scene_last_grid(self.h, C.byref(g), C.byref(b)))
        return g.value, b.value

    @property
    def time(self):
        return float(self.L.zr_scene_time(self.h))

    @property
    def count(self):
        return int(self.L.zr_scene_count(self.h))

    def binning(self):
        n = self.count
        keys = np.zeros(n, np.uint64)
        order = np.zeros(n, np.int32)
        gf = np.zeros(n, np.int32)
        pages = np.zeros(8 * n, np.uint64)
        ng, npg = C.c_int64(), C.c_int64()
        self._check(self.L.zr_scene_binning(self.h, keys.ctypes.data_as(C.POINTER(C.c_uint64)), order.ctypes.data_as(C.POINTER(C.c_int32)),
                                            gf.ctypes.data_as(C.POINTER(C.c_int32)), C.byref(ng), pages.ctypes.data_as(C.POINTER(C.c_uint64)),
                                            C.byref(npg)))
        return {"sorted": keys, "order": order, "group_first": gf[: ng.value], "pages": pages[: npg.value]}

    def set_timing(self, on):
        self._check(self.L.zr_scene_set_timing(self.h, int(on)))

    def timing(self):
        out = np.zeros(5)
        steps = C.c_int64()
        self._check(self.L.zr_scene_get_timing(self.h, _dp(out), C.byref(steps)))
        return dict(zip(("sort", "activate", "p2g", "grid", "g2p"), out)), steps.value

    def set_autotune(self, mode):
        """0 fixed default schedule, 1 autotuned and cached per workload class, 2 re-measured per batch."""
        self._check(self.L.zr_scene_set_autotune(self.h, int(mode)))

    def save_state(self):
        """The scene's dynamic state as a binary image (bytes)."""
        n = self.L.zr_scene_state_bytes(self.h)
        if n < 0:
            raise ZrError(ZR_ERR_STATE, "no particles")
        buf = C.create_string_buffer(n)
        self._check(self.L.zr_scene_save_state(self.h, buf, n))
        return buf.raw

    def load_state(self, image):
        buf = C.create_string_buffer(bytes(image), len(image))
        self._check(self.L.zr_scene_load_state(self.h, buf, len(image)))

    def write_state(self, path):
        self._check(self.L.zr_scene_write_state_file(self.h, os.fsencode(path)))

    def read_state(self, path):
        self._check(self.L.zr_scene_read_state_file(self.h, os.fsencode(path)))

    def write_bgeo(self, path, v=False, d=False, a1=False):
        """Frame file for visualisation (.bgeo): positions and, as chosen, velocity "v", damage "d" and the current
        fibre director "a_1" (the reference's writePartio / anisoFrax frames)."""
        flags = (BGEO_V if v else 0) | (BGEO_D if d else 0) | (BGEO_A1 if a1 else 0)
        self._check(self.L.zr_scene_write_bgeo(self.h, os.fsencode(path), flags))

    def advance_frames(self, frames, frame_dt, min_dt=1e-6, cfl_dt=False):
        """Whole frames with the reference's time stepping and CFL restarts; returns the number of restarts."""
        r = C.c_int()
        self._check(self.L.zr_scene_advance_frames(self.h, int(frames), float(frame_dt), float(min_dt), int(cfl_dt), C.byref(r)))
        return r.value

    def set_schedule(self, chunk, buffers, p2g_ctas_per_sm, g2p_threads, fused=0, g2p_tight=0):
        """chunk/buffers select the split P2G form's staging; fused=1 selects the one-kernel P2G, fused=2 the
        same with registers cut for one more CTA per SM, fused=3 its warp-specialised form (producer and consumer
        warps); g2p_tight: +1 cuts G2P
        registers likewise, +2 stages the velocities of the 8 neighbouring blocks by bulk asynchronous copies."""
        arr = (C.c_int32 * 6)(int(fused), chunk, buffers, p2g_ctas_per_sm, g2p_threads, int(g2p_tight))
        self._check(self.L.zr_scene_set_schedule(self.h, arr))

    def schedule(self):
        rc, out = _schedule(self.L.zr_scene_get_schedule, self.h)
        self._check(rc)
        return out

    def stats(self):
        a, b, c = C.c_int64(), C.c_int64(), C.c_int64()
        self._check(self.L.zr_scene_stats(self.h, C.byref(a), C.byref(b), C.byref(c)))
        return {"launches_per_step": a.value, "device_bytes": b.value, "fallbacks": c.value}


class Batch:
    """Many independent scenes advanced together (one launch per kernel for the whole batch)."""

    def __init__(self, precision=F32):
        self.L = load_library()
        self.h = C.c_void_p()
        self._check(self.L.zr_batch_create(precision, C.byref(self.h)))

    def _check(self, rc):
        if rc:
            raise ZrError(rc, self.L.zr_batch_last_error(self.h).decode())
        return rc

    def close(self):
        if self.h:
            self.L.zr_batch_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_scene(self, scene):
        slot = C.c_int()
        self._check(self.L.zr_batch_add_scene(self.h, scene.h, C.byref(slot)))
        return slot.value

    def add_recipe(self, r):
        slot = C.c_int()
        self._check(self.L.zr_batch_add_recipe(self.h, C.byref(r), C.byref(slot)))
        return slot.value

    def commit(self):
        self._check(self.L.zr_batch_commit(self.h))

    def step(self, n=1):
        done = C.c_int()
        rc = self.L.zr_batch_step(self.h, n, C.byref(done))
        self.last_done = done.value
        self._check(rc)
        return done.value

    def count(self, slot):
        return int(self.L.zr_batch_count(self.h, slot))

    @property
    def last_step_ms(self):
        return float(self.L.zr_batch_last_step_ms(self.h))

    def get(self, slot, name, dtype=np.float64):
        fid, nc = FIELD[name]
        n = self.count(slot)
        out = np.zeros((n, nc) if nc > 1 else n, dtype=dtype)
        self._check(self.L.zr_batch_get_field(self.h, slot, fid, out.ctypes.data_as(C.c_void_p), F64 if dtype == np.float64 else F32))
        return out

    def reductions(self, slot):
        out = np.zeros(7)
        self._check(self.L.zr_batch_reductions(self.h, slot, _dp(out)))
        return out

    def set_timing(self, on):
        self._check(self.L.zr_batch_set_timing(self.h, int(on)))

    def timing(self):
        out = np.zeros(5)
        steps = C.c_int64()
        self._check(self.L.zr_batch_get_timing(self.h, _dp(out), C.byref(steps)))
        return dict(zip(("sort", "activate", "p2g", "grid", "g2p"), out)), steps.value

    def set_autotune(self, mode):
        self._check(self.L.zr_batch_set_autotune(self.h, int(mode)))

    def schedule(self):
        rc, out = _schedule(self.L.zr_batch_get_schedule, self.h)
        self._check(rc)
        return out

    def stats(self):
        a, b, c = C.c_int64(), C.c_int64(), C.c_int64()
        self._check(self.L.zr_batch_stats(self.h, C.byref(a), C.byref(b), C.byref(c)))
        return {"launches_per_step": a.value, "device_bytes": b.value, "fallbacks": c.value}


def _schedule(fn, h):
    out = (C.c_int32 * 7)()
    rc = fn(h, out)
    return rc, {"fused": out[0], "chunk": out[1], "buffers": out[2], "p2g_ctas_per_sm": out[3], "g2p_threads": out[4], "g2p_tight": out[5],
                "tuned": bool(out[6])}



class Server:
    """Continuous-batching request loop: requests (scene recipe + substeps) are admitted by a device-memory
    budget, advanced together with the resident scenes, and retired with their final state on the host."""

    QUEUED, RUNNING, DONE, FAILED = 0, 1, 2, 3

    def __init__(self, precision=F32, budget_bytes=60e9, tick_substeps=10, max_scenes=256):
        self.L = load_library()
        self.h = C.c_void_p()
        rc = self.L.zr_server_create(precision, float(budget_bytes), tick_substeps, max_scenes, C.byref(self.h))
        if rc:
            raise ZrError(rc, "bad server configuration")

    def _check(self, rc):
        if rc:
            raise ZrError(rc, self.L.zr_server_last_error(self.h).decode())
        return rc

    def close(self):
        if self.h:
            self.L.zr_server_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, r, substeps):
        rid = C.c_int64()
        self._check(self.L.zr_server_submit_recipe(self.h, C.byref(r), substeps, C.byref(rid)))
        return rid.value

    def submit_scene(self, scene, substeps):
        rid = C.c_int64()
        self._check(self.L.zr_server_submit_scene(self.h, scene.h, substeps, C.byref(rid)))
        return rid.value

    def tick(self):
        a, b, c = C.c_int(), C.c_int(), C.c_int()
        self._check(self.L.zr_server_tick(self.h, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    def request(self, rid):
        st, lat, n, k = C.c_int(), C.c_double(), C.c_int64(), C.c_int()
        self._check(self.L.zr_server_request(self.h, rid, C.byref(st), C.byref(lat), C.byref(n), C.byref(k)))
        return {"state": st.value, "latency_s": lat.value, "particles": n.value, "substeps": k.value}

    def result(self, rid, name, dtype=np.float64):
        fid, nc = FIELD[name]
        n = self.request(rid)["particles"]
        out = np.zeros((n, nc) if nc > 1 else n, dtype=dtype)
        self._check(self.L.zr_server_result(self.h, rid, fid, out.ctypes.data_as(C.c_void_p), F64 if dtype == np.float64 else F32))
        return out

    def release(self, rid):
        self._check(self.L.zr_server_release(self.h, rid))

    def stats(self):
        a, b, c = C.c_double(), C.c_double(), C.c_int64()
        self._check(self.L.zr_server_stats(self.h, C.byref(a), C.byref(b), C.byref(c)))
        return {"particle_substeps": a.value, "device_ms": b.value, "device_bytes": c.value}


def version():
    return load_library().zr_version().decode()


def write_bgeo(path, x, attributes=None):
    """Write n points (x: (n, 3)) and named float attributes ({name: (n,) or (n, k) array}) as a .bgeo file."""
    x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, 3)
    attributes = attributes or {}
    names, sizes, arrays = [], [], []
    for k, a in attributes.items():
        a = np.ascontiguousarray(a, dtype=np.float64).reshape(len(x), -1)
        names.append(k.encode())
        sizes.append(a.shape[1])
        arrays.append(a)
    na = len(names)
    cn = (C.c_char_p * max(1, na))(*names)
    cs = (C.c_int32 * max(1, na))(*sizes)
    cd = (C.POINTER(C.c_double) * max(1, na))(*[_dp(a) for a in arrays])
    rc = load_library().zr_write_bgeo(os.fsencode(path), len(x), _dp(x), na, cn, cs, cd)
    if rc:
        raise ZrError(rc, f"cannot write {path}")
