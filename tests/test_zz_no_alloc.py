"""GPU: the binning entry point that allocates no device memory (zr_bin_device_noalloc).

It serves callers that may not allocate device memory while they run (a host that reserved one arena at
start-up, a loop with a fixed budget, a callback inside another runtime); all its scratch is a static
device array shared by every call. This file is collected last so that a failure here comes after every
other test has run. Its output must equal, bit for bit, the binning of the allocating scene API
(zr_scene_binning) on the same positions, on two consecutive calls (the second smaller than the first,
so stale scratch from the first call would show up); a call after the warm-up calls must leave the device's
free memory unchanged; a particle outside the stated domain is reported."""
import ctypes as C
import glob
import os

import numpy as np
import pytest

import ziran2020_gb300 as zr

pytestmark = pytest.mark.gpu


def positions(seed, n_side, dx, origin):
    rng = np.random.default_rng(seed)
    g = np.stack(np.meshgrid(*[np.arange(n_side)] * 3, indexing="ij"), -1).reshape(-1, 3)
    x = (g + rng.random(g.shape)) * (dx / 2) + np.asarray(origin)
    rng.shuffle(x)
    return x


def scene_binning(prec, x, dx):
    s = zr.Scene(prec)
    s.set_params(dx, 1e-4)
    n = len(x)
    first = s.add_particles(x, np.ones(n), np.ones(n))
    s.add_corotated(first, n, 1e4, 0.3)
    return s.binning()


def noalloc_binning(prec, x, dx):
    import torch

    L = zr.load_library()
    n = len(x)
    dtype = torch.float32 if prec == zr.F32 else torch.float64
    xd = torch.tensor(np.ascontiguousarray(x).reshape(-1), dtype=dtype, device="cuda")
    keys = torch.empty(n, dtype=torch.int64, device="cuda")
    order = torch.empty(n, dtype=torch.int32, device="cuda")
    first = torch.empty(n, dtype=torch.int32, device="cuda")
    ng = C.c_int64(-1)
    stream = torch.cuda.current_stream().cuda_stream
    rc = L.zr_bin_device_noalloc(prec, n, C.c_void_p(xd.data_ptr()), dx, 0, C.c_void_p(keys.data_ptr()), C.c_void_p(order.data_ptr()),
                                 C.c_void_p(first.data_ptr()), C.byref(ng), C.c_void_p(stream))
    assert rc == zr.ZR_OK, rc
    return {"sorted": keys.cpu().numpy().view(np.uint64), "order": order.cpu().numpy(), "group_first": first.cpu().numpy()[: ng.value]}


@pytest.mark.parametrize("prec", [zr.F32, zr.F64])
def test_noalloc_binning_equals_scene_binning_on_two_calls(prec):
    dx = 1 / 128
    cases = [positions(1, 40, dx, (0.2, 0.3, 0.25)), positions(2, 23, dx, (0.41, 0.22, 0.5))]  # 64000 then 12167 particles
    for x in cases:
        if prec == zr.F32:
            x = x.astype(np.float32).astype(np.float64)  # both paths bin the same float values
        want = scene_binning(prec, x, dx)
        got = noalloc_binning(prec, x, dx)
        assert np.array_equal(got["sorted"], want["sorted"])
        assert np.array_equal(got["order"], want["order"])
        assert np.array_equal(got["group_first"], want["group_first"])


GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "binning_*.npz")))


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[8:-4] for p in GOLDEN])
def test_noalloc_binning_matches_reference_spgrid(path):
    """The golden vectors made by the reference's own SPGrid code (cell-face positions, duplicates, coordinates up
    to ~4000 cells, cell sizes whose reciprocal is inexact): sorted keys, order and group starts bit for bit."""
    g = np.load(path)
    got = noalloc_binning(int(g["precision"]), g["x"], float(g["dx"]))
    assert np.array_equal(got["sorted"], g["sorted"])
    assert np.array_equal(got["order"], g["order"])
    assert np.array_equal(got["group_first"], g["group_first"])


def test_noalloc_rejects_sizes_beyond_its_static_scratch():
    import torch

    L = zr.load_library()
    big = (1 << 20) + 1
    dummy = torch.empty(16, dtype=torch.float32, device="cuda")
    p = C.c_void_p(dummy.data_ptr())
    ng = C.c_int64()
    assert L.zr_bin_device_noalloc(zr.F32, big, p, 1 / 64, 0, p, p, p, C.byref(ng), None) == zr.ZR_ERR_ARG


def _noalloc_call(L, prec, xd, n, dx, domain_cells, keys, order, first, ng, stream):
    return L.zr_bin_device_noalloc(prec, n, C.c_void_p(xd.data_ptr()), dx, domain_cells, C.c_void_p(keys.data_ptr()),
                                   C.c_void_p(order.data_ptr()), C.c_void_p(first.data_ptr()), C.byref(ng), C.c_void_p(stream))


def test_noalloc_call_leaves_free_device_memory_unchanged():
    """The property the entry point exists for: once each precision has been called (set-up and kernel
    loading), a call changes the device's free memory by nothing (cudaMemGetInfo before and after)."""
    import torch

    L = zr.load_library()
    dx = 1 / 128
    x = positions(5, 32, dx, (0.3, 0.3, 0.3))
    n = len(x)
    bufs = {}
    for prec, dtype in ((zr.F32, torch.float32), (zr.F64, torch.float64)):
        bufs[prec] = (torch.tensor(x.reshape(-1), dtype=dtype, device="cuda"), torch.empty(n, dtype=torch.int64, device="cuda"),
                      torch.empty(n, dtype=torch.int32, device="cuda"), torch.empty(n, dtype=torch.int32, device="cuda"))
    stream = torch.cuda.current_stream().cuda_stream
    ng = C.c_int64(-1)
    for prec in (zr.F32, zr.F64):  # warm-up: per-device set-up and each precision's kernels
        xd, keys, order, first = bufs[prec]
        assert _noalloc_call(L, prec, xd, n, dx, 0, keys, order, first, ng, stream) == zr.ZR_OK
    torch.cuda.synchronize()
    for prec in (zr.F32, zr.F64):
        xd, keys, order, first = bufs[prec]
        free0 = torch.cuda.mem_get_info()[0]
        assert _noalloc_call(L, prec, xd, n, dx, 0, keys, order, first, ng, stream) == zr.ZR_OK
        torch.cuda.synchronize()
        assert torch.cuda.mem_get_info()[0] == free0, prec


def test_noalloc_reports_particles_outside_the_domain():
    """A base node at or beyond domain_cells gives ZR_ERR_OUT_OF_DOMAIN (the reference's SPGrid range
    assertion); the next call with in-domain positions succeeds again (the flag is cleared per call)."""
    import torch

    L = zr.load_library()
    dx = 1 / 64
    x = positions(9, 12, dx, (0.2, 0.2, 0.2))
    x[7] = (1.5, 0.3, 0.3)  # base node 95 in x, beyond a 68-cell domain
    n = len(x)
    xd = torch.tensor(x.reshape(-1), dtype=torch.float64, device="cuda")
    keys = torch.empty(n, dtype=torch.int64, device="cuda")
    order = torch.empty(n, dtype=torch.int32, device="cuda")
    first = torch.empty(n, dtype=torch.int32, device="cuda")
    ng = C.c_int64(-1)
    stream = torch.cuda.current_stream().cuda_stream
    assert _noalloc_call(L, zr.F64, xd, n, dx, 68, keys, order, first, ng, stream) == zr.ZR_ERR_OUT_OF_DOMAIN
    x[7] = (0.25, 0.3, 0.3)
    xd.copy_(torch.tensor(x.reshape(-1), dtype=torch.float64))
    assert _noalloc_call(L, zr.F64, xd, n, dx, 68, keys, order, first, ng, stream) == zr.ZR_OK
