"""The C++ shim (include/ziran_gb300.hpp) compiles against the C ABI and links to the in-tree library; on a
GPU the demo scenes run: a corotated cube conserves momentum up to the gravity impulse, and a QR-stable
Neo-Hookean piece with fibre stiffness and anisotropic damage tears when pulled."""
import os
import subprocess

import pytest

import ziran2020_gb300 as zr

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "shim_demo.cpp")


def build_demo(tmp_path):
    lib = zr.library_path()
    exe = str(tmp_path / "shim_demo")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), SRC, "-o", exe, lib,
                           "-Wl,-rpath," + os.path.dirname(lib)])
    return exe


def test_shim_compiles_and_links(tmp_path):
    zr.load_library()
    assert os.path.exists(build_demo(tmp_path))


@pytest.mark.gpu
def test_shim_demo_runs(tmp_path):
    exe = build_demo(tmp_path)
    out = subprocess.check_output([exe], text=True).split()
    n, t, py = int(out[1]), float(out[3]), float(out[5])
    assert n == 4096
    assert abs(t - 20 * 1e-4) < 1e-9
    m_total = n * 1000 * (1 / 64) ** 3 / 8
    assert abs(py - m_total * (-1.0 - 9.8 * 20e-4)) < 1e-4 * m_total
    # the QR-stable Neo-Hookean piece with fibre stiffness and anisotropic damage: pulled at 1 m/s, it tears
    n2, dmax = int(out[7]), float(out[9])
    assert n2 == 12 * 4 * 4 * 8
    assert 0 < dmax <= 1
    # the same piece with the implicit damage solve (sim.implicit = true): damage grows, the CG iterated
    n3, dmax3, cg3 = int(out[13]), float(out[15]), int(out[17])
    assert n3 == n2 and 0 < dmax3 <= 1 and cg3 > 0
    # two one-substep jobs of the same state through stepJobs (zr_scene_step_stream): the same result, and it moved
    jobs_diff, moved, reruns = float(out[19]), float(out[21]), int(out[23])
    assert jobs_diff < 1e-6 and 1e-5 < moved < 1e-3
    assert reruns == 0  # the second job ran on the pipelined path
