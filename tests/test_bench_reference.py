"""CPU: the bench's reference arm (the oracle restatement of the reference's CPU algorithm) runs the same
workload as the GPU arm, with inputs from the oracle's own generator, and loads no product library."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_same_workload_without_product_library():
    code = ("import sys; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '1', '--workload', 'aniso_slab_dx128']; "
            "import bench; bench.main(); print('PRODUCT_LOADED', 'libziran_gb300' in open('/proc/self/maps').read())")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = r.stdout.splitlines()
    line = json.loads(next(l for l in lines if l.startswith("{")))
    assert "PRODUCT_LOADED False" in lines
    assert line["impl"] == "reference" and line["dtype"] == "f64"
    cfg = line["config"]
    assert cfg["workload"] == "aniso_slab_dx128" and cfg["particles"] == 425984 and cfg["precision_path"] == "fp64"
    assert line["cpu_baseline"]["kind"] == "port" and line["value"] > 0
