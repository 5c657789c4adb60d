#!/usr/bin/env python
"""Benchmark of the explicit MPM substep on GB300: particle-substeps/s, FP32 path beside the plain FP64
GPU path, with the FP32-vs-FP64 error, the roofline of the dominant kernel and the CPU baseline.

Workload (one GPU): the AnisoMPM slab at dx = 1/256 — 0.5 x 0.1 x 0.5 m, 8 particles per cell
(128 x 26 x 128 cells = 3,407,872 particles), Neo-Hookean (Borden) E=5e4 Pa, nu=0.25, rho=800,
fibres vMF(kappa=20) about +x, anisotropic damage alpha=-1, l0=0.5 dx, sigma_c ~ N(400, 40) Pa,
ends pulled apart at +-0.5 m/s, dt = 5e-5, seeded synthetic inputs. One "step" is one substep of the
whole scene. The particle state (~0.8 GB in FP32, two alternating copies) is larger than L2, so no L2
flush is needed between substeps.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
Under torchrun each rank advances its own scene (replicas, weak scaling); rank 0 prints one JSON line.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # name: (recipe kind, overrides)
    "aniso_slab_dx256": (1, dict(dx=1 / 256, l0=0.5 / 256)),
    "aniso_slab_dx128": (1, dict()),
    "elastic_box_dx64": (0, dict()),
    # the same slab with the QR-stable Neo-Hookean model and fibre stiffness 10 mu (examples/tubepull.h:104-107)
    "aniso_slab_qr_dx256": (1, dict(dx=1 / 256, l0=0.5 / 256, model=2, fiber_stiffness=10.0)),
    # the same slab with the implicit damage solve (AnisoFractureSimulation.h:437-626) instead of the explicit update
    "aniso_slab_implicit_dx256": (1, dict(dx=1 / 256, l0=0.5 / 256, implicit_damage=1)),
}
def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="aniso_slab_dx256", choices=sorted(WORKLOADS) + ["batch256", "serve"])
    ap.add_argument("--rates", default="4,16,64", help="serve: Poisson arrival rates (requests/s) to sweep")
    ap.add_argument("--requests", type=int, default=48, help="serve: requests per arrival rate")
    ap.add_argument("--tick", type=int, default=25, help="serve: substeps per serving tick")
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--no-e2e-sequential", dest="e2e_sequential", action="store_false",
                    help="skip the end-to-end variant that uploads and downloads one after the other")
    ap.add_argument("--accuracy-steps", default="100,500", help="substeps at which FP32 is compared with the FP64 path")
    ap.add_argument("--oracle-steps", type=int, default=200, help="substeps of the elastic-cube check against the FP64 oracle")
    ap.add_argument("--fp64-steps", type=int, default=10)
    ap.add_argument("--oracle-slab-steps", type=int, default=100,
                    help="substeps of the whole workload on the FP64 oracle: the GPU paths' error against it, and the CPU baseline")
    ap.add_argument("--no-batch", action="store_true", help="default workload: skip the 256-scene batch summary")
    ap.add_argument("--no-serve", action="store_true", help="default workload: skip the serving summary")
    ap.add_argument("--batch-steps", type=int, default=20, help="default workload: timed substeps of the batch summary")
    ap.add_argument("--serve-rates", default="8,32", help="default workload: arrival rates (requests/s) of the serving summary")
    ap.add_argument("--serve-requests", type=int, default=24, help="default workload: requests per rate in the serving summary")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--eager", action="store_true", help="with --profile-only: launch kernels one at a time, not as graphs")
    ap.add_argument("--profile-only", action="store_true", help="one scene only: warmup + timed substeps (for ncu captures)")
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"], help="with --profile-only: the scene's precision")
    ap.add_argument("--state-out", default=None, help="with --profile-only: write the scene's state to this file at the end")
    ap.add_argument("--state-in", default=None,
                    help="with --profile-only: start from a state file written by --state-out (a late state to profile after "
                         "few launches)")
    ap.add_argument("--schedule", default="auto",
                    help="auto (the autotuner), or fused:CTAS:G2P[:TIGHT], fused2:CTAS:G2P[:TIGHT], ws:CTAS:G2P[:TIGHT] or "
                         "split:CHUNK:BUFFERS:CTAS:G2P[:TIGHT] "
                         "(a fixed launch schedule)")
    return ap.parse_args()


# ------------------------------------------------------------------------------------------- helpers
def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        vis = os.environ.get("CUDA_VISIBLE_DEVICES")
        devs = vis.split(",") if vis else [str(i) for i in range(64)]
        os.environ["CUDA_VISIBLE_DEVICES"] = devs[local]
        import torch.distributed as td

        td.init_process_group("gloo")  # host-side barrier and max only: scenes are independent replicas
    return world, rank


def barrier(world):
    if world > 1:
        import torch.distributed as td

        td.barrier()


def allreduce_max(world, v):
    if world == 1:
        return v
    import torch
    import torch.distributed as td

    t = torch.tensor([float(v)], dtype=torch.float64)
    td.all_reduce(t, op=td.ReduceOp.MAX)
    return float(t.item())


def allreduce_sum(world, v):
    if world == 1:
        return v
    import torch
    import torch.distributed as td

    t = torch.tensor([float(v)], dtype=torch.float64)
    td.all_reduce(t, op=td.ReduceOp.SUM)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clock / throttle samples while the GPU works (started before, stopped after). The SM clock reported
    is the median over samples taken under load (GPU utilisation >= 50%); a timed region of a few milliseconds is
    shorter than the 100 ms sampling period, so the window also covers the measurement passes that follow it."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap,"
              "utilization.gpu")

    def __init__(self):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "100"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.p.kill()
        self.f.flush()
        vis = os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0]
        rows = []
        with open(self.f.name) as fh:
            for line in fh:
                parts = [t.strip() for t in line.split(",")]
                if len(parts) == 10 and parts[0] == vis:
                    rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        num = lambda t: t.replace(".", "").isdigit()  # noqa: E731
        loaded = [r for r in rows if num(r[9]) and float(r[9]) >= 50.0]
        sm = [float(r[1]) for r in (loaded or rows) if num(r[1])]
        mx = [float(r[2]) for r in rows if num(r[2])]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows), "samples_under_load": len(loaded),
                "power_w_max": max((float(r[3]) for r in rows if num(r[3])), default=None)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as fh:
            pk = json.load(fh)
        return float(pk["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic(kernel, workload):
    """DRAM bytes per launch of `kernel` from the committed ncu summary (profiles/*.txt), or None."""
    pdir = os.path.join(ROOT, "profiles")
    if not os.path.isdir(pdir):
        return None
    for fn in sorted(os.listdir(pdir)):
        if not fn.endswith(".txt"):
            continue
        with open(os.path.join(pdir, fn)) as fh:
            for line in fh:
                # line format: "traffic_per_launch <kernel> <workload> <bytes>"
                t = line.split()
                if len(t) == 4 and t[0] == "traffic_per_launch" and t[1] == kernel and t[2] == workload:
                    return float(t[3])
    return None


def algorithmic_bytes(s_bytes, n, blocks, nodes_per_block, damage):
    """Compulsory DRAM bytes per launch of each phase (inputs read once, outputs written once).

    particle fields: x3 v3 C9 F9 m V0 (+ d, sigma_c with damage), a 4-byte id; grid accumulators:
    m, m v (3), f (3), phase field (2); grid velocities: v (3) + phase field."""
    ns = n * s_bytes
    nodes = blocks * nodes_per_block
    dmg = 1 if damage else 0
    p2g = ns * (26 + dmg) + 4 * n + nodes * s_bytes * 9
    grid = nodes * s_bytes * (9 + 9 + 4)  # read accumulators, clear them, write velocities
    g2p_read = ns * (12 + 2 + 2 * dmg) + 4 * n + nodes * s_bytes * 4
    g2p_write = ns * (24 + 2 + 2 * dmg) + 4 * n + 8 * n
    return {"p2g": p2g, "grid": grid, "g2p": g2p_read + g2p_write, "sort": n * (8 + 4) * 2}


# ------------------------------------------------------------------------------------------- arms
# recipe fields of WORKLOADS -> the oracle's scene-family parameters (oracle/pyoracle.py RECIPE_DEFAULTS)
_ORACLE_KEYS = {"dx": "dx", "l0": "l0", "model": "model", "fiber_stiffness": "fiber", "implicit_damage": "implicit", "size": "size"}


def oracle_workload(kind, over, seed, inputs=None):
    """The workload as an FP64 oracle scene (test infrastructure, the CPU baseline). With inputs=None the
    particles come from the oracle's own seeded generator (the reference arm loads no product library);
    otherwise from the given arrays (the same inputs as the GPU run)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as po

    kw = {_ORACLE_KEYS[k]: v for k, v in over.items() if k in _ORACLE_KEYS}
    if "implicit" in kw:
        kw["implicit"] = bool(kw["implicit"])
    return po.recipe_scene(kind, 8, seed=seed, inputs=inputs, **kw)


def run_reference(args, world, rank):
    """The reference's CPU algorithm on all host threads: the oracle restatement (the reference itself cannot be
    built here or on Arm), FP64 as the reference's AnisoMPM driver is compiled (anisofracture.cpp:13-14), on the
    same workload, seed and particle count as the GPU arm, with inputs from the oracle's own generator."""
    if rank != 0:
        return None
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as po

    kind, over = WORKLOADS[args.workload]
    o, n = oracle_workload(kind, over, seed=12345)
    t0 = time.perf_counter()
    o.step(max(1, args.warmup))
    per_step = (time.perf_counter() - t0) / max(1, args.warmup)
    # every requested substep is timed unless that would take more than REF_TIMED_S (a run with the default
    # 1000 substeps); the line then states how many were timed
    steps = args.steps if per_step * args.steps <= REF_TIMED_S else max(1, int(REF_TIMED_S / per_step))
    t0 = time.perf_counter()
    o.step(steps)
    el = time.perf_counter() - t0
    val = n * steps / el
    cfg = _config(args, "fp64")
    cfg["particles"] = int(n)
    cfg["substeps_timed"] = steps
    return {"impl": "reference", "metric": "particle-substeps/sec", "value": val, "unit": "particle-substeps/s", "n_gpus": args.gpus,
            "steps": steps, "warmup": args.warmup, "ms_per_step": el / steps * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded; inputs from the oracle's own generator)", "config": cfg,
            "cpu_baseline": {"value": val, "unit": "particle-substeps/s", "cores": po.num_threads(), "kind": "port", "precision": "f64",
                             "sample": f"the whole workload ({n} particles), {steps} substeps after {max(1, args.warmup)} warm-up substeps"},
            "e2e": {"value": val, "unit": "particle-substeps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


REF_TIMED_S = 240.0


def error_vs_oracle(steps):
    """Max and RMS error of x, v, F, d of the FP32 and FP64 GPU paths against the FP64 oracle (host cores)
    after `steps` substeps of the elastic cube: side 0.25 centred at (0.5, 0.6, 0.5), dx = 1/64, 8 particles
    per cell (32,768), E = 1e4, nu = 0.3, rho = 1000, v0 = (0, -1, 0), gravity, sticky ground at y = 0.05,
    dt = 1e-4."""
    import numpy as np

    import ziran2020_gb300 as zr

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import scenes

    desc = scenes.elastic_box(size=0.25, dx=1 / 64, seed=20200)
    o = scenes.oracle_scene(desc, 8)
    t0 = time.perf_counter()
    o.step(steps)
    ref = o.state()
    out = {"scene": f"elastic cube, {len(desc['m'])} particles, dx=1/64, {steps} substeps", "oracle_seconds": round(time.perf_counter() - t0, 2),
           "x_unit": "metres in a unit domain (domain-relative)"}
    for prec, name in ((zr.F32, "fp32"), (zr.F64, "fp64")):
        g = scenes.gpu_scene(desc, prec)
        g.step(steps)
        st = scenes.gpu_state(g)
        out[name] = {}
        for f in ("x", "v", "F", "d"):
            e = np.abs(np.asarray(st[f], dtype=np.float64) - np.asarray(ref[f], dtype=np.float64))
            out[name][f] = {"max": float(e.max()), "rms": float(np.sqrt(np.mean(e * e)))}
        del g
    return out


def field_errors(a, b):
    """max and RMS of |a - b| for x, v, F and d (float64)."""
    import numpy as np

    out = {}
    for f in ("x", "v", "F", "d"):
        e = np.abs(np.asarray(a[f], dtype=np.float64) - np.asarray(b[f], dtype=np.float64))
        out[f] = {"max": float(e.max()) if e.size else 0.0, "rms": float(np.sqrt(np.mean(e * e))) if e.size else 0.0}
    return out


def apply_schedule(obj, spec):
    """Fix the launch schedule of a scene from --schedule (the autotuner otherwise picks it)."""
    if spec == "auto":
        return
    f = spec.split(":")
    if f[0] in ("fused", "fused2", "ws"):
        obj.set_schedule(0, 0, int(f[1]), int(f[2]), fused={"fused": 1, "fused2": 2, "ws": 3}[f[0]],
                         g2p_tight=int(f[3]) if len(f) > 3 else 0)
    else:
        obj.set_schedule(int(f[1]), int(f[2]), int(f[3]), int(f[4]), g2p_tight=int(f[5]) if len(f) > 5 else 0)


def _config(args, precision="fp32"):
    return {"workload": args.workload, "particles": None, "substeps_timed": args.steps, "precision_path": precision,
            "l2": "particle state larger than L2 (no flush needed)", "parallelism": f"replicas x{args.gpus}"}


def measure_batch(recs, steps, warmup, world=1, fp64_steps=10):
    """Advance the batch of recipes (one launch per kernel for all scenes): timed substeps, per-phase kernel times,
    the roofline of the dominant transfer kernel, and the plain FP64 GPU path on the same batch."""
    import ziran2020_gb300 as zr
    from ziran2020_gb300 import workloads

    n = workloads.total_particles(recs)
    b = zr.Batch(zr.F32)
    for r in recs:
        b.add_recipe(r)
    b.commit()
    clocks = ClockSampler()
    clocks.start()
    b.step(warmup)
    barrier(world)
    b.step(steps)
    ms = b.last_step_ms
    barrier(world)
    stats = b.stats()
    b.set_timing(True)
    b.step(min(steps, 20))
    phases, ksteps = b.timing()
    b.set_timing(False)
    per = {k: v / ksteps for k, v in phases.items()}
    schedule = b.schedule()
    del b
    peak, peak_kind = measured_peaks()
    alg = algorithmic_bytes(4, n, 0, 64, False)  # particle bytes only: the batch reports no block count
    dom = max(("p2g", "g2p"), key=lambda k: per[k])
    achieved = alg[dom] / (per[dom] / 1e3) / 1e9
    roof = {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
            "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)", "traffic": profiled_traffic(dom, "batch256"),
            "algorithmic_bytes": alg[dom], "kernel_ms": round(per[dom], 4), "phase_ms_per_substep": {k: round(v, 4) for k, v in per.items()},
            "frac_by_phase": {k: round(alg[k] / (per[k] / 1e3) / 1e9 / peak, 4) for k in ("p2g", "g2p") if per.get(k)},
            "note": "algorithmic bytes count particle traffic only (grid nodes excluded)"}
    b64 = zr.Batch(zr.F64)
    for r in recs:
        b64.add_recipe(r)
    b64.step(2)
    b64.step(fp64_steps)
    fp64_value = n * fp64_steps / (b64.last_step_ms / 1e3)
    del b64
    clock_info = clocks.stop()
    clock_info["window"] = "warm-up, timed substeps, per-phase timing pass, FP64 path"
    return {"particles": int(n), "ms": ms, "stats": stats, "clocks": clock_info, "roofline": roof, "schedule": schedule, "fp64_value": fp64_value}


def batch_summary(args):
    """The 256-scene batch of elastic boxes (N log-uniform in 5k-400k) beside the single-scene line: throughput,
    roofline fraction and the plain FP64 GPU path on the same batch."""
    from ziran2020_gb300 import workloads

    recs = workloads.batch_recipes(seed=20200713)
    m = measure_batch(recs, args.batch_steps, max(3, args.warmup), fp64_steps=args.fp64_steps)
    value = m["particles"] * args.batch_steps / (m["ms"] / 1e3)
    return {"workload": "batch256", "scenes": len(recs), "particles": m["particles"], "metric": "particle-substeps/sec", "value": value,
            "unit": "particle-substeps/s", "steps": args.batch_steps, "ms_per_step": m["ms"] / args.batch_steps, "roofline": m["roofline"],
            "clocks": m["clocks"], "schedule": m["schedule"], "gpu_launches": int(m["stats"]["launches_per_step"]) * args.batch_steps,
            "fp64_path": {"value": m["fp64_value"], "unit": "particle-substeps/s", "fp32_over_fp64": value / m["fp64_value"]}}


def run_batch(args, world, rank):
    """256 independent elastic boxes (N log-uniform in 5k-400k, E ~ U(5e3, 5e4), centre ~ U[0.3,0.7]^3,
    v0 ~ U[-1,1]^3; dx = 1/64, dt = 1e-4) advanced together: one launch per kernel for the whole batch."""
    from ziran2020_gb300 import workloads

    recs = workloads.batch_recipes(seed=20200713 + rank)
    m = measure_batch(recs, args.steps, args.warmup, world, fp64_steps=args.fp64_steps)
    n = m["particles"]
    ms_max = allreduce_max(world, m["ms"])
    value = allreduce_sum(world, n) * args.steps / (ms_max / 1e3)
    cpu = None
    if rank == 0 and not args.no_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import pyoracle as po

        o, ns = po.recipe_scene(0, 8, seed=12345)
        o.step(1)
        t0 = time.perf_counter()
        o.step(20)
        el = time.perf_counter() - t0
        cpu = {"value": ns * 20 / el, "unit": "particle-substeps/s", "cores": po.num_threads(), "kind": "port", "precision": "f64",
               "sample": f"one {ns}-particle elastic box of the family (dx=1/64), 20 substeps; the batch would run its scenes one by one"}
    cfg = {"workload": "batch256", "scenes": len(recs), "particles": int(n), "substeps_timed": args.steps, "precision_path": "fp32",
           "l2": "particle state larger than L2 (no flush needed)", "parallelism": f"replicas x{world}", "schedule": m["schedule"]}
    line = {"metric": "particle-substeps/sec", "value": value, "unit": "particle-substeps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded recipe family)", "config": cfg, "roofline": m["roofline"], "cpu_baseline": cpu,
            "e2e": {"value": None, "unit": "particle-substeps/s", "h2d_bytes_per_step": None, "d2h_bytes_per_step": None,
                    "note": "measured on the single-scene workload"},
            "gpu_launches": int(m["stats"]["launches_per_step"]) * args.steps, "kernels_per_substep": int(m["stats"]["launches_per_step"]),
            "clocks": m["clocks"], "fp64_fallbacks": m["stats"]["fallbacks"],
            "fp64_path": {"value": m["fp64_value"], "unit": "particle-substeps/s", "fp32_over_fp64": value / world / m["fp64_value"]}}
    return line if rank == 0 else None


def serve_sweep(rates, count, tick, seed_base=4242):
    """Poisson stream of scene-advance requests (elastic or AnisoMPM family, 10k-2M particles log-uniform,
    50-500 substeps uniform), FP32, state resident on the device, admission by a 60 GB budget; per arrival rate
    the p50/p99 request latency (submit -> result on the host) and the aggregate particle-substeps/s."""
    import numpy as np

    import ziran2020_gb300 as zr
    from ziran2020_gb300 import workloads

    sweep = []
    for ri, lam in enumerate(rates):
        reqs = workloads.request_stream(seed=seed_base + 17 * ri, count=count)
        built = []
        for r, steps in reqs:
            sc = zr.Scene(zr.F32)
            sc.from_recipe(r)  # host-side scene construction happens before the clock starts
            built.append((sc, steps, zr.recipe_count(r)))
        arrivals = np.cumsum(np.random.default_rng(99 + ri).exponential(1.0 / lam, len(reqs)))
        sv = zr.Server(zr.F32, budget_bytes=60e9, tick_substeps=tick, max_scenes=256)
        ids, k = [], 0
        t0 = time.perf_counter()
        while True:
            now = time.perf_counter() - t0
            while k < len(built) and arrivals[k] <= now:
                ids.append(sv.submit_scene(built[k][0], built[k][1]))
                k += 1
            running, queued, _ = sv.tick()
            if k == len(built) and running == 0 and queued == 0:
                break
            if running == 0 and queued == 0 and k < len(built):
                time.sleep(max(0.0, arrivals[k] - (time.perf_counter() - t0)))
        wall = time.perf_counter() - t0
        lats = np.array([sv.request(i)["latency_s"] for i in ids])
        st = sv.stats()
        ps = float(sum(n * steps for _, steps, n in built))
        sweep.append({"rate_per_s": lam, "requests": len(ids), "p50_latency_s": float(np.percentile(lats, 50)),
                      "p99_latency_s": float(np.percentile(lats, 99)), "particle_substeps": ps, "makespan_s": wall,
                      "throughput": ps / wall, "device_throughput": st["particle_substeps"] / (st["device_ms"] / 1e3),
                      "peak_device_bytes": st["device_bytes"]})
        del sv, built
    return sweep


def serve_summary(args):
    """Continuous batching under a Poisson request stream, beside the single-scene line (bounded: a few rates and
    requests)."""
    rates = [float(r) for r in args.serve_rates.split(",") if r.strip()]
    sweep = serve_sweep(rates, args.serve_requests, args.tick)
    return {"workload": "serve", "metric": "p50/p99 request latency (s) and aggregate particle-substeps/s", "requests_per_rate": args.serve_requests,
            "budget_bytes": 60e9, "tick_substeps": args.tick, "precision_path": "fp32", "rates": sweep}


def run_serve(args, world, rank):
    """The serving workload on its own line: the sweep over --rates with --requests per rate."""
    sweep = serve_sweep([float(r) for r in args.rates.split(",")], args.requests, args.tick, seed_base=4242 + 1000 * rank)
    best = max(sweep, key=lambda e: e["throughput"])
    cfg = {"workload": "serve", "requests_per_rate": args.requests, "rates_per_s": [e["rate_per_s"] for e in sweep], "budget_bytes": 60e9,
           "tick_substeps": args.tick, "precision_path": "fp32", "parallelism": f"replicas x{world}"}
    line = {"metric": "particle-substeps/sec", "value": allreduce_sum(world, best["throughput"]), "unit": "particle-substeps/s",
            "n_gpus": world, "steps": None, "warmup": 0, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded request stream)", "config": cfg, "serving": sweep,
            "p50_latency_s": best["p50_latency_s"], "p99_latency_s": best["p99_latency_s"]}
    return line if rank == 0 else None


def run_ours(args, world, rank):
    import numpy as np

    import ziran2020_gb300 as zr

    if args.workload == "batch256":
        return run_batch(args, world, rank)
    if args.workload == "serve":
        return run_serve(args, world, rank)

    kind, over = WORKLOADS[args.workload]
    r = zr.recipe(kind, seed=12345 + rank, **over)
    n = zr.recipe_count(r)
    damage = kind == 1

    s = zr.Scene(zr.F64 if args.profile_only and args.precision == "fp64" else zr.F32)
    s.from_recipe(r)
    apply_schedule(s, args.schedule)
    if args.profile_only:
        if args.state_in:
            s.read_state(args.state_in)
        if args.eager:  # substeps launched one kernel at a time (ncu lists no kernel of a graph holding a conditional loop)
            s.set_timing(True)
        s.step(args.warmup)
        s.step(args.steps)
        if args.state_out:
            s.write_state(args.state_out)
        g, b = s.last_grid()
        print(json.dumps({"profile_only": True, "particles": n, "groups": g, "blocks": b, "ms_per_step": s.last_step_ms / max(1, args.steps)}))
        return None
    clocks = ClockSampler()
    clocks.start()
    s.step(args.warmup)
    # per-phase kernel durations (CUDA events on the engine's stream, substeps run without graphs) on the state the
    # timed region starts from and, after it, on the state it ends with; the start pass runs on a saved image of the
    # state, which is then restored, so the timed substeps are exactly those after the warm-up
    kt_steps = min(args.steps, 20)

    def phase_pass():
        s.set_timing(True)  # also clears the accumulated phase times
        s.step(kt_steps)
        phases, ksteps = s.timing()
        s.set_timing(False)
        return {k: v / ksteps for k, v in phases.items()}

    image = s.save_state()
    per_start = phase_pass()
    s.load_state(image)
    s.step(1)  # the first substep after a restore sorts from scratch: kept out of the timed region like the warm-up
    del image
    barrier(world)
    s.step(args.steps)
    ms = s.last_step_ms
    barrier(world)
    ms_max = allreduce_max(world, ms)
    n_total = allreduce_sum(world, n)
    value = n_total * args.steps / (ms_max / 1e3)
    stats = s.stats()
    groups, blocks = s.last_grid()
    schedule = s.schedule()
    per_end = phase_pass()
    per = {k: 0.5 * (per_start[k] + per_end[k]) for k in per_start}
    peak, peak_kind = measured_peaks()
    alg = algorithmic_bytes(4, n, blocks, 64, damage)
    dom = max(("p2g", "g2p"), key=lambda k: per[k])
    achieved = alg[dom] / (per[dom] / 1e3) / 1e9
    traffic = profiled_traffic(dom, args.workload)
    roof = {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
            "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else "fallback 6800 GB/s",
            "traffic": traffic, "algorithmic_bytes": alg[dom], "kernel_ms": round(per[dom], 4),
            "phase_ms_per_substep": {k: round(v, 4) for k, v in per.items()},
            "phase_ms_per_substep_start": {k: round(v, 4) for k, v in per_start.items()},
            "phase_ms_per_substep_end": {k: round(v, 4) for k, v in per_end.items()},
            "phase_timing": f"CUDA events per phase over {kt_steps} substeps on the timed region's first state (restored after) and "
                            f"{kt_steps} after its last; the kernel time is the mean of the two",
            "frac_by_phase": {k: round(alg[k] / (per[k] / 1e3) / 1e9 / peak, 4) for k in ("p2g", "g2p", "grid") if per.get(k)}}

    # end to end through the C ABI with pinned host buffers: every step's state uploaded, one substep, its result
    # downloaded
    e2e = None
    try:
        import torch

        K = args.e2e_steps
        host = torch.empty((n, 25), dtype=torch.float32).pin_memory().numpy()
        res = [torch.empty((n, 25), dtype=torch.float32).pin_memory().numpy() for _ in range(2)]
        s.get_state(host)
        s.step_stream([host] * 2, res)  # warm-up: copy streams, device slots, the one-substep graph
        s.set_state(host)
        s.step(1)
        s.exchange_state(host, res[0])
        s.step(1)
        s.get_state(res[0])
        # jobs through zr_scene_step_stream: the copies of later inputs and earlier results overlap the substeps. The
        # host link is shared with the node's other work (a first full pipeline after the warm-up has run at half
        # speed with no job rerun), so one untimed run of the K jobs comes first, then five timed runs, and the median
        # is reported (all five beside it)
        s.step_stream([host] * K, [res[k % 2] for k in range(K)])
        runs = []
        for _ in range(5):
            t0 = time.perf_counter()
            s.step_stream([host] * K, [res[k % 2] for k in range(K)])
            runs.append(allreduce_sum(world, n) * K / allreduce_max(world, time.perf_counter() - t0))
        # the same jobs with zr_scene_exchange_state: each step's download and the next upload in one kernel
        t0 = time.perf_counter()
        s.set_state(host)  # step 0's input
        for k in range(K):
            s.step(1)
            if k + 1 < K:
                s.exchange_state(host, res[0])  # step k's result out while step k+1's input comes in
            else:
                s.get_state(res[0])  # the last result
        e2e_x = allreduce_sum(world, n) * K / allreduce_max(world, time.perf_counter() - t0)
        nbytes = n * 25 * 4
        e2e_seq = None
        if args.e2e_sequential:
            t0 = time.perf_counter()
            for _ in range(K):
                s.set_state(host)
                s.step(1)
                s.get_state(res[0])
            e2e_seq = allreduce_sum(world, n) * K / allreduce_max(world, time.perf_counter() - t0)
        e2e = {"value": sorted(runs)[len(runs) // 2], "unit": "particle-substeps/s",
               "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
               "what": f"{K} jobs, each the whole FP32 state (x,v,C,F,d) uploaded from pinned host memory, one substep, the "
                       "result downloaded to pinned host memory, through zr_scene_step_stream (the copies of the next inputs and "
                       "the last results run on the copy engines during the substeps); the median of five runs of the jobs",
               "runs": runs, "reruns": s.stream_reruns, "exchange_value": e2e_x, "sequential_value": e2e_seq}
    except Exception as ex:  # pinned memory needs torch; report instead of failing the line
        e2e = {"value": None, "unit": "particle-substeps/s", "h2d_bytes_per_step": None, "d2h_bytes_per_step": None, "error": str(ex)}
    cg_iterations = s.cg_iterations
    del s

    # plain FP64 GPU path on the same workload
    s64 = zr.Scene(zr.F64)
    s64.from_recipe(r)
    s64.step(2)
    s64.step(args.fp64_steps)
    fp64_value = n * args.fp64_steps / (s64.last_step_ms / 1e3)
    del s64
    clock_info = clocks.stop()
    clock_info["window"] = "warm-up, timed substeps, per-phase timing pass, end-to-end steps, FP64 path"

    # FP32 against the FP64 GPU path at the --accuracy-steps marks, and both GPU paths against the FP64 oracle
    # on the whole workload (the same inputs) after --oracle-slab-steps substeps; that oracle run, timed over
    # its substeps after the first, is also the CPU baseline (the oracle on all host threads, kind "port")
    acc, slab_vs_oracle, cpu, late = None, None, None, None
    marks = sorted({int(v) for v in str(args.accuracy_steps).split(",") if v.strip() and int(v) > 0})
    K = 0 if args.no_cpu else max(0, args.oracle_slab_steps)
    if rank == 0 and (marks or K):
        ref = None
        if K:
            o, no = oracle_workload(kind, over, seed=12345 + rank, inputs=zr.recipe_generate(r))
            import pyoracle as po

            t0 = time.perf_counter()
            o.step(1)
            first = time.perf_counter() - t0
            t0 = time.perf_counter()
            if K > 1:
                o.step(K - 1)
            el = time.perf_counter() - t0
            ref = o.state()
            del o
            timed, secs = (K - 1, el) if K > 1 else (1, first)
            cpu = {"value": no * timed / secs, "unit": "particle-substeps/s", "cores": po.num_threads(), "kind": "port", "precision": "f64",
                   "sample": f"the whole workload ({no} particles, same inputs), substeps {2 if K > 1 else 1}-{K}: {secs:.1f} s"}
        a32, a64 = zr.Scene(zr.F32), zr.Scene(zr.F64)
        a32.from_recipe(r)
        a64.from_recipe(r)
        acc = {"reference": "FP64 GPU path", "x_unit": "metres in a unit domain (domain-relative)", "at": []} if marks else None
        done = 0
        for mk in sorted(set(marks) | ({K} if K else set())):
            a32.step(mk - done)
            seg_ms = a32.last_step_ms
            a64.step(mk - done)
            if mk == max(marks or [0]) and mk - done >= 50:
                # the timed value covers the first substeps of the pull; the damage grows later (more particles take
                # the tensile split): device throughput over the last segment of this run, graph-launched as well
                late = {"substeps": f"{done + 1}-{mk}", "value": n * (mk - done) / (seg_ms / 1e3), "unit": "particle-substeps/s"}
            done = mk
            s32 = {f: a32.get(f) for f in ("x", "v", "F", "d")}
            s64 = {f: a64.get(f) for f in ("x", "v", "F", "d")}
            if mk in marks:
                acc["at"].append({"substeps": mk, **field_errors(s32, s64)})
            if mk == K:
                slab_vs_oracle = {"scene": f"{args.workload}, {n} particles, {K} substeps, inputs shared with the oracle",
                                  "reference": "FP64 oracle (CPU)", "x_unit": "metres in a unit domain (domain-relative)",
                                  "fp32": field_errors(s32, ref), "fp64": field_errors(s64, ref)}
        del a32, a64

    # FP32 and FP64 GPU paths against the FP64 oracle on the elastic cube (32,768 particles, dx = 1/64,
    # corotated E = 1e4, sticky ground), the scene the 1e-4 position bound is stated on
    vs_oracle = None
    if rank == 0 and not args.no_cpu and args.oracle_steps > 0:
        vs_oracle = error_vs_oracle(args.oracle_steps)

    cfg = _config(args)
    cfg["particles"] = int(n)
    cfg["active_blocks"] = int(blocks)
    cfg["particle_groups"] = int(groups)
    cfg["schedule"] = schedule
    if over.get("implicit_damage"):
        # the CG loop runs as a conditional node of the substep graph: 5 kernels per iteration, not counted in
        # kernels_per_substep; the phase "grid" includes the whole damage solve
        cfg["damage_solve"] = {"cg_iterations_last_substep": cg_iterations, "kernels_per_cg_iteration": 5}
    line = {"metric": "particle-substeps/sec", "value": value, "unit": "particle-substeps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded recipe)", "config": cfg, "roofline": roof, "cpu_baseline": cpu, "e2e": e2e,
            "gpu_launches": int(stats["launches_per_step"]) * args.steps, "kernels_per_substep": int(stats["launches_per_step"]),
            "clocks": clock_info, "fp64_path": {"value": fp64_value, "unit": "particle-substeps/s", "fp32_over_fp64": value / world / fp64_value},
            "late_state": late, "fp32_vs_fp64_error": acc, "error_vs_fp64_oracle": vs_oracle, "error_vs_fp64_oracle_slab": slab_vs_oracle,
            "fp64_fallbacks": stats["fallbacks"]}
    if rank == 0 and not args.no_batch:
        line["batch"] = batch_summary(args)
    if rank == 0 and not args.no_serve:
        line["serving"] = serve_summary(args)
    return line if rank == 0 else None


def main():
    args = parse()
    world, rank = dist_setup()
    if args.impl == "reference":
        line = run_reference(args, world, rank)
    else:
        line = run_ours(args, world, rank)
    if line is not None:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as td

        td.destroy_process_group()


if __name__ == "__main__":
    main()
