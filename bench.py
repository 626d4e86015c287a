#!/usr/bin/env python
"""Benchmark: tet-element-steps/s of the corotational-tet implicit-Euler step on one GB300.

Workload (default): the 40x40x160 cube-grid bar of edge h = 4 mm, 5 tets per cube (1,280,000 tets,
270,641 nodes, 811,923 dofs), per-tet E log-uniform in [1e4, 1e6] Pa and nu uniform in [0.40, 0.49], z = 0
clamped, the z = 160h face driven by a 20% compression ramp over 50 steps, gravity, dt = 1e-3,
CG tolerance 1e-10. A step is one FemRepresentation::update(dt). Inputs are synthetic (seeded).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--precision fp64|mixed] [--impl reference]

One JSON line on rank 0. Under torchrun every rank steps its own replica of the bar on its own GPU
(replicas only: a single mesh does not shard without a halo exchange) and the job value is the sum.
"""

from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "tet-element-steps/s"
PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0
CG_CAP = 10000


def log(msg):
    sys.stderr.write(f"[bench {time.strftime('%H:%M:%S')}] {msg}\n")
    sys.stderr.flush()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Dist:
    """Control-plane barrier and max/sum reductions over ranks (gloo; no data-path collective)."""

    def __init__(self, world):
        self.world = world
        self.pg = None
        if world > 1:
            import torch.distributed as dist

            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo")
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def reduce(self, value, op):
        if not self.pg:
            return value
        import torch

        t = torch.tensor([float(value)], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX if op == "max" else self.pg.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.out = None

    def start(self):
        try:
            self.out = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.out, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.out.flush()
        self.out.seek(0)
        rows = [r.split(",") for r in self.out.read().strip().splitlines() if r.strip()]
        os.unlink(self.out.name)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [c.strip() for c in r]
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                smax = float(r[2])
            except ValueError:
                continue
            for nm, val in zip(names, r[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def load_peak():
    try:
        with open(PEAKS_FILE) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def load_traffic(kernel_key):
    """Per-launch DRAM bytes of a kernel from the committed ncu summary (profiles/traffic.json)."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            return json.load(f).get(kernel_key)
    except Exception:
        return None


def build_scene(args):
    from opensurgsim_gb300 import mesh

    # The explicit CG iteration cap only bounds the run if a solve ever stagnates; at the
    # benchmark's states CG converges in a few hundred iterations, far below it.
    if args.config == "bar":
        return mesh.scene_bar_compression(cg_max_iterations=CG_CAP)
    return mesh.scene_cube(10, 10, 10, cg_max_iterations=CG_CAP)


def scenario_velocities(scene, step):
    return scene.driven_values(step) if scene.driven_dofs is not None else None


def run_ours(args, rank, world, local, dist):
    import numpy as np
    import torch

    from opensurgsim_gb300 import _lib, build
    from opensurgsim_gb300.body import Body

    build.build()
    torch.cuda.set_device(local)
    scene = build_scene(args)
    m = scene.mesh
    log(f"scene {scene.name}: {m.num_tets} tets, {m.num_nodes} nodes")
    prec = _lib.PRECISION_MIXED if args.precision == "mixed" else _lib.PRECISION_FP64
    body = Body.from_scene(scene, precision=prec, device=local)
    stream = torch.cuda.ExternalStream(body.stream(), device=local)
    dt = scene.dt
    driven = scene.driven_dofs is not None
    if driven:
        d_dofs = torch.from_numpy(scene.driven_dofs.astype(np.int32)).cuda(local)
        ramp = torch.from_numpy(scene.driven_values(0)).cuda(local)
        hold = torch.zeros_like(ramp)

    def set_driven(step):
        if driven:
            vals = ramp if step < scene.ramp_steps else hold
            body_lib.gbfem_set_velocities_device(body.handle, d_dofs.numel(), d_dofs.data_ptr(), vals.data_ptr())

    body_lib = _lib.load()
    flags = _lib.STEP_TIME_KERNELS
    log(f"body created: nnz {body.nnz}")
    step = 0
    for _ in range(args.warmup):
        set_driven(step)
        body.step(dt, 1, flags)
        step += 1
    torch.cuda.synchronize(local)
    log(f"warm-up done ({args.warmup} steps)")
    dist.barrier()
    sampler = ClockSampler(local)
    sampler.start()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    agg = dict(cg_iterations=0, kernel_launches=0, ms_spmv=0.0, spmv_timed=0, refinement_sweeps=0,
               polar_fallbacks=0, cg_max_iterations_hit=0)
    statuses = []
    ev0.record(stream)
    for _ in range(args.steps):
        set_driven(step)
        statuses.append(body.step(dt, 1, flags))
        s = body.stats()
        for k in agg:
            agg[k] += s[k]
        agg["kernel_launches"] += 1 if driven else 0
        step += 1
    ev1.record(stream)
    torch.cuda.synchronize(local)
    clocks = sampler.stop()
    dist.barrier()
    ms = ev0.elapsed_time(ev1)
    log(f"timed region: {args.steps} steps in {ms:.1f} ms")
    ms_max = dist.reduce(ms, "max")
    total_units = dist.reduce(m.num_tets * args.steps, "sum")
    value = total_units / (ms_max / 1e3)

    # End to end through the public API with host buffers: prescribed velocities copied in from
    # pinned host memory, positions and velocities read back every step.
    h_dofs = torch.from_numpy(scene.driven_dofs.astype(np.int32)).pin_memory() if driven else None
    h_vals = torch.empty(scene.driven_dofs.size if driven else 0, dtype=torch.float64).pin_memory()
    h_x = torch.empty(body.n, dtype=torch.float64).pin_memory().numpy()
    h_v = torch.empty(body.n, dtype=torch.float64).pin_memory().numpy()
    torch.cuda.synchronize(local)
    dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        if driven:
            h_vals.numpy()[:] = scene.driven_values(step)
            body.set_velocities(h_dofs.numpy(), h_vals.numpy())
        body.step(dt, 1, 0)
        body_lib.gbfem_get_state(body.handle, _lib.dptr(h_x), _lib.dptr(h_v))
        step += 1
    torch.cuda.synchronize(local)
    e2e_s = dist.reduce(time.perf_counter() - t0, "max")
    log(f"e2e region: {args.steps} steps in {e2e_s:.3f} s")
    e2e_value = total_units / e2e_s
    h2d = (scene.driven_dofs.size * (4 + 8)) if driven else 0
    d2h = 2 * body.n * 8

    # Roofline of the dominant kernel: the CG matrix-vector product on the symmetric BSR matrix.
    nb = body.nnz // 9
    val_bytes = 8 if prec == _lib.PRECISION_FP64 else 4
    spmv_bytes = body.nnz * val_bytes + nb * 4 + (body.num_nodes + 1) * 4 + 2 * body.n * val_bytes
    spmv_ms = agg["ms_spmv"] / max(1, agg["spmv_timed"])
    peak, peak_kind = load_peak()
    achieved = spmv_bytes / (spmv_ms / 1e3) / 1e9 if spmv_ms > 0 else None
    traffic = load_traffic(f"spmv_sell_{args.precision}_{args.config}")
    cg_per_step = agg["cg_iterations"] / max(1, args.steps)
    line = {
        "metric": METRIC,
        "value": value,
        "unit": "tet-element-steps/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_max / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64" if prec == _lib.PRECISION_FP64 else "f32+f64",
        "data": "synthetic (seeded cube-grid meshes)",
        "config": {
            "workload": ("bar40x40x160 (h 4 mm) 20% compression ramp: 1,280,000 tets, 270,641 nodes, "
                         "nnz 30,865,689, E log-U[1e4,1e6], nu U[0.40,0.49], gravity, dt 1e-3, CG tol 1e-10"
                         if args.config == "bar" else "cube10x10x10: 5,000 tets, E 1e5, nu 0.45"),
            "tets": m.num_tets, "nodes": m.num_nodes, "dofs": body.n, "nnz": body.nnz,
            "precision": args.precision, "scenario_steps": [args.warmup, args.warmup + args.steps],
            "l2": "working set larger than L2 (no flush needed)" if args.config == "bar" else
                  "working set L2-resident (small case)",
            "parallelism": f"replicas x{world}",
        },
        "gpu_launches": int(agg["kernel_launches"]),
        "cg_iterations_per_step": cg_per_step,
        "step_status": sorted(set(int(s) for s in statuses)),
        "clocks": clocks,
        "e2e": {"value": e2e_value, "unit": "tet-element-steps/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "roofline": {
            "kernel": f"k_cg_spmv_sell ({args.precision})",
            "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": (achieved / peak) if achieved else None, "traffic": traffic,
            "algorithmic_bytes_per_launch": spmv_bytes, "avg_launch_ms": spmv_ms,
            "launches_timed": agg["spmv_timed"], "peak_source": f"{peak_kind} (hbm_gbs)",
        },
    }
    body.close()
    return line, scene


def cpu_baseline(scene, steps=1):
    """The oracle (FP64 C++ restatement of the reference step) on the host: `steps` steps of the
    same scene from the same start state, one thread (a representation is single-threaded)."""
    from oracle import oracle as O

    model = O.OracleModel.from_scene(scene)
    t_total = 0.0
    for s in range(steps):
        if scene.driven_dofs is not None:
            x, v = model.state()
            v[scene.driven_dofs] = scene.driven_values(s)
            model.set_state(None, v)
        t0 = time.perf_counter()
        model.step(scene.dt)
        t_total += time.perf_counter() - t0
    return scene.mesh.num_tets * steps / t_total, t_total


def run_reference(args, rank, world):
    """Reference arm: the CPU implementation of the path (the oracle restatement; the reference
    itself cannot be built without Eigen/Boost) on the host, bounded in wall time."""
    from opensurgsim_gb300 import mesh  # noqa: F401
    from oracle import oracle as O

    if rank != 0:
        return None
    O.build()
    scene = build_scene(args)
    model = O.OracleModel.from_scene(scene)
    budget_s = float(os.environ.get("GBFEM_REFERENCE_BUDGET_S", "150"))
    step = 0

    def one():
        nonlocal step
        if scene.driven_dofs is not None:
            x, v = model.state()
            v[scene.driven_dofs] = scene.driven_values(step)
            model.set_state(None, v)
        t0 = time.perf_counter()
        model.step(scene.dt)
        step += 1
        return time.perf_counter() - t0

    t_warm = one() if args.warmup > 0 else 0.0
    times = []
    while len(times) < args.steps and (sum(times) + t_warm) < budget_s:
        times.append(one())
    value = scene.mesh.num_tets * len(times) / sum(times)
    sample = (f"{len(times)} timed step(s) (+{min(args.warmup, 1)} warm-up) of the same scene, capped at "
              f"{budget_s:.0f} s of CPU time; oracle FP64 C++ restatement, -O3, 1 thread")
    line = {
        "metric": METRIC, "value": value, "unit": "tet-element-steps/s", "n_gpus": world, "steps": len(times),
        "warmup": min(args.warmup, 1), "ms_per_step": 1e3 * sum(times) / len(times), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded cube-grid meshes)",
        "config": {"workload": "bar40x40x160 compression" if args.config == "bar" else "cube10x10x10",
                   "tets": scene.mesh.num_tets, "precision": "fp64"},
        "impl": "reference",
        "cpu_baseline": {"value": value, "unit": "tet-element-steps/s", "cores": 1, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "tet-element-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    return line


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--config", default="bar", choices=["bar", "cube"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    rank, world, local = dist_env()
    if args.impl == "reference":
        line = run_reference(args, rank, world)
        if rank == 0:
            print(json.dumps(line), flush=True)
        return
    dist = Dist(world)
    line, scene = run_ours(args, rank, world, local, dist)
    if rank == 0:
        if world == 1 and not args.no_cpu_baseline:
            from oracle import oracle as O

            O.build()
            log("cpu baseline: oracle on the host")
            v, t = cpu_baseline(scene, 1)
            log(f"cpu baseline: 1 step in {t:.1f} s")
            line["cpu_baseline"] = {"value": v, "unit": "tet-element-steps/s", "cores": 1, "kind": "port",
                                    "sample": f"1 step of the same scene on the host ({t:.1f} s), oracle FP64 "
                                              "C++ restatement, -O3, 1 thread"}
        print(json.dumps(line), flush=True)
    dist.close()


if __name__ == "__main__":
    main()
