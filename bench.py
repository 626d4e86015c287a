#!/usr/bin/env python
"""Benchmark: tet-element-steps/s of the corotational-tet implicit-Euler step on one GB300.

Default workload (--config batch): 256 independent cube-grid meshes of edge 1 cm, 5 tets per cube,
node counts log-uniform in [500, 50000] (11,543,720 tets, 2,613,280 nodes from seed 3), per-mesh E
log-uniform in [1e4, 1e6] Pa, nu 0.45, rho 1000, bottom faces fixed, gravity -9.81 z, Rayleigh
alpha 0.01 / beta 0.001, dt 1e-3, CG tolerance 1e-10, one Newton iteration. A step is one
FemRepresentation::update(dt) of every mesh. The measured form is the batched mixed-precision step
(FP32 element / assembly / CG, FP64 residual refreshes, all meshes in one persistent launch); the
same meshes are also stepped through the plain FP64 GPU path one mesh at a time, and the line
carries that path's throughput, the speed-up over it and the mixed-vs-FP64 displacement error.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--config batch|bar|cube|hex]
                    [--precision fp64|mixed] [--impl reference]

--config bar is the 40x40x160 compression bar (h 4 mm, 1.28M tets), --config cube the 10x10x10 cube
(5,000 tets), --config hex the reference's own performance-test model (DivisibleCubeRepresentation,
Fem3DElementCube hexahedra) at 64 nodes per axis (250,047 hexahedra); all three take --precision. Inputs are synthetic (seeded). One JSON line on rank 0. Under
torchrun the batch's meshes shard over the ranks by greedy bin-packing (one GPU each, no data-path
collective; strong scaling: the job value is all meshes' tet-steps over the slowest rank's time); the
single-mesh workloads run one replica per rank (weak scaling).
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
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "tet-element-steps/s, mixed+batched vs plain FP64 GPU path at <=1e-6 rel disp err"
UNIT = "tet-element-steps/s"
HEX_METRIC = "hex-element-steps/s (Fem3DElementCube, the reference's DivisibleCube performance-test model)"
HEX_UNIT = "hex-element-steps/s"
PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0
CG_CAP = 10000
BAR_SCENARIO_STEPS = 200  # --config bar --steps 200: the whole compression scenario, both forms
# Cube edge of the bar. The scenario leaves it open; the driven face moves 0.64 edges a step whatever h
# is, an elastic wave crosses sqrt(E/rho) dt / h edges a step. At 4 mm the 50 ramp steps stay
# well-posed. In the hold phase of the whole 200-step scenario, elements invert by the hundred
# thousand (per-element E spans two decades, nu reaches 0.49) and the FP64 CG stops converging (on
# GB300: from step ~60 at 4 mm, ~130 at 2 mm, the trajectories diverging after); the whole-scenario run
# reports the step where the FP64 solve first fails and the error up to it.
BAR_H_WINDOW = 0.004
BAR_H_FULL = 0.004
BATCH = dict(count=256, lo=500, hi=50000, seed=3)
BATCH_PARAMS = dict(rayleigh_mass=0.01, rayleigh_stiffness=0.001, gravity=(0.0, 0.0, -9.81), cg_tolerance=1e-10)
COMPARE_STEPS = 4  # steps of the per-mesh FP64 path's timing (1 untimed + 3 timed)
ERROR_RUN_STEPS = 100  # the batch scenario's length: the mixed-vs-FP64 error is taken over all of it


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


# FP64 arithmetic of the corotational element kernel (k_element_fp64), per tet: 1,717 DFMA, 742 DMUL
# and 189 DADD executed (ncu counters sm__sass_thread_inst_executed_op_{dfma,dmul,dadd}_pred_on.sum
# over one launch on the 10x10x10 cube, 5,000 tets) = 2 * 1717 + 742 + 189 FLOPs. The kernel does
# the polar decomposition, the corotational tangent and the force in closed form, so this is below
# the reference's ~6-7k FMAs per tet for the same element update.
ELEMENT_FP64_FLOPS_PER_TET = 2 * 1717 + 742 + 189
# GB300 FP64 (non-tensor) peak, NVIDIA's nominal figure; no measured FP64 peak is available.
FP64_PEAK_TFLOPS = 1.25


def load_traffic(kernel_key):
    """Per-launch DRAM bytes of a kernel from the committed ncu summary (profiles/traffic.json)."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            return json.load(f).get(kernel_key)
    except Exception:
        return None


def host_threads():
    return max(1, math.ceil(0.5 * (os.cpu_count() or 1)))


def host_info():
    """The host the CPU numbers were taken on: nproc and the lscpu summary lines."""
    info = {"nproc": os.cpu_count()}
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        keep = ("Architecture", "Model name", "Socket(s)", "Core(s) per socket", "Thread(s) per core", "CPU(s)",
                "CPU max MHz")
        for ln in out.splitlines():
            k, _, v = ln.partition(":")
            if k.strip() in keep:
                info[k.strip()] = v.strip()
    except Exception as exc:  # lscpu missing: nproc alone
        info["lscpu"] = f"unavailable ({exc.__class__.__name__})"
    return info


# ------------------------------------------------------------------------------------------------
# Algorithmic bytes (HBM) of the solve, per CG iteration and per FP64 residual refresh, for one
# mesh with scalar non-zeros nnz, N nodes and n = 3N dofs; s = bytes per matrix value. Block
# sparse storage reads one 4-byte column index per 3x3 block (nnz / 9 of them) and one offset per
# block row; vector passes per iteration by CG schedule (two-phase: p, z in, p out, q out and in,
# x_delta and r in and out, invdiag in: ten; one-phase: r, w, s in and out, p and x_delta in and out,
# invdiag in: eleven); a refresh reads x, b and writes r in FP64.

SCHEDULE_NAMES = {0: "two-phase", 1: "fp64", 2: "one-phase"}


def pin_schedule(body, args):
    """--cg-schedule: after the autotuning warm-up step, keep its block sizes and grid but run the
    persistent solve in the named CG schedule (for comparing the schedules on one workload)."""
    if args.cg_schedule == "auto":
        return
    e, c, r, _ = body.tuning()
    body.set_tuning(e, c, r, {v: k for k, v in SCHEDULE_NAMES.items()}[args.cg_schedule])


def vector_passes(schedule):
    return 11 if schedule == 2 else 10


def bytes_per_iteration(nnz, N, s, vectors=10):
    return nnz * s + (nnz // 9) * 4 + 4 * (N + 1) + vectors * s * 3 * N


def bytes_per_refresh(nnz, N, s):
    return nnz * s + (nnz // 9) * 4 + 4 * (N + 1) + 3 * 8 * 3 * N


# ------------------------------------------------------------------------------------------------
# Batched workload

def batch_scenes(count=BATCH["count"]):
    """The batch workload; a smaller `count` takes the first meshes of the same seeded sequence."""
    from opensurgsim_gb300 import mesh

    return mesh.scenes_batch(**dict(BATCH, count=count))


def batch_body(meshes, precision, device, autotune=False):
    from opensurgsim_gb300.body import Body

    return Body(meshes, precision=precision, device=device, autotune=autotune, **BATCH_PARAMS)


def rel_disp_err(x_mixed, x64, rest):
    import numpy as np

    d64 = x64 - rest
    return float(np.linalg.norm((x_mixed - rest) - d64) / max(np.linalg.norm(d64), 1e-300))


def fp64_path_comparison(meshes, local):
    """The plain FP64 GPU path on the same meshes, one handle per mesh stepped in turn (the
    reference steps representations one by one): COMPARE_STEPS steps, the last ones timed."""
    import torch

    from opensurgsim_gb300 import _lib
    from opensurgsim_gb300.body import Body

    bodies = [Body(m, precision=_lib.PRECISION_FP64, device=local, cg_max_iterations=0, **BATCH_PARAMS)
              for m in meshes]
    for b in bodies:
        b.step(1e-3, 1)
    torch.cuda.synchronize(local)
    t0 = time.perf_counter()
    its = 0
    for _ in range(COMPARE_STEPS - 1):
        for b in bodies:
            b.step(1e-3, 1)
            its += b.stats()["cg_iterations"]
    torch.cuda.synchronize(local)
    sec = (time.perf_counter() - t0) / (COMPARE_STEPS - 1)
    tets = sum(m.num_tets for m in meshes)
    for b in bodies:
        b.close()
    return {"value": tets / sec, "unit": UNIT, "ms_per_step": 1e3 * sec,
            "cg_iterations_per_step": its / (COMPARE_STEPS - 1),
            "how": (f"plain FP64 form, one handle per mesh stepped in turn; steps 2-{COMPARE_STEPS} timed "
                    "(host clock around device-synchronised steps)")}


def fp64_batch_and_error(meshes, local, steps, warmup, mixed_tuning):
    """(1) The plain FP64 form batched like the mixed one: all meshes in one handle, every mesh's Eigen
    CG in one persistent FP64 launch, graph steps, autotuned; `steps` steps device-timed after
    `warmup`. (2) The mixed-vs-FP64 displacement error over the whole 100-step scenario: that FP64
    batch and a mixed batch (the timed run's tuning) stepped side by side from rest, the per-mesh
    relative error ||u_mixed - u_fp64|| / ||u_fp64|| taken on the device after every step."""
    import numpy as np
    import torch

    from opensurgsim_gb300 import _lib
    from opensurgsim_gb300.autograd import state_views

    tets = sum(m.num_tets for m in meshes)
    b64 = batch_body(meshes, _lib.PRECISION_FP64, local, autotune=True)
    stream = torch.cuda.ExternalStream(b64.stream(), device=local)
    for _ in range(warmup):
        b64.step(1e-3, 1, _lib.STEP_GRAPH)
    torch.cuda.synchronize(local)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    st = b64.step(1e-3, steps, _lib.STEP_GRAPH)
    ev1.record(stream)
    torch.cuda.synchronize(local)
    ms = ev0.elapsed_time(ev1)
    its = int(b64.segment_stats()["iterations"].max())
    fp64_batch = {"value": tets * steps / (ms / 1e3), "unit": UNIT, "ms_per_step": ms / steps,
                  "cg_iterations_per_step": its / steps, "step_status": int(st), "tuning_ctas_per_sm": b64.tuning()[1],
                  "how": ("plain FP64 form batched: one handle, FP64 element kernel and assembly, every mesh's Eigen "
                          "CG in one persistent FP64 launch, graph steps; device-timed like the mixed line")}
    # Side-by-side run from rest over the whole scenario.
    bm = batch_body(meshes, _lib.PRECISION_MIXED, local)
    bm.set_tuning(*mixed_tuning)
    rest = torch.from_numpy(np.concatenate([m.nodes.ravel() for m in meshes])).cuda(local)
    x64, v64 = state_views(b64)
    xm, _ = state_views(bm)
    x64.copy_(rest)
    v64.zero_()
    torch.cuda.synchronize(local)
    counts = np.array([3 * m.num_nodes for m in meshes])
    seg = torch.from_numpy(np.repeat(np.arange(len(meshes)), counts)).cuda(local)
    worst_per_mesh = torch.zeros(len(meshes), dtype=torch.float64, device=f"cuda:{local}")
    worst_per_step = []
    for _ in range(ERROR_RUN_STEPS):
        bm.step(1e-3, 1, _lib.STEP_GRAPH)
        b64.step(1e-3, 1, _lib.STEP_GRAPH)
        u = x64 - rest
        d = xm - x64
        num = torch.zeros(len(meshes), dtype=torch.float64, device=u.device).index_add_(0, seg, d * d)
        den = torch.zeros(len(meshes), dtype=torch.float64, device=u.device).index_add_(0, seg, u * u)
        e = torch.sqrt(num / den.clamp_min(1e-300))
        worst_per_mesh = torch.maximum(worst_per_mesh, e)
        worst_per_step.append(float(e.max()))
    final = e.cpu().numpy()
    bm.close()
    b64.close()
    err = {"max": float(max(worst_per_step)), "final_max": float(final.max()), "final_median": float(np.median(final)),
           "median_of_per_mesh_max": float(np.median(worst_per_mesh.cpu().numpy())),
           "every_10_steps": [float(v) for v in worst_per_step[9::10]], "steps": ERROR_RUN_STEPS,
           "definition": ("||u_mixed - u_fp64|| / ||u_fp64|| per mesh, u = x - x_rest, after every step of the "
                          f"{ERROR_RUN_STEPS}-step scenario from rest; max = worst mesh over all steps, final_* at the "
                          "last step; FP64 reference: the FP64 batch (persistent FP64 CG, tolerance 1e-10)")}
    return fp64_batch, err


def run_batch(args, rank, world, local, dist):
    import numpy as np
    import torch

    from opensurgsim_gb300 import _lib, build

    from opensurgsim_gb300 import shard

    build.build()
    torch.cuda.set_device(local)
    all_scenes = batch_scenes(args.meshes)
    total_tets = sum(s.mesh.num_tets for s in all_scenes)
    total_nodes = sum(s.mesh.num_nodes for s in all_scenes)
    scenes = all_scenes
    if world > 1:
        # The meshes shard over the ranks by greedy bin-packing; no data-path collective.
        bins = shard.partition([shard.mesh_weight(s.mesh) for s in all_scenes], world)
        scenes = [all_scenes[i] for i in bins[rank]]
    meshes = [s.mesh for s in scenes]
    tets = sum(m.num_tets for m in meshes)
    nodes = sum(m.num_nodes for m in meshes)
    log(f"batch: rank {rank}/{world} steps {len(meshes)} of {len(all_scenes)} meshes, {tets} tets, {nodes} nodes")
    body = batch_body(meshes, _lib.PRECISION_MIXED, local, autotune=True)
    stream = torch.cuda.ExternalStream(body.stream(), device=local)
    # Steps run as a captured CUDA graph; the first warm-up step autotunes (outside the graph).
    flags = _lib.STEP_TIME_KERNELS | _lib.STEP_GRAPH
    for w in range(args.warmup):
        body.step(1e-3, 1, flags)
        if w == 0:
            pin_schedule(body, args)
    torch.cuda.synchronize(local)
    tuning = body.tuning()
    log(f"tuning: {tuning[0]} elements per block, {tuning[1]} CTAs per SM, refresh weight {tuning[2]}, "
        f"CG schedule {SCHEDULE_NAMES[tuning[3]]}")
    vpass = vector_passes(tuning[3])
    dist.barrier()
    sampler = ClockSampler(local)
    sampler.start()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    launches, solve_ms, statuses = 0, 0.0, []
    alg_bytes = 0.0
    nnz = body.nnz_per_mesh
    nn = np.diff(body.node_offsets)
    it_bytes = np.array([bytes_per_iteration(int(z), int(N), 4, vpass) for z, N in zip(nnz, nn)], dtype=np.float64)
    rf_bytes = np.array([bytes_per_refresh(int(z), int(N), 4) for z, N in zip(nnz, nn)], dtype=np.float64)
    io_bytes = float(np.sum(16 * 3 * nn))  # b in, x out (FP64)
    ev0.record(stream)
    statuses.append(body.step(1e-3, args.steps, flags))
    ev1.record(stream)
    s = body.stats()
    launches = s["kernel_launches"]
    solve_ms = s["ms_spmv"]
    ss = body.segment_stats()  # summed over the call's steps
    alg_bytes = float(np.dot(ss["iterations"], it_bytes) + np.dot(ss["refreshes"], rf_bytes)) + io_bytes * args.steps
    iters_total = int(ss["iterations"].max())
    torch.cuda.synchronize(local)
    clocks = sampler.stop()
    dist.barrier()
    ms = ev0.elapsed_time(ev1)
    ms_max = dist.reduce(ms, "max")
    value = dist.reduce(tets * args.steps, "sum") / (ms_max / 1e3)
    log(f"timed region: {args.steps} steps in {ms:.1f} ms ({tets * args.steps / ms * 1e3 / 1e6:.1f} M tet-steps/s)")

    # End to end through the public API with host buffers: every step the state of all meshes is
    # copied in from pinned host memory (gbfem_set_state), stepped, and read back (gbfem_get_state).
    h_x = torch.empty(body.n, dtype=torch.float64).pin_memory().numpy()
    h_v = torch.empty(body.n, dtype=torch.float64).pin_memory().numpy()
    body_lib = _lib.load()
    body_lib.gbfem_get_state(body.handle, _lib.dptr(h_x), _lib.dptr(h_v))
    torch.cuda.synchronize(local)
    dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        body_lib.gbfem_set_state(body.handle, _lib.dptr(h_x), _lib.dptr(h_v))
        body.step(1e-3, 1, _lib.STEP_GRAPH)
        body_lib.gbfem_get_state(body.handle, _lib.dptr(h_x), _lib.dptr(h_v))
    torch.cuda.synchronize(local)
    e2e_s = dist.reduce(time.perf_counter() - t0, "max")
    e2e_value = dist.reduce(tets * args.steps, "sum") / e2e_s
    log(f"e2e region: {args.steps} steps in {e2e_s:.3f} s")
    body.close()

    peak, peak_kind = load_peak()
    launch_ms = solve_ms / max(1, args.steps)
    per_launch = alg_bytes / max(1, args.steps)
    achieved = per_launch / (launch_ms / 1e3) / 1e9 if launch_ms > 0 else None
    line = {
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_max / args.steps,
        "higher_is_better": True,
        "scaling": "strong",
        "vs_baseline": None,
        "dtype": "f32+f64",
        "data": "synthetic (seeded cube-grid meshes)",
        "config": {
            "workload": (f"batch{len(all_scenes)}: {len(all_scenes)} cube-grid meshes (h 1 cm, 5 tets per cube, "
                         f"nodes log-U[500,50000], seed 3), {total_tets} tets, {total_nodes} nodes, E log-U[1e4,1e6] "
                         "per mesh, nu 0.45, bottom faces fixed, "
                         "gravity, alpha 0.01, beta 0.001, dt 1e-3, CG tol 1e-10; batched mixed precision, one "
                         "persistent solve launch per step, steps launched as a CUDA graph"),
            "tuning": {"elements_per_block": tuning[0], "ctas_per_sm": tuning[1], "refresh_weight": tuning[2],
                       "cg_schedule": SCHEDULE_NAMES[tuning[3]], "how": "autotuned on the first warm-up step"},
            "meshes": len(all_scenes), "tets": total_tets, "nodes": total_nodes, "precision": "mixed",
            "l2": "working set (~2 GB) larger than L2: no flush needed",
            "parallelism": (f"meshes sharded over {world} ranks by greedy bin-packing (opensurgsim_gb300.shard), "
                            "no data-path collective" if world > 1 else "one GPU, all meshes in one batch"),
        },
        "gpu_launches": int(launches),
        "cg_iterations_per_step": iters_total / max(1, args.steps),  # the slowest mesh
        "step_status": sorted(set(int(s) for s in statuses)),
        "clocks": clocks,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 2 * body.n * 8,
                "d2h_bytes_per_step": 2 * body.n * 8},
        "roofline": {
            "kernel": "k_pcg_persistent (whole batched mixed-precision solve, one launch per step)",
            "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": (achieved / peak) if achieved else None,
            "traffic": load_traffic(f"pcg_persistent_batch{len(all_scenes)}") if world == 1 else None,
            "algorithmic_bytes_per_launch": per_launch, "avg_launch_ms": launch_ms,
            "peak_source": f"{peak_kind} (hbm_gbs)",
            "bytes_model": (f"per mesh: CG iterations x (nnz*4 + nnz/9*4 + 4(N+1) + {vpass}*4*3N) + refreshes x "
                            "(nnz*4 + nnz/9*4 + 4(N+1) + 3*8*3N) + 16*3N"),
        },
    }
    return line, scenes


# ------------------------------------------------------------------------------------------------
# Single-mesh workloads (bar, cube)

HEX_NODES_PER_AXIS = 64  # --config hex: 63^3 = 250,047 hexahedra, 262,144 nodes


def build_scene(config, h=None):
    from opensurgsim_gb300 import mesh

    if config == "hex":
        # The reference's own performance-test model (DivisibleCubeRepresentation + Fem3DPerformanceTest:
        # rho 980, nu 0.499, E 15.3e3, nodes 0-2 fixed, CG tolerance 1e-3, maxIter 0.1 n, dt 1e-3, 10
        # frames), scaled from its 2..8 nodes per axis to 64.
        return mesh.scene_divisible_cube(HEX_NODES_PER_AXIS)
    # The explicit CG iteration cap only bounds the run if a solve ever stagnates; at the
    # benchmark's states CG converges in a few hundred iterations, far below it.
    if config == "bar":
        return mesh.scene_bar_compression(h=h or BAR_H_WINDOW, cg_max_iterations=CG_CAP)
    return mesh.scene_cube(10, 10, 10, cg_max_iterations=CG_CAP)


def run_single(args, rank, world, local, dist):
    import numpy as np
    import torch

    from opensurgsim_gb300 import _lib, build
    from opensurgsim_gb300.body import Body

    build.build()
    torch.cuda.set_device(local)
    scene = build_scene(args.config, args.bar_h)
    m = scene.mesh
    log(f"scene {scene.name}: {m.num_tets} tets, {m.num_nodes} nodes")
    prec = _lib.PRECISION_MIXED if args.precision == "mixed" else _lib.PRECISION_FP64
    body = Body.from_scene(scene, precision=prec, device=local, autotune=(prec == _lib.PRECISION_MIXED))
    stream = torch.cuda.ExternalStream(body.stream(), device=local)
    dt = scene.dt
    driven = scene.driven_dofs is not None
    body_lib = _lib.load()
    if driven:
        d_dofs = torch.from_numpy(scene.driven_dofs.astype(np.int32)).cuda(local)
        ramp = torch.from_numpy(scene.driven_values(0)).cuda(local)
        hold = torch.zeros_like(ramp)

    def set_driven(step):
        if driven:
            vals = ramp if step < scene.ramp_steps else hold
            body_lib.gbfem_set_velocities_device(body.handle, d_dofs.numel(), d_dofs.data_ptr(), vals.data_ptr())

    # The mixed form's steps run as a captured CUDA graph (the prescribed velocities are written into
    # the state between graph launches); the first warm-up step autotunes.
    graph = _lib.STEP_GRAPH if prec == _lib.PRECISION_MIXED else 0
    flags = _lib.STEP_TIME_KERNELS | graph
    step = 0
    for w in range(args.warmup):
        set_driven(step)
        body.step(dt, 1, flags)
        if w == 0 and prec == _lib.PRECISION_MIXED:
            pin_schedule(body, args)
        step += 1
    torch.cuda.synchronize(local)
    dist.barrier()
    sampler = ClockSampler(local)
    sampler.start()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    agg = dict(cg_iterations=0, kernel_launches=0, ms_spmv=0.0, spmv_timed=0, refinement_sweeps=0)
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
    metric, unit = (HEX_METRIC, HEX_UNIT) if args.config == "hex" else (METRIC, UNIT)
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
        body.step(dt, 1, graph)
        body_lib.gbfem_get_state(body.handle, _lib.dptr(h_x), _lib.dptr(h_v))
        step += 1
    torch.cuda.synchronize(local)
    e2e_s = dist.reduce(time.perf_counter() - t0, "max")
    e2e_value = total_units / e2e_s
    fp64_alu = None
    if prec == _lib.PRECISION_FP64 and args.config != "hex":
        # The element kernel is bound by the FP64 pipe, not HBM: one more (untimed) step with phase
        # events gives its device time.
        set_driven(step)
        body.step(dt, 1, _lib.STEP_TIME_PHASES)
        step += 1
        el_ms = body.stats()["ms_element"]
        if el_ms > 0:
            tflops = m.num_tets * ELEMENT_FP64_FLOPS_PER_TET / (el_ms / 1e3) / 1e12
            fp64_alu = {"kernel": "k_element_fp64", "bound": "fp64 pipe", "achieved": tflops,
                        "peak": FP64_PEAK_TFLOPS, "unit": "TFLOP/s", "frac": tflops / FP64_PEAK_TFLOPS,
                        "flops_per_tet": ELEMENT_FP64_FLOPS_PER_TET, "launch_ms": el_ms,
                        "peak_source": "nominal (no measured FP64 peak)"}
    workload = {
        "bar": ("bar40x40x160 (h 4 mm) 20% compression ramp: 1,280,000 tets, 270,641 nodes, "
                "nnz 30,865,689, E log-U[1e4,1e6], nu U[0.40,0.49], gravity, dt 1e-3, CG tol 1e-10"),
        "cube": "cube10x10x10: 5,000 tets, E 1e5, nu 0.45",
        "hex": (f"divisiblecube{HEX_NODES_PER_AXIS} (Fem3DElementCube): {m.num_tets:,} hexahedra, {m.num_nodes:,} "
                "nodes, rho 980, nu 0.499, E 15.3e3, nodes 0-2 fixed, gravity (0,-9.81,0), no damping, dt 1e-3, "
                "CG tol 1e-3, maxIter 0.1 n"),
    }[args.config]
    h2d = (scene.driven_dofs.size * (4 + 8)) if driven else 0
    d2h = 2 * body.n * 8
    peak, peak_kind = load_peak()
    cg_per_step = agg["cg_iterations"] / max(1, args.steps)
    if prec == _lib.PRECISION_FP64:
        # Dominant kernel: the CG SpMV on the SELL-32 block matrix, timed per launch.
        spmv_bytes = body.nnz * 8 + (body.nnz // 9) * 4 + (body.num_nodes + 1) * 4 + 2 * body.n * 8
        launch_ms = agg["ms_spmv"] / max(1, agg["spmv_timed"])
        kernel, per_launch, key = "k_cg_spmv_sell (fp64)", spmv_bytes, f"spmv_sell_fp64_{args.config}"
        model = "nnz*8 + nnz/9*4 + 4(N+1) + 2*8*n per SpMV"
    else:
        # Dominant kernel: the persistent mixed-precision solve, one launch per step.
        launch_ms = agg["ms_spmv"] / max(1, args.steps)
        iters = agg["cg_iterations"] / max(1, args.steps)
        sweeps = agg["refinement_sweeps"] / max(1, args.steps)
        vpass = vector_passes(body.tuning()[3])
        per_launch = (iters * bytes_per_iteration(body.nnz, body.num_nodes, 4, vpass)
                      + sweeps * bytes_per_refresh(body.nnz, body.num_nodes, 4) + 16 * body.n)
        kernel, key = "k_pcg_persistent (mixed)", f"pcg_persistent_{args.config}"
        model = (f"CG iterations x (nnz*4 + nnz/9*4 + 4(N+1) + {vpass}*4*n) + refreshes x (nnz*4 + nnz/9*4 + 4(N+1) "
                 "+ 3*8*n) + 16n")
    achieved = per_launch / (launch_ms / 1e3) / 1e9 if launch_ms > 0 else None
    line = {
        "metric": metric,
        "value": value,
        "unit": unit,
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
            "workload": workload,
            "elements": m.num_tets, "nodes": m.num_nodes, "dofs": body.n, "nnz": body.nnz,
            "precision": args.precision, "scenario_steps": [args.warmup, args.warmup + args.steps],
            "l2": "working set larger than L2 (no flush needed)" if args.config in ("bar", "hex") else
                  "working set L2-resident (small case)",
            "parallelism": f"replicas x{world}",
        },
        "gpu_launches": int(agg["kernel_launches"]),
        "cg_iterations_per_step": cg_per_step,
        "step_status": sorted(set(int(s) for s in statuses)),
        "clocks": clocks,
        "e2e": {"value": e2e_value, "unit": unit, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "roofline": {
            "kernel": kernel, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": (achieved / peak) if achieved else None, "traffic": load_traffic(key),
            "algorithmic_bytes_per_launch": per_launch, "avg_launch_ms": launch_ms,
            "peak_source": f"{peak_kind} (hbm_gbs)", "bytes_model": model,
        },
    }
    if fp64_alu:
        line["fp64_alu"] = fp64_alu
    body.close()
    return line, scene


def run_bar_full(args, rank, world, local, dist):
    """The 40x40x160 compression bar over its whole scenario (50 ramp steps, then hold; 200 steps),
    plain FP64 and mixed forms side by side on the same GPU. After every step the mixed form's
    displacement is compared with the FP64 form's on the device; both forms are timed per step with
    CUDA events on their own streams. W warm-up steps run first (the mixed form autotunes), then both
    bodies are put back at rest and the timed run starts at step 0 of the scenario."""
    import numpy as np
    import torch

    from opensurgsim_gb300 import _lib, build
    from opensurgsim_gb300.autograd import state_views
    from opensurgsim_gb300.body import Body

    build.build()
    torch.cuda.set_device(local)
    scene = build_scene("bar", args.bar_h or BAR_H_FULL)
    m = scene.mesh
    log(f"bar full run: {m.num_tets} tets, {m.num_nodes} nodes, h {scene.mesh.h * 1e3:g} mm, {args.steps} steps, "
        "both forms")
    bodies = {"fp64": Body.from_scene(scene, precision=_lib.PRECISION_FP64, device=local),
              "mixed": Body.from_scene(scene, precision=_lib.PRECISION_MIXED, device=local, autotune=True)}
    flags = {"fp64": 0, "mixed": _lib.STEP_GRAPH}
    L = _lib.load()
    d_dofs = torch.from_numpy(scene.driven_dofs.astype(np.int32)).cuda(local)
    ramp = torch.from_numpy(scene.driven_values(0)).cuda(local)
    hold = torch.zeros_like(ramp)
    rest = torch.from_numpy(m.nodes.ravel().copy()).cuda(local)
    views = {k: state_views(b) for k, b in bodies.items()}
    streams = {k: torch.cuda.ExternalStream(b.stream(), device=local) for k, b in bodies.items()}

    def drive(b, step):
        vals = ramp if step < scene.ramp_steps else hold
        L.gbfem_set_velocities_device(b.handle, d_dofs.numel(), d_dofs.data_ptr(), vals.data_ptr())

    for k, b in bodies.items():
        for s in range(args.warmup):
            drive(b, s)
            b.step(scene.dt, 1, flags[k])
            if s == 0 and k == "mixed":
                pin_schedule(b, args)
    torch.cuda.synchronize(local)
    for k, b in bodies.items():  # back to rest: the timed run is the scenario from its first step
        x, v = views[k]
        x.copy_(rest)
        v.zero_()
    torch.cuda.synchronize(local)
    tuning = bodies["mixed"].tuning()
    dist.barrier()
    sampler = ClockSampler(local)
    sampler.start()
    evs = {k: [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(args.steps)] for k in bodies}
    agg = {k: dict(cg_iterations=0, kernel_launches=0, polar_fallbacks=0, singular_g=0, ms_spmv=0.0,
                   refinement_sweeps=0) for k in bodies}
    statuses = {k: set() for k in bodies}
    errs = []
    u64n = []
    per_step = {k: [] for k in bodies}  # (status, CG iterations, SVD fallbacks) per step
    for s in range(args.steps):
        for k, b in bodies.items():
            drive(b, s)
            e0, e1 = evs[k][s]
            e0.record(streams[k])
            timing = _lib.STEP_TIME_KERNELS if k == "mixed" else 0  # the persistent solve's own events
            status = int(b.step(scene.dt, 1, flags[k] | timing))
            statuses[k].add(status)
            e1.record(streams[k])
            st = b.stats()
            for key in agg[k]:
                agg[k][key] += st[key]
            per_step[k].append((status, st["cg_iterations"], st["polar_fallbacks"]))
        # Relative displacement error of the mixed form against the FP64 form, on the device.
        u64 = views["fp64"][0] - rest
        d = views["mixed"][0] - views["fp64"][0]
        n64 = float(torch.linalg.vector_norm(u64))
        errs.append(float(torch.linalg.vector_norm(d)) / max(n64, 1e-300))
        u64n.append(n64)
    torch.cuda.synchronize(local)
    clocks = sampler.stop()
    dist.barrier()
    ms = {k: sum(e0.elapsed_time(e1) for e0, e1 in evs[k]) for k in bodies}
    units = m.num_tets * args.steps
    val = {k: dist.reduce(units, "sum") / (dist.reduce(ms[k], "max") / 1e3) for k in bodies}
    log(f"fp64 {val['fp64'] / 1e6:.1f} M, mixed {val['mixed'] / 1e6:.1f} M tet-steps/s; max err {max(errs):.2e}")

    # End to end (mixed, public API, host buffers) over 10 further hold steps: prescribed velocities
    # in from pinned host memory, x and v read back every step.
    bm = bodies["mixed"]
    h_dofs = scene.driven_dofs.astype(np.int32)
    h_vals = torch.zeros(h_dofs.size, dtype=torch.float64).pin_memory().numpy()
    h_x = torch.empty(bm.n, dtype=torch.float64).pin_memory().numpy()
    h_v = torch.empty(bm.n, dtype=torch.float64).pin_memory().numpy()
    e2e_steps = 10
    torch.cuda.synchronize(local)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        bm.set_velocities(h_dofs, h_vals)
        bm.step(scene.dt, 1, _lib.STEP_GRAPH)
        L.gbfem_get_state(bm.handle, _lib.dptr(h_x), _lib.dptr(h_v))
    torch.cuda.synchronize(local)
    e2e_value = m.num_tets * e2e_steps / (time.perf_counter() - t0)

    peak, peak_kind = load_peak()
    am = agg["mixed"]
    solve_ms = am["ms_spmv"] / args.steps
    vpass = vector_passes(tuning[3])
    per_launch = (am["cg_iterations"] / args.steps * bytes_per_iteration(bm.nnz, bm.num_nodes, 4, vpass)
                  + am["refinement_sweeps"] / args.steps * bytes_per_refresh(bm.nnz, bm.num_nodes, 4) + 16 * bm.n)
    achieved = per_launch / (solve_ms / 1e3) / 1e9 if solve_ms > 0 else None
    errs_a = np.array(errs)
    ramp_end = min(scene.ramp_steps, args.steps)
    # The first step whose FP64 solve stopped at its iteration cap: from there the FP64 reference's
    # own step no longer converges (the scene's hold phase inverts elements by the hundred thousand and
    # the tangent stops being positive definite), and the two forms follow diverging trajectories.
    cap64 = next((i for i, r in enumerate(per_step["fp64"]) if r[0] != 0), None)
    well_posed = errs_a[:cap64] if cap64 is not None else errs_a
    line = {
        "metric": METRIC, "value": val["mixed"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms["mixed"] / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic (seeded cube-grid mesh)",
        "config": {
            "workload": (f"bar40x40x160 (h {scene.mesh.h * 1e3:g} mm) whole scenario: 20% compression ramp over 50 "
                         "steps, then held; "
                         f"{args.steps} steps from rest; 1,280,000 tets, 270,641 nodes, E log-U[1e4,1e6], "
                         "nu U[0.40,0.49], gravity, dt 1e-3, CG tol 1e-10; plain FP64 and mixed forms side by side"),
            "elements": m.num_tets, "nodes": m.num_nodes, "dofs": bm.n, "nnz": bm.nnz, "precision": "mixed",
            "tuning": {"elements_per_block": tuning[0], "ctas_per_sm": tuning[1], "refresh_weight": tuning[2],
                       "cg_schedule": SCHEDULE_NAMES[tuning[3]]},
            "l2": "working set larger than L2 (no flush needed)", "parallelism": f"replicas x{world}",
        },
        "gpu_launches": int(am["kernel_launches"]),
        "cg_iterations_per_step": am["cg_iterations"] / args.steps,
        "step_status": sorted(statuses["mixed"]),
        "clocks": clocks,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h_dofs.size * (4 + 8)),
                "d2h_bytes_per_step": 2 * bm.n * 8,
                "how": f"{e2e_steps} hold steps after the timed run, host clock"},
        "roofline": {
            "kernel": "k_pcg_persistent (mixed)", "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": (achieved / peak) if achieved else None,
            "traffic": load_traffic("pcg_persistent_bar") if abs(scene.mesh.h - BAR_H_WINDOW) < 1e-12 else None,
            "algorithmic_bytes_per_launch": per_launch, "avg_launch_ms": solve_ms,
            "peak_source": f"{peak_kind} (hbm_gbs)",
            "bytes_model": (f"CG iterations x (nnz*4 + nnz/9*4 + 4(N+1) + {vpass}*4*n) + refreshes x "
                            "(nnz*4 + nnz/9*4 + 4(N+1) + 3*8*n) + 16n"),
        },
        "fp64_path": {"value": val["fp64"], "unit": UNIT, "ms_per_step": ms["fp64"] / args.steps,
                      "cg_iterations_per_step": agg["fp64"]["cg_iterations"] / args.steps,
                      "step_status": sorted(statuses["fp64"]),
                      "how": "plain FP64 form, same scenario and steps, device-timed per step"},
        "speedup_vs_fp64_path": val["mixed"] / val["fp64"],
        "rel_disp_err_vs_fp64": {
            "max": float(errs_a.max()), "final": float(errs_a[-1]), "max_ramp": float(errs_a[:ramp_end].max()),
            "max_hold": float(errs_a[ramp_end:].max()) if args.steps > ramp_end else None,
            "every_10_steps": [float(e) for e in errs_a[9::10]],
            "first_step_fp64_not_converged": cap64,
            "max_while_fp64_converges": float(well_posed.max()) if well_posed.size else None,
            "definition": "||u_mixed - u_fp64|| / ||u_fp64||, u = x - x_rest, after every step"},
        "per_step_every_10": {k: [list(r) for r in v[9::10]] for k, v in per_step.items()},
        "inversions": {"polar_fallbacks_fp64": agg["fp64"]["polar_fallbacks"],
                       "polar_fallbacks_mixed": am["polar_fallbacks"],
                       "singular_g_fp64": agg["fp64"]["singular_g"], "singular_g_mixed": am["singular_g"],
                       "how": "element updates that took the SVD polar path (det F <= 0), summed over the run"},
    }
    for b in bodies.values():
        b.close()
    return line, scene


# ------------------------------------------------------------------------------------------------
# Differentiation workload (--config adjoint): identification of per-element log E on a 20x20x40
# cube grid (80,000 tets) from 64 marker positions after 50 steps.

ADJ_STEPS, ADJ_CHECKPOINT, ADJ_MARKERS, ADJ_FD_ELEMENTS, ADJ_FD_H = 50, 10, 64, 32, 1e-6


def adjoint_problem(seed=5):
    """theta_e = ln(1e5) + N(0, 0.3), v0 ~ N(0, 0.01) m/s per free dof, 64 seeded marker nodes, targets
    from a second (ground-truth) theta field after 50 steps; bottom face fixed, gravity, alpha 0.01,
    beta 0.001, dt 1e-3; CG tolerance 1e-12 (finite differences at h = 1e-6 need tight solves)."""
    import numpy as np

    from opensurgsim_gb300 import mesh

    scene = mesh.scene_cube(20, 20, 40, seed=seed, cg_tolerance=1e-12)
    m = scene.mesh
    rng = np.random.default_rng(seed)
    theta = math.log(1e5) + rng.normal(0, 0.3, m.num_tets)
    theta_true = math.log(1e5) + rng.normal(0, 0.3, m.num_tets)
    v0 = rng.normal(0, 0.01, 3 * m.num_nodes)
    v0[m.bc_dofs] = 0.0
    bc_nodes = set((m.bc_dofs // 3).tolist())
    free = np.array([i for i in range(m.num_nodes) if i not in bc_nodes])
    markers = np.sort(rng.choice(free, ADJ_MARKERS, replace=False))
    return scene, theta, theta_true, v0, markers


def run_adjoint(args, local):
    """Forward + backward throughput of the 50-step rollout (FP64 and mixed), the gradient against
    central finite differences on 32 random elements, and the mixed gradient against the FP64 one."""
    import numpy as np
    import torch

    from opensurgsim_gb300 import _lib, build
    from opensurgsim_gb300.autograd import rollout
    from opensurgsim_gb300.body import Body

    build.build()
    torch.cuda.set_device(local)
    dev = torch.device(f"cuda:{local}")
    scene, theta_np, theta_true_np, v0_np, markers = adjoint_problem()
    m = scene.mesh
    x0 = torch.tensor(m.nodes.ravel(), dtype=torch.float64, device=dev)
    v0 = torch.tensor(v0_np, dtype=torch.float64, device=dev)
    theta = torch.tensor(theta_np, dtype=torch.float64, device=dev)
    mk = torch.tensor(np.stack([3 * markers, 3 * markers + 1, 3 * markers + 2], 1).ravel(), dtype=torch.long,
                      device=dev)
    bodies = {p: Body.from_scene(scene, precision=(_lib.PRECISION_MIXED if p == "mixed" else _lib.PRECISION_FP64),
                                 device=local) for p in ("fp64", "mixed")}
    with torch.no_grad():
        xT, _ = rollout(bodies["fp64"], torch.tensor(theta_true_np, dtype=torch.float64, device=dev), x0, v0,
                        scene.dt, ADJ_STEPS, ADJ_CHECKPOINT)
        target = xT[mk].clone()

    def loss(body, th, flags=0):
        xT_, _ = rollout(body, th, x0, v0, scene.dt, ADJ_STEPS, ADJ_CHECKPOINT, flags)
        return ((xT_[mk] - target) ** 2).sum()

    results = {}
    for p, body in bodies.items():
        def fwd_bwd():
            th = theta.clone().requires_grad_(True)
            L = loss(body, th)
            L.backward()
            return float(L.detach()), th.grad.detach().clone()
        fwd_bwd()  # warm-up
        torch.cuda.synchronize(dev)
        reps = 2
        t0 = time.perf_counter()
        for _ in range(reps):
            Lval, g = fwd_bwd()
        torch.cuda.synchronize(dev)
        sec = (time.perf_counter() - t0) / reps
        t0 = time.perf_counter()
        with torch.no_grad():
            loss(body, theta)
        torch.cuda.synchronize(dev)
        sec_fwd = time.perf_counter() - t0
        # Phase split of the adjoint steps of the last (first-in-time) checkpoint segment: the stats
        # restart at every forward step, so they hold that segment's adjoint steps.
        from opensurgsim_gb300.autograd import graph_rollouts

        if graph_rollouts(body):
            split = {"how": "forward and backward each run as one CUDA graph in the library; no per-phase times"}
        else:
            th = theta.clone().requires_grad_(True)
            loss(body, th, _lib.STEP_TIME_PHASES).backward()
            st = body.stats()
            nadj = min(ADJ_CHECKPOINT, ADJ_STEPS)
            split = {"system_ms": st["ms_element"] / nadj, "transposed_solve_ms": st["ms_solve"] / nadj,
                     "element_derivatives_ms": st["ms_update"] / nadj}
        results[p] = {"loss": Lval, "grad": g, "sec": sec, "sec_forward": sec_fwd, "split": split}
        log(f"adjoint {p}: forward+backward {sec:.3f} s, forward {sec_fwd:.3f} s, loss {Lval:.6e}, split {split}")
    # Central finite differences in log E on 32 random elements (FP64 form).
    rng = np.random.default_rng(17)
    els = np.sort(rng.choice(m.num_tets, ADJ_FD_ELEMENTS, replace=False))
    g64 = results["fp64"]["grad"].cpu().numpy()
    fd = np.zeros(len(els))
    with torch.no_grad():
        for i, e in enumerate(els):
            tp, tm = theta.clone(), theta.clone()
            tp[e] += ADJ_FD_H
            tm[e] -= ADJ_FD_H
            fd[i] = (float(loss(bodies["fp64"], tp)) - float(loss(bodies["fp64"], tm))) / (2 * ADJ_FD_H)
    diff = np.abs(g64[els] - fd)
    gm = results["mixed"]["grad"].cpu().numpy()
    mixed_err = float(np.linalg.norm(gm - g64) / np.linalg.norm(g64))
    E = m.num_tets
    line = {
        "metric": "tet-element-steps/s (forward + backward of a 50-step rollout, adjoint form)",
        "value": E * ADJ_STEPS / results["fp64"]["sec"],
        "unit": UNIT,
        "n_gpus": 1, "steps": 2, "warmup": 1,
        "ms_per_step": 1e3 * results["fp64"]["sec"] / ADJ_STEPS,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded cube-grid mesh, seeded parameters)",
        "config": {"workload": ("adjoint20x20x40: 80,000 tets, log E = ln 1e5 + N(0, 0.3), v0 ~ N(0, 0.01), 64 "
                                "markers, targets from a ground-truth log E field, 50 steps, checkpoints every "
                                "10, CG tol 1e-12"), "tets": E, "nodes": m.num_nodes},
        "adjoint_step_split_ms": results["fp64"]["split"],
        "mixed": {"value": E * ADJ_STEPS / results["mixed"]["sec"],
                  "ms_per_step": 1e3 * results["mixed"]["sec"] / ADJ_STEPS,
                  "grad_rel_err_vs_fp64": mixed_err, "adjoint_step_split_ms": results["mixed"]["split"]},
        "forward_only": {"fp64": E * ADJ_STEPS / results["fp64"]["sec_forward"],
                         "mixed": E * ADJ_STEPS / results["mixed"]["sec_forward"]},
        "fd_check": {"elements": ADJ_FD_ELEMENTS, "h": ADJ_FD_H,
                     "norm_rel_err": float(np.linalg.norm(g64[els] - fd) / np.linalg.norm(fd)),
                     "max_err_rel_to_max_grad": float(diff.max() / np.abs(fd).max()),
                     "median_rel_err": float(np.median(diff / np.abs(fd))), "gate": 1e-4},
        "loss": results["fp64"]["loss"],
        "timing": "host clock around device-synchronised forward+backward (2 repetitions after 1 warm-up)",
    }
    for b in bodies.values():
        b.close()
    return line


# ------------------------------------------------------------------------------------------------
# Batched differentiation workload (--config adjoint-batch): 64 meshes, node counts log-uniform in
# [2000, 100000], per-element log E, 30 steps, FP32 bulk with FP64 refreshes in one batch handle; the
# gradient of every mesh is compared with the FP64 adjoint of that mesh alone.

# Every state of the 30 steps is kept (checkpoint after every step, ~2 GB of HBM for the 6.2M-tet batch),
# so the reverse sweep runs no step again; the same rollout with checkpoints every 10 steps (segments
# re-run) is timed beside it and gives the same gradient bit for bit.
ADJB = dict(count=64, lo=2000, hi=100000, seed=11, steps=30, checkpoint=1, checkpoint_rerun=10, markers=16)


def run_adjoint_batch(args, local):
    import numpy as np
    import torch

    from opensurgsim_gb300 import _lib, build
    from opensurgsim_gb300.autograd import rollout
    from opensurgsim_gb300.body import Body
    from opensurgsim_gb300 import mesh as M

    build.build()
    torch.cuda.set_device(local)
    dev = torch.device(f"cuda:{local}")
    scenes = M.scenes_batch(count=ADJB["count"], lo=ADJB["lo"], hi=ADJB["hi"], seed=ADJB["seed"])
    meshes = [s.mesh for s in scenes]
    rng = np.random.default_rng(ADJB["seed"])
    theta = [np.log(m.young) + rng.normal(0, 0.3, m.num_tets) for m in meshes]
    theta_true = [np.log(m.young) + rng.normal(0, 0.3, m.num_tets) for m in meshes]
    v0 = []
    markers = []
    for m in meshes:
        v = rng.normal(0, 0.01, 3 * m.num_nodes)
        v[m.bc_dofs] = 0.0
        v0.append(v)
        bc_nodes = set((m.bc_dofs // 3).tolist())
        free = np.array([i for i in range(m.num_nodes) if i not in bc_nodes])
        markers.append(np.sort(rng.choice(free, min(ADJB["markers"], free.size), replace=False)))
    steps, ck = ADJB["steps"], ADJB["checkpoint"]
    tets = sum(m.num_tets for m in meshes)
    log(f"adjoint batch: {len(meshes)} meshes, {tets} tets, {sum(m.num_nodes for m in meshes)} nodes")

    def t64(a):
        return torch.tensor(a, dtype=torch.float64, device=dev)

    # Batch handle (mixed precision): concatenated parameters and states.
    batch = Body(meshes, precision=_lib.PRECISION_MIXED, device=local, **BATCH_PARAMS)
    no = batch.node_offsets
    mk = np.concatenate([np.stack([3 * (no[k] + mm), 3 * (no[k] + mm) + 1, 3 * (no[k] + mm) + 2], 1).ravel()
                         for k, mm in enumerate(markers)])
    mk_t = torch.tensor(mk, dtype=torch.long, device=dev)
    x0 = t64(np.concatenate([m.nodes.ravel() for m in meshes]))
    v0b = t64(np.concatenate(v0))
    with torch.no_grad():
        xT, _ = rollout(batch, t64(np.concatenate(theta_true)), x0, v0b, 1e-3, steps, ck)
        target = xT[mk_t].clone()
    th_b = t64(np.concatenate(theta))

    def fwd_bwd(every):
        th = th_b.clone().requires_grad_(True)
        xT_, _ = rollout(batch, th, x0, v0b, 1e-3, steps, every)
        L = ((xT_[mk_t] - target) ** 2).sum()
        L.backward()
        return th.grad.detach().cpu().numpy()

    def timed(every):
        # Warm-up: the same rollout (the library captures the forward and the backward graphs once).
        for _ in range(max(1, args.warmup)):
            g = fwd_bwd(every)
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        for _ in range(reps):
            g = fwd_bwd(every)
        torch.cuda.synchronize(dev)
        return g, (time.perf_counter() - t0) / reps

    reps = max(1, min(args.steps, 3))
    g_batch, sec = timed(ck)
    log(f"batched mixed forward+backward: {sec:.2f} s (checkpoint every {ck} step)")
    g_rerun, sec_rerun = timed(ADJB["checkpoint_rerun"])
    same = bool(np.array_equal(g_rerun, g_batch))
    log(f"  with checkpoints every {ADJB['checkpoint_rerun']} steps (segments re-run): {sec_rerun:.2f} s, "
        f"gradient bit-identical: {same}")
    batch.close()

    def grads_fp64_batch():
        b = Body(meshes, precision=_lib.PRECISION_FP64, device=local, **BATCH_PARAMS)
        th = th_b.clone().requires_grad_(True)
        xk, _ = rollout(b, th, x0, v0b, 1e-3, steps, ck)
        ((xk[mk_t] - target) ** 2).sum().backward()
        torch.cuda.synchronize(dev)
        b.close()
        return th.grad.detach().cpu().numpy()

    # FP64 reference adjoint: the same meshes as one FP64 batch (FP64 element derivatives, every
    # mesh's Eigen CG in FP64), also as CUDA-graph rollouts.
    grads_fp64_batch()  # capture and warm-up
    t0 = time.perf_counter()
    g64 = grads_fp64_batch()
    sec64 = time.perf_counter() - t0
    to = np.concatenate([[0], np.cumsum([m.num_tets for m in meshes])])
    errs = [float(np.linalg.norm(g_batch[to[k]:to[k + 1]] - g64[to[k]:to[k + 1]]) /
                  max(np.linalg.norm(g64[to[k]:to[k + 1]]), 1e-300)) for k in range(len(meshes))]
    log(f"FP64 reference adjoint (FP64 batch): {sec64:.2f} s; gradient error max {max(errs):.2e}")
    # Cross-check of the FP64 batch against FP64 handles, one per mesh, on the first 4 meshes.
    cross = []
    mo = np.concatenate([[0], np.cumsum([3 * len(mm) for mm in markers])])
    for k in range(min(4, len(meshes))):
        m = meshes[k]
        b = Body(m, precision=_lib.PRECISION_FP64, device=local, **BATCH_PARAMS)
        mkk = torch.tensor(np.stack([3 * markers[k], 3 * markers[k] + 1, 3 * markers[k] + 2], 1).ravel(),
                           dtype=torch.long, device=dev)
        th = t64(theta[k]).requires_grad_(True)
        xk, _ = rollout(b, th, t64(m.nodes.ravel()), t64(v0[k]), 1e-3, steps, ck)
        ((xk[mkk] - target[mo[k]:mo[k + 1]]) ** 2).sum().backward()
        gk = th.grad.detach().cpu().numpy()
        cross.append(float(np.linalg.norm(g64[to[k]:to[k + 1]] - gk) / max(np.linalg.norm(gk), 1e-300)))
        b.close()
    log(f"FP64 batch vs FP64 single handles (first {len(cross)} meshes): max {max(cross):.2e}")
    return {
        "metric": "tet-element-steps/s (forward + backward, batched adjoint, 30 steps)",
        "value": tets * steps / sec, "unit": UNIT, "n_gpus": 1, "steps": reps, "warmup": max(1, args.warmup),
        "ms_per_step": 1e3 * sec / steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64", "data": "synthetic (seeded cube-grid meshes, seeded parameters)",
        "config": {"workload": (f"adjoint batch: {len(meshes)} meshes, nodes log-U[2000,100000] (seed {ADJB['seed']}), "
                                f"{tets} tets, per-element log E = ln E_mesh + N(0, 0.3), {ADJB['markers']} markers "
                                f"per mesh, {steps} steps, every state kept (checkpoint after every step), mixed "
                                "precision batch handle; forward and backward each one CUDA graph in the library"),
                   "tets": tets},
        "grad_rel_err_vs_fp64_adjoint": {"max": max(errs), "median": float(np.median(errs)),
                                         "definition": "per mesh ||g_batch - g_fp64|| / ||g_fp64||, FP64 batch reference"},
        "checkpoints_every_10": {"value": tets * steps / sec_rerun, "sec": sec_rerun,
                                 "grad_bit_identical": same,
                                 "how": "the same rollout with checkpoints every 10 steps, the backward re-running "
                                        "each segment's steps"},
        "fp64_reference_adjoint": {"value": tets * steps / sec64,
                                   "how": "the same meshes as one FP64 batch handle, graph rollouts, host clock"},
        "fp64_batch_vs_single_handles": {"max": max(cross), "meshes": len(cross),
                                         "definition": "per mesh gradient, FP64 batch vs one FP64 handle"},
        "timing": f"host clock around {reps} device-synchronised forward+backward passes after the warm-up",
    }


# ------------------------------------------------------------------------------------------------
# CPU side: the oracle (FP64 C++ restatement of the reference step), the only CPU implementation
# of the path that runs here (the reference needs Eigen and Boost).

def batch_cpu_sample(scenes):
    """Every 4th mesh of the batch (a bounded, size-representative sample)."""
    return scenes[::4]


def cpu_batch_steps(scenes, steps):
    """`steps` steps of every sampled mesh, one mesh per task on ceil(0.5 * cores) host threads."""
    import numpy as np
    from oracle import oracle as O

    models = [O.OracleModel.from_scene(s) for s in scenes]
    threads = host_threads()
    t0 = time.perf_counter()
    O.step_many(models, 1e-3, steps, threads)
    sec = time.perf_counter() - t0
    tets = sum(s.mesh.num_tets for s in scenes)
    split = np.sum([m.last_step_times() for m in models], axis=0)
    return tets * steps / sec, sec, threads, phase_split(split, "CPU seconds of the last step summed over the meshes")


def phase_split(t3, how):
    """The CPU step by part, as the oracle times it."""
    tot = float(sum(t3))
    names = ("element_and_assembly", "system_bc_rhs", "pcg")
    return {"seconds": {k: float(v) for k, v in zip(names, t3)},
            "share": {k: (float(v) / tot if tot > 0 else 0.0) for k, v in zip(names, t3)}, "how": how}


def cpu_single_steps(scene, steps):
    import numpy as np
    from oracle import oracle as O

    model = O.OracleModel.from_scene(scene)
    t_total = 0.0
    split = np.zeros(3)
    for s in range(steps):
        if scene.driven_dofs is not None:
            x, v = model.state()
            v[scene.driven_dofs] = scene.driven_values(s)
            model.set_state(None, v)
        t0 = time.perf_counter()
        model.step(scene.dt)
        t_total += time.perf_counter() - t0
        split += model.last_step_times()
    return scene.mesh.num_tets * steps / t_total, t_total, phase_split(split, f"seconds over {steps} step(s)")


def run_reference(args, rank, world):
    """Reference arm: the CPU implementation of the path on the host cores, bounded samples."""
    from oracle import oracle as O

    if rank != 0:
        return None
    O.build()
    if args.config == "batch":
        scenes = batch_cpu_sample(batch_scenes(args.meshes))
        from oracle import oracle as O2

        models = [O2.OracleModel.from_scene(s) for s in scenes]
        threads = host_threads()
        tets = sum(s.mesh.num_tets for s in scenes)
        O2.step_many(models, 1e-3, max(0, args.warmup), threads)
        times = []
        budget_s = float(os.environ.get("GBFEM_REFERENCE_BUDGET_S", "150"))
        while len(times) < args.steps and sum(times) < budget_s:
            t0 = time.perf_counter()
            O2.step_many(models, 1e-3, 1, threads)
            times.append(time.perf_counter() - t0)
        value = tets * len(times) / sum(times)
        sample = (f"every 4th mesh of the 256-mesh batch ({len(scenes)} meshes, {tets} tets), {len(times)} timed "
                  f"step(s), one mesh per task on {threads} host threads; oracle FP64 C++ restatement, -O3")
        cores, workload = threads, "batch256 (every 4th mesh)"
        ms = 1e3 * sum(times) / len(times)
        split = phase_split([sum(m.last_step_times()[i] for m in models) for i in range(3)],
                            "CPU seconds of the last step summed over the meshes")
    else:
        scene = build_scene(args.config, args.bar_h)
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

        for _ in range(max(0, args.warmup)):
            one()
        times = []
        parts = [0.0, 0.0, 0.0]
        while len(times) < args.steps and sum(times) < budget_s:
            times.append(one())
            parts = [p + t for p, t in zip(parts, model.last_step_times())]
        value = scene.mesh.num_tets * len(times) / sum(times)
        split = phase_split(parts, f"seconds over the {len(times)} timed step(s)")
        sample = (f"{len(times)} timed step(s) of the same scene, capped at {budget_s:.0f} s; oracle FP64 C++ "
                  "restatement, -O3, 1 thread (a representation is single-threaded)")
        cores, workload = 1, args.config
        ms = 1e3 * sum(times) / len(times)
    metric, unit = (HEX_METRIC, HEX_UNIT) if args.config == "hex" else (METRIC, UNIT)
    return {
        "metric": metric, "value": value, "unit": unit, "n_gpus": world, "steps": len(times),
        "warmup": max(0, args.warmup), "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded cube-grid meshes)",
        "config": {"workload": workload, "precision": "fp64"},
        "impl": "reference",
        "cpu_baseline": {"value": value, "unit": unit, "cores": cores, "threads": cores, "kind": "port",
                         "sample": sample, "phase_split": split, "host": host_info()},
        "e2e": {"value": value, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="batch", choices=["batch", "bar", "cube", "hex", "adjoint", "adjoint-batch"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"],
                    help="bar and cube only; the batch is always mixed precision")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-compare", action="store_true", help="skip the plain FP64 path comparison (batch)")
    ap.add_argument("--cg-schedule", default="auto", choices=["auto", "two-phase", "one-phase"],
                    help="mixed form: run the persistent solve in this CG schedule instead of the autotuner's")
    ap.add_argument("--meshes", type=int, default=BATCH["count"], help="batch size (smaller cases for profiling)")
    ap.add_argument("--bar-h", type=float, default=None,
                    help=f"bar cube edge in m (default {BAR_H_WINDOW} for a step window, {BAR_H_FULL} for the whole run)")
    args = ap.parse_args()
    rank, world, local = dist_env()
    if args.impl == "reference":
        line = run_reference(args, rank, world)
        if rank == 0:
            print(json.dumps(line), flush=True)
        return
    if args.config in ("adjoint", "adjoint-batch"):
        if rank == 0:
            fn = run_adjoint if args.config == "adjoint" else run_adjoint_batch
            print(json.dumps(fn(args, local)), flush=True)
        return
    dist = Dist(world)
    if args.config == "batch":
        line, scenes = run_batch(args, rank, world, local, dist)
    elif args.config == "bar" and args.steps >= BAR_SCENARIO_STEPS:
        line, scene = run_bar_full(args, rank, world, local, dist)
    else:
        line, scene = run_single(args, rank, world, local, dist)
    if rank == 0:
        if args.config == "batch" and not args.no_compare and world == 1:
            meshes = [s.mesh for s in scenes]
            log("plain FP64 path on the same meshes, one handle per mesh")
            fp64 = fp64_path_comparison(meshes, local)
            line["fp64_path"] = fp64
            line["speedup_vs_fp64_path"] = line["value"] / (fp64["value"] * world)
            log("plain FP64 form batched, and the mixed-vs-FP64 error over the whole scenario")
            tun = line["config"]["tuning"]
            fb, err = fp64_batch_and_error(meshes, local, args.steps, args.warmup,
                                           (tun["elements_per_block"], tun["ctas_per_sm"], tun["refresh_weight"],
                                            {v: k for k, v in SCHEDULE_NAMES.items()}[tun["cg_schedule"]]))
            line["fp64_batched"] = fb
            line["rel_disp_err_vs_fp64"] = err
            line["speedup_split"] = {
                "batching": fb["value"] / fp64["value"], "precision": line["value"] / fb["value"],
                "total": line["value"] / fp64["value"],
                "how": ("batching = FP64 batched / FP64 one handle per mesh; precision = mixed batched / FP64 "
                        "batched; total = their product")}
            log(f"fp64 path {fp64['value'] / 1e6:.1f} M, fp64 batched {fb['value'] / 1e6:.1f} M tet-steps/s; "
                f"speed-up {line['speedup_vs_fp64_path']:.2f} (batching {line['speedup_split']['batching']:.2f} x "
                f"precision {line['speedup_split']['precision']:.2f}); max rel disp err {err['max']:.2e} over "
                f"{ERROR_RUN_STEPS} steps")
        if world == 1 and not args.no_cpu_baseline:
            from oracle import oracle as O

            O.build()
            log("cpu baseline: oracle on the host")
            if args.config == "batch":
                sample = batch_cpu_sample(scenes)
                v, t, threads, split = cpu_batch_steps(sample, 1)
                line["cpu_baseline"] = {
                    "value": v, "unit": UNIT, "cores": threads, "threads": threads, "kind": "port",
                    "host": host_info(),
                    "sample": (f"1 step of every 4th mesh of the batch ({len(sample)} meshes, "
                               f"{sum(s.mesh.num_tets for s in sample)} tets) in {t:.1f} s, one mesh per task on "
                               f"{threads} host threads; oracle FP64 C++ restatement, -O3"),
                    "phase_split": split}
            else:
                v, t, split = cpu_single_steps(scene, 1)
                line["cpu_baseline"] = {"value": v, "unit": line["unit"], "cores": 1, "threads": 1, "kind": "port",
                                        "host": host_info(),
                                        "sample": f"1 step of the same scene on the host ({t:.1f} s), oracle FP64 "
                                                  "C++ restatement, -O3, 1 thread", "phase_split": split}
            log(f"cpu baseline: {v / 1e3:.1f} k tet-steps/s")
        print(json.dumps(line), flush=True)
    dist.close()


if __name__ == "__main__":
    main()
