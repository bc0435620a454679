#!/usr/bin/env python
"""Benchmark: 1M-particle 3-D PBF dam break, steps/s on one GB300.

Workload: 128 x 128 x 64 = 1,048,576 fluid particles, lattice spacing h/2
(h = 0.1), jitter U(-0.01h, 0.01h), in the corner of a 4:1 box; poly6 /
spiky kernels, 4 Jacobi iterations with the neighbour grid rebuilt every
iteration, s_corr k = 0.1 n = 4 dq = 0.2h, XSPH c = 0.01, dt = 1/120, FP32.
Synthetic seeded data (the reference publishes no dataset or numbers).

One "step" is one full pbd update (prediction, 4 x (grid build, lambda,
fused delta + walls), velocity, XSPH), replayed from a captured CUDA graph.
Steps are timed one by one with CUDA events on the launching stream; L2 is
flushed (256 MiB write) before each timed step, outside the timed span.

--impl reference times the reference path on the host cores: the oracle
(the FP64 C restatement of the reference step, all host threads) on the
same workload -- the reference's own GPU code does not build on CUDA 13 and
its CPU solver is 2-D and O(N^2).

Under torchrun (N > 1) every rank runs its own replica of the scene (the
single-scene step has no independent partition), and value is the total
steps/s over all replicas ("scaling": "weak").
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "1M-particle PBF steps/s: plain vs batched/adjoint, same GPU, <=1e-5 proj err"
UNIT = "steps/s"

LIST_ASSEMBLY = {0: "row chunks in shared memory", 1: "row chunks in global memory"}

# Algorithmic bytes (compulsory FP32 traffic, each array touched once per pass)
B_LAMBDA = 20      # read x* 16 + write lambda 4, per particle
B_DELTA = 36       # read x* 16 + read lambda_i 4 + write x 16, per particle
B_STEP_FIXED = 189  # predict 48 + grid 77 + finalize 64
B_ITER = 56        # lambda + delta


def dist_env():
    return int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")), \
        int(os.environ.get("LOCAL_RANK", "0"))


def max_over_ranks(seconds: float, world: int, device=None) -> float:
    """The slowest rank's time: the job ends when it does (replicas run
    independently, so this is the only cross-rank exchange)."""
    if world <= 1:
        return seconds
    import torch
    import torch.distributed as dist

    t = torch.tensor([seconds], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_rank: float, world: int, seconds: float) -> float:
    """Whole-job units per second: every rank's units over the slowest
    rank's time (weak scaling: per-rank work is fixed)."""
    return world * units_per_rank / seconds


def read_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def fp32_peak_gflops(stream) -> float | None:
    """FP32 FMA throughput of this GPU (GFLOP/s) from the benchmark's probe
    library (bench_fp32_peak.cu, built beside the product library)."""
    import ctypes

    from particlesolver_gb300 import _build

    try:
        lib = ctypes.CDLL(str(_build.build_probe()))
    except Exception:
        return None
    g = ctypes.c_double()
    fn = lib.fp32_peak_gflops
    fn.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.c_void_p]
    fn.restype = ctypes.c_int
    return g.value if fn(ctypes.byref(g), stream) == 0 else None


def read_traffic():
    p = ROOT / "profiles" / "ncu_traffic.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except Exception:
            return None
    return None


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.file = None

    def __enter__(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.file, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.proc or not self.file:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        rows = []
        for line in Path(self.file.name).read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append(dict(sm=float(parts[1]), smax=float(parts[2]), power=float(parts[3]),
                                 hw=parts[5], hwt=parts[6], swt=parts[7], pcap=parts[8]))
            except ValueError:
                continue
        os.unlink(self.file.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        reasons = set()
        for r in rows:
            for key, name in (("hw", "hw_slowdown"), ("hwt", "hw_thermal_slowdown"),
                              ("swt", "sw_thermal_slowdown"), ("pcap", "sw_power_cap")):
                if r[key].lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(r["sm"] for r in rows), "sm_max_mhz": max(r["smax"] for r in rows),
                "power_w_max": max(r["power"] for r in rows), "samples": len(rows), "reasons": sorted(reasons)}


def cpu_baseline_sample(scene, threads: int):
    """One oracle update of the full workload on the host cores."""
    from oracle import Oracle
    from particlesolver_gb300 import default_params
    from particlesolver_gb300 import workloads as W

    o = Oracle(default_params(**scene.params), scene.n, threads=threads)
    W.apply_to(scene, o)
    t0 = time.perf_counter()
    o.update(scene.dt)
    return time.perf_counter() - t0


def workload_config(args, sc) -> dict:
    """The workload keys both arms report (identical by construction)."""
    return {"workload": f"pbf_dam_break_{sc.n}", "particles": sc.n, "lattice": [args.nx, args.ny, args.nz],
            "h": sc.params["kernel_radius"], "iterations": sc.params["iterations"],
            "grid_rebuild": "every iteration", "xsph_c": sc.params["xsph_c"], "dt": sc.dt,
            "l2": "GPU arm: flushed before each timed step (256 MiB write); host arm: n/a"}


def density_invariant(pos, sc, after_steps: int, sample_size: int = 20000):
    """rho / rho0 - 1 over a seeded sample of particles (rho = poly6 sum
    within h, the particle itself included, FP64 on the host): mean
    compression (mean of the positive part), mean signed error, largest."""
    import numpy as np

    try:
        from scipy.spatial import cKDTree
    except ImportError:
        return None
    xs = np.asarray(pos, np.float64)[:, :3]
    n = len(xs)
    sample = np.random.default_rng(7).choice(n, min(n, sample_size), replace=False)
    h = sc.params["kernel_radius"]
    c6 = 315.0 / (64.0 * np.pi * h ** 9)
    nbrs = cKDTree(xs).query_ball_point(xs[sample], r=h)
    rho = np.array([np.sum(c6 * np.clip(h * h - np.sum((xs[q] - xs[i]) ** 2, 1), 0.0, None) ** 3)
                    for i, q in zip(sample, nbrs)])
    err = rho / np.asarray(sc.rest_density, np.float64)[sample] - 1.0
    return {"mean_compression_pct": round(100.0 * float(np.mean(np.clip(err, 0.0, None))), 3),
            "mean_signed_pct": round(100.0 * float(np.mean(err)), 3),
            "max_pct": round(100.0 * float(np.max(err)), 2),
            "after_steps": after_steps, "sample": int(len(sample))}


def run_reference(args, world, rank):
    if rank != 0:
        return
    from particlesolver_gb300 import workloads as W

    sc = W.dam_break(args.nx, args.ny, args.nz, cell_div=args.cell_div)
    threads = os.cpu_count() or 1
    from oracle import Oracle
    from particlesolver_gb300 import host_params

    # the same parameters as the GPU arm's default_params(**sc.params),
    # without loading the CUDA library
    o = Oracle(host_params(**sc.params), sc.n, threads=threads)
    W.apply_to(sc, o)
    budget = args.ref_budget_s
    t_start = time.perf_counter()
    warm = max(3, args.warmup)
    for _ in range(warm):
        o.update(sc.dt)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        o.update(sc.dt)
        times.append(time.perf_counter() - t0)
        if time.perf_counter() - t_start > budget:
            break
    v = len(times) / sum(times)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world,
            "steps": len(times), "warmup": warm, "ms_per_step": 1e3 * sum(times) / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded dam break, splitmix64)",
            "config": workload_config(args, sc),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{len(times)} full oracle updates of the {sc.n}-particle dam break "
                                       f"(the reference GPU path does not build on CUDA 13; its CPU path is "
                                       f"2-D O(N^2)); steps capped by a {budget:.0f} s budget"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def load_scenes(scenes, max_particles=None):
    """All scenes in one system, scene k from slot sum(n_0 .. n_(k-1))."""
    from particlesolver_gb300 import ParticleSystem, default_params
    from particlesolver_gb300 import workloads as W

    total = sum(sc.n for sc in scenes)
    sysm = ParticleSystem(default_params(**scenes[0].params), max_particles or total)
    for k, sc in enumerate(scenes):
        if k:
            sysm.begin_scene(default_params(**sc.params))
        first = sysm.num_particles
        W.apply_to(W.Scene(sc.name, sc.params, sc.pos_w, sc.phase, vel=sc.vel, rest_density=sc.rest_density,
                           pairs=None if sc.pairs is None else sc.pairs + first, rest=sc.rest,
                           stiffness=sc.stiffness, pins=None if sc.pins is None else sc.pins + first,
                           pin_points=sc.pin_points, bodies=[(f + first, c, st) for f, c, st in sc.bodies],
                           open_gas=[(f + first, c) for f, c in sc.open_gas], sdf=sc.sdf), sysm)
    return sysm


def run_batched(args, dev, stream, flush):
    """Batched scenes (512 PBF blocks / granular columns, log-uniform 1k-64k
    particles): one system stepping every scene with one launch per stage,
    replayed from a CUDA graph, against the plain per-scene solver (one
    system per scene, stepped one after another on the same stream)."""
    import torch

    from particlesolver_gb300 import ParticleSystem, default_params
    from particlesolver_gb300 import workloads as W

    scenes = W.batched_scenes(args.batch_scenes)
    S = len(scenes)
    total = sum(sc.n for sc in scenes)
    dt = 1.0 / 60.0
    sh = stream.cuda_stream
    batch = load_scenes(scenes)
    for _ in range(3):
        batch.update(dt, sh)
    batch.autotune(dt, 2, sh)
    batch.update_graph(dt, 1, sh)
    torch.cuda.synchronize()
    K = args.batch_steps
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    batch.reset_profile()
    with torch.cuda.stream(stream):
        for a, b in ev:
            flush.zero_()
            a.record(stream)
            batch.update_graph(dt, 1, sh)
            b.record(stream)
    torch.cuda.synchronize()
    t_batch = sum(a.elapsed_time(b) for a, b in ev) / 1e3
    launches = batch.profile()["kernel_launches"]
    tun = batch.tuning()
    tuning = {"threads_per_particle": int(tun.threads_per_particle), "neighbor_skin": round(float(tun.neighbor_skin), 4),
              "neighbor_list_capacity": int(tun.neighbor_list_capacity),
              "list_assembly": LIST_ASSEMBLY.get(int(tun.list_assembly), str(int(tun.list_assembly))),
              "list_reuses_last_step": batch.list_reuses()}
    batch.check_finite(sh)
    del batch

    singles = []
    for sc in scenes:
        sy = ParticleSystem(default_params(**sc.params), sc.n)
        W.apply_to(sc, sy)
        singles.append(sy)
    for sy in singles:
        sy.update(dt, sh)

    def per_scene(graph: bool, steps: int):
        for sy in singles:  # warm (and capture)
            sy.update_graph(dt, 1, sh) if graph else sy.update(dt, sh)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            flush.zero_()
            a.record(stream)
            for _ in range(steps):
                for sy in singles:
                    sy.update_graph(dt, 1, sh) if graph else sy.update(dt, sh)
            b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / 1e3

    k_single = max(1, min(K, args.batch_single_steps))
    t_eager = per_scene(False, k_single)
    t_graph = per_scene(True, k_single)
    for sy in singles:
        sy.close()
    kinds = [sc.name for sc in scenes]
    v_batch = S * K / t_batch
    v_eager = S * k_single / t_eager
    v_graph = S * k_single / t_graph
    return {"unit": "scenes*steps/s", "value": v_batch, "scenes": S, "particles": total,
            "pbf_blocks": kinds.count("pbf_block"), "granular_columns": kinds.count("granular_column"),
            "steps": K, "ms_per_step": 1e3 * t_batch / K, "gpu_launches": launches, "tuning": tuning,
            "per_scene_plain": {"value": v_eager, "steps": k_single, "ms_per_step": 1e3 * t_eager / k_single,
                                "how": "one system per scene, pbd_update each, same stream"},
            "per_scene_graph": {"value": v_graph, "steps": k_single, "ms_per_step": 1e3 * t_graph / k_single,
                                "how": "one system per scene, its own captured step graph"},
            "speedup_vs_plain": v_batch / v_eager, "speedup_vs_per_scene_graph": v_batch / v_graph,
            "dt": dt, "workload": f"{S} scenes, counts round(exp(U(ln 1024, ln 65536))), PBF block or 2-D "
                                  f"granular column by coin flip (seeded)"}


def time_scene(sc, stream, flush, steps, warmup=3):
    """Steps/s of one scene replayed from its CUDA graph (per-step events,
    L2 flushed before each step), with its per-stage times and launches."""
    import torch

    from particlesolver_gb300 import ParticleSystem, default_params
    from particlesolver_gb300 import workloads as W

    sh = stream.cuda_stream
    sysm = ParticleSystem(default_params(**sc.params), sc.n)
    W.apply_to(sc, sysm)
    for _ in range(warmup):
        sysm.update(sc.dt, sh)
    sysm.autotune(sc.dt, 2, sh)
    sysm.update_graph(sc.dt, 1, sh)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    sysm.reset_profile()
    with torch.cuda.stream(stream):
        for a, b in ev:
            flush.zero_()
            a.record(stream)
            sysm.update_graph(sc.dt, 1, sh)
            b.record(stream)
    torch.cuda.synchronize()
    t = sum(a.elapsed_time(b) for a, b in ev) / 1e3
    launches = sysm.profile()["kernel_launches"]
    sysm.set_profiling(True)
    sysm.reset_profile()
    for _ in range(3):
        sysm.update(sc.dt, sh)
    prof = sysm.profile()
    sysm.check_finite(sh)
    sysm.close()
    return {"value": steps / t, "unit": "steps/s", "ms_per_step": 1e3 * t / steps, "steps": steps,
            "particles": sc.n, "gpu_launches": launches,
            "stage_ms_per_step": {k: v / 3 for k, v in prof["stage_ms"].items() if v}}


def run_other_configs(args, stream, flush):
    """The mixed cloth / rope / rigid scene (833,536 particles) and the 2-D
    granular column (1,600 particles, 600-step runs in the reference), each
    on the GPU, the column also with the oracle on one host thread."""
    from particlesolver_gb300 import workloads as W

    out = {}
    mixed = W.mixed_scene()
    r = time_scene(mixed, stream, flush, args.other_steps)
    r.update(workload=f"mixed: 256x256 cloth (stretch/shear/bend, pinned edges), 2000 ropes x 64, 10000 random-pose "
                      f"4x4x4 shape-matched bodies; {mixed.info['constraints']} distance constraints, 4 iterations, "
                      f"dt 1/60")
    out["mixed_scene"] = r
    # the CPU sand-pile path: the CPU reference's contact and wall
    # projectors (PBD_FLAG_CPU_CONTACTS)
    col = W.granular_column(cpu_contacts=True)
    r = time_scene(col, stream, flush, args.other_steps)
    from oracle import Oracle, refcpu
    from particlesolver_gb300 import default_params

    o = Oracle(default_params(**col.params), col.n, threads=1)
    W.apply_to(col, o)
    t0 = time.perf_counter()
    k = 0
    while k < 600 and time.perf_counter() - t0 < 10.0:
        o.update(col.dt)
        k += 1
    cpu = k / (time.perf_counter() - t0)
    r.update(workload="2-D granular column: 40x40 lattice spacing 2r, jitter U(+-0.01r), mu_s 0.5, mu_k 0.3, "
                      "3 iterations, dt 1/60, the CPU reference's contact and wall projectors",
             cpu_oracle_1_thread={"value": cpu, "unit": "steps/s", "steps": k, "kind": "port"})
    # the reference's own 2-D CPU solver, where its sources were built on
    # this machine (oracle/_ref); single-threaded as written
    if refcpu.available():
        ref = refcpu.RefCPU(col.pos_w[:, :2], mass=1.0, s_friction=0.5, k_friction=0.3)
        t0 = time.perf_counter()
        k = 0
        while k < 600 and time.perf_counter() - t0 < 10.0:
            ref.tick(col.dt)
            k += 1
        r["cpu_reference_1_thread"] = {"value": k / (time.perf_counter() - t0), "unit": "steps/s", "steps": k,
                                       "kind": "reference"}
    else:
        r["cpu_reference_1_thread"] = {"unavailable": "the reference's CPU sources are not on this machine "
                                                      "(oracle/_ref not built)"}
    out["granular_2d"] = r
    return out


def run_adjoint(args, dev, stream):
    """Differentiation: 64 batched cloth / rope / grain scenes (4,552
    particles each), 120 steps of 1/60 with checkpoints every 10.  Times one
    forward rollout and one backward pass, then recovers the hidden
    per-constraint stiffness and initial velocities from the hidden run's
    final positions by Adam through the adjoint."""
    import numpy as np
    import torch

    from particlesolver_gb300 import workloads as W
    from particlesolver_gb300.autograd import fit, rollout

    scenes = W.differentiation_scenes(args.adjoint_scenes)
    sysm = load_scenes(scenes)
    n = sysm.num_particles
    m = sysm.num_distance_constraints
    dt, T, every = 1.0 / 60.0, args.adjoint_steps, 10
    cat = lambda key: np.concatenate([getattr(sc, key) for sc in scenes])  # noqa: E731

    x0 = torch.tensor(cat("pos_w"), device=dev)
    v_hidden = torch.tensor(cat("vel"), device=dev)
    s_hidden = torch.tensor(cat("stiffness"), device=dev)
    # on torch's current stream: the autograd engine runs the backward on
    # the stream of the forward, and timing is wall clock between device
    # synchronisations (the backward is a host-driven sequence of segments)
    with torch.no_grad():
        target, _ = rollout(sysm, s_hidden, x0, v_hidden, dt, T, every)
    s0 = torch.full((m,), 0.6, device=dev)
    v_init = torch.zeros_like(v_hidden)
    # warm-up forward + backward (first launches, work-array allocation)
    for _ in range(2):
        st = s0.clone().requires_grad_(True)
        v0 = v_init.clone().requires_grad_(True)
        xT, _ = rollout(sysm, st, x0, v0, dt, T, every)
        xT[:, :3].sum().backward()
    fwd, bwd = [], []
    for _ in range(3):
        st = s0.clone().requires_grad_(True)
        v0 = v_init.clone().requires_grad_(True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        xT, _ = rollout(sysm, st, x0, v0, dt, T, every)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        loss = ((xT[:, :3] - target[:, :3]) ** 2).sum(1).mean()
        loss.backward()
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        fwd.append(1e3 * (t1 - t0))
        bwd.append(1e3 * (t2 - t1))
    fwd_ms, bwd_ms = statistics.median(fwd), statistics.median(bwd)
    grains = torch.tensor(np.concatenate([sc.phase == 3 for sc in scenes]), device=dev)

    def errors(st, vv):
        return (float((st - s_hidden).abs().mean()), float((vv - v_hidden)[grains, :3].norm(dim=1).mean()))

    def loss_at(st, vv, steps, tgt):
        with torch.no_grad():
            xT, _ = rollout(sysm, st, x0, vv, dt, steps, every)
            return float(((xT[:, :3] - tgt[:, :3]) ** 2).sum(1).mean())

    # the hidden run's positions after a short horizon, for the curriculum
    T1 = min(30, T)
    with torch.no_grad():
        target1, _ = rollout(sysm, s_hidden, x0, v_hidden, dt, T1, every)
    # identifiability: how much the final positions change with stiffness
    # alone and with velocities alone (the other set at its hidden value)
    sens = {}
    for steps, tgt in ((T1, target1), (T, target)):
        sens[f"steps_{steps}"] = {"loss_stiffness_wrong": loss_at(s0, v_hidden, steps, tgt),
                                  "loss_velocities_wrong": loss_at(s_hidden, v_init, steps, tgt),
                                  "loss_both_wrong": loss_at(s0, v_init, steps, tgt)}
    base = {"scenes": len(scenes), "particles": n, "constraints": m, "steps": T, "checkpoint_every": every,
            "dt": dt, "forward_ms": fwd_ms, "backward_ms": bwd_ms,
            "timing": "wall clock between device synchronisations, median of 3 after 2 warm-up passes",
            "backward_over_forward": bwd_ms / fwd_ms, "particle_steps_per_s_fwd_bwd": n * T / ((fwd_ms + bwd_ms) * 1e-3),
            "workload": f"{len(scenes)} scenes of a 64x64 cloth (stretch, pinned edges) + 8 ropes x 32 + 200 "
                        f"grains, hidden stiffness U(0.2, 1) and grain velocities; fit from stiffness 0.6 and "
                        f"zero velocities by Adam through the adjoint, on the hidden run's positions after "
                        f"{T1} steps, then after {T}"}
    e0 = errors(s0, v_init)
    base["start"] = {"stiffness_mae": e0[0], "grain_velocity_err": e0[1], "loss": sens[f"steps_{T}"]["loss_both_wrong"]}
    if args.adjoint_iters <= 0:  # timing only: no recovery
        return {**base, "sensitivity": sens}
    t0 = time.perf_counter()
    # recovery by a horizon curriculum: both parameter sets fitted to the
    # hidden run's positions after T1 steps, then after T
    st1, v1, losses1 = fit(sysm, x0, target1, s0, v_init, dt, T1, every, 2 * args.adjoint_iters, 0.02, 0.05)
    st2, v2, losses2 = fit(sysm, x0, target, st1, v1, dt, T, every, args.adjoint_iters, 0.01, 0.005)
    torch.cuda.synchronize()
    fit_s = time.perf_counter() - t0
    # stiffness alone, from the hidden velocities, on the final positions
    st3, _, losses3 = fit(sysm, x0, target, s0, v_hidden, dt, T, every, args.adjoint_iters, 0.02, 0.0)
    e1, e2, e3 = errors(st1, v1), errors(st2, v2), errors(st3, v_hidden)
    return {**base,
            "curriculum": [
                {"steps": T1, "iterations": len(losses1), "loss_first": losses1[0], "loss_last": losses1[-1],
                 "stiffness_mae": e1[0], "grain_velocity_err": e1[1], f"loss_at_{T}": loss_at(st1, v1, T, target)},
                {"steps": T, "iterations": len(losses2), "loss_first": losses2[0], "loss_last": losses2[-1],
                 "stiffness_mae": e2[0], "grain_velocity_err": e2[1]}],
            "fit_s": fit_s,
            "stiffness_only_from_hidden_velocities": {"steps": T, "iterations": len(losses3),
                                                      "loss_first": losses3[0], "loss_last": losses3[-1],
                                                      "stiffness_mae_start": e0[0], "stiffness_mae_end": e3[0]},
            "sensitivity": sens}


def run_ours(args, world, rank, local_rank):
    import numpy as np
    import torch

    from particlesolver_gb300 import ParticleSystem, default_params
    from particlesolver_gb300 import workloads as W

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    sc = W.dam_break(args.nx, args.ny, args.nz, cell_div=args.cell_div)
    n = sc.n
    sysm = ParticleSystem(default_params(**sc.params), n)
    W.apply_to(sc, sysm)
    stream = torch.cuda.Stream(device=dev)
    sh = stream.cuda_stream
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def barrier():
        if world > 1:
            import torch.distributed as dist

            dist.barrier()

    # warm-up, then the lanes-per-particle choice (autotuned on the warmed-up
    # state unless --tpp fixes it), then the step graph capture
    warm = max(3, args.warmup)
    if args.tpp:
        sysm.set_threads_per_particle(args.tpp)
    for _ in range(warm):
        sysm.update(sc.dt, sh)
    if not args.tpp:
        sysm.autotune(sc.dt, 2, sh)
    tpp = sysm.threads_per_particle
    tuning = sysm.tuning()
    held = sysm.get_params()  # cell size and grid after the autotuner
    sysm.update_graph(sc.dt, 1, sh)
    torch.cuda.synchronize()
    # the end-to-end run below restarts from this state, so that both
    # numbers cover the same steps of the flow
    state0 = sysm.save_state()

    # ---- timed region: K steps, L2 flushed before each, device events
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    sysm.reset_profile()
    barrier()
    torch.cuda.synchronize()
    t_wall0 = time.perf_counter()
    with ClockSampler(local_rank) as clocks:
        with torch.cuda.stream(stream):
            for k in range(args.steps):
                flush.zero_()
                starts[k].record(stream)
                sysm.update_graph(sc.dt, 1, sh)
                ends[k].record(stream)
        torch.cuda.synchronize()
    barrier()
    wall = time.perf_counter() - t_wall0
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    total_s = sum(step_ms) / 1e3
    launches = sysm.profile()["kernel_launches"]
    total_s = max_over_ranks(total_s, world, dev)
    value = job_throughput(args.steps, world, total_s)

    # ---- density invariant after the timed steps: rho / rho0 - 1 over a
    # seeded sample of particles (rho = poly6 sum within h, FP64 on the host)
    density = density_invariant(sysm.positions(), sc, warm + 1 + args.steps)

    # ---- per-stage device times over the timed region's steps, replayed
    # eagerly (events between stage groups) from the same start state
    sysm.load_state(state0)
    sysm.set_profiling(True)
    sysm.reset_profile()
    prof_steps = args.steps
    for _ in range(prof_steps):
        flush.zero_()
        sysm.update(sc.dt, sh)
    prof = sysm.profile()
    sysm.set_profiling(False)

    # ---- end to end through the public API with host buffers: the caller
    # owns the state in pinned host memory; every step uploads positions and
    # velocities, runs the update and downloads both.  Same start state and
    # step count as the timed region.
    sysm.load_state(state0)
    pos_h = torch.empty((n, 4), dtype=torch.float32).pin_memory()
    vel_h = torch.empty((n, 4), dtype=torch.float32).pin_memory()
    lib = sysm.lib
    sysm._check(lib.pbd_get_positions_velocities(sysm.h, 0, n, pos_h.data_ptr(), vel_h.data_ptr(), 0, sh))
    e2e_steps = max(3, args.steps)
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        # the state goes up and comes back every step, positions and
        # velocities copied concurrently (pbd_set/get_positions_velocities)
        sysm._check(lib.pbd_set_positions_velocities(sysm.h, 0, n, pos_h.data_ptr(), vel_h.data_ptr(), 0, sh))
        sysm.update_graph(sc.dt, 1, sh)
        sysm._check(lib.pbd_get_positions_velocities(sysm.h, 0, n, pos_h.data_ptr(), vel_h.data_ptr(), 0, sh))
    e2e_s = max_over_ranks(time.perf_counter() - t0, world, dev)
    e2e_value = job_throughput(e2e_steps, world, e2e_s)
    sysm.check_finite(sh)
    reuses = sysm.list_reuses()

    # ---- a later window of the same flow: from the timed region's start
    # state, advance args.later_advance steps untimed, then time
    # args.later_steps steps as above (the column compresses and neighbour
    # lists lengthen as the flow develops, so steps get costlier)
    later = None
    if args.later_steps:
        sysm.load_state(state0)
        for _ in range(args.later_advance):
            sysm.update_graph(sc.dt, 1, sh)
        lev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(args.later_steps)]
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            for a, b in lev:
                flush.zero_()
                a.record(stream)
                sysm.update_graph(sc.dt, 1, sh)
                b.record(stream)
        torch.cuda.synchronize()
        later_s = max_over_ranks(sum(a.elapsed_time(b) for a, b in lev) / 1e3, world, dev)
        sysm.check_finite(sh)
        first = warm + 1 + args.later_advance
        later = {"value": job_throughput(args.later_steps, world, later_s), "unit": UNIT,
                 "ms_per_step": 1e3 * later_s / args.later_steps, "first_step": first + 1,
                 "steps": args.later_steps, "untimed_advance": args.later_advance,
                 "density_error": density_invariant(sysm.positions(), sc, first + args.later_steps)}
    batched = None
    if args.batch_scenes:
        sysm.close()
        batched = run_batched(args, dev, stream, flush)
    adjoint = run_adjoint(args, dev, stream) if args.adjoint_scenes else None
    others = run_other_configs(args, stream, flush) if args.other_steps else None

    if rank != 0:
        return

    # roofline of the dominant single-kernel stage
    per_launch = {}
    for st, b in (("lambda", B_LAMBDA), ("solve", B_DELTA)):
        nl = prof["stage_launches"][st]
        if nl:
            per_launch[st] = (prof["stage_ms"][st] / nl, b * n)
    dom = max(per_launch, key=lambda k: per_launch[k][0] * prof["stage_launches"][k])
    dom_ms, dom_bytes = per_launch[dom]
    peak, peak_kind = read_peaks()
    achieved = dom_bytes / (dom_ms * 1e-3) / 1e9
    traffic_tab = read_traffic()
    traffic = None
    if traffic_tab and dom in traffic_tab.get("per_launch_bytes", {}):
        traffic = traffic_tab["per_launch_bytes"][dom]
    step_bytes = (B_STEP_FIXED + 4 * B_ITER) * n
    ms_per_step = 1e3 * total_s / args.steps
    # FP32 beside HBM: the dominant kernel's FP32 flops per particle (an
    # ncu instruction mix carried over from an earlier capture, not
    # measured in this run) over its launch time here, against the FP32 FMA
    # throughput measured here by the benchmark's own probe
    fp32 = None
    flops_pp = (traffic_tab or {}).get("fp32_flops_per_particle", {}).get(dom)
    if flops_pp:
        peak32 = fp32_peak_gflops(sh)
        ach32 = flops_pp * n / (dom_ms * 1e-3) / 1e9
        fp32 = {"kernel": dom, "flops_per_particle": flops_pp, "achieved_gflops": ach32,
                "peak_gflops": peak32, "frac": ach32 / peak32 if peak32 else None,
                "peak_source": "measured in this run (FP32 FMA probe, bench_fp32_peak.cu)",
                "flops_source": "carried over: " + traffic_tab.get("fp32_source_short", "ncu instruction mix")}

    cpu = None
    if world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        dt_cpu = cpu_baseline_sample(sc, threads)
        cpu = {"value": 1.0 / dt_cpu, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"1 full oracle update (FP64 restatement of the reference step) of the {n}-particle "
                         f"dam break on {threads} host threads"}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": warm, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded dam break, splitmix64)",
        "config": workload_config(args, sc),
        "tuning": {"cell_size": round(float(held.cell_size), 6), "grid": list(held.grid_size),
                   "cell_source": "autotuned" if not args.tpp else "given",
                   "threads_per_particle": tpp, "tpp_source": "fixed" if args.tpp else "autotuned",
                   "neighbor_skin": float(tuning.neighbor_skin),
                   "neighbor_list_capacity": int(tuning.neighbor_list_capacity),
                   "list_assembly": LIST_ASSEMBLY.get(int(tuning.list_assembly), str(int(tuning.list_assembly))),
                   "list_reuses_last_step": reuses},
        "timing": {"how": "per-step CUDA events on the launching stream, CUDA graph replay",
                   "particle_iterations_per_s": value * n * 4,
                   "step_bytes_algorithmic": step_bytes,
                   "step_achieved_gbs": step_bytes / (ms_per_step * 1e-3) / 1e9,
                   "wall_s_timed_region": wall},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
                     "traffic_source": ("carried over, not measured in this run: " +
                                        (traffic_tab or {}).get("traffic_source_short", "ncu capture"))
                     if traffic is not None else None,
                     "bytes_per_launch": dom_bytes, "ms_per_launch": dom_ms},
        "fp32": fp32,
        # (stages that launched nothing are left out: with XSPH on, the
        # velocity update runs inside the XSPH stage)
        "stage_ms_per_step": {k: v / prof_steps for k, v in prof["stage_ms"].items()
                              if prof["stage_launches"][k]},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 2 * 16 * n, "d2h_bytes_per_step": 2 * 16 * n,
                "steps": e2e_steps},
        "gpu_launches": launches,
        "clocks": clocks.summary(),
        "cpu_baseline": cpu,
        "density_error": density,
        "later_window": later,
        "batched": batched,
        "adjoint": adjoint,
        "other_configs": others,
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--nx", type=int, default=128)
    ap.add_argument("--ny", type=int, default=128)
    ap.add_argument("--nz", type=int, default=64)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--tpp", type=int, default=0, help="lanes per particle (0 = autotune)")
    ap.add_argument("--cell-div", type=int, default=1, help="grid cell size = h / cell_div")
    ap.add_argument("--ref-budget-s", type=float, default=120.0)
    ap.add_argument("--later-advance", type=int, default=50, help="untimed steps before the later window")
    ap.add_argument("--later-steps", type=int, default=20, help="timed steps of the later window (0 = skip)")
    ap.add_argument("--batch-scenes", type=int, default=512, help="batched-scenes measurement (0 = skip)")
    ap.add_argument("--batch-steps", type=int, default=20)
    ap.add_argument("--batch-single-steps", type=int, default=3)
    ap.add_argument("--adjoint-scenes", type=int, default=64, help="differentiation measurement (0 = skip)")
    ap.add_argument("--adjoint-steps", type=int, default=120)
    ap.add_argument("--adjoint-iters", type=int, default=20)
    ap.add_argument("--other-steps", type=int, default=20, help="mixed scene / 2-D column measurement (0 = skip)")
    args = ap.parse_args()
    world, rank, local_rank = dist_env()
    if args.impl == "reference":
        run_reference(args, world, rank)
        return
    if world > 1:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl", init_method="env://")
    try:
        run_ours(args, world, rank, local_rank)
    finally:
        if world > 1:
            import torch.distributed as dist

            dist.destroy_process_group()


if __name__ == "__main__":
    main()
