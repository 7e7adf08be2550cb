#!/usr/bin/env python
"""Benchmark of the SPH sub-step on one GB300: particle-updates/s.

Workload (default): the 1,048,576-particle double dambreak — two 64x128x64
lattice blocks at spacing 2r (r = 0.0025, h = 4r) at opposite corners of the
box [0,1]^3, jittered by U(+-0.1 spacing) from seed 20171; rest density 1000,
k = 50 (p = k (rho - rho0)), viscosity 0.01, gravity -9.8, dt = 1e-4.

Printed JSON line (rank 0):
  value      particle-updates/s with the state resident in HBM: N x K / the
             summed device time (CUDA events on the solver's stream) of K
             graph-replayed sub-steps; a 256 MiB buffer is overwritten before
             every step, outside the timed intervals, so each step starts with
             a cold L2.
  e2e        the same metric through the C ABI with host buffers: per step
             sf_set_state (pinned host AoS pos+vel -> device) + sf_advance_frame
             + sf_get_state (device -> pinned host), wall clock; parts_ms
             gives each call's own time (synchronised, medians of 10).
  roofline   the dominant kernel's algorithmic bytes per launch / its average
             launch time (CUDA events between stages over K profiled steps),
             against the measured HBM copy bandwidth.
  cpu_baseline  the CPU oracle (the reference's solver cannot be built: its
             SPH library is not part of the reference) on the host cores.

``--impl reference`` times that CPU implementation as the reference arm.
``--only adjoint`` runs the differentiable section alone and prints its record,
and ``--only batched`` advances the batched-cube workload for --batch-steps
steps (default 10) with the default kernel choices (no autotuning, no
per-scene comparison): commands to profile; they do not print the bench line.
``--tuning L,D,F,P,W`` sets the headline solver's kernel choices (sf_tuning:
list mode, density and force block sizes, gather batch, L2 window) instead of
the defaults, and ``--pre-steps N`` measures from the state N sub-steps on.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import platform
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-updates/s at 1M (1 GB300); batched vs per-scene; adjoint/forward time"
UNIT = "particle-updates/s"
FLUSH_BYTES = 256 << 20  # > 129 MB L2

# Algorithmic (compulsory) bytes per particle of each stage: vec3 = 12 B,
# scalar = 4 B, neighbour reads counted once.  Scan stages are per cell.
STAGE_BYTES_PER_PARTICLE = {
    "density": 12 + 8,                       # read pos; write rho, p
    "force_integrate": 12 + 12 + 8 + 12 + 12 + 8,  # read pos, vel, (p, 1/rho); write pos, vel, key+slot
    "scatter": 8 + 4 + 4,                    # read key+slot, cell start; write index
    "rank_gather": 8 + 8 + 24 + 24,          # read key, cell range; read pos+vel; write pos+vel
}
STAGE_BYTES_PER_CELL = {"scan": 4 + 4}  # read the cell histogram, write the cell table
# Adjoint force pass (k_adj_forces) per particle: read its own step record
# (x, p | v, 1/rho) 32, adjoint record (apb | avb) 32, (p, 1/rho) 8, rho 4 and
# list count 4; write (x, rho_bar), (x_bar, k_bar) and v_bar 48.
ADJ_FORCES_BYTES_PER_PARTICLE = 32 + 32 + 8 + 4 + 4 + 48
STEP_BYTES_PER_UPDATE = 213  # canonical whole-step figure (hash 20 + sort 16 + reorder 48 + cells 5 + density 20 + force 44 + integrate 60)

# single-scene workloads, batch and adjoint: simplefluid_gb300/workloads/*.json
from simplefluid_gb300 import configs  # noqa: E402

WORKLOADS = configs.available("scene")


def measured_peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons while running."""

    QUERY = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []
        self.t = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            time.sleep(0.3)
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            if self.t:
                self.t.join(timeout=2)

    def summary(self) -> dict:
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx = float(f[1])
            except ValueError:
                continue
            for nm, v in zip(names, f[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        loaded = [x for x in sm if x >= 0.5 * (mx or max(sm))] or sm
        return {"sm_mhz": statistics.median(loaded), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def make_params(workload: str):
    return configs.params(workload)


def host_cpu() -> dict:
    """The host the CPU baselines ran on: architecture, CPU model and logical CPUs."""
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                model = line.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    if model is None:
        try:
            with open("/proc/cpuinfo") as f:
                for line in f:
                    if line.lower().startswith("model name"):
                        model = line.split(":", 1)[1].strip()
                        break
        except OSError:
            pass
    return {"machine": platform.machine(), "cpu_model": model, "logical_cpus": os.cpu_count()}


def cpu_oracle_rate(pos: np.ndarray, prm, budget_s: float, max_steps: int, warmup: int = 1):
    """Oracle sub-steps on the host cores: (updates/s, steps timed, threads)."""
    from oracle import oracle as O
    O.build()
    st = O.State(pos)
    cp = prm.to_c()
    if warmup:
        st.step(cp, warmup)
    steps, t0 = 0, time.perf_counter()
    while steps < max_steps:
        st.step(cp, 1)
        steps += 1
        if time.perf_counter() - t0 >= budget_s:
            break
    dt = time.perf_counter() - t0
    return pos.shape[0] * steps / dt, steps, O.max_threads()


def measure_batched(args, dist=None, rank: int = 0, ws: int = 1) -> dict:
    """Batched cubes: 256 scenes (counts log-uniform in [2000, 65536], seed
    20171) advanced together, one graph launch per step, in the configuration
    the autotuner chooses (grid granularity, and either the five launches'
    kernel variants or the persistent step's cluster and block size).  Beside
    it, on the same clock (wall time between synchronisations, the same steps
    from the same state): the five-launch step and the persistent step with
    each cluster and block size, every scene stepped on its own context one
    after another, and all those contexts interleaved on their own streams.
    With several ranks the scenes are spread over them (largest first, no
    communication) and each throughput is all ranks' particle-updates over the
    slowest rank's time."""
    from simplefluid_gb300 import SPHBatch, SPHParameters, SPHSolver, batch_cubes, shard_batch
    from simplefluid_gb300 import _capi as C
    cfg = configs.load("batched_cubes")
    steps = args.batch_steps if args.batch_steps else cfg["steps"]
    params, counts, pos = batch_cubes(cfg["seed"], cfg["scenes"], configs.params(cfg))
    total_scenes = len(params)
    if ws > 1:
        params, counts, pos, _ = shard_batch(params, counts, pos, rank, ws)
    n = int(counts.sum())

    def rate(run) -> float:
        """All ranks' particle-updates of `steps` steps over the slowest rank's
        wall-clock time of run() (synchronised on both sides)."""
        t0 = time.perf_counter()
        run()
        t_s, u = aggregate_over_ranks(dist, time.perf_counter() - t0, n * steps)
        return u / t_s

    variants = {}
    with SPHBatch(params) as b:
        b.setState(counts, pos)
        b.step(3)
        t0 = time.perf_counter()
        tune, K, _ = b.autotune(5)
        tune_s = time.perf_counter() - t0
        snap = b.getState()

        def timed(t):
            b.setTuning(t)
            b.setState(counts, *snap)
            b.step(3)
            b.synchronize()

            def run():
                b.step(steps)
                b.synchronize()
            return rate(run)

        chosen = C.sf_tuning()
        ctypes.memmove(ctypes.byref(chosen), ctypes.byref(tune), ctypes.sizeof(tune))
        batched = timed(chosen)
        variants["five_launches"] = timed(C.sf_tuning(C.SF_LIST_TILE, 128, 128, 2, 0, 0, 0))
        for cl in (4, 8):
            for bb in (256, 1024):
                variants[f"persistent_cluster{cl}_block{bb}"] = timed(
                    C.sf_tuning(C.SF_LIST_TILE, 256, 128, 2, 0, cl, bb))
        # the chosen configuration again, for the device-time figure
        b.setTuning(chosen)
        b.setState(counts, *snap)
        b.step(3)
        b.synchronize()
        dev_ms = b.timedSteps(steps)
    off = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    ctxs = []
    try:
        for s in range(len(params)):
            pp = SPHParameters.from_c(params[s])
            pp.cellsPerH = K
            c = SPHSolver(pp)
            c.setParticles(snap[0][off[s]:off[s + 1]], snap[1][off[s]:off[s + 1]])
            c.makeReady()
            ctxs.append(c)
        for c in ctxs:
            c.step(3)
        for c in ctxs:
            c.synchronize()

        def sequential():
            for c in ctxs:
                c.step(steps)
                c.synchronize()

        def interleaved():
            for _ in range(steps):
                for c in ctxs:
                    c.step(1)
            for c in ctxs:
                c.synchronize()
        seq = rate(sequential)
        rr = rate(interleaved)
    finally:
        for c in ctxs:
            c.close()
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        # the CPU oracle over the scenes one after another, on a sample of them
        ups = secs = 0.0
        threads = 1
        sample = range(0, len(params), 32)
        for s in sample:
            pp = SPHParameters.from_c(params[s])
            pp.cellsPerH = K
            rate_s, st, threads = cpu_oracle_rate(pos[off[s]:off[s + 1]], pp, args.cpu_seconds / 8, 20)
            ups += (off[s + 1] - off[s]) * st
            secs += (off[s + 1] - off[s]) * st / rate_s
        cpu = {"value": ups / secs, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"scenes {list(sample)} one after another, up to 20 sub-steps each (after 1 warm-up)"}
    dev_t, units = aggregate_over_ranks(dist, dev_ms, n * steps)
    return {"value": batched, "unit": UNIT, "scenes": total_scenes, "particles": units // steps, "steps": steps,
            "ranks": ws,
            "sequential_value": seq, "ratio_vs_sequential": batched / seq, "interleaved_streams_value": rr,
            "ratio_vs_interleaved_streams": batched / rr, "variants": variants,
            "device_time_value": units / (dev_t * 1e-3),
            "cpu_baseline": cpu,
            "autotuned": {"cells_per_h": K, "list_mode": tune.list_mode, "density_block": tune.density_block,
                          "force_block": tune.force_block, "prefetch": tune.prefetch,
                          "batch_cluster": tune.batch_cluster, "batch_block": tune.batch_block,
                          "seconds": tune_s},
            "timing": "value, variants, sequential and interleaved: wall clock between synchronisations over the "
                      "same steps from the same state; device_time_value: CUDA events over the chosen "
                      "configuration's graph-replayed steps"}


def profile_batched(args) -> dict:
    """The batched-cube workload alone: upload, 3 warm-up steps, then
    --batch-steps steps (default 10) with the default kernel choices; device
    time by CUDA events.  A command to profile the batched kernels."""
    from simplefluid_gb300 import SPHBatch, batch_cubes
    cfg = configs.load("batched_cubes")
    steps = args.batch_steps or 10
    params, counts, pos = batch_cubes(cfg["seed"], cfg["scenes"], configs.params(cfg))
    with SPHBatch(params) as b:
        if args.tuning:
            from simplefluid_gb300 import _capi as C
            b.setTuning(C.sf_tuning(*[int(x) for x in args.tuning.split(",")]))
        b.setState(counts, pos)
        b.step(3)
        b.synchronize()
        ms = b.timedSteps(steps)
    n = int(counts.sum())
    return {"scenes": len(params), "particles": n, "steps": steps, "ms_per_step": ms / steps,
            "value": n * steps / (ms * 1e-3), "unit": UNIT, "tuning": args.tuning}


def measure_adjoint(args) -> dict:
    """Differentiable dambreak: 65,536 particles, 200 steps, checkpoints every 20;
    loss = squared distance of the 32^3 CIC histogram to a seeded target.  Reports
    the plain forward (graph replays, CUDA events), the forward with checkpoints,
    the loss and the adjoint (wall clock, synchronised), and adjoint / forward."""
    from simplefluid_gb300 import SPHSolver, scene_positions
    cfg = configs.load("adjoint_64k")
    prm = configs.params(cfg)
    pos = scene_positions(prm, prm.scene, cfg["seed"])
    rng = np.random.default_rng(cfg["seed"])
    vel = rng.normal(scale=cfg["initial_velocity_sigma"], size=pos.shape).astype(np.float32)
    target = rng.uniform(size=cfg["histogram_resolution"] ** 3)
    target = (target / target.sum()).astype(np.float32)
    steps, ckpt = cfg["steps"], cfg["checkpoint_every"]
    from simplefluid_gb300 import _capi as C
    lib = C.load()
    with SPHSolver(prm) as s:
        s.setParticles(pos, vel)
        s.makeReady()
        s.step(3)
        s.setParticles(pos, vel)
        ms = ctypes.c_float()
        C.check(lib.sf_step_timed(s.handle, steps, 0, ctypes.byref(ms), None))
        fwd_ms = ms.value
        best = None
        for _ in range(3):
            s.setParticles(pos, vel)
            s.synchronize()
            t0 = time.perf_counter()
            s.forward(steps, ckpt)
            s.synchronize()
            t1 = time.perf_counter()
            L, dldx = s.lossHistogram(target)
            t2 = time.perf_counter()
            _, dv0, dmu, dk = s.adjoint(dldx)
            t3 = time.perf_counter()
            cur = ((t1 - t0) * 1e3, (t2 - t1) * 1e3, (t3 - t2) * 1e3)
            best = cur if best is None or cur[2] < best[2] else best
        # per-pass device times of the reverse sweep (one segment, CUDA events)
        npass = lib.sf_adjoint_pass_count()
        pass_ms = np.zeros(npass, np.float32)
        seg_steps = ctypes.c_uint32()
        C.check(lib.sf_adjoint_profile(s.handle, pass_ms.ctypes.data_as(ctypes.c_void_p), npass,
                                       ctypes.byref(seg_steps)))
    passes = {lib.sf_adjoint_pass_name(p).decode(): float(pass_ms[p]) / seg_steps.value for p in range(npass)}
    n = int(pos.shape[0])
    fbytes = ADJ_FORCES_BYTES_PER_PARTICLE * n
    avg = passes["adj_forces"]
    peaks = measured_peaks()
    achieved = fbytes / (avg * 1e-3) / 1e9
    roof = {"bound": "hbm", "kernel": "k_adj_forces", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
            "frac": achieved / peaks["hbm_gbs"], "algorithmic_bytes_per_launch": fbytes, "avg_launch_ms": avg,
            "peak_source": peaks["source"],
            "note": ("not HBM-bound: 65,536 particles fill about 13 warps per SM; ncu shows 35% issue-active at "
                     "9.2 cycles per instruction (about 7,000 instructions per warp)")}
    return {"particles": int(pos.shape[0]), "steps": steps, "ckpt_every": ckpt, "forward_ms": fwd_ms,
            "forward_with_checkpoints_ms": best[0], "loss_ms": best[1], "adjoint_ms": best[2],
            "ratio_adjoint_over_forward": best[2] / fwd_ms, "loss": float(L),
            "dloss_dviscosity": float(dmu), "dloss_dstiffness": float(dk),
            "passes_ms_per_step": passes, "roofline": roof,
            "timing": "forward: CUDA events over graph-replayed steps; others: wall clock, best of 3, "
                      "adjoint includes the checkpointed forward recompute"}


def measure_frames_and_render(args) -> dict:
    """The reference's frame loop and renderer, each beside the CPU oracle:
    whole 1/30 s frames with the adaptive sub-step on the device (one graph
    launch per frame, 16,000-particle dambreak), and the sphere-impostor
    image of the 1M double dambreak at 1280 x 720 (splat + shade on the
    device, outputs left in device memory)."""
    from oracle import oracle as O
    from simplefluid_gb300 import SPHSolver, render_params, scene_positions
    from simplefluid_gb300 import _capi as C
    lib = C.load()
    out = {}
    prm = make_params("dambreak_16k")
    prm.adaptiveTimeStep = True
    pos = scene_positions(prm, prm.scene)
    frames = 10
    with SPHSolver(prm) as s:
        s.setParticles(pos)
        s.makeReady()
        s.advanceFrames(1)
        s.setParticles(pos)
        t0 = time.perf_counter()
        _, sub = s.advanceFrames(frames)
        gpu_s = time.perf_counter() - t0
    rec = {"particles": int(pos.shape[0]), "frames": frames, "substeps": int(sub),
           "frames_per_s": frames / gpu_s, "timing": "wall clock, synchronised"}
    if not args.no_cpu_baseline:
        O.build()
        st = O.State(pos)
        t0 = time.perf_counter()
        _, csub, _ = st.frames(prm.to_c(), 1)
        rec["cpu_baseline"] = {"frames_per_s": 1.0 / (time.perf_counter() - t0), "substeps": int(csub),
                               "cores": O.max_threads(), "kind": "port", "sample": "the first frame"}
    out["frames_16k_adaptive"] = rec

    prm = make_params("double_dambreak_1m")
    pos = scene_positions(prm, prm.scene)
    rp = render_params(width=1280, height=720, eye=(0.5, 1.3, 2.6), focus=(0.5, 0.3, 0.5))
    with SPHSolver(prm) as s:
        s.setParticles(pos)
        for _ in range(3):
            C.check(lib.sf_render(s.handle, ctypes.byref(rp), None, None, None))
        s.synchronize()
        reps = 20
        t0 = time.perf_counter()
        for _ in range(reps):
            C.check(lib.sf_render(s.handle, ctypes.byref(rp), None, None, None))
        s.synchronize()
        ms = (time.perf_counter() - t0) * 1e3 / reps
    rec = {"particles": int(pos.shape[0]), "pixels": [1280, 720], "ms_per_image": ms,
           "timing": "wall clock over 20 images, synchronised"}
    if not args.no_cpu_baseline:
        t0 = time.perf_counter()
        O.render(prm.to_c(), rp, pos)
        rec["cpu_baseline"] = {"ms_per_image": (time.perf_counter() - t0) * 1e3, "cores": O.max_threads(),
                               "kind": "port", "sample": "one image"}
    out["render_1m_1280x720"] = rec
    return out


def measure_other_workloads(args, skip: str) -> dict:
    """The other single-scene workloads on the GPU (graph-replayed sub-steps,
    CUDA events, L2 flushed before every step) beside the CPU oracle on the
    host cores (a time-bounded sample from the initial state)."""
    from simplefluid_gb300 import SPHSolver, scene_positions
    from simplefluid_gb300 import _capi as C
    lib = C.load()
    plan = {wl: configs.load(wl)["steps"] for wl in ("dambreak_16k", "sphere_pool")}
    out = {}
    for wl, steps in plan.items():
        if wl == skip:
            continue
        prm = make_params(wl)
        pos = scene_positions(prm, prm.scene)
        n = int(pos.shape[0])
        with SPHSolver(prm) as s:
            s.setParticles(pos)
            s.makeReady()
            s.step(3)
            s.setParticles(pos)
            ms = ctypes.c_float()
            C.check(lib.sf_step_timed(s.handle, steps, FLUSH_BYTES, ctypes.byref(ms), None))
        rec = {"particles": n, "steps": steps, "value": n * steps / (ms.value * 1e-3), "unit": UNIT,
               "ms_per_step": ms.value / steps}
        if not args.no_cpu_baseline:
            rate, csteps, threads = cpu_oracle_rate(pos, prm, args.cpu_seconds / 3, steps)
            rec["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
                                   "sample": f"{csteps} sub-steps from the initial state (after 1 warm-up)"}
        out[wl] = rec
    return out


def aggregate_over_ranks(dist, local_ms: float, local_units: int):
    """Whole-job timing of replicas: the slowest rank's time and the units all
    ranks processed (weak scaling: every rank runs its own copy of the
    workload).  `dist` is torch.distributed (initialised) or None."""
    if dist is None:
        return local_ms, local_units
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([local_ms], dtype=torch.float64, device=dev)
    u = torch.tensor([float(local_units)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(t.item()), int(round(float(u.item())))


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    return ws, int(os.environ.get("RANK", "0")), int(os.environ.get("LOCAL_RANK", "0"))


def workload_config(workload: str, prm, n: int, grid, ws: int) -> dict:
    """The `config` object of both arms' lines (the same keys and values)."""
    return {"workload": workload, "particles": int(n), "kernel_radius": prm.kernelRadius,
            "particle_radius": prm.particleRadius, "dt": prm.timeStep, "grid": [int(g) for g in grid],
            "parallelism": f"replicas{ws}" if ws > 1 else "single",
            "l2": "flushed before every timed GPU step (256 MiB write outside the timed intervals); "
                  "the state (0.4 GB at 1M particles) exceeds the 129 MB L2"}


def run_reference(args, workload):
    """The reference arm: the CPU restatement of the SPH step (the reference's
    own solver library is not part of the reference tree), on all host
    threads, over the same workload, warm-up and step count as the GPU arm.
    Its input comes from the oracle's scene generator, which reproduces the
    reference's Source/SceneManager.cpp bit for bit; nothing of the product
    library is loaded."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    from oracle import oracle as O
    O.build()
    cfg = configs.load(workload)
    prm = make_params(workload)
    cp = prm.to_c()
    pos = O.scene(cp, prm.scene, cfg["seed"])
    d = O.derive(cp)
    grid = (d["nx"], d["ny"], d["nz"])
    budget = min(240.0, max(10.0, 1.0 * args.steps))
    rate, steps, threads = cpu_oracle_rate(pos, prm, budget, args.steps, warmup=args.warmup)
    sample = (f"{steps} of {args.steps} sub-steps of the {pos.shape[0]}-particle {workload} "
              f"(after {args.warmup} warm-up), time-bounded at {budget:.0f} s")
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": args.gpus, "steps": steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * pos.shape[0] / rate, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded scene generator: jittered lattice blocks, seed 20171)",
        "config": workload_config(workload, prm, pos.shape[0], grid, ws),
        "gpu_launches": 0,
        "cpu_baseline": {"value": rate, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample,
                         "note": "CPU restatement (reference TBB solver library unavailable: not in the reference tree)",
                         "host": host_cpu()},
        "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args, workload):
    ws, rank, local_rank = dist_env()
    from simplefluid_gb300 import SPHSolver, scene_positions
    from simplefluid_gb300 import _capi as C
    lib = C.load()
    C.check(lib.sf_select_device(local_rank))
    prm = make_params(workload)
    pos = scene_positions(prm, prm.scene, configs.load(workload)["seed"])
    n = pos.shape[0]
    solver = SPHSolver(prm)
    if args.tuning:
        t = C.sf_tuning(*[int(x) for x in args.tuning.split(",")])
        C.check(lib.sf_set_tuning(solver.handle, ctypes.byref(t)))
    solver.setParticles(pos)
    solver.makeReady()
    ctx = solver.handle

    dist = None
    if ws > 1:
        import torch
        import torch.distributed as dist_mod
        torch.cuda.set_device(local_rank)
        dist_mod.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        dist = dist_mod

    def barrier():
        if dist is not None:
            dist.barrier()

    def max_over_ranks(x: float) -> float:
        return aggregate_over_ranks(dist, x, 0)[0]

    # later states of the workload (--pre-steps), then the warm-up; the state
    # after it starts each of the three passes below
    if args.pre_steps:
        C.check(lib.sf_step(ctx, args.pre_steps))
    C.check(lib.sf_step(ctx, max(args.warmup, 3)))
    solver.synchronize()
    snap_pos, snap_vel = solver.getState()

    # headline: K graph-replayed sub-steps, cold L2 before each, device time
    total_ms = ctypes.c_float()
    step_ms = np.zeros(args.steps, np.float32)
    barrier()
    with ClockSampler(local_rank) as clk:
        C.check(lib.sf_step_timed(ctx, args.steps, FLUSH_BYTES, ctypes.byref(total_ms),
                                  step_ms.ctypes.data_as(ctypes.c_void_p)))
        # warm-L2 variant over the same steps, back-to-back (informational)
        solver.setParticles(snap_pos, snap_vel)
        warm_ms = ctypes.c_float()
        C.check(lib.sf_step_timed(ctx, args.steps, 0, ctypes.byref(warm_ms), None))
    barrier()
    t_ms, units = aggregate_over_ranks(dist, total_ms.value, n * args.steps)
    value = units / (t_ms * 1e-3)

    # per-stage device times over the same K steps, profiled (non-graph)
    solver.setParticles(snap_pos, snap_vel)
    nst = lib.sf_stage_count()
    stage_ms = np.zeros(nst, np.float32)
    C.check(lib.sf_profile_steps(ctx, args.steps, FLUSH_BYTES, stage_ms.ctypes.data_as(ctypes.c_void_p), nst))
    names = [lib.sf_stage_name(i).decode() for i in range(nst)]
    avg_ms = {nm: float(stage_ms[i]) / args.steps for i, nm in enumerate(names)}
    dom = max(avg_ms, key=avg_ms.get)
    nx, ny, nz = solver.gridDims()
    ncells = nx * ny * nz
    if dom in STAGE_BYTES_PER_PARTICLE:
        bytes_per_launch = STAGE_BYTES_PER_PARTICLE[dom] * n
    else:
        bytes_per_launch = STAGE_BYTES_PER_CELL.get(dom, 0) * ncells
    peaks = measured_peaks()
    achieved = bytes_per_launch / (avg_ms[dom] * 1e-3) / 1e9
    # DRAM traffic and issue figures of one ncu capture of the same kernel
    # (profiles/ncu_figures.json; per launch, step 7 of this workload)
    traffic, ncu_fig = None, {}
    tpath = os.path.join(ROOT, "profiles", "ncu_figures.json")
    if os.path.exists(tpath):
        with open(tpath) as f:
            ncu_fig = json.load(f).get(workload, {}).get(dom, {})
        traffic = ncu_fig.get("traffic_bytes")

    # e2e through the C ABI with pinned host buffers
    nbytes = n * 3 * 4
    hp, hv = ctypes.c_void_p(), ctypes.c_void_p()
    C.check(lib.sf_host_alloc(nbytes, ctypes.byref(hp)))
    C.check(lib.sf_host_alloc(nbytes, ctypes.byref(hv)))
    pos_h = np.ctypeslib.as_array((ctypes.c_float * (3 * n)).from_address(hp.value)).reshape(n, 3)
    vel_h = np.ctypeslib.as_array((ctypes.c_float * (3 * n)).from_address(hv.value)).reshape(n, 3)
    pos_h[:] = snap_pos  # the same trajectory as the passes above (after its warm-up steps)
    vel_h[:] = snap_vel
    dtv = ctypes.c_float()
    e2e_steps = args.steps
    for _ in range(max(args.warmup, 3)):
        C.check(lib.sf_set_state(ctx, hp, hv, n))
        C.check(lib.sf_advance_frame(ctx, ctypes.byref(dtv)))
        C.check(lib.sf_get_state(ctx, hp, hv, n))
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        C.check(lib.sf_set_state(ctx, hp, hv, n))
        C.check(lib.sf_advance_frame(ctx, ctypes.byref(dtv)))
        C.check(lib.sf_get_state(ctx, hp, hv, n))
    e2e_s = max_over_ranks(time.perf_counter() - t0)
    barrier()
    finite = bool(np.isfinite(pos_h).all() and np.isfinite(vel_h).all())
    # where an end-to-end step's time goes: each call on its own, synchronised
    # (medians of 10; the upload returns when its copies end, its sort after)
    parts = {"set_state_return": [], "set_state": [], "advance_frame": [], "get_state": []}
    for _ in range(10):
        t1 = time.perf_counter()
        C.check(lib.sf_set_state(ctx, hp, hv, n))
        t2 = time.perf_counter()
        C.check(lib.sf_synchronize(ctx))
        t3 = time.perf_counter()
        C.check(lib.sf_advance_frame(ctx, ctypes.byref(dtv)))
        C.check(lib.sf_synchronize(ctx))
        t4 = time.perf_counter()
        C.check(lib.sf_get_state(ctx, hp, hv, n))
        t5 = time.perf_counter()
        for k, dt_ in (("set_state_return", t2 - t1), ("set_state", t3 - t1), ("advance_frame", t4 - t3),
                       ("get_state", t5 - t4)):
            parts[k].append(dt_ * 1e3)
    e2e_parts = {k: statistics.median(v) for k, v in parts.items()}
    lib.sf_host_free(hp)
    lib.sf_host_free(hv)
    e2e_value = ws * n * e2e_steps / e2e_s

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        rate, steps, threads = cpu_oracle_rate(pos, prm, args.cpu_seconds, 200)
        cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{steps} sub-steps of the {n}-particle {workload} from its initial state (after 1 warm-up), "
                         f"CPU oracle with {threads} OpenMP threads; reference TBB solver library unavailable",
               "host": host_cpu()}

    solver.close()
    batched = measure_batched(args, dist, rank, ws) if not args.no_batched else None
    adjoint = measure_adjoint(args) if (rank == 0 and not args.no_adjoint) else None
    others = measure_other_workloads(args, workload) if (rank == 0 and not args.no_other_workloads) else None
    if others is not None:
        others.update(measure_frames_and_render(args))
    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return
    kernels_per_step = nst
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded scene generator: jittered lattice blocks, seed 20171)",
        "config": workload_config(workload, prm, n, (nx, ny, nz), ws),
        "value_warm_l2": ws * n * args.steps / (max_over_ranks(warm_ms.value) * 1e-3),
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": achieved / peaks["hbm_gbs"], "traffic": traffic,
                     "peak_source": peaks["source"], "algorithmic_bytes_per_launch": bytes_per_launch,
                     "avg_launch_ms": avg_ms[dom],
                     "step_frac": STEP_BYTES_PER_UPDATE * value / 1e9 / peaks["hbm_gbs"],
                     "ncu": {k: ncu_fig[k] for k in ("issue_active_pct", "ipc", "warps_active_pct",
                                                     "long_scoreboard_per_issue") if k in ncu_fig},
                     "note": ("bound by instruction issue, not HBM (ncu issue-active above)"
                              if ncu_fig.get("issue_active_pct", 0) >= 70 else
                              "bound by the latency of dependent loads, not HBM bandwidth (ncu above)")},
        "stages_ms": avg_ms,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 2 * nbytes, "d2h_bytes_per_step": 2 * nbytes,
                "path": "sf_set_state(pinned host) + sf_advance_frame + sf_get_state(pinned host)",
                "state_finite": finite, "parts_ms": e2e_parts},
        "gpu_launches": kernels_per_step * args.steps,
        "tuning": args.tuning,
        "pre_steps": args.pre_steps,
        "clocks": clk.summary(),
        "cpu_baseline": cpu,
        "batched": batched,
        "adjoint": adjoint,
        "other_workloads": others,
    }
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="double_dambreak_1m")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-other-workloads", action="store_true")
    ap.add_argument("--batch-steps", type=int, default=0, help="default: the batched_cubes configuration's steps")
    ap.add_argument("--only", choices=["adjoint", "batched"], default=None,
                    help="run one section alone and print its record (for profiling); not the bench line")
    ap.add_argument("--pre-steps", type=int, default=0,
                    help="advance the headline workload this many sub-steps before the warm-up (later states)")
    ap.add_argument("--tuning", default=None,
                    help="kernel choices: list_mode,density_block,force_block,prefetch,l2_window"
                         "[,batch_cluster,batch_block]")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.only == "adjoint":
        print(json.dumps({"section": "adjoint", **measure_adjoint(args)}), flush=True)
    elif args.only == "batched":
        print(json.dumps({"section": "batched", **profile_batched(args)}), flush=True)
    elif args.impl == "reference":
        run_reference(args, args.workload)
    else:
        run_ours(args, args.workload)


if __name__ == "__main__":
    main()
