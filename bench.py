#!/usr/bin/env python
"""Throughput benchmark of the PBF substep pipeline (particle-iterations/s).

Workload: the 1,048,576-particle dam break (position-based-fluids_gb300/
scenarios/dam_break_1m.par: a 128x64x128 block at spacing 0.05 with seeded
jitter in a 12.8 x 6.4 x 6.4 box, h = 0.1, 4 solver iterations).  One bench
step is one 1/60 s frame = 2 substeps of Simulation::Step.

  value  : particle-iterations/s = N * iterations * substeps / time, with the
           state resident in HBM; CUDA events on the library's stream around
           K frames (after W warm-up frames), max over ranks.
  e2e    : the same metric through the C-ABI with host buffers, over the same
           frames (replayed from the state the timed frames started from):
           every frame copies positions + velocities in from pinned host
           memory, steps, and copies them back out, the positions while the
           last substep's XSPH and vorticity run (wall clock).
  roofline: the dominant kernel's algorithmic bytes per launch over its
           average launch time (CUDA events between stages on the library's
           stream, in a separate pass of the same frames), against the
           measured HBM copy bandwidth.

--impl reference times the reference's own kernels on the host cores (its
OpenCL C compiled through a C++ shim, OpenMP over all cores; the CPU
restatement where they were not compiled) on the same scene instead.
Multi-GPU (torchrun): every rank advances its own replica of the scene;
value sums the particles of all ranks over the slowest rank's time.
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

REPO = Path(__file__).resolve().parent
PKG = REPO / "position-based-fluids_gb300"
for _p in (str(REPO), str(PKG)):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "particle-iterations/s at 1M particles (plain PBF substep pipeline)"
UNIT = "particle-iterations/s"
SCENE = "dam_break_1m"
FALLBACK_HBM_GBS = 6800.0

# Per-particle algorithmic bytes of one launch of each stage (compulsory
# reads and writes of the particle records, the keys and the neighbour list;
# neighbour records gathered through the caches are not counted).  `nl` / `nd`
# are the mean neighbour-list lengths of the density pass / the other passes.
STAGE_BYTES = {
    "predictPositions": lambda nl, nd, it=4: 72.0,
    "sortParticles": lambda nl, nd, it=4: 68.0,
    "updateCells": lambda nl, nd, it=4: 12.0,
    "buildFriendsList": lambda nl, nd, it=4: 20.0 + 4.0 * nl,
    "resetPartList": lambda nl, nd, it=4: 12.0,
    # per density pass: the friend entries read; the first pass of a substep
    # also writes them as flat rows for the passes after it (it = iterations)
    "computeScaling": lambda nl, nd, it=4: 40.0 + 4.0 * nl + 4.0 * nl / max(it, 1),
    "computeDelta": lambda nl, nd, it=4: 40.0 + 4.0 * nd,
    "updateVelocities": lambda nl, nd, it=4: 80.0,
    "applyViscosity": lambda nl, nd, it=4: 68.0 + 4.0 * nd,
    "applyVorticity": lambda nl, nd, it=4: 68.0 + 4.0 * nd,
}

# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) and warp
# instructions (smsp__inst_executed.sum) per launch, the mean over the four
# launches of each pass in one substep (for the density pass: the one that
# records the flat friend rows and three that read them), from ncu captures of
# the dam_break_1m scene in the first substep of frame 51 (256-thread blocks,
# plain thread map), with the mean list lengths of that substep (density pass
# nl, other passes nd).  Scaled to the measured list lengths: the traffic by
# the stage's algorithmic bytes, the instructions in proportion to the list
# length of the pass.
TRAFFIC_CAPTURE = {"computeScaling": {"bytes": 311.79e6, "nl": 38.88, "nd": 33.07},
                   "computeDelta": {"bytes": 219.73e6, "nl": 38.88, "nd": 33.07}}
ISSUE_CAPTURE = {"computeScaling": {"inst": 152.28e6, "nl": 38.88, "nd": 33.07},
                 "computeDelta": {"inst": 148.34e6, "nl": 38.88, "nd": 33.07}}
SM_COUNT = 152
SCHEDULERS_PER_SM = 4

CLOCK_FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")


def measured_peaks() -> tuple[float, str]:
    path = REPO / "MEASURED_PEAKS.json"
    try:
        return float(json.loads(path.read_text())["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    def __init__(self, device_index: int):
        self.device = device_index
        self.proc = None
        self.path = None
        self.out = None
        self._summary = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.out = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={CLOCK_FIELDS}", "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.out, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        deadline = time.time() + 3.0  # the first sample before the timed region starts
        while self.proc is not None and time.time() < deadline:
            try:
                if Path(self.path).stat().st_size > 0:
                    break
            except OSError:
                pass
            time.sleep(0.05)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        if self.out is not None:
            self.out.close()

    def summary(self) -> dict:
        if self._summary is None:
            self._summary = self._read()
        return self._summary

    def _read(self) -> dict:
        rows = []
        try:
            for line in Path(self.path).read_text().splitlines():
                f = [x.strip() for x in line.split(",")]
                if len(f) >= 9 and f[0] == str(self.device):
                    rows.append(f)
        except Exception:
            pass
        finally:
            try:
                os.unlink(self.path)
            except Exception:
                pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["clocks not sampled"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def stage_roofline(sim, n: int, iters: int, sub: int, frames: int, peak: float, peak_kind: str):
    """Per-stage device times of `frames` eager frames (events between
    stages) and the roofline of the dominant neighbour kernel: its
    algorithmic bytes per launch (with the current mean list lengths) over
    its mean launch time.  Returns (nl, nd, stage_ms, dominant, launch_ms,
    roofline dict)."""
    counts, _ = sim.read_friends(slots=1)
    nl, nd = float(counts[:, 0].mean()), float(counts[:, 1].mean())
    sim.enable_stage_timing(True)
    totals: dict[str, float] = {}
    for _ in range(frames):
        sim.Step(sub)
        for k, v in sim.stage_timings().items():
            totals[k] = totals.get(k, 0.0) + v
    sim.enable_stage_timing(False)
    per_frame_launches = {"computeScaling": iters * sub, "computeDelta": iters * sub}
    stage_ms = {k: v / frames for k, v in totals.items()}
    dominant = max((k for k in stage_ms if k in STAGE_BYTES), key=lambda k: stage_ms[k])
    launch_ms = stage_ms[dominant] / per_frame_launches.get(dominant, sub)
    algo_bytes = STAGE_BYTES[dominant](nl, nd, iters) * n
    achieved = algo_bytes / (launch_ms / 1000.0) / 1e9
    traffic = None
    if dominant in TRAFFIC_CAPTURE:
        cap = TRAFFIC_CAPTURE[dominant]
        traffic = cap["bytes"] * STAGE_BYTES[dominant](nl, nd, iters) / STAGE_BYTES[dominant](cap["nl"], cap["nd"], 4)
    roof = {"bound": "hbm", "kernel": dominant, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_source": peak_kind, "traffic": traffic,
            "algorithmic_bytes_per_launch": algo_bytes, "avg_launch_ms": launch_ms}
    return nl, nd, stage_ms, dominant, launch_ms, roof


def cpu_reference_sample(params, pos, vel, seconds: float, max_substeps: int | None = None,
                         warmup: int = 1) -> tuple[float, dict]:
    """Time the reference's CPU path on a bounded sample of the scene: the
    reference's own kernels through the OpenCL-C shim (oracle/_ref) on all host
    threads where they were compiled, else the CPU restatement (the oracle
    port, bit-identical to them).  `warmup` (at least 1) untimed substeps
    come first.  Returns (particle-iterations/s, the cpu_baseline fields kind /
    cores / sample / substeps / seconds / warmup)."""
    from oracle import oracle
    n, iters = int(params.particleCount), int(params.simIterations)
    w = max(1, int(warmup))
    if oracle.ref_available():
        try:
            # a w-substep run and a (w+k)-substep run from the same state:
            # their difference is k substeps after w warm-up substeps, and the
            # buffer setup of each run cancels
            t0 = time.perf_counter()
            oracle.ref_step(params, pos, vel, w, threads=0)
            tw = time.perf_counter() - t0
            threads = oracle.ref_max_threads()
            k = max(1, int(seconds / max(tw / w, 1e-3)))
            if max_substeps:
                k = min(k, max_substeps)
            t0 = time.perf_counter()
            oracle.ref_step(params, pos, vel, w + k, threads=0)
            el = max(time.perf_counter() - t0 - tw, 1e-9)
            return n * iters * k / el, {
                "kind": "reference", "cores": threads, "substeps": k, "seconds": el, "warmup": w,
                "sample": f"{k} substep(s) of the {n}-particle scene after {w} warm-up substep(s) from its initial "
                          f"state, through the reference's own kernels (OpenCL-C shim, work-items on {threads} "
                          f"threads): a {w + k}-substep run less a {w}-substep run, {el:.1f} s"}
        except (OSError, RuntimeError, FileNotFoundError):
            pass  # no compiler or no generated unit here: the restatement below
    threads = oracle.max_threads()
    p, v, _ = oracle.step(params, pos, vel, w, threads=threads)
    done, t0 = 0, time.perf_counter()
    while True:
        p, v, _ = oracle.step(params, p, v, 1, threads=threads)
        done += 1
        el = time.perf_counter() - t0
        if el >= seconds or (max_substeps and done >= max_substeps):
            break
    return n * iters * done / el, {
        "kind": "port", "cores": threads, "substeps": done, "seconds": el, "warmup": w,
        "sample": f"{done} substep(s) of the {n}-particle scene after {w} warm-up substep(s) from its initial "
                  f"state, through the CPU restatement, {el:.1f} s"}


def cpu_baseline(params, pos, vel, seconds: float) -> dict:
    """The reference's CPU path on a bounded sample of the scene."""
    value, info = cpu_reference_sample(params, pos, vel, seconds)
    return {"value": value, "unit": UNIT, "cores": info["cores"], "kind": info["kind"], "sample": info["sample"]}


def workload_name(scene: str, n: int, iters: int, sub: int) -> str:
    return (f"{scene}: {n} particles (128x64x128 block, spacing 0.05, seeded jitter) in a 12.8x6.4x6.4 box; "
            f"{iters} iterations x {sub} substeps per step (frame)")


def reference_arm(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import pbf
    params, pos, vel = pbf.make_scene(args.scene)
    n, iters = int(params.particleCount), int(params.simIterations)
    value, info = cpu_reference_sample(params, pos, vel, args.cpu_budget, max_substeps=args.steps,
                                       warmup=args.warmup)
    done, el = info["substeps"], info["seconds"]
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": done, "warmup": info["warmup"], "ms_per_step": 1000.0 * el / done,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": workload_name(args.scene, n, iters, int(params.subSteps)),
                   "reference_step": "one substep per timed step (a bounded sample of the frame)",
                   "particles": n, "iterations": iters, "threads": info["cores"]},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": info["cores"], "kind": info["kind"],
                         "sample": info["sample"] + f" (time budget {args.cpu_budget:.0f} s)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def replica_rate(units: float, seconds: float, dist=None, device: str = "cpu") -> tuple[float, float]:
    """Whole-job rate of replicas: the units of all ranks over the slowest
    rank's time.  Returns (rate, slowest seconds); without a process group,
    this rank's own."""
    import torch
    if dist is None:
        return units / seconds, seconds
    t = torch.tensor([seconds], dtype=torch.float64, device=device)
    u = torch.tensor([units], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(u.item()) / float(t.item()), float(t.item())


# The stage groups the per-stage times are also reported in: keys, sort,
# permutation and cell table / friend lists and the density pass / the
# position-correction pass / velocities, XSPH and vorticity.
STAGE_GROUPS = {
    "sort": ("predictPositions", "radixsort", "sortParticles", "updateCells", "resetPartList"),
    "friends+lambda": ("buildFriendsList", "computeScaling"),
    "delta_p": ("computeDelta", "packData"),
    "xsph+vorticity": ("updateVelocities", "applyViscosity", "applyVorticity"),
}


def gpu_arm(args) -> None:
    import numpy as np
    import torch
    import pbf

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    params, pos, vel = pbf.make_scene(args.scene)
    params.relaxedMath = 1 if args.math == "relaxed" else 0
    n, iters, sub = int(params.particleCount), int(params.simIterations), int(params.subSteps)
    sim = pbf.Simulation.create(params, pos, vel, device=local)
    stream = torch.cuda.ExternalStream(sim.stream(), device=torch.device("cuda", local))

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()

    for _ in range(args.warmup):
        sim.step_async(sub)
    sim.synchronize()
    blocks = sim.autotune(trial_substeps=2) if not args.no_autotune else sim.launch_shape()
    # the state the timed frames start from, for the end-to-end replay below
    h0pos = torch.empty((n, 4), dtype=torch.float32, pin_memory=True)
    h0vel = torch.empty((n, 4), dtype=torch.float32, pin_memory=True)
    sim.read_state_into(h0pos.data_ptr(), h0vel.data_ptr())

    # ---- timed region: K frames, state resident in HBM ----
    barrier()
    launches0 = sim.launch_count()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clocks:
        torch.cuda.nvtx.range_push("timed frames")  # lets a profiler capture exactly these launches
        ev0.record(stream)
        for _ in range(args.steps):
            sim.step_async(sub)
        ev1.record(stream)
        torch.cuda.nvtx.range_pop()
        ev1.synchronize()
    sim.synchronize()
    barrier()
    ms = ev0.elapsed_time(ev1)
    launches = sim.launch_count() - launches0
    value, ms = replica_rate(n * iters * sub * args.steps, ms / 1000.0, dist, "cuda")
    ms *= 1000.0

    # ---- end to end through the C-ABI with pinned host buffers ----
    # The same frames again: the state the timed frames started from is
    # uploaded and stepped frame by frame, so both numbers time the same work.
    end_pos = np.empty((n, 4), np.float32)
    end_vel = np.empty((n, 4), np.float32)
    sim.read_state_into(end_pos.ctypes.data, end_vel.ctypes.data)
    hpos = torch.empty((n, 4), dtype=torch.float32, pin_memory=True)
    hvel = torch.empty((n, 4), dtype=torch.float32, pin_memory=True)
    hpos.copy_(torch.from_numpy(end_pos))
    hvel.copy_(torch.from_numpy(end_vel))
    e2e_steps = max(1, min(args.steps, args.e2e_steps or args.steps))
    def e2e_frame():  # upload, step, download through the C-ABI; one wait per frame
        sim.write_state_async(hpos.data_ptr(), hvel.data_ptr())
        sim.step_read_async(sub, hpos.data_ptr(), hvel.data_ptr())  # positions copied during XSPH/vorticity
        sim.synchronize()

    for _ in range(3):  # warm-up frames beyond the timed ones
        e2e_frame()
    hpos.copy_(h0pos)
    hvel.copy_(h0vel)
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_frame()
    e2e_s = time.perf_counter() - t0
    e2e_value, _ = replica_rate(n * iters * sub * e2e_steps, e2e_s, dist, "cuda")
    # a full replay must end on the timed frames' final state, bit for bit
    e2e_replay_identical = None
    if e2e_steps == args.steps:
        e2e_replay_identical = bool(np.array_equal(hpos.numpy().view(np.uint32), end_pos.view(np.uint32)) and
                                    np.array_equal(hvel.numpy().view(np.uint32), end_vel.view(np.uint32)))

    # ---- density error of the state after the timed frames ----
    _, _, dpred = sim.read_state()
    rel = np.abs(dpred[:, 3].astype(np.float64) / float(params.restDensity) - 1.0)
    rel = rel[np.isfinite(rel)]
    density_error = {"mean": float(rel.mean()), "p95": float(np.percentile(rel, 95)), "max": float(rel.max()),
                     "note": "|rho / rho0 - 1| per particle, density of the last solver iteration"}

    # ---- per-stage device times (eager launches, events between stages) ----
    peak, peak_kind = measured_peaks()
    nl, nd, stage_ms, dominant, launch_ms, roof = stage_roofline(sim, n, iters, sub, max(1, min(args.steps, 20)),
                                                                 peak, peak_kind)
    issue = None
    if dominant in ISSUE_CAPTURE and args.math == "exact":
        cap = ISSUE_CAPTURE[dominant]
        inst = cap["inst"] * (nl / cap["nl"] if dominant == "computeScaling" else nd / cap["nd"])
        clk = clocks.summary().get("sm_mhz") or 2070.0
        peak_issue = SM_COUNT * SCHEDULERS_PER_SM * clk * 1e6
        issue = {"kernel": dominant, "warp_instructions_per_launch": inst,
                 "achieved": inst / (launch_ms / 1000.0), "peak": peak_issue, "unit": "warp instructions/s",
                 "frac": inst / (launch_ms / 1000.0) / peak_issue,
                 "source": "ncu smsp__inst_executed.sum of one launch in the first substep of frame 51 (256-thread "
                           "blocks, plain thread map, list length 38.88 / 33.07), scaled by list length"}
    # ---- the other arithmetic mode, same scene state, its own block sizes ----
    other_line = None
    if not args.no_other_mode:
        other = "exact" if args.math == "relaxed" else "relaxed"
        p2 = params.copy()
        p2.relaxedMath = 1 if other == "relaxed" else 0
        sim.set_params(p2)
        for _ in range(3):
            sim.step_async(sub)
        sim.synchronize()
        other_blocks = sim.autotune(trial_substeps=2) if not args.no_autotune else sim.launch_shape()
        barrier()
        o0, o1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        o0.record(stream)
        for _ in range(args.steps):
            sim.step_async(sub)
        o1.record(stream)
        o1.synchronize()
        other_ms = o0.elapsed_time(o1) / args.steps
        *_, other_stages, _, _, other_roof = stage_roofline(sim, n, iters, sub, max(1, min(args.steps, 10)), peak,
                                                            peak_kind)
        other_line = {"mode": other, "value": n * iters * sub / (other_ms / 1000.0), "ms_per_step": other_ms,
                      "blocks": dict(zip(["friends", "scaling", "delta", "viscosity", "vorticity", "friends_algorithm",
                                          "balance"], other_blocks)),
                      "roofline": other_roof,
                      "stage_ms_per_step": {k: round(v, 4) for k, v in sorted(other_stages.items(), key=lambda kv: -kv[1])}}
        sim.set_params(params)
        sim.set_launch_shape(blocks)

    frame_ms = ms / args.steps
    bytes_sub = (444.0 + 56.0 * iters) * n  # whole-substep compulsory bytes, P = 3 sort passes
    pipeline_gbs = bytes_sub * sub / (frame_ms / 1000.0) / 1e9

    if rank != 0:
        sim.close()
        if dist is not None:
            dist.destroy_process_group()
        return
    base = None
    if world == 1 and not args.no_cpu_baseline:
        base = cpu_baseline(params, pos, vel, args.cpu_seconds)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": frame_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": workload_name(args.scene, n, iters, sub),
                   "particles": n, "iterations": iters, "substeps_per_step": sub,
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                   "l2": "working set larger than L2 (no flush)", "mode": MODES[args.math],
                   "cuda_graph": True,
                   "blocks": dict(zip(["friends", "scaling", "delta", "viscosity", "vorticity", "friends_algorithm", "balance"], blocks))},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 32 * n, "d2h_bytes_per_step": 32 * n,
                "steps": e2e_steps, "frames": "the timed frames replayed from their start state",
                "replay_bit_identical": e2e_replay_identical},
        "gpu_launches": int(launches),
        "roofline": roof,
        "pipeline_roofline": {"bytes_per_particle_substep": 444.0 + 56.0 * iters, "achieved": pipeline_gbs,
                              "frac": pipeline_gbs / peak},
        **({"issue_roofline": issue} if issue else {}),
        "particle_substeps_per_s": value / iters,
        "stage_ms_per_step": {k: round(v, 4) for k, v in sorted(stage_ms.items(), key=lambda kv: -kv[1])},
        "stage_groups_ms_per_step": {g: round(sum(stage_ms.get(k, 0.0) for k in ks), 4) for g, ks in STAGE_GROUPS.items()},
        "neighbours": {"density_pass": nl, "other_passes": nd},
        "density_error": density_error,
        **({"other_mode": other_line} if other_line else {}),
        "clocks": clocks.summary(),
    }
    if base is not None:
        line["cpu_baseline"] = base
    print(json.dumps(line), flush=True)
    sim.close()
    if dist is not None:
        dist.destroy_process_group()
    if dist is not None:
        dist.destroy_process_group()


MODES = {
    "relaxed": "relaxedMath 1: the four neighbour passes in relaxed FP32 (one rsqrt per pair, FMA), as the "
               "reference's -cl-fast-relaxed-math build; one substep of positions within 1e-5 relative of the "
               "exact oracle, velocities within exact FP32's own error against FP64",
    "exact": "relaxedMath 0: strict IEEE FP32 in the reference's operation order, bit-identical to the oracle",
}


# Stage groups of the particle-count sweep.
SWEEP_GROUPS = {
    "sort": ["predictPositions", "radixsort", "sortParticles", "updateCells", "resetPartList"],
    "gather": ["buildFriendsList"],
    "constraint": ["computeScaling", "computeDelta"],
    "velocity": ["updateVelocities", "applyViscosity", "applyVorticity"],
}


def sweep(args) -> None:
    """Particle-count sweep on the double dam break: one JSON line per
    (particles, iterations) with stage-group times against HBM peak."""
    import torch
    import pbf
    peak, peak_kind = measured_peaks()
    counts = [int(x) for x in args.sweep_counts.split(",")]
    for n in counts:
        for iters in (2, 4, 8):
            params, pos, vel = pbf.make_double_dam_break(n, iterations=iters)
            sub = int(params.subSteps)
            sim = pbf.Simulation.create(params, pos, vel, device=0)
            stream = torch.cuda.ExternalStream(sim.stream())
            for _ in range(args.sweep_warmup):
                sim.step_async(sub)
            sim.synchronize()
            blocks = sim.autotune(trial_substeps=2) if not args.no_autotune else sim.launch_shape()
            ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            ev0.record(stream)
            for _ in range(args.sweep_steps):
                sim.step_async(sub)
            ev1.record(stream)
            ev1.synchronize()
            sim.synchronize()
            frame_ms = ev0.elapsed_time(ev1) / args.sweep_steps
            counts_, _ = sim.read_friends(slots=1)
            nl, nd = float(counts_[:, 0].mean()), float(counts_[:, 1].mean())
            sim.enable_stage_timing(True)
            totals: dict[str, float] = {}
            for _ in range(3):
                sim.Step(sub)
                for k, v in sim.stage_timings().items():
                    totals[k] = totals.get(k, 0.0) + v / 3.0
            sim.close()
            launches = {"computeScaling": iters * sub, "computeDelta": iters * sub}
            groups = {}
            for g, names in SWEEP_GROUPS.items():
                ms = sum(totals.get(k, 0.0) for k in names)
                byts = 0.0
                for k in names:
                    if k in STAGE_BYTES:
                        byts += STAGE_BYTES[k](nl, nd, iters) * n * launches.get(k, sub)
                    elif k == "radixsort":
                        byts += (16.0 * 3 + 4.0) * n * sub  # 3 passes of 8-bit digits
                groups[g] = {"ms_per_step": round(ms, 4), "gb_per_s": byts / (ms / 1e3) / 1e9 if ms else None,
                             "hbm_frac": (byts / (ms / 1e3) / 1e9) / peak if ms else None}
            line = {"sweep": "double_dam_break", "particles": n, "iterations": iters,
                    "value": n * iters * sub / (frame_ms / 1e3), "unit": UNIT, "ms_per_step": frame_ms,
                    "steps": args.sweep_steps, "warmup": args.sweep_warmup, "neighbours": {"density_pass": nl,
                    "other_passes": nd}, "groups": groups, "peak_gbs": peak, "peak_source": peak_kind,
                    "blocks": dict(zip(["friends", "scaling", "delta", "viscosity", "vorticity", "friends_algorithm",
                                        "balance"], blocks))}
            print(json.dumps(line), flush=True)


def batched(args) -> None:
    """256 independent dam breaks (pbf.make_batch_scenes) advanced together,
    each substep one CUDA graph over all scenes with autotuned block sizes;
    compared with the same scenes run one at a time on the plain path and
    with the single-scene 1M dam break."""
    import numpy as np
    import torch
    import pbf

    def rate(sim, n, frames, warm):
        sub = int(sim.params.subSteps)
        stream = torch.cuda.ExternalStream(sim.stream())
        for _ in range(warm):
            sim.step_async(sub)
        sim.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(frames):
            sim.step_async(sub)
        e1.record(stream)
        e1.synchronize()
        sim.synchronize()
        ms = e0.elapsed_time(e1) / frames
        return n * int(sim.params.simIterations) * sub / (ms / 1e3), ms

    scenes, positions = pbf.make_batch_scenes(count=args.batch_scenes)
    pos = np.concatenate(positions)
    total = int(pos.shape[0])
    sim = pbf.Simulation.create(scenes, pos, np.zeros_like(pos), device=0)
    for _ in range(args.warmup):
        sim.step_async(int(sim.params.subSteps))
    sim.synchronize()
    blocks = sim.autotune(trial_substeps=2)
    launches0 = sim.launch_count()
    batch_rate, batch_ms = rate(sim, total, args.steps, 0)
    launches = sim.launch_count() - launches0
    sim.close()
    seq_ms = 0.0
    for p, x in zip(scenes, positions):
        one = pbf.Simulation.create(p, x, np.zeros_like(x), device=0)
        _, ms = rate(one, int(p.particleCount), args.batch_seq_steps, 3)
        seq_ms += ms
        one.close()
    seq_rate = total * int(scenes[0].simIterations) * int(scenes[0].subSteps) / (seq_ms / 1e3)
    params, p1, v1 = pbf.make_scene(SCENE)
    single = pbf.Simulation.create(params, p1, v1, device=0)
    single_rate, _ = rate(single, int(params.particleCount), args.steps, args.warmup)
    single.close()
    line = {"batched": f"{len(scenes)} dam-break scenes", "particles": total, "value": batch_rate, "unit": UNIT,
            "ms_per_step": batch_ms, "steps": args.steps, "warmup": args.warmup, "gpu_launches": int(launches),
            "autotuned_blocks": dict(zip(["friends", "scaling", "delta", "viscosity", "vorticity", "friends_algorithm", "balance"], blocks)),
            "sequential_value": seq_rate, "ratio_vs_sequential": batch_rate / seq_rate,
            "single_scene_value": single_rate, "ratio_vs_single_scene": batch_rate / single_rate,
            "config": {"scenes": len(scenes), "counts": "log-uniform in [4096, 65536], seed 7",
                       "fill": 0.3, "tilt_deg": "U(0, 10)", "xsph_c": "U(0.005, 0.05)", "iterations": 4,
                       "substeps_per_step": 2, "cuda_graph": True}}
    print(json.dumps(line), flush=True)


def rollout(args) -> None:
    """Differentiable rollout: the 65,536-particle dam break (64x32x32
    block) for 60 frames of 2 substeps, checkpoints every 10 substeps.  Loss:
    MSE between the final positions and those of a target run with gravity
    tilted 5 degrees and XSPH c = 0.03.  Times pbf_rollout_forward and
    pbf_rollout_backward (which recomputes each segment from its checkpoint
    before running the adjoint kernels over it) with CUDA events on the
    simulation's stream, next to the plain path's 120 substeps."""
    import numpy as np
    import torch
    import pbf

    frames, every = args.rollout_frames, args.rollout_every
    params, pos, vel = pbf.make_rollout_scene(64, 32, 32)
    n = int(params.particleCount)
    substeps = frames * int(params.subSteps)
    tparams = pbf.rollout_target_params(params)
    with pbf.Simulation.create(tparams, pos, vel, device=0) as tsim:
        tsim.Step(substeps)
        target = tsim.positions_by_id().astype(np.float64)
    sim = pbf.Simulation.create(params, pos, vel, device=0)
    stream = torch.cuda.ExternalStream(sim.stream())

    def timed(fn):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        out = fn()
        e1.record(stream)
        e1.synchronize()
        return out, e0.elapsed_time(e1)

    def dl_dx(x):
        g = np.zeros((n, 4), np.float32)
        g[:, :3] = (2.0 * (x[:, :3].astype(np.float64) - target[:, :3]) / (3.0 * n)).astype(np.float32)
        return g

    fwd, bwd, plain = [], [], []
    launches = 0
    blocks = sim.launch_shape()
    for rep in range(args.warmup_rollouts + args.rollouts):
        sim.write_state(pos, vel)
        _, ms_plain = timed(lambda: sim.Step(substeps))
        sim.write_state(pos, vel)
        l0 = sim.launch_count()
        _, ms_f = timed(lambda: sim.rollout_forward(substeps, every))
        x = sim.positions_by_id()
        loss = float(np.mean((x[:, :3].astype(np.float64) - target[:, :3]) ** 2))
        g = dl_dx(x)
        (dv, dc, dg), ms_b = timed(lambda: sim.rollout_backward(g))
        if rep + 1 == args.warmup_rollouts and not args.no_autotune:
            blocks = sim.autotune(trial_substeps=4)
        if rep >= args.warmup_rollouts:
            fwd.append(ms_f)
            bwd.append(ms_b)
            plain.append(ms_plain)
            launches = sim.launch_count() - l0
    sim.close()
    f, bk, pl = float(np.median(fwd)), float(np.median(bwd)), float(np.median(plain))
    list_bytes = 4 * n * int(params.friendsCircles) * int(params.particlesPerCircle)
    tape_bytes = every * (4 * n + list_bytes + 8 * n + 16 * n * (int(params.simIterations) + 3)
                          + (n * int(params.simIterations) if params.boxClamp else 0))
    line = {"rollout": f"{n}-particle dam break (64x32x32), {frames} frames x {int(params.subSteps)} substeps",
            "metric": "backward / forward time", "value": bk / f, "higher_is_better": False,
            "forward_ms": f, "backward_ms": bk, "plain_steps_ms": pl,
            "forward_us_per_substep": 1e3 * f / substeps, "backward_us_per_substep": 1e3 * bk / substeps,
            "rollouts": args.rollouts, "warmup": args.warmup_rollouts, "gpu_launches": int(launches),
            "forward_blocks": dict(zip(["friends", "scaling", "delta", "viscosity", "vorticity", "friends_algorithm", "balance"], blocks)),
            "loss": loss, "grad_norms": {"v0": float(np.linalg.norm(dv[:, :3])), "c": float(dc),
                                         "g": [float(v) for v in dg]},
            "memory_bytes": {"tape_one_segment": tape_bytes, "checkpoints": (substeps // every + 1) * 36 * n},
            "dtype": "f32",
            "config": {"particles": n, "substeps": substeps, "checkpoint_every": every, "iterations":
                       int(params.simIterations), "target": "gravity tilted 5 deg, XSPH c = 0.03",
                       "gradients": "initial velocities, XSPH c, gravity vector"}}
    print(json.dumps(line), flush=True)


def render(args) -> None:
    """The headless renderer on the 1M dam break after the warm-up frames:
    splat + visible scan + grid + depth smoothing + shading (mode 0) and the
    two colour modes, at 1280 x 720, CUDA events on the library's stream."""
    import numpy as np
    import torch
    import pbf

    params, pos, vel = pbf.make_scene(SCENE)
    sim = pbf.Simulation.create(params, pos, vel, device=0)
    for _ in range(args.warmup):
        sim.step_async(int(params.subSteps))
    sim.synchronize()
    stream = torch.cuda.ExternalStream(sim.stream())
    cam = pbf.render_camera((6.4, 5.0, 18.0), (6.4, 1.0, 3.2), (0.0, 1.0, 0.0), 45.0, 1280, 720, 0.03)
    modes = {}
    for mode in (0, 1, 2):
        for _ in range(3):
            sim.render_frame(cam, mode)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.render_frames):
            sim.render_frame(cam, mode)
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1) / args.render_frames
        img = sim.render_read(cam, 1)
        covered = float(((img[..., 1] > 0) if mode == 0 else (img[..., 3] > 0)).mean())
        modes[str(mode)] = {"ms_per_frame": ms, "covered_pixels": covered}
    sim.close()
    line = {"render": f"{int(params.particleCount)}-particle dam break after {args.warmup} frames, 1280x720",
            "metric": "ms per rendered frame", "value": modes["0"]["ms_per_frame"], "higher_is_better": False,
            "modes": modes, "frames": args.render_frames, "dtype": "f32",
            "config": {"mode 0": "splat + visible scan + grid + depth smoothing + shading",
                       "mode 1": "splat coloured by speed", "mode 2": "splat coloured by index",
                       "point_size": 0.03, "fovy_deg": 45.0}}
    print(json.dumps(line), flush=True)


def friends_compare(args) -> None:
    """The friends build of the 1M dam break after the warm-up frames, once
    with each algorithm from the same state (a short run to profile: one
    substep with the shared-memory brick gather, one with the L1 scan)."""
    import pbf
    params, pos, vel = pbf.make_scene(SCENE)
    sim = pbf.Simulation.create(params, pos, vel, device=0)
    for _ in range(args.warmup):
        sim.step_async(int(params.subSteps))
    sim.synchronize()
    for algorithm in (2, 0):
        sim.set_launch_shape([256, 128, 128, 128, 128, algorithm, 0])
        sim.Step(1)
    sim.synchronize()
    sim.close()
    print(json.dumps({"friends_compare": "one substep each with friends algorithms 2 and 0", "warmup": args.warmup}))


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=50)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--scene", default=SCENE)
    ap.add_argument("--e2e-steps", type=int, default=0, help="end-to-end frames (0: as many as --steps)")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--cpu-budget", type=float, default=150.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default block sizes")
    ap.add_argument("--no-other-mode", action="store_true", help="skip timing the other arithmetic mode")
    ap.add_argument("--math", choices=["relaxed", "exact"], default="exact",
                    help="relaxedMath of the timed scene (the other mode is timed beside it)")
    ap.add_argument("--sweep", action="store_true", help="particle-count sweep (double dam break) instead")
    ap.add_argument("--sweep-counts", default="262144,2097152,8388608")
    ap.add_argument("--sweep-steps", type=int, default=20)
    ap.add_argument("--sweep-warmup", type=int, default=10)
    ap.add_argument("--batched", action="store_true", help="256 batched scenes instead")
    ap.add_argument("--batch-scenes", type=int, default=256)
    ap.add_argument("--batch-seq-steps", type=int, default=10)
    ap.add_argument("--rollout", action="store_true", help="differentiable rollout forward/backward instead")
    ap.add_argument("--render", action="store_true", help="headless renderer timings instead")
    ap.add_argument("--friends-compare", action="store_true", help="one substep per friends algorithm (to profile)")
    ap.add_argument("--render-frames", type=int, default=20)
    ap.add_argument("--rollout-frames", type=int, default=60)
    ap.add_argument("--rollout-every", type=int, default=10)
    ap.add_argument("--rollouts", type=int, default=3)
    ap.add_argument("--warmup-rollouts", type=int, default=1)
    args = ap.parse_args()
    if args.rollout:
        rollout(args)
        return
    if args.render:
        render(args)
        return
    if args.friends_compare:
        friends_compare(args)
        return
    if args.batched:
        batched(args)
        return
    if args.sweep:
        sweep(args)
        return
    if args.impl == "gb300":
        args.warmup = max(3, args.warmup)  # at least 3 untimed frames
    if args.impl == "reference":
        reference_arm(args)
    else:
        gpu_arm(args)


if __name__ == "__main__":
    main()
