#!/usr/bin/env python
"""Throughput benchmark of the PBF substep pipeline (particle-iterations/s).

Workload: the 1,048,576-particle dam break (position-based-fluids_gb300/
scenarios/dam_break_1m.par: a 128x64x128 block at spacing 0.05 with seeded
jitter in a 12.8 x 6.4 x 6.4 box, h = 0.1, 4 solver iterations).  One bench
step is one 1/60 s frame = 2 substeps of Simulation::Step.

  value   : particle-iterations/s = N * iterations * substeps / time, with the
            state resident in HBM; CUDA events on the library's stream around
            K frames (after W warm-up frames), max over ranks.
  e2e     : the same metric through the C-ABI with host buffers, over the same
            frames (replayed from the state the timed frames started from):
            every frame copies positions + velocities in from pinned host
            memory, steps, and copies them back out, the positions while the
            last substep's XSPH and vorticity run (wall clock).
  roofline: the dominant kernel's compulsory bytes per launch over its
            average launch time.  The launch times come from a replay of the
            same K frames from the same start state, one substep at a time
            with CUDA events between the stages; the list lengths are the
            means over those substeps.  Peak: the measured HBM copy bandwidth.
  batched / rollout: the 256-scene batch and the differentiable rollout,
            each timed with CUDA events and its own clock record.

--impl reference times the reference's own kernels on the host cores (its
OpenCL C compiled through a C++ shim, OpenMP over all cores; the CPU
restatement where they were not compiled) on the same scene and the same
frames (W warm-up frames, then up to K timed ones within a time budget); the
scene is built by the oracle, without the product library.
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

# Compulsory bytes per particle of one launch of each stage in the path's
# byte model: float4 particle records (16 B) and 32-bit keys read or written
# once, neighbour records gathered through the caches not counted, and no
# friend list (the model's gather streams the neighbour cells).  Fused
# stages carry the sum of what they fuse: predict (R32 W32) + keys (R16 W8);
# the sort's P passes of 8-bit digits (16 P + 4, per substep, all of its
# launches); the permutation of pos / pred / vel (R4 + 48 W48); the cell
# table (R4 + 8 x occupied cells / N); per solver iteration the density pass
# R16 W4 and the position pass R16+4 W16; velocities R32 W32; XSPH with
# vorticity R32 W32; vorticity confinement R48 W16.  Whole substep:
# 444 + 56 I bytes per particle at P = 3.
def survey_bytes(stage: str, passes: int = 3):
    return {"predictPositions": 88.0, "radixsort": 16.0 * passes + 4.0, "sortParticles": 100.0,
            "updateCells": 12.0, "computeScaling": 20.0, "computeDelta": 36.0, "updateVelocities": 64.0,
            "applyViscosity": 64.0, "applyVorticity": 64.0}.get(stage)


# Bytes per particle of one launch of each stage as this build moves them:
# the model's bytes plus the friend list it keeps (4 B per entry written or
# read).  `nl` / `nd` are the mean list lengths of the density pass / the
# other passes.
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
# instructions (smsp__inst_executed.sum) per launch from an ncu capture of the
# dam_break_1m scene in the first substep of frame 51, with the mean list
# lengths of that frame (density pass nl, other passes nd): the friends build,
# and the mean over the four launches of each solver pass in the substep (for
# the density pass: the one that records the flat friend rows and three that
# read them).  Launch shape of the capture: the autotuner's for that state
# under ncu (friends 128-thread blocks, density passes 128, position passes
# 64, plain thread map).
# Scaled to the measured list lengths: the traffic by the stage's
# list-inclusive bytes, the instructions in proportion to the list length of
# the pass (for the friends build, whose candidates grow with the density,
# to nl).
CAPTURE_SOURCE = ("ncu capture of the first substep of frame 51 (friends 128-thread blocks, density passes 128, "
                  "position passes 64, list lengths 38.52 / 32.79), scaled by list length")
TRAFFIC_CAPTURE = {"buildFriendsList": {"bytes": 813.3e6, "nl": 38.52, "nd": 32.79},
                   "computeScaling": {"bytes": 308.8e6, "nl": 38.52, "nd": 32.79},
                   "computeDelta": {"bytes": 216.4e6, "nl": 38.52, "nd": 32.79}}
ISSUE_CAPTURE = {"buildFriendsList": {"inst": 650.0e6, "nl": 38.52, "nd": 32.79},
                 "computeScaling": {"inst": 114.5e6, "nl": 38.52, "nd": 32.79},
                 "computeDelta": {"inst": 116.6e6, "nl": 38.52, "nd": 32.79}}
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


def replay_stages(sim, start_pos, start_vel, frames: int, sub: int):
    """Replays `frames` frames from the given start state one substep at a
    time with CUDA events between the stages (pbf_enable_stage_timing), so
    that the per-stage device times belong to exactly those frames.  Returns
    (stage ms per frame, mean density-pass list length, mean other-pass list
    length, final pos, final vel), the list lengths averaged over every
    substep of the replay."""
    import numpy as np
    sim.write_state(start_pos, start_vel)
    sim.enable_stage_timing(True)
    totals: dict[str, float] = {}
    nl = nd = 0.0
    for _ in range(frames):
        for _ in range(sub):
            sim.Step(1)
            for k, v in sim.stage_timings().items():
                totals[k] = totals.get(k, 0.0) + v
            counts, _ = sim.read_friends(slots=0)
            nl += float(counts[:, 0].mean(dtype=np.float64))
            nd += float(counts[:, 1].mean(dtype=np.float64))
    sim.enable_stage_timing(False)
    pos, vel, _ = sim.read_state()
    k = max(1, frames * sub)
    return {name: v / frames for name, v in totals.items()}, nl / k, nd / k, pos, vel


def launches_per_frame(stage: str, iters: int, sub: int) -> int:
    return iters * sub if stage in ("computeScaling", "computeDelta") else sub


def stage_rooflines(stage_ms: dict, n: int, iters: int, sub: int, nl: float, nd: float, peak: float) -> dict:
    """Per stage: its time per frame and per launch, and its bandwidth by the
    path's byte model (`frac`) and by the bytes this build moves, friend
    lists included (`frac_with_lists`)."""
    out = {}
    for k, ms in stage_ms.items():
        per = launches_per_frame(k, iters, sub)
        launch_ms = ms / per
        model = survey_bytes(k)
        own = STAGE_BYTES[k](nl, nd, iters) if k in STAGE_BYTES else None
        if k == "radixsort":
            model_bytes = model * n  # all passes of one substep's sort
        else:
            model_bytes = model * n if model is not None else None
        row = {"ms_per_step": round(ms, 4), "launches_per_step": per, "ms_per_launch": round(launch_ms, 5)}
        if model_bytes is not None and launch_ms > 0:
            gbs = model_bytes / (launch_ms / 1e3) / 1e9
            row.update(bytes_per_launch=model_bytes, gbs=round(gbs, 1), frac=round(gbs / peak, 4))
        if own is not None and launch_ms > 0:
            gbs = own * n / (launch_ms / 1e3) / 1e9
            row.update(bytes_with_lists_per_launch=own * n, gbs_with_lists=round(gbs, 1),
                       frac_with_lists=round(gbs / peak, 4))
        out[k] = row
    return out


def dominant_roofline(stage_ms: dict, n: int, iters: int, sub: int, nl: float, nd: float, peak: float,
                      peak_kind: str) -> dict:
    """The roofline of the stage with the most time per frame: its
    compulsory bytes per launch (the path's byte model; for the friends
    build, which the model does not have, the positions it reads and the
    list it writes) over its mean launch time."""
    dominant = max((k for k in stage_ms if k in STAGE_BYTES), key=lambda k: stage_ms[k])
    launch_ms = stage_ms[dominant] / launches_per_frame(dominant, iters, sub)
    model = survey_bytes(dominant)
    own = STAGE_BYTES[dominant](nl, nd, iters) * n
    algo = model * n if model is not None else own
    achieved = algo / (launch_ms / 1e3) / 1e9
    traffic = None
    if dominant in TRAFFIC_CAPTURE:
        cap = TRAFFIC_CAPTURE[dominant]
        traffic = cap["bytes"] * STAGE_BYTES[dominant](nl, nd, iters) / STAGE_BYTES[dominant](cap["nl"], cap["nd"], 4)
    return {"bound": "hbm", "kernel": dominant, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_source": peak_kind, "traffic": traffic,
            "algorithmic_bytes_per_launch": algo,
            "bytes_model": ("the path's compulsory particle-record bytes per particle" if model is not None
                            else "positions read and friend list written (no friend list in the path's model)"),
            "bytes_with_lists_per_launch": own, "achieved_with_lists": own / (launch_ms / 1e3) / 1e9,
            "frac_with_lists": own / (launch_ms / 1e3) / 1e9 / peak, "avg_launch_ms": launch_ms,
            "launches_per_step": launches_per_frame(dominant, iters, sub),
            "list_lengths": {"density_pass": nl, "other_passes": nd}}


def cpu_reference_sample(params, pos, vel, warm_substeps: int, group: int, max_substeps: int,
                         seconds: float) -> tuple[float, dict]:
    """Time the reference's CPU path on a bounded sample: `warm_substeps`
    untimed substeps from (pos, vel), then substeps timed a frame (`group`
    substeps) at a time until `max_substeps` or `seconds` is reached.  The
    reference's own kernels through the OpenCL-C shim (oracle/_ref) on all
    host threads where they were compiled, else the CPU restatement (the
    oracle port, bit-identical to them).  Returns (particle-iterations/s,
    the fields kind / cores / sample / substeps / seconds)."""
    from oracle import oracle
    n, iters = int(params.particleCount), int(params.simIterations)
    if oracle.ref_available():
        try:
            done, el, _, _ = oracle.ref_run_timed(params, pos, vel, warm_substeps, group, max_substeps, seconds)
            threads = oracle.ref_max_threads()
            return n * iters * done / el, {
                "kind": "reference", "cores": threads, "substeps": done, "seconds": el,
                "sample": f"{done} substep(s) of the {n}-particle scene after {warm_substeps} untimed substep(s) "
                          f"from the given start state, through the reference's own kernels (OpenCL-C shim, "
                          f"work-items on {threads} threads), {el:.1f} s"}
        except (OSError, RuntimeError, FileNotFoundError):
            pass  # no compiler or no generated unit here: the restatement below
    threads = oracle.max_threads()
    p, v = pos, vel
    if warm_substeps:
        p, v, _ = oracle.step(params, p, v, warm_substeps, threads=threads)
    done, t0 = 0, time.perf_counter()
    while True:
        p, v, _ = oracle.step(params, p, v, group, threads=threads)
        done += group
        el = time.perf_counter() - t0
        if el >= seconds or done >= max_substeps:
            break
    return n * iters * done / el, {
        "kind": "port", "cores": threads, "substeps": done, "seconds": el,
        "sample": f"{done} substep(s) of the {n}-particle scene after {warm_substeps} untimed substep(s) from the "
                  f"given start state, through the CPU restatement, {el:.1f} s"}


def solver_constants(params) -> str:
    return (f"solver constants epsilon {params.epsilon:g}, s_corr k {-params.surfaceTenstionK:g}, XSPH c "
            f"{params.viscosityFactor:.6g} (= 0.01 / 6378) in place of the dam-break set's 600, 0.1 and 0.01, "
            f"which the reference's own kernels run unstably (NaN within about 10 substeps); box clamp "
            f"{'on' if params.boxClamp else 'off'}, zero-distance guard {'on' if params.zeroDistanceGuard else 'off'}")


def workload_name(scene: str, params) -> str:
    n, iters, sub = int(params.particleCount), int(params.simIterations), int(params.subSteps)
    block = "?"
    for line in (PKG / "scenarios" / f"{scene}.par").read_text().splitlines():
        f = line.split("#")[0].split()
        if len(f) == 4 and f[0].lower() == "blockdims":
            block = "x".join(f[1:])
    box = "x".join(f"{float(hi) - float(lo):g}" for lo, hi in ((params.xMin, params.xMax), (params.yMin, params.yMax),
                                                               (params.zMin, params.zMax)))
    return (f"{scene}: {n} particles ({block} block, spacing {params.h * params.setupSpacing:g}, seeded jitter) "
            f"in a {box} box; {iters} iterations x {sub} substeps per step (frame); {solver_constants(params)}")


def reference_scene(name: str):
    """(params, pos, vel) of a bundled scenario, built by the oracle from the
    scenario file (the product library stays unloaded)."""
    from oracle import oracle
    import pbf  # the ctypes mirror of PbfParameters only; its library is loaded lazily and not here
    return oracle.make_scene(PKG / "scenarios" / f"{name}.par", pbf.PbfParameters)


def reference_arm(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    params, pos, vel = reference_scene(args.scene)
    n, iters, sub = int(params.particleCount), int(params.simIterations), int(params.subSteps)
    value, info = cpu_reference_sample(params, pos, vel, args.warmup * sub, sub, args.steps * sub, args.cpu_budget)
    frames = max(1, info["substeps"] // sub)
    el = info["seconds"]
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": frames, "warmup": args.warmup, "ms_per_step": 1000.0 * el / frames,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": workload_name(args.scene, params),
                   "reference_step": f"one frame of {sub} substeps, after {args.warmup} untimed warm-up frames "
                                     f"from the initial state (the frames the GPU arm times), up to --steps frames "
                                     f"within {args.cpu_budget:.0f} s",
                   "particles": n, "iterations": iters, "substeps_per_step": sub, "threads": info["cores"]},
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


def finish_rank(sim, dist=None) -> None:
    """End of a rank's run: its simulation closed, then its process group
    (if any) destroyed, once."""
    if sim is not None:
        sim.close()
    if dist is not None and dist.is_initialized():
        dist.destroy_process_group()


# The stage groups the per-stage times are also reported in: keys, sort,
# permutation and cell table / friend lists and the density pass / the
# position-correction pass / velocities, XSPH and vorticity.
STAGE_GROUPS = {
    "sort": ("predictPositions", "radixsort", "sortParticles", "updateCells", "resetPartList"),
    "friends+lambda": ("buildFriendsList", "computeScaling"),
    "delta_p": ("computeDelta", "packData"),
    "xsph+vorticity": ("updateVelocities", "applyViscosity", "applyVorticity"),
}

SHAPE_KEYS = ["friends", "scaling", "delta", "viscosity", "vorticity", "friends_algorithm", "balance", "persistent"]


def timed_frames(sim, stream, frames: int, sub: int, device_index: int):
    """CUDA events on the simulation's stream around `frames` frames, with
    the clocks sampled meanwhile.  Returns (ms per frame, clock summary)."""
    import torch
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    sim.synchronize()
    with ClockSampler(device_index) as clocks:
        e0.record(stream)
        for _ in range(frames):
            sim.step_async(sub)
        e1.record(stream)
        e1.synchronize()
    sim.synchronize()
    return e0.elapsed_time(e1) / frames, clocks.summary()


def batched_block(args, single_value: float, device_index: int) -> dict:
    """The 256-scene batch (pbf.make_batch_scenes: counts log-uniform in
    [4096, 65536] from seed 7, ~5.7M particles) advanced together, one graph
    per substep with autotuned block sizes, against the single-scene rate of
    this run and against the same scenes run one at a time on the plain
    path."""
    import numpy as np
    import torch
    import pbf
    scenes, positions = pbf.make_batch_scenes(count=args.batch_scenes)
    pos = np.concatenate(positions)
    total = int(pos.shape[0])
    sub, iters = int(scenes[0].subSteps), int(scenes[0].simIterations)
    sim = pbf.Simulation.create(scenes, pos, np.zeros_like(pos), device=device_index)
    stream = torch.cuda.ExternalStream(sim.stream(), device=torch.device("cuda", device_index))
    warmup = args.batch_warmup if args.batch_warmup >= 0 else args.warmup  # as many frames as the single scene
    for _ in range(warmup):
        sim.step_async(sub)
    sim.synchronize()
    blocks = sim.autotune(trial_substeps=2)
    # the same shape with one block per particle tile and with persistent
    # grids walking the tiles, from the same state (the headline keeps the
    # autotuner's choice)
    start_pos, start_vel, _ = sim.read_state()
    grid_ms = {}
    for persistent in (0, 1):
        sim.write_state(start_pos, start_vel)
        sim.set_launch_shape(list(blocks[:7]) + [persistent])
        grid_ms["persistent" if persistent else "block_per_tile"], _ = timed_frames(sim, stream, args.batch_steps,
                                                                                   sub, device_index)
    sim.write_state(start_pos, start_vel)
    sim.set_launch_shape(blocks)
    launches0 = sim.launch_count()
    ms, clocks = timed_frames(sim, stream, args.batch_steps, sub, device_index)
    launches = sim.launch_count() - launches0
    stage_ms, bnl, bnd, _, _ = replay_stages(sim, start_pos, start_vel, args.batch_steps, sub)
    sim.close()
    rate = total * iters * sub / (ms / 1e3)
    seq_ms = 0.0
    for p, x in zip(scenes, positions):
        one = pbf.Simulation.create(p, x, np.zeros_like(x), device=device_index)
        st = torch.cuda.ExternalStream(one.stream(), device=torch.device("cuda", device_index))
        for _ in range(3):
            one.step_async(sub)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        one.synchronize()
        e0.record(st)
        for _ in range(args.batch_seq_steps):
            one.step_async(sub)
        e1.record(st)
        e1.synchronize()
        seq_ms += e0.elapsed_time(e1) / args.batch_seq_steps
        one.close()
    seq_rate = total * iters * sub / (seq_ms / 1e3)
    return {"workload": f"{len(scenes)} dam-break scenes, {total} particles, counts log-uniform in [4096, 65536] "
                        f"(seed 7), box fill 0.3, gravity tilted U(0, 10) deg, XSPH c U(0.005, 0.05); {iters} "
                        f"iterations x {sub} substeps per frame, one CUDA graph per substep",
            "particles": total, "value": rate, "unit": UNIT, "ms_per_step": ms, "steps": args.batch_steps,
            "warmup": warmup, "gpu_launches": int(launches),
            "stage_ms_per_step": {k: round(v, 4) for k, v in sorted(stage_ms.items(), key=lambda kv: -kv[1])},
            "neighbours": {"density_pass": bnl, "other_passes": bnd},
            "ratio_vs_single_scene": rate / single_value, "single_scene_value": single_value,
            "sequential_value": seq_rate, "ratio_vs_sequential": rate / seq_rate,
            "sequential_steps": args.batch_seq_steps,
            "grid_ms_per_step": grid_ms,
            "blocks": dict(zip(SHAPE_KEYS, blocks)), "clocks": clocks}


def rollout_block(args, device_index: int) -> dict:
    """The differentiable rollout: the 65,536-particle dam break (64x32x32
    block) for 60 frames of 2 substeps, checkpoints every 10 substeps; loss
    the MSE to a target run with gravity tilted 5 degrees and XSPH c = 0.03.
    pbf_rollout_forward and pbf_rollout_backward (which recomputes each
    segment from its checkpoint before its adjoint kernels) timed with CUDA
    events on the simulation's stream; the median of `rollouts` runs after
    one warm-up run."""
    import numpy as np
    import torch
    import pbf
    frames, every = args.rollout_frames, args.rollout_every
    params, pos, vel = pbf.make_rollout_scene(64, 32, 32)
    n = int(params.particleCount)
    substeps = frames * int(params.subSteps)
    with pbf.Simulation.create(pbf.rollout_target_params(params), pos, vel, device=device_index) as tsim:
        tsim.Step(substeps)
        target = tsim.positions_by_id().astype(np.float64)
    sim = pbf.Simulation.create(params, pos, vel, device=device_index)
    stream = torch.cuda.ExternalStream(sim.stream(), device=torch.device("cuda", device_index))

    def timed(fn):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        sim.synchronize()
        e0.record(stream)
        out = fn()
        e1.record(stream)
        e1.synchronize()
        return out, e0.elapsed_time(e1)

    fwd, bwd, plain = [], [], []
    loss, dv, dc, dg, launches = 0.0, None, 0.0, (0.0, 0.0, 0.0), 0
    with ClockSampler(device_index) as clocks:
        for rep in range(1 + args.rollouts):
            sim.write_state(pos, vel)
            _, ms_plain = timed(lambda: sim.Step(substeps))
            sim.write_state(pos, vel)
            l0 = sim.launch_count()
            _, ms_f = timed(lambda: sim.rollout_forward(substeps, every))
            x = sim.positions_by_id()
            loss = float(np.mean((x[:, :3].astype(np.float64) - target[:, :3]) ** 2))
            g = np.zeros((n, 4), np.float32)
            g[:, :3] = (2.0 * (x[:, :3].astype(np.float64) - target[:, :3]) / (3.0 * n)).astype(np.float32)
            (dv, dc, dg), ms_b = timed(lambda: sim.rollout_backward(g))
            if rep >= 1:
                fwd.append(ms_f)
                bwd.append(ms_b)
                plain.append(ms_plain)
                launches = sim.launch_count() - l0
    sim.close()
    f, bk, pl = float(np.median(fwd)), float(np.median(bwd)), float(np.median(plain))
    return {"workload": f"{n}-particle dam break (64x32x32 block), {frames} frames x {int(params.subSteps)} "
                        f"substeps, checkpoint every {every} substeps, loss MSE to a target run (gravity tilted 5 "
                        f"deg, XSPH c 0.03); gradients w.r.t. initial velocities, XSPH c and the gravity vector",
            "metric": "backward / forward time", "value": bk / f, "higher_is_better": False,
            "forward_ms": f, "backward_ms": bk, "plain_steps_ms": pl,
            "forward_us_per_substep": 1e3 * f / substeps, "backward_us_per_substep": 1e3 * bk / substeps,
            "rollouts": args.rollouts, "warmup": 1, "gpu_launches": int(launches), "loss": loss,
            "grad_norms": {"v0": float(np.linalg.norm(dv[:, :3])), "c": float(dc), "g": [float(v) for v in dg]},
            "clocks": clocks.summary()}


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
    # the state the timed frames start from: the end-to-end and stage replays
    # below run the same frames from it
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
    frame_ms = ms / args.steps

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

    # ---- per-stage device times of the same frames (eager, events between stages) ----
    peak, peak_kind = measured_peaks()
    stage_ms, nl, nd, rpos, rvel = replay_stages(sim, h0pos.numpy(), h0vel.numpy(), args.steps, sub)
    stage_replay_identical = bool(np.array_equal(rpos.view(np.uint32), end_pos.view(np.uint32)) and
                                  np.array_equal(rvel.view(np.uint32), end_vel.view(np.uint32)))
    stage_sum = sum(stage_ms.values())
    roof = dominant_roofline(stage_ms, n, iters, sub, nl, nd, peak, peak_kind)
    per_stage = stage_rooflines(stage_ms, n, iters, sub, nl, nd, peak)
    dominant, launch_ms = roof["kernel"], roof["avg_launch_ms"]

    # ---- density error of the state after the timed frames ----
    _, _, dpred = sim.read_state()
    rel = np.abs(dpred[:, 3].astype(np.float64) / float(params.restDensity) - 1.0)
    rel = rel[np.isfinite(rel)]
    density_error = {"mean": float(rel.mean()), "p95": float(np.percentile(rel, 95)), "max": float(rel.max()),
                     "note": "|rho / rho0 - 1| per particle, density of the last solver iteration"}

    # the issue rate of every captured stage (the exact passes' bound), the dominant one as issue_roofline
    clk = clocks.summary().get("sm_mhz") or 2070.0
    peak_issue = SM_COUNT * SCHEDULERS_PER_SM * clk * 1e6
    stage_issue = {}
    for k, cap in ISSUE_CAPTURE.items():
        if k not in stage_ms or (args.math != "exact" and k != "buildFriendsList"):
            continue
        inst = cap["inst"] * (nl / cap["nl"] if k in ("computeScaling", "buildFriendsList") else nd / cap["nd"])
        k_ms = stage_ms[k] / launches_per_frame(k, iters, sub)
        stage_issue[k] = {"kernel": k, "warp_instructions_per_launch": inst, "ms_per_launch": k_ms,
                          "achieved": inst / (k_ms / 1000.0), "peak": peak_issue, "unit": "warp instructions/s",
                          "frac": inst / (k_ms / 1000.0) / peak_issue,
                          "source": "smsp__inst_executed.sum of the " + CAPTURE_SOURCE}
    issue = stage_issue.get(dominant)

    # ---- the other arithmetic mode, same start state, its own block sizes ----
    other_line = None
    if not args.no_other_mode:
        other = "exact" if args.math == "relaxed" else "relaxed"
        p2 = params.copy()
        p2.relaxedMath = 1 if other == "relaxed" else 0
        sim.set_params(p2)
        sim.write_state(h0pos.numpy(), h0vel.numpy())
        for _ in range(3):
            sim.step_async(sub)
        sim.synchronize()
        other_blocks = sim.autotune(trial_substeps=2) if not args.no_autotune else sim.launch_shape()
        sim.write_state(h0pos.numpy(), h0vel.numpy())
        barrier()
        other_ms, other_clocks = timed_frames(sim, stream, args.steps, sub, local)
        other_stages, onl, ond, _, _ = replay_stages(sim, h0pos.numpy(), h0vel.numpy(), min(args.steps, 20), sub)
        other_line = {"mode": other, "value": n * iters * sub / (other_ms / 1000.0), "ms_per_step": other_ms,
                      "frames": "the timed frames, from their start state",
                      "blocks": dict(zip(SHAPE_KEYS, other_blocks)),
                      "roofline": dominant_roofline(other_stages, n, iters, sub, onl, ond, peak, peak_kind),
                      "stage_ms_per_step": {k: round(v, 4) for k, v in sorted(other_stages.items(), key=lambda kv: -kv[1])},
                      "stage_frames": min(args.steps, 20), "clocks": other_clocks}
        sim.set_params(params)
        sim.set_launch_shape(blocks)

    bytes_sub = (444.0 + 56.0 * iters) * n  # whole-substep compulsory bytes, P = 3 sort passes
    pipeline_gbs = bytes_sub * sub / (frame_ms / 1000.0) / 1e9

    if rank != 0:
        finish_rank(sim, dist)
        return
    sim.close()
    sim = None
    batched = rollout = base = None
    if world == 1 and not args.no_batched:
        batched = batched_block(args, value, local)
    if world == 1 and not args.no_rollout:
        rollout = rollout_block(args, local)
    if world == 1 and not args.no_cpu_baseline:
        # the reference's kernels from the start state of the timed frames
        cpu_value, info = cpu_reference_sample(params, h0pos.numpy(), h0vel.numpy(), 0, sub, args.steps * sub,
                                               args.cpu_seconds)
        base = {"value": cpu_value, "unit": UNIT, "cores": info["cores"], "kind": info["kind"],
                "sample": info["sample"] + " (the start state of the timed frames)"}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": frame_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": workload_name(args.scene, params),
                   "particles": n, "iterations": iters, "substeps_per_step": sub,
                   "epsilon": float(params.epsilon), "s_corr_k": -float(params.surfaceTenstionK),
                   "xsph_c": float(params.viscosityFactor),
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                   "l2": "working set larger than L2 (no flush)", "mode": MODES[args.math],
                   "cuda_graph": True, "blocks": dict(zip(SHAPE_KEYS, blocks))},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 32 * n, "d2h_bytes_per_step": 32 * n,
                "steps": e2e_steps, "frames": "the timed frames replayed from their start state",
                "replay_bit_identical": e2e_replay_identical},
        "gpu_launches": int(launches),
        "roofline": roof,
        "pipeline_roofline": {"bytes_per_particle_substep": 444.0 + 56.0 * iters, "achieved": pipeline_gbs,
                              "frac": pipeline_gbs / peak},
        **({"issue_roofline": issue} if issue else {}),
        **({"stage_issue_rooflines": stage_issue} if stage_issue else {}),
        "particle_substeps_per_s": value / iters,
        "stage_replay": {"frames": args.steps, "bit_identical_to_timed_frames": stage_replay_identical,
                         "stage_sum_ms_per_step": stage_sum, "ratio_to_ms_per_step": stage_sum / frame_ms},
        "stage_ms_per_step": {k: round(v, 4) for k, v in sorted(stage_ms.items(), key=lambda kv: -kv[1])},
        "stage_groups_ms_per_step": {g: round(sum(stage_ms.get(k, 0.0) for k in ks), 4) for g, ks in STAGE_GROUPS.items()},
        "stage_rooflines": per_stage,
        "neighbours": {"density_pass": nl, "other_passes": nd, "averaged_over": f"the {args.steps * sub} substeps of the timed frames"},
        "density_error": density_error,
        **({"other_mode": other_line} if other_line else {}),
        **({"batched": batched} if batched else {}),
        **({"rollout": rollout} if rollout else {}),
        "clocks": clocks.summary(),
    }
    if base is not None:
        line["cpu_baseline"] = base
    print(json.dumps(line), flush=True)
    finish_rank(sim, dist)


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
            sim_state = sim.read_state()
            counts_, _ = sim.read_friends(slots=0)
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
            base = None
            if n <= args.sweep_cpu_max:  # the reference's kernels from the state the timed frames ended on
                end_pos, end_vel, _ = sim_state
                cpu_value, info = cpu_reference_sample(params, end_pos, end_vel, 0, sub, 8 * sub, args.cpu_seconds)
                base = {"value": cpu_value, "unit": UNIT, "cores": info["cores"], "kind": info["kind"],
                        "sample": info["sample"]}
            line = {"sweep": "double_dam_break", "particles": n, "iterations": iters,
                    "value": n * iters * sub / (frame_ms / 1e3), "unit": UNIT, "ms_per_step": frame_ms,
                    "steps": args.sweep_steps, "warmup": args.sweep_warmup, "neighbours": {"density_pass": nl,
                    "other_passes": nd}, "groups": groups, "peak_gbs": peak, "peak_source": peak_kind,
                    "blocks": dict(zip(SHAPE_KEYS, blocks)), **({"cpu_baseline": base} if base else {})}
            print(json.dumps(line), flush=True)


def batched(args) -> None:
    """--batched: the batch block alone, against the single-scene 1M rate
    measured in the same process."""
    import torch
    import pbf
    params, p1, v1 = pbf.make_scene(SCENE)
    sub = int(params.subSteps)
    single = pbf.Simulation.create(params, p1, v1, device=0)
    for _ in range(args.warmup):
        single.step_async(sub)
    single.autotune(trial_substeps=2)
    ms, _ = timed_frames(single, torch.cuda.ExternalStream(single.stream()), args.steps, sub, 0)
    single.close()
    rate = int(params.particleCount) * int(params.simIterations) * sub / (ms / 1e3)
    print(json.dumps({"batched": batched_block(args, rate, 0)}), flush=True)


def rollout(args) -> None:
    """--rollout: the rollout block alone."""
    print(json.dumps({"rollout": rollout_block(args, 0)}), flush=True)


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
        sim.set_launch_shape([256, 128, 128, 128, 128, algorithm, 0, 0])
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
    ap.add_argument("--sweep-cpu-max", type=int, default=262144,
                    help="largest sweep size that also times the reference's CPU kernels")
    ap.add_argument("--batched", action="store_true", help="256 batched scenes alone")
    ap.add_argument("--no-batched", action="store_true", help="leave the batched block out of the default run")
    ap.add_argument("--batch-scenes", type=int, default=256)
    ap.add_argument("--batch-steps", type=int, default=10, help="timed frames of the batch")
    ap.add_argument("--batch-warmup", type=int, default=-1,
                    help="warm-up frames of the batch (default: --warmup, as the single scene)")
    ap.add_argument("--batch-seq-steps", type=int, default=5, help="timed frames of each scene run alone")
    ap.add_argument("--rollout", action="store_true", help="differentiable rollout forward/backward alone")
    ap.add_argument("--no-rollout", action="store_true", help="leave the rollout block out of the default run")
    ap.add_argument("--render", action="store_true", help="headless renderer timings instead")
    ap.add_argument("--friends-compare", action="store_true", help="one substep per friends algorithm (to profile)")
    ap.add_argument("--render-frames", type=int, default=20)
    ap.add_argument("--rollout-frames", type=int, default=60)
    ap.add_argument("--rollout-every", type=int, default=10)
    ap.add_argument("--rollouts", type=int, default=3, help="timed rollouts (after one warm-up rollout)")
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
