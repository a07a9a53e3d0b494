"""The bounds-checked build (build.py --checked, -DPBF_CHECK_BOUNDS): every
index the kernels read from device memory (friend-list entries, the sort
permutation, keys) is checked before use and an out-of-range one is reported
through the error word, which pbf_step turns into an error.  Over the cases
that stress those paths (hash collisions, a modulo hash, odd sizes, saturated
and many circles, all three friends algorithms, a batch of scenes, the
rollout's reverse pass) it must report nothing and give the oracle's results
bit for bit.  The library a process loads is fixed at import, so the cases
run in a child process with PBF_CHECK_BOUNDS=1."""
from __future__ import annotations

import importlib.util
import os
import subprocess
import sys
import textwrap
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

REPO = Path(__file__).resolve().parent.parent
PKG = REPO / "position-based-fluids_gb300"

SCRIPT = textwrap.dedent("""
    import sys
    sys.path[:0] = [{repo!r}, {pkg!r}]
    import numpy as np
    import pbf
    from oracle import oracle

    assert pbf.LIB_PATH.name == "libpbf_gb300_checked.so", pbf.LIB_PATH

    def same(a, b):
        a = np.array(a, np.float32); b = np.array(b, np.float32)
        a[np.isnan(a)] = 0; b[np.isnan(b)] = 0
        return np.array_equal(a.view(np.uint32), b.view(np.uint32))

    def scene(dims, **ov):
        params = pbf.load_scenario("dam_break_32k")
        for k, v in ov.items():
            setattr(params, k, v)
        params.particleCount = dims[0] * dims[1] * dims[2]
        pos = pbf.scene_block(*dims, 0.05, (0.025,) * 3, 0.005, 20240601)
        return params, pos, np.zeros_like(pos)

    cases = [((16, 16, 16), dict(gridBufSize=64)),
             ((16, 16, 16), dict(gridBufSize=1000)),
             ((17, 13, 11), dict()),
             ((16, 16, 16), dict(friendsCircles=7, particlesPerCircle=3)),
             ((12, 12, 12), dict(friendsCircles=8, particlesPerCircle=64))]
    for dims, ov in cases:
        params, pos, vel = scene(dims, **ov)
        op, ovv, opr = oracle.step(params, pos, vel, 3)
        for algorithm in (0, 1, 2):
            with pbf.Simulation.create(params, pos, vel, device=0) as sim:
                sim.set_launch_shape(sim.launch_shape()[:5] + [algorithm, 1 if algorithm == 1 else 0])
                sim.Step(3)  # raises if a kernel reported an index out of range
                gp, gv, gpr = sim.read_state()
            assert same(gp, op) and same(gv, ovv) and same(gpr, opr), (dims, ov, algorithm)

    scenes, positions = pbf.make_batch_scenes(first=6)
    pos = np.concatenate(positions)
    with pbf.Simulation.create(scenes, pos, np.zeros_like(pos), device=0) as sim:
        offs = sim.scene_offsets()
        sim.Step(2)
        bp, bv, _ = sim.read_state()
    for s, (p, x) in enumerate(zip(scenes, positions)):
        op, ovv, _ = oracle.step(p, x, np.zeros_like(x), 2)
        sl = slice(int(offs[s]), int(offs[s + 1]))
        assert same(bp[sl], op) and same(bv[sl], ovv), ("batch scene", s)

    params, pos, vel = scene((16, 16, 16))
    with pbf.Simulation.create(params, pos, vel, device=0) as sim:
        sim.rollout_forward(6, 3)
        sim.rollout_backward(np.ones((params.particleCount, 4), np.float32))  # raises on a reported index
    print("checked build ok")
""")


def test_checked_build_matches_oracle_and_reports_nothing():
    spec = importlib.util.spec_from_file_location("pbf_pkg_build", PKG / "build.py")
    pkg_build = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(pkg_build)
    pkg_build.build(checked=True)
    env = dict(os.environ, PBF_CHECK_BOUNDS="1")
    run = subprocess.run([sys.executable, "-c", SCRIPT.format(repo=str(REPO), pkg=str(PKG))], env=env,
                         capture_output=True, text=True, timeout=900)
    assert run.returncode == 0, run.stdout[-3000:] + run.stderr[-3000:]
    assert "checked build ok" in run.stdout
