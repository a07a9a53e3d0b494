"""The CUDA path against the oracle, through the C-ABI (needs a GPU).

Contract: the sort permutation, keys and cell table are bit-exact; one and
many substeps of positions, velocities and predictions are bit-exact as
well (NaN payloads aside: every NaN is compared as NaN).  The tolerance the
path promises is 1e-5 relative (max |gpu - oracle| / max |oracle| per array),
which bit-exact results meet trivially; the relative error is computed and
checked as well so a regression reports a figure, not only a mismatch.
"""
from __future__ import annotations

import hashlib
import importlib.util
import json
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
REL_TOL = 1e-5


def _mg():
    spec = importlib.util.spec_from_file_location("make_golden", GOLDEN / "make_golden.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


MG = None


def mg():
    global MG
    if MG is None:
        MG = _mg()
    return MG


def assert_same(name, got, want):
    g, w = mg().canonical(got), mg().canonical(want)
    same = np.array_equal(g.view(np.uint32), w.view(np.uint32))
    if not same:
        finite = np.isfinite(w) & np.isfinite(g)
        scale = float(np.max(np.abs(w[finite]))) if finite.any() else 1.0
        rel = float(np.max(np.abs(g[finite] - w[finite]))) / max(scale, 1e-30) if finite.any() else np.inf
        nbad = int(np.sum(g.view(np.uint32) != w.view(np.uint32)))
        nan_mismatch = int(np.sum(np.isnan(g) != np.isnan(w)))
        raise AssertionError(f"{name}: {nbad} words differ (rel err {rel:.3e}, NaN mismatches {nan_mismatch})")


def run_gpu(pbf, params, pos, vel, substeps, device, graph=True, friends=True, algorithm=None, sort=None):
    """`sort` (a dict, optional) receives the keys, permutation and cell table
    of the last substep (pbf_read_sort)."""
    with pbf.Simulation.create(params, pos, vel, device=device) as sim:
        sim.use_graph(graph)
        if algorithm is not None:  # friends algorithm; the balanced map with the warp one
            sim.set_launch_shape(sim.launch_shape()[:5] + [algorithm, 1 if algorithm == 1 else 0])
        sim.Step(substeps)
        p, v, pr = sim.read_state()
        counts, lst = sim.read_friends() if friends else (None, None)
        if sort is not None:
            sort["keys"], sort["perm"], sort["cells"] = sim.read_sort()
    return p, v, pr, counts, lst


def scene(pbf, dims, base="dam_break_32k", spacing=0.05, origin=(0.025,) * 3, jitter=0.005, seed=20240601, **ov):
    params = pbf.load_scenario(base)
    for k, v in ov.items():
        setattr(params, k, v)
    params.particleCount = dims[0] * dims[1] * dims[2]
    pos = pbf.scene_block(*dims, spacing, origin, jitter, seed)
    return params, pos, np.zeros_like(pos)


# ------------------------------------------------------------------ sort --
@pytest.mark.parametrize("case", [
    dict(dims=(32, 32, 32)),
    dict(dims=(17, 13, 11)),                      # N not a multiple of 32 / 2048
    dict(dims=(16, 16, 16), gridBufSize=64),      # hash collisions
    dict(dims=(16, 16, 16), gridBufSize=1000),    # modulo, not a power of two
    dict(dims=(2, 1, 1)),                         # two particles
    dict(dims=(12, 12, 12), origin=(-0.3,) * 3),  # negative coordinates: cells truncate toward zero
    dict(dims=(8, 8, 8), origin=(102.2, 0.025, 0.025)),  # x cells past 1023: Morton bits wrap
])
def test_sort_and_cells_bit_exact(case, pbf_mod, oracle_mod, cuda_device):
    case = dict(case)
    dims = case.pop("dims")
    params, pos, vel = scene(pbf_mod, dims, **case)
    rng = np.random.default_rng(3)
    pred = pos.copy()
    pred[:, :3] += rng.uniform(-0.02, 0.02, (len(pos), 3)).astype(np.float32)
    with pbf_mod.Simulation.create(params, pos, vel, device=cuda_device) as sim:
        gk, gp, gc = sim.sort_state(pred)
    ok, op, oc = oracle_mod.sort(params, pred)
    assert np.array_equal(gk, ok), "keys"
    assert np.array_equal(gp, op), "permutation"
    assert np.array_equal(gc, oc), "cell table"


def test_sort_at_full_scale_properties(pbf_mod, oracle_mod, cuda_device):
    """1M particles: bit-exact against the oracle, plus the properties of a
    stable sort (sorted keys, a permutation, stable ties)."""
    params, pos, vel = pbf_mod.make_scene("dam_break_1m")
    with pbf_mod.Simulation.create(params, pos, vel, device=cuda_device) as sim:
        gk, gp, gc = sim.sort_state(pos)
    n = len(pos)
    assert np.all(np.diff(gk[:n].astype(np.int64)) >= 0)
    assert np.array_equal(np.sort(gp[:n]), np.arange(n, dtype=np.uint32))
    same = gk[1:n] == gk[:n - 1]
    assert np.all(gp[1:n][same] > gp[:n - 1][same]), "ties keep input order"
    ok, op, oc = oracle_mod.sort(params, pos)
    assert np.array_equal(gk, ok) and np.array_equal(gp, op) and np.array_equal(gc, oc)


# -------------------------------------------------------- golden digests --
MANIFEST = json.loads((GOLDEN / "golden.json").read_text())


@pytest.mark.parametrize("algorithm", [0, 1, 2], ids=["scan", "warp", "brick"])
@pytest.mark.parametrize("case", MANIFEST["cases"], ids=[c["name"] for c in MANIFEST["cases"]])
def test_gpu_matches_reference_kernel_digests(case, algorithm, pbf_mod, cuda_device):
    """Outputs of the reference's own kernels (tests/golden) reproduced on the
    GPU: positions, velocities and predictions after the last substep, and
    that substep's sorted keys, permutation and cell table (the reference's
    histogram / scan / paste / reorder and updateCells, radixsort.cl:61-308,
    update_cells.cl) as the GPU pipeline computed them."""
    params, pos, vel = mg().scene(tuple(case["block"]), case["overrides"])
    sort = {}
    p, v, pr, _, _ = run_gpu(pbf_mod, params, pos, vel, case["substeps"], cuda_device, friends=False,
                             algorithm=algorithm, sort=sort)
    for name, arr in (("pos", p), ("vel", v), ("pred", pr), ("keys", sort["keys"]), ("perm", sort["perm"]),
                      ("cells", sort["cells"])):
        assert mg().digest(arr) == case["sha256"][name], f"{case['name']}: {name}"


# ------------------------------------------------------- substep parity --
SUBSTEP_CASES = {
    "dam32k_clamped_1": (dict(dims=(32, 32, 32)), 1),
    "dam32k_clamped_4": (dict(dims=(32, 32, 32)), 4),
    "literal_clamped_6": (dict(dims=(24, 24, 24), base="dam_break_32k_literal"), 6),
    "gravity_vector": (dict(dims=(20, 16, 12), gravityVectorEnable=1, gravityX=1.2, gravityY=-9.0, gravityZ=0.5), 3),
    "zero_iterations": (dict(dims=(16, 16, 16), simIterations=0), 2),
    "one_iteration_odd": (dict(dims=(19, 7, 23), simIterations=1), 2),
    "collisions_clamped": (dict(dims=(16, 16, 16), gridBufSize=128), 2),
    "eight_circles_64": (dict(dims=(16, 16, 16), friendsCircles=8, particlesPerCircle=64), 2),
    "seven_circles_saturated": (dict(dims=(16, 16, 16), friendsCircles=7, particlesPerCircle=3), 2),
    "two_particles": (dict(dims=(2, 1, 1)), 3),
    "one_particle": (dict(dims=(1, 1, 1)), 2),
    # unclamped blocks where the reference's cell arithmetic is at its edges:
    # straddling the origin (cell 0 spans (-h, h), the -1 neighbours' Morton
    # bits come from negative integers) and past 1024 cells along x (the
    # 10-bit Morton coordinates wrap, so distant cells share hashes)
    "across_origin": (dict(dims=(12, 12, 12), origin=(-0.3,) * 3, boxClamp=0), 3),
    # no jitter: many neighbours share a coordinate, so the numerators of the
    # exact passes' quotients by |r| are exactly zero
    "lattice_without_jitter": (dict(dims=(14, 14, 14), jitter=0.0), 3),
    "beyond_morton_range": (dict(dims=(8, 8, 8), origin=(102.2, 0.025, 0.025), boxClamp=0), 3),
}


@pytest.mark.parametrize("algorithm", [0, 1, 2], ids=["scan", "warp", "brick"])
@pytest.mark.parametrize("name", list(SUBSTEP_CASES))
def test_substeps_bit_exact(name, algorithm, pbf_mod, oracle_mod, cuda_device):
    """Both friends algorithms (per-particle scan, warp-cooperative runs),
    with the plain and the balanced thread map of the solver passes."""
    spec, substeps = SUBSTEP_CASES[name]
    spec = dict(spec)
    dims = spec.pop("dims")
    params, pos, vel = scene(pbf_mod, dims, **spec)
    gp, gv, gpr, gcounts, glist = run_gpu(pbf_mod, params, pos, vel, substeps, cuda_device, algorithm=algorithm)
    op, ov, opr, dbg = oracle_mod.step(params, pos, vel, substeps, debug=True)
    assert np.array_equal(gcounts, dbg["counts"]), "friend counts"
    slots = int(dbg["counts"][:, 0].max()) if len(dbg["counts"]) else 0
    for s in range(slots):
        used = dbg["counts"][:, 0] > s
        assert np.array_equal(glist[s][used], dbg["list"][s][used]), f"friend list slot {s}"
    assert_same("pos", gp, op)
    assert_same("vel", gv, ov)
    assert_same("pred", gpr, opr)


@pytest.mark.parametrize("algorithm", [0, 1, 2], ids=["scan", "warp", "brick"])
def test_tiny_coordinates_bit_exact(algorithm, pbf_mod, oracle_mod, cuda_device):
    """Predicted coordinates in (0, 2^-27): their differences can be too small
    for the exact passes' quotients through one reciprocal, so the particles
    that may hold such a friend (the 27 cells around it) divide the IEEE way
    for the rest of the substep.  A block at the origin (no clamp) with some
    particles moved onto tiny coordinates next to neighbours at exactly 0;
    each friends build marks the cells around them itself."""
    params, pos, vel = scene(pbf_mod, (10, 10, 10), origin=(0.0, 0.0, 0.0), jitter=0.0, boxClamp=0)
    pos[1, 0] = np.float32(3e-13)       # x next to particle 0 at x = 0
    pos[10, 1] = np.float32(1e-30)      # y, a normal float far below 2^-27
    pos[100, 2] = np.float32(2e-42)     # z, subnormal
    pos[111, :3] = np.float32(5e-39)
    gp, gv, gpr, gcounts, glist = run_gpu(pbf_mod, params, pos, vel, 3, cuda_device, algorithm=algorithm)
    op, ov, opr, dbg = oracle_mod.step(params, pos, vel, 3, debug=True)
    assert np.array_equal(gcounts, dbg["counts"]), "friend counts"
    assert_same("pos", gp, op)
    assert_same("vel", gv, ov)
    assert_same("pred", gpr, opr)


def test_tiny_coordinates_arising_in_a_dam_break_bit_exact(pbf_mod, oracle_mod, cuda_device):
    """Coordinates in (0, 2^-27) also arise by themselves: particles resting a
    hair's breadth off a wall.  In the 65,536-particle double dam break with
    4 iterations they appear from about substep 150 on, the oracle's states
    show them, and the GPU's state equals the oracle's every 32 substeps
    through substep 224."""
    params, pos, vel = pbf_mod.make_double_dam_break(65536, iterations=4)
    tiny = 0
    p, v = pos, vel
    with pbf_mod.Simulation.create(params, pos, vel, device=cuda_device) as sim:
        for chunk in range(7):
            for _ in range(32):
                p, v, q = oracle_mod.step(params, p, v, 1)
                x = np.abs(np.concatenate([p[:, :3], q[:, :3]]))
                tiny += int(((x > 0) & (x < 2.0 ** -27)).sum())
            sim.Step(32)
            gp, gv, gq = sim.read_state()
            assert_same(f"pos after {32 * (chunk + 1)} substeps", gp, p)
            assert_same(f"vel after {32 * (chunk + 1)} substeps", gv, v)
            assert_same(f"pred after {32 * (chunk + 1)} substeps", gq, q)
    assert tiny > 0, "no coordinate in (0, 2^-27) arose: the case no longer covers them"


def test_persistent_grids_bit_identical(pbf_mod, cuda_device):
    """Persistent grids (at most the resident blocks, walking the particle
    tiles grid-stride) against one block per tile: the 1M dam break with
    64-thread blocks has 16,384 tiles, more than a GB300 keeps resident, so
    every block walks several tiles; with and without the balanced thread map."""
    params, pos, vel = pbf_mod.make_scene("dam_break_1m")
    for balance in (0, 1):
        out = []
        for persistent in (0, 1):
            with pbf_mod.Simulation.create(params, pos, vel, device=cuda_device) as sim:
                sim.set_launch_shape([64, 64, 64, 64, 64, 0, balance, persistent])
                sim.Step(4)
                out.append(sim.read_state())
        for name, x, y in zip(("pos", "vel", "pred"), out[0], out[1]):
            assert_same(f"{name} (balance {balance})", y, x)


def test_graph_and_eager_paths_agree(pbf_mod, cuda_device):
    params, pos, vel = scene(pbf_mod, (20, 20, 20))
    a = run_gpu(pbf_mod, params, pos, vel, 5, cuda_device, graph=True)
    b = run_gpu(pbf_mod, params, pos, vel, 5, cuda_device, graph=False)
    for name, x, y in zip(("pos", "vel", "pred"), a[:3], b[:3]):
        assert_same(name, x, y)


def test_paused_steps_match_oracle(pbf_mod, oracle_mod, cuda_device):
    """bPauseSim: no gravity, no sort; the previous sorted keys are reused."""
    params, pos, vel = scene(pbf_mod, (16, 16, 12))
    with pbf_mod.Simulation.create(params, pos, vel, device=cuda_device) as sim:
        sim.Step(2)
        sim.bPauseSim = True
        sim.Step(2)
        sim.bPauseSim = False
        sim.Step(1)
        gp, gv, gpr = sim.read_state()
    keys = np.zeros(oracle_mod.n_keys(len(pos)), np.uint32)
    p, v, _ = oracle_mod.step(params, pos, vel, 2, keys_state=keys)
    p, v, _ = oracle_mod.step(params, p, v, 2, paused=True, keys_state=keys)
    p, v, pr = oracle_mod.step(params, p, v, 1, keys_state=keys)
    assert_same("pos", gp, p)
    assert_same("vel", gv, v)
    assert_same("pred", gpr, pr)


def test_rollout_300_frames_bit_exact(pbf_mod, oracle_mod, cuda_device):
    """The 32,768-particle dam break for 300 frames (600 substeps): identical
    to the oracle at every checkpoint, with density error and energy stated."""
    params, pos, vel = pbf_mod.make_scene("dam_break_32k")
    checkpoints = [2, 20, 200, 600]
    with pbf_mod.Simulation.create(params, pos, vel, device=cuda_device) as sim:
        op, ov = pos, vel
        done = 0
        for cp in checkpoints:
            sim.Step(cp - done)
            op, ov, opr = oracle_mod.step(params, op, ov, cp - done)
            done = cp
            gp, gv, gpr = sim.read_state()
            assert_same(f"pos@{cp}", gp, op)
            assert_same(f"vel@{cp}", gv, ov)
            assert_same(f"pred@{cp}", gpr, opr)
            rho = gpr[:, 3]
            ok = np.isfinite(gp).all(axis=1) & np.isfinite(gv).all(axis=1) & np.isfinite(rho)
            err = np.abs(rho[ok] / params.restDensity - 1.0)
            ke = 0.5 * np.sum(gv[ok, :3].astype(np.float64) ** 2)
            pe = params.garvity * np.sum(gp[ok, 1].astype(np.float64))
            print(f"substep {cp}: density error mean {err.mean():.4f} max {err.max():.3f}; "
                  f"kinetic {ke:.2f} potential {pe:.2f}; non-finite {int((~ok).sum())}")
            assert ok.all(), "the guarded scene keeps every particle finite"


def test_one_substep_at_1m_bit_exact_and_fp64_error(pbf_mod, oracle_mod, cuda_device):
    """1,048,576 particles: one substep bit-exact against the FP32 oracle; the
    max error against the FP64 oracle is stated."""
    params, pos, vel = pbf_mod.make_scene("dam_break_1m")
    gp, gv, gpr, _, _ = run_gpu(pbf_mod, params, pos, vel, 1, cuda_device, friends=False)
    op, ov, opr = oracle_mod.step(params, pos, vel, 1)
    assert_same("pos", gp, op)
    assert_same("vel", gv, ov)
    assert_same("pred", gpr, opr)
    dp, dv, _ = oracle_mod.step_f64(params, pos, vel, 1)
    for name, g, d in (("pos", gp, dp), ("vel", gv, dv)):
        err = np.abs(g[:, :3].astype(np.float64) - d[:, :3])
        rel = err.max() / np.abs(d[:, :3]).max()
        print(f"1M, one substep, {name}: max |fp32 - fp64| = {err.max():.3e} (relative {rel:.3e})")


def test_stage_timings_and_launch_count(pbf_mod, cuda_device):
    params, pos, vel = scene(pbf_mod, (16, 16, 16))
    with pbf_mod.Simulation.create(params, pos, vel, device=cuda_device) as sim:
        sim.enable_stage_timing(True)
        sim.Step(1)
        t = sim.stage_timings()
        for name in ("predictPositions", "radixsort", "sortParticles", "updateCells", "buildFriendsList",
                     "computeScaling", "computeDelta", "updateVelocities", "applyViscosity", "applyVorticity"):
            assert name in t and t[name] >= 0.0
        assert sim.launch_count() > 0


def test_argument_errors(pbf_mod, cuda_device):
    params, pos, vel = scene(pbf_mod, (8, 8, 8))
    with pbf_mod.Simulation.create(params, pos, vel, device=cuda_device) as sim:
        bad = params.copy()
        bad.particleCount = 999
        with pytest.raises(pbf_mod.PbfError):
            sim.set_params(bad)
        bad = params.copy()
        bad.friendsCircles = 9
        with pytest.raises(pbf_mod.PbfError):
            sim.set_params(bad)
        with pytest.raises(pbf_mod.PbfError) as e:
            sim.LoadForceMasks(np.ones((0, 4), np.uint32))  # an empty image
        assert e.value.code == pbf_mod.PBF_ERR_INVALID
        with pytest.raises(pbf_mod.PbfError):
            sim.set_wave_position(-1.0)
    s = pbf_mod.Simulation(params, cuda_device)
    with pytest.raises(pbf_mod.PbfError) as e:
        s.Step(1)
    assert e.value.code == pbf_mod.PBF_ERR_STATE
    s.close()


def test_force_planes_match_reference_digests(pbf_mod, cuda_device):
    """The reference's 14 force planes as data (pbf_set_force_quads) with a
    mask (pbf_load_force_masks): bit-exact against the reference's own
    computeDelta with its hard-coded planes."""
    manifest = json.loads((GOLDEN / "golden.json").read_text())
    force = manifest["force_planes"]
    params, pos, vel = mg().force_scene()
    quads = mg().quads_array(force["quads"])
    with pbf_mod.Simulation(params, cuda_device) as sim:
        sim.InitBuffers(pos, vel)
        sim.InitCells()
        sim.LoadForceMasks(mg().force_mask(force["mask"]))
        sim.InitKernels()
        sim.set_force_quads(quads)
        sim.Step(force["substeps"])
        p, v, pr = sim.read_state()
        sim.set_force_quads(None)   # removing the planes restores the plain path
        with pytest.raises(pbf_mod.PbfError):
            sim.set_force_quads(np.zeros(65, pbf_mod.QUAD_DTYPE))
    for name, arr in (("pos", p), ("vel", v), ("pred", pr)):
        assert mg().digest(arr) == force["sha256"][name], name


def test_rollout_1m_100_frames_bit_exact(pbf_mod, oracle_mod, cuda_device):
    """The 1,048,576-particle dam break for 100 frames (200 substeps) on the
    GPU and in the oracle: identical state at the end."""
    params, pos, vel = pbf_mod.make_scene("dam_break_1m")
    with pbf_mod.Simulation.create(params, pos, vel, device=cuda_device) as sim:
        sim.autotune(trial_substeps=1)  # any launch shape gives the same bits
        sim.Step(200)
        gp, gv, gpr = sim.read_state()
    op, ov, opr = oracle_mod.step(params, pos, vel, 200)
    assert_same("pos", gp, op)
    assert_same("vel", gv, ov)
    assert_same("pred", gpr, opr)
    rho = gpr[:, 3].astype(np.float64) / params.restDensity - 1.0
    print(f"1M after 200 substeps: density error mean {np.abs(rho).mean():.4f}, "
          f"kinetic {0.5 * np.sum(gv[:, :3].astype(np.float64) ** 2):.1f}")


@pytest.mark.parametrize("algorithm", [0, 2], ids=["scan", "brick"])
def test_complete_neighbours_bit_exact(pbf_mod, oracle_mod, cuda_device, algorithm):
    """completeNeighbours 1 (every friend circle in every pass, self in the
    density): GPU and oracle agree bit for bit, and the rule does change the
    result against the reference's truncated sets."""
    params, pos, vel = scene(pbf_mod, (24, 24, 24))
    params.completeNeighbours = 1
    gp, gv, gpr, _, _ = run_gpu(pbf_mod, params, pos, vel, 4, cuda_device, algorithm=algorithm)
    op, ov, opr = oracle_mod.step(params, pos, vel, 4)
    assert_same("pos", gp, op)
    assert_same("vel", gv, ov)
    assert_same("pred", gpr, opr)
    params.completeNeighbours = 0
    rp, _, _ = oracle_mod.step(params, pos, vel, 4)
    assert not np.array_equal(rp, op)
    with pbf_mod.Simulation.create(params, pos, vel, device=cuda_device) as sim:
        p2 = params.copy()
        p2.completeNeighbours = 1
        sim.set_params(p2)
        with pytest.raises(pbf_mod.PbfError):
            sim.rollout_forward(2, 1)  # rollouts follow the reference's sets
