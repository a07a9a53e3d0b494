"""Seeded random configurations, each stepped on the GPU and by the oracle and
compared bit for bit (needs a GPU).  Every draw varies everything at once:
lattice size and spacing, h, the hash-grid size (collisions included), friend
circles and their limit, iterations, substeps, box clamp, zero-distance guard,
complete neighbour sets, a gravity vector, random initial velocities, the
friends algorithm and the solver thread map."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SEEDS = list(range(48))


def _canonical(a):
    a = np.array(a, np.float32, copy=True)
    a[np.isnan(a)] = np.float32("nan")  # one NaN pattern: payloads differ between CPU and GPU
    return a.view(np.uint32)


def draw(pbf, seed):
    rng = np.random.default_rng(1000 + seed)
    params = pbf.load_scenario("dam_break_32k")
    dims = tuple(int(x) for x in rng.integers(1, 21, 3))
    spacing = float(rng.uniform(0.035, 0.065))
    h = np.float32(rng.uniform(0.07, 0.16))
    params.h = float(h)
    params.h_2 = float(h * h)
    params.gridBufSize = int(rng.choice([64, 100, 1000, 4096, 1 << 15, 1 << 19]))
    params.friendsCircles = int(rng.integers(1, 9))
    params.particlesPerCircle = int(rng.integers(1, 65))
    params.simIterations = int(rng.integers(0, 6))
    params.boxClamp = int(rng.integers(0, 2))
    params.zeroDistanceGuard = int(rng.integers(0, 2))
    params.completeNeighbours = int(rng.integers(0, 2))
    if rng.integers(0, 2):
        params.gravityVectorEnable = 1
        g = rng.normal(0.0, 1.0, 3)
        params.gravityX, params.gravityY, params.gravityZ = (float(x) for x in 9.8 * g / np.linalg.norm(g))
    params.particleCount = dims[0] * dims[1] * dims[2]
    pos = pbf.scene_block(*dims, spacing, (0.025,) * 3, float(rng.uniform(0.0, 0.01)), int(rng.integers(1 << 30)))
    vel = np.zeros_like(pos)
    vel[:, :3] = rng.normal(0.0, 0.5, (len(pos), 3)).astype(np.float32)
    substeps = int(rng.integers(1, 4))
    algorithm = int(rng.integers(0, 3))
    balance = int(rng.integers(0, 2))
    return params, pos, vel, substeps, algorithm, balance


@pytest.mark.parametrize("seed", SEEDS)
def test_random_configuration_bit_exact(seed, pbf_mod, oracle_mod, cuda_device):
    params, pos, vel, substeps, algorithm, balance = draw(pbf_mod, seed)
    with pbf_mod.Simulation.create(params, pos, vel, device=cuda_device) as sim:
        sim.set_launch_shape(sim.launch_shape()[:5] + [algorithm, balance])
        sim.Step(substeps)
        gp, gv, gpr = sim.read_state()
    op, ov, opr = oracle_mod.step(params, pos, vel, substeps)
    for name, g, o in (("pos", gp, op), ("vel", gv, ov), ("pred", gpr, opr)):
        bad = int(np.sum(_canonical(g) != _canonical(o)))
        assert bad == 0, (f"seed {seed}: {name} differs in {bad} words "
                          f"(N {params.particleCount}, grid {params.gridBufSize}, circles {params.friendsCircles}x"
                          f"{params.particlesPerCircle}, iterations {params.simIterations}, algorithm {algorithm})")


@pytest.mark.parametrize("seed", SEEDS)
def test_random_configuration_relaxed_within_tolerance(seed, pbf_mod, oracle_mod, cuda_device):
    """relaxedMath 1 on the same draws, one substep: positions within 1e-5
    relative (max |gpu - exact| / max |exact|) of the exact oracle."""
    params, pos, vel, _, algorithm, balance = draw(pbf_mod, seed)
    params.relaxedMath = 1
    with pbf_mod.Simulation.create(params, pos, vel, device=cuda_device) as sim:
        sim.set_launch_shape(sim.launch_shape()[:5] + [algorithm, balance])
        sim.Step(1)
        gp, _, _ = sim.read_state()
    exact = params.copy()
    exact.relaxedMath = 0
    op, _, _ = oracle_mod.step(exact, pos, vel, 1)
    g, o = gp[:, :3].astype(np.float64), op[:, :3].astype(np.float64)
    finite = np.isfinite(o).all(axis=1)
    assert np.array_equal(finite, np.isfinite(g).all(axis=1)), f"seed {seed}: non-finite positions differ"
    if finite.any():
        rel = np.max(np.abs(g[finite] - o[finite])) / max(np.max(np.abs(o[finite])), 1e-30)
        print(f"seed {seed}: relaxed vs exact, one substep: {rel:.2e}")
        assert rel < 1e-5, f"seed {seed}: {rel:.2e}"
