"""Batched scenes: many dam breaks advanced together, every stage one launch
over all of them.  Each scene's result must be bit-identical to running that
scene alone with the same gridBufSize; the autotuner must not change results."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _same(a, b):
    a = a.copy(); b = b.copy()
    a[np.isnan(a)] = 0; b[np.isnan(b)] = 0
    return np.array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.mark.parametrize("contract", [{}, {"relaxedMath": 1}, {"completeNeighbours": 1}],
                         ids=["exact", "relaxed", "complete"])
def test_batch_equals_scenes_run_alone(pbf_mod, cuda_device, contract):
    """Under every arithmetic contract and neighbour rule, each scene of a
    batch is bit-identical to the same scene run alone."""
    scenes, positions = pbf_mod.make_batch_scenes(first=12)
    for p in scenes:
        for k, v in contract.items():
            setattr(p, k, v)
    pos = np.concatenate(positions)
    with pbf_mod.Simulation.create(scenes, pos, np.zeros_like(pos), device=cuda_device) as sim:
        offs = sim.scene_offsets()
        assert list(np.diff(offs)) == [p.particleCount for p in scenes]
        sim.Step(3)
        bp, bv, bpr = sim.read_state()
    for s, (p, x) in enumerate(zip(scenes, positions)):
        with pbf_mod.Simulation.create(p, x, np.zeros_like(x), device=cuda_device) as one:
            one.Step(3)
            op, ov, opr = one.read_state()
        sl = slice(int(offs[s]), int(offs[s + 1]))
        assert _same(bp[sl], op) and _same(bv[sl], ov) and _same(bpr[sl], opr), f"scene {s}"


def test_batch_matches_oracle_per_scene(pbf_mod, oracle_mod, cuda_device):
    scenes, positions = pbf_mod.make_batch_scenes(first=4)
    pos = np.concatenate(positions)
    with pbf_mod.Simulation.create(scenes, pos, np.zeros_like(pos), device=cuda_device) as sim:
        offs = sim.scene_offsets()
        sim.Step(2)
        bp, bv, _ = sim.read_state()
    for s, (p, x) in enumerate(zip(scenes, positions)):
        op, ov, _ = oracle_mod.step(p, x, np.zeros_like(x), 2)
        sl = slice(int(offs[s]), int(offs[s + 1]))
        assert _same(bp[sl], op) and _same(bv[sl], ov), f"scene {s}"


def test_autotune_keeps_results_and_state(pbf_mod, cuda_device):
    scenes, positions = pbf_mod.make_batch_scenes(first=16)
    pos = np.concatenate(positions)
    with pbf_mod.Simulation.create(scenes, pos, np.zeros_like(pos), device=cuda_device) as a, \
         pbf_mod.Simulation.create(scenes, pos, np.zeros_like(pos), device=cuda_device) as b:
        a.Step(1)
        b.Step(1)
        blocks = b.autotune(trial_substeps=1)
        assert b.launch_shape() == blocks and all(x in (64, 128, 256, 512) for x in blocks[:5])
        assert blocks[5] in (0, 1, 2) and blocks[6] in (0, 1) and blocks[7] in (0, 1)
        a.Step(2)
        b.Step(2)
        for x, y in zip(a.read_state(), b.read_state()):
            assert _same(x, y)
        assert np.array_equal(a.read_ids(), b.read_ids())  # the trials' permutations are undone too
        b.set_launch_shape([96, 160, 224, 288, 352, (blocks[5] + 1) % 3, 1 - blocks[6], 1 - blocks[7]])  # another shape
        b.Step(1)
        a.Step(1)
        for x, y in zip(a.read_state(), b.read_state()):
            assert _same(x, y)


def test_batch_step_read_async_matches_step_then_read(pbf_mod, cuda_device):
    """The overlapped step-and-read-back on a batch: the same state as
    stepping and reading after, frame by frame, with the read graph reused."""
    torch = pytest.importorskip("torch")
    scenes, positions = pbf_mod.make_batch_scenes(first=8)
    pos = np.concatenate(positions)
    n = len(pos)
    hp = torch.empty((n, 4), dtype=torch.float32).pin_memory()
    hv = torch.empty((n, 4), dtype=torch.float32).pin_memory()
    with pbf_mod.Simulation.create(scenes, pos, np.zeros_like(pos), device=cuda_device) as a, \
         pbf_mod.Simulation.create(scenes, pos, np.zeros_like(pos), device=cuda_device) as b:
        for _ in range(3):
            a.Step(2)
            pa, va, _ = a.read_state()
            b.step_read_async(2, hp.data_ptr(), hv.data_ptr())
            b.synchronize()
            assert _same(pa, hp.numpy()) and _same(va, hv.numpy())


def test_batch_rejects_incompatible_scenes(pbf_mod, cuda_device):
    scenes, _ = pbf_mod.make_batch_scenes(first=2)
    scenes[1].epsilon = 123.0
    with pytest.raises(pbf_mod.PbfError) as e:
        pbf_mod.Simulation(scenes, cuda_device)
    assert "scene 1" in str(e.value)
