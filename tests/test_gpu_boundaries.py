"""Boundaries and state files beyond the reference's fixed scene (needs a
GPU): the wave generator's moving wall and the binary state file, each
against the oracle / the uninterrupted run, bit for bit."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _same(a, b):
    return np.array_equal(np.ascontiguousarray(a).view(np.uint32), np.ascontiguousarray(b).view(np.uint32))


def test_wave_wall_matches_oracle(pbf_mod, oracle_mod, cuda_device):
    """The box clamp's low x wall at xMin + wavePos, moved between frames as
    the reference's Runner computes it (src/Runner.cpp:100-116)."""
    params, pos, vel = pbf_mod.make_scene("dam_break_32k")
    params.waveGenAmp, params.waveGenFreq, params.waveGenDuty = 0.05, 1.0, 1.0
    frames, sub = 12, int(params.subSteps)
    walls = [pbf_mod.wave_position(params, 0.25 + f * params.timeStep) for f in range(frames)]
    assert max(walls) > 0.05
    op, ov = pos, vel
    with pbf_mod.Simulation.create(params, pos, vel, device=cuda_device) as sim:
        try:
            for w in walls:
                sim.set_wave_position(w)
                sim.Step(sub)
                oracle_mod.set_wave_position(w)
                op, ov, _ = oracle_mod.step(params, op, ov, sub)
        finally:
            oracle_mod.set_wave_position(0.0)
        gp, gv, _ = sim.read_state()
    assert _same(gp, op) and _same(gv, ov)
    assert gp[:, 0].min() >= params.xMin + walls[-1]


def test_state_file_round_trip(pbf_mod, cuda_device, tmp_path):
    """Save mid-run, keep stepping; a second context loads the file and
    steps the same substeps: identical state and particle ids."""
    params, pos, vel = pbf_mod.make_scene("dam_break_32k")
    path = tmp_path / "state.pbfstate"
    with pbf_mod.Simulation.create(params, pos, vel, device=cuda_device) as a:
        a.Step(10)
        a.save_state(path)
        a.Step(7)
        pa, va, _ = a.read_state()
        ia = a.read_ids()
    with pbf_mod.Simulation.create(params, np.zeros_like(pos), None, device=cuda_device) as b:
        b.load_state(path)
        b.Step(7)
        pb, vb, _ = b.read_state()
        ib = b.read_ids()
    assert _same(pa, pb) and _same(va, vb)
    np.testing.assert_array_equal(ia, ib)
    small, spos, svel = pbf_mod.make_scene("dam_break_32k")
    small.particleCount = 4096
    with pbf_mod.Simulation.create(small, spos[:4096], svel[:4096], device=cuda_device) as c:
        with pytest.raises(pbf_mod.PbfError):
            c.load_state(path)              # another particle count
        (tmp_path / "junk").write_bytes(b"not a state file")
        with pytest.raises(pbf_mod.PbfError):
            c.load_state(tmp_path / "junk")


def test_perf_trackers_follow_the_reference_monitor(pbf_mod, cuda_device):
    """Trackers named as OCLPerfMon names them, smoothed with weight 0.5
    (src/OCLPerfMon.cpp:33-49), exported as JSON for dashboards."""
    import json
    params, pos, vel = pbf_mod.make_scene("dam_break_32k")
    with pbf_mod.Simulation.create(params, pos, vel, device=cuda_device) as sim:
        sim.enable_stage_timing(True)
        sim.Step(1)
        first = {t[0]: t for t in sim.perf_trackers()}
        sim.Step(1)
        second = sim.perf_trackers()
        doc = json.loads(sim.perf_json())
    iters = int(params.simIterations)
    names = [t[0] for t in second]
    want = (["predictPositions", "radixsort", "sortParticles", "updateCells", "buildFriendsList", "resetPartList"] +
            [x for i in range(iters) for x in (f"computeScaling_{i}", f"computeDelta_{i}")] +
            ["updateVelocities", "applyViscosity", "applyVorticity"])
    assert names == want
    for name, start, end, total, last in second:
        assert end >= start and total > 0 and total == last
        assert end > first[name][2]                     # timestamps advance
        # total = 0.5 * current + 0.5 * previous, with current >= 0
        assert total >= 0.5 * first[name][3] - 1e-9
    assert [t["eventName"] for t in doc["trackers"]] == want
    assert abs(doc["total_time"] - sum(t[3] for t in second)) < 1e-3


def test_async_state_copies_match_sync(pbf_mod, cuda_device):
    """write_state_async / step_async / read_state_async / synchronize gives
    the frames the synchronous calls give."""
    torch = pytest.importorskip("torch")
    params, pos, vel = pbf_mod.make_scene("dam_break_32k")
    n = len(pos)
    hp = torch.from_numpy(pos.copy()).pin_memory()
    hv = torch.zeros((n, 4), dtype=torch.float32).pin_memory()
    with pbf_mod.Simulation.create(params, pos, vel, device=cuda_device) as a, \
         pbf_mod.Simulation.create(params, pos, vel, device=cuda_device) as b:
        p, v = pos.copy(), vel.copy()
        for _ in range(3):
            a.write_state(p, v)
            a.Step(2)
            p, v, _ = a.read_state()
            b.write_state_async(hp.data_ptr(), hv.data_ptr())
            b.step_async(2)
            b.read_state_async(hp.data_ptr(), hv.data_ptr())
            b.synchronize()
        assert _same(p, hp.numpy()) and _same(v, hv.numpy())


@pytest.mark.parametrize("mode", ["graph", "eager", "pageable", "paused", "stage_timing"])
def test_step_read_async_matches_step_then_read(pbf_mod, cuda_device, mode):
    """pbf_step_read_async (the position copy overlapping the last substep's
    XSPH and vorticity) against pbf_step + pbf_read_state, frame by frame:
    page-locked buffers replay a captured substep with its copies (swapping
    the buffers recaptures it); pageable buffers, graphs off, a paused
    simulation and stage timing take the eager path.  The launch count grows
    as pbf_step_async's does, plus one: the read-back substep runs its
    vorticity pass in two launches, so that the first half's velocities copy
    out while the second half runs (stage timing reads back after the step,
    with one launch)."""
    torch = pytest.importorskip("torch")
    params, pos, vel = pbf_mod.make_scene("dam_break_32k")
    n = len(pos)
    if mode == "pageable":
        bufs = [(np.empty((n, 4), np.float32), np.empty((n, 4), np.float32)) for _ in range(2)]
        ptrs = [(p.ctypes.data, v.ctypes.data) for p, v in bufs]
        views = [(p, v) for p, v in bufs]
    else:
        bufs = [(torch.empty((n, 4), dtype=torch.float32).pin_memory(),
                 torch.empty((n, 4), dtype=torch.float32).pin_memory()) for _ in range(2)]
        ptrs = [(p.data_ptr(), v.data_ptr()) for p, v in bufs]
        views = [(p.numpy(), v.numpy()) for p, v in bufs]
    with pbf_mod.Simulation.create(params, pos, vel, device=cuda_device) as a, \
         pbf_mod.Simulation.create(params, pos, vel, device=cuda_device) as b:
        for sim in (a, b):
            if mode == "eager":
                sim.use_graph(False)
            if mode == "paused":
                sim.bPauseSim = True
            if mode == "stage_timing":
                sim.enable_stage_timing(True)
        for frame, (sub, k) in enumerate([(1, 0), (2, 0), (2, 0), (3, 1), (2, 0)]):
            la, lb = a.launch_count(), b.launch_count()
            a.step_async(sub)
            a.synchronize()
            pa, va, _ = a.read_state()
            b.step_read_async(sub, *ptrs[k])
            b.synchronize()
            assert _same(pa, views[k][0]) and _same(va, views[k][1]), f"frame {frame}"
            assert b.launch_count() - lb == a.launch_count() - la + (0 if mode == "stage_timing" else 1)
        pb, vb, _ = b.read_state()
        assert _same(pa, pb) and _same(va, vb)
        b.step_read_async(1, ptrs[0][0], None)  # positions only
        a.Step(1)
        b.synchronize()
        assert _same(a.read_state()[0], views[0][0])
        with pytest.raises(pbf_mod.PbfError):
            b.step_read_async(0, *ptrs[0])


def test_non_finite_injection_matches_oracle(pbf_mod, oracle_mod, cuda_device):
    """A NaN and an infinite particle written into the state: the pipeline
    runs on, identically to the oracle (NaN compared as NaN), and the error
    word stays clear (NaN positions hash to a valid cell)."""
    params, pos, vel = pbf_mod.make_scene("dam_break_32k")
    pos = pos.copy()
    pos[100, 0] = np.float32("nan")
    pos[2000, 1] = np.float32("inf")
    with pbf_mod.Simulation.create(params, pos, vel, device=cuda_device) as sim:
        sim.Step(3)
        gp, gv, gpr = sim.read_state()
    op, ov, opr = oracle_mod.step(params, pos, vel, 3)

    def canon(a):
        a = np.array(a, np.float32, copy=True)
        a.view(np.uint32)[np.isnan(a)] = 0x7FC00000
        return a.view(np.uint32)
    assert np.array_equal(canon(gp), canon(op)) and np.array_equal(canon(gv), canon(ov))
    assert np.isnan(gp).any()


class _DeviceArray:
    """A device buffer described by the CUDA array interface (no copy)."""

    def __init__(self, ptr: int, n: int):
        self.__cuda_array_interface__ = {"shape": (n, 4), "typestr": "<f4", "data": (ptr, False),
                                         "strides": None, "version": 2}


def test_device_positions_stream_and_nvtx(pbf_mod, cuda_device):
    """pbf_device_positions hands out the current position buffer (the headless
    stand-in for the GL buffer the reference shares with its renderer); work
    queued on the library's stream (pbf_get_stream) after an asynchronous step
    sees the stepped positions without a wait; NVTX ranges around the stages
    change nothing."""
    torch = pytest.importorskip("torch")
    params, pos, vel = pbf_mod.make_scene("dam_break_32k")
    n = int(params.particleCount)
    dev = torch.device("cuda", cuda_device)
    with pbf_mod.Simulation.create(params, pos, vel, device=cuda_device) as a, \
         pbf_mod.Simulation.create(params, pos, vel, device=cuda_device) as b:
        a.step_async(3)
        stream = torch.cuda.ExternalStream(a.stream(), device=dev)
        with torch.cuda.stream(stream):
            view = torch.as_tensor(_DeviceArray(a.device_positions(), n), device=dev)
            copy = view.clone()  # ordered after the step on the library's stream
        stream.synchronize()
        p, _, _ = a.read_state()
        assert _same(copy.cpu().numpy(), p)
        # eager steps with and without NVTX ranges
        a.use_graph(False)
        b.use_graph(False)
        b.Step(3)
        b.enable_nvtx(True)
        a.Step(2)
        b.Step(2)
        for x, y in zip(a.read_state(), b.read_state()):
            assert _same(x, y)
