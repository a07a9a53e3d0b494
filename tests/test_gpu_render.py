"""The headless renderer (pbf_render_frame) against the oracle's
restatement of the reference's particle shaders (needs a GPU): splat,
smoothed depth and final images bit for bit (NaN compared as NaN: the
smoothing shader divides by a zero gradient on background pixels, as in
the reference)."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _canon(a):
    a = np.array(a, np.float32, copy=True)
    a[np.isnan(a)] = np.float32("nan")
    a.view(np.uint32)[np.isnan(a)] = 0x7FC00000
    return a.view(np.uint32)


def _coarse_scene(pbf_mod):
    """The reference's scene scale (dam_coarse: smoothing length 2, spacing
    0.55), where the smoothing shader's target density 1 is a surface."""
    params = pbf_mod.load_scenario("dam_break_32k")
    params.h, params.h_2 = 2.0, 4.0
    pos = pbf_mod.scene_block(16, 16, 16, 0.55, (0.3, 0.3, 0.3), 0.05, 7)
    params.particleCount = len(pos)
    pos[:, 3] = np.linspace(0.0, 40.0, len(pos), dtype=np.float32)  # speeds for the colour mode
    return params, pos


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_render_matches_oracle(pbf_mod, oracle_mod, cuda_device, mode):
    params, pos = _coarse_scene(pbf_mod)
    cam = pbf_mod.render_camera((4.4, 8.0, 30.0), (4.4, 4.0, 4.4), (0.0, 1.0, 0.0), 45.0, 160, 120, 1.0)
    with pbf_mod.Simulation.create(params, pos, np.zeros_like(pos), device=cuda_device) as sim:
        sim.render_frame(cam, mode)
        out, splat = sim.render_read(cam, 0), sim.render_read(cam, 1)
        smooth = sim.render_read(cam, 2) if mode == 0 else None
    osplat, osmooth, oout = oracle_mod.render(cam, mode, params, pos)
    assert np.array_equal(_canon(splat), _canon(osplat)), "splat"
    if mode == 0:
        assert np.array_equal(_canon(smooth), _canon(osmooth)), "smoothed depth"
    assert np.array_equal(_canon(out), _canon(oout)), "frame"
    covered = (splat[..., 1] > 0) if mode == 0 else (splat[..., 3] > 0)
    assert 0.05 < covered.mean() < 0.9


def test_render_after_steps_matches_oracle(pbf_mod, oracle_mod, cuda_device):
    """The dam break stepped on the GPU, then rendered from its positions."""
    params, pos, vel = pbf_mod.make_scene("dam_break_32k")
    cam = pbf_mod.render_camera((1.6, 1.2, 5.0), (1.0, 0.4, 0.8), (0.0, 1.0, 0.0), 45.0, 128, 96, 0.03)
    with pbf_mod.Simulation.create(params, pos, vel, device=cuda_device) as sim:
        sim.Step(20)
        p, _, _ = sim.read_state()
        sim.render_frame(cam, 0)
        out = sim.render_read(cam, 0)
        with pytest.raises(pbf_mod.PbfError):
            sim.render_frame(cam, 3)
    _, _, oout = oracle_mod.render(cam, 0, params, p)
    assert np.array_equal(_canon(out), _canon(oout))


def test_render_read_needs_a_frame(pbf_mod, cuda_device):
    params, pos = _coarse_scene(pbf_mod)
    cam = pbf_mod.render_camera((4.4, 8.0, 30.0), (4.4, 4.0, 4.4), (0.0, 1.0, 0.0), 45.0, 32, 24, 1.0)
    with pbf_mod.Simulation.create(params, pos, np.zeros_like(pos), device=cuda_device) as sim:
        with pytest.raises(pbf_mod.PbfError):
            sim.render_read(cam, 0)
