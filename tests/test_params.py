"""Parameters, the `.par` loader and the scene generators (host code, CPU only)."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest


def test_prefix_layout_matches_reference_struct(pbf_mod):
    """PbfParameters keeps src/Parameters.hpp:5-56 byte for byte as its prefix."""
    P = pbf_mod.PbfParameters
    names = [f for f, _ in P._fields_]
    ref_order = ["resetSimOnChange", "particleCount", "xMin", "xMax", "yMin", "yMax", "zMin", "zMax",
                 "waveGenAmp", "waveGenFreq", "waveGenDuty", "timeStep", "simIterations", "subSteps", "h",
                 "restDensity", "epsilon", "garvity", "vorticityFactor", "viscosityFactor", "surfaceTenstionK",
                 "surfaceTenstionDist", "friendsCircles", "particlesPerCircle", "gridBufSize", "setupSpacing",
                 "segmentSize", "sortIterations", "particleRenderSize", "h_2", "EnableCachedBuffers"]
    assert names[:len(ref_order)] == ref_order
    for k, name in enumerate(ref_order[:-1]):
        assert getattr(P, name).offset == 4 * k
    assert P.EnableCachedBuffers.offset == 120
    assert P.gravityVectorEnable.offset == 124  # appended after the reference's 124-byte struct


def test_loader_semantics(pbf_mod):
    text = ("# comment line\n"
            "ParticleCount 1234   # trailing comment\n"
            "SMOOTHLEN 0.2\n"
            "Garvity 3.5\n"
            "NoSuchKey 7\n"
            "   \n"
            "GridBufferSize 4096\n"
            "GravityY -2.0\n"
            "BoxClamp 1\n")
    p = pbf_mod.load_parameters(text)
    assert p.particleCount == 1234
    assert p.h == pytest.approx(0.2)
    assert p.h_2 == np.float32(np.float32(0.2) * np.float32(0.2))
    assert p.garvity == pytest.approx(3.5)
    assert p.friendsCircles == 5 and p.particlesPerCircle == 50
    assert p.gridBufSize == 4096
    assert p.gravityVectorEnable == 1 and p.gravityY == pytest.approx(-2.0)
    assert p.boxClamp == 1
    assert p._unknown_keys == 1


def test_loader_keeps_unset_fields_and_drops_unterminated_last_line(pbf_mod):
    base = pbf_mod.load_parameters("RestDensity 100\n")
    p = pbf_mod.load_parameters("Epsilon 5\nViscosityFactor 0.5", base)  # no trailing newline
    assert p.restDensity == pytest.approx(100.0)   # kept from base
    assert p.epsilon == pytest.approx(5.0)
    assert p.viscosityFactor == 0.0                # last line dropped, as src/ParamUtils.cpp:34-38


def test_bundled_scenarios(pbf_mod):
    for name in pbf_mod.SCENES:
        params, pos, vel = pbf_mod.make_scene(name)
        n = params.particleCount
        assert pos.shape == (n, 4) and vel.shape == (n, 4)
        lo = np.array([params.xMin, params.yMin, params.zMin], np.float32)
        hi = np.array([params.xMax, params.yMax, params.zMax], np.float32)
        assert np.all(pos[:, :3] > lo) and np.all(pos[:, :3] < hi)
        assert params.boxClamp == 1 and params.simIterations == 4 and params.subSteps == 2
        # the hash range covers every cell of the box: no modulo collisions
        cells = np.ceil((hi - lo) / params.h).astype(int)
        bits = sum(int(np.ceil(np.log2(c))) for c in cells)
        assert (1 << bits) <= params.gridBufSize


def test_scene_block_is_deterministic(pbf_mod):
    a = pbf_mod.scene_block(4, 3, 2, 0.05, (0.1, 0.2, 0.3), 0.005, 99)
    b = pbf_mod.scene_block(4, 3, 2, 0.05, (0.1, 0.2, 0.3), 0.005, 99)
    c = pbf_mod.scene_block(4, 3, 2, 0.05, (0.1, 0.2, 0.3), 0.005, 100)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    lattice = pbf_mod.scene_block(4, 3, 2, 0.05, (0.1, 0.2, 0.3), 0.0, 99)
    assert np.all(np.abs(a - lattice)[:, :3] <= 0.005 + 1e-7)
    f64 = lambda v: np.float64(np.float32(v))  # float arguments, promoted to double
    assert lattice[1, 0] == np.float32(f64(0.1) + 1 * f64(0.05))
    assert lattice[4, 1] == np.float32(f64(0.2) + 1 * f64(0.05))
    assert lattice[12, 2] == np.float32(f64(0.3) + 1 * f64(0.05))


def test_reference_lattice(pbf_mod):
    """Simulation::CreateParticles (src/Simulation.cpp:71-101)."""
    p = pbf_mod.load_parameters("ParticleCount 30\nSmoothLen 2.0\nSetupSpacing 0.55\n")
    pos = pbf_mod.reference_lattice(p)
    per_axis = 4  # ceil(cbrt(30))
    d = np.float32(np.float32(2.0) * np.float32(0.55))
    off = np.float32((np.float32(1.0) - np.float32(per_axis) * d) / np.float32(2.0))
    for i in (0, 1, 5, 17, 29):
        x, y, z = (i // per_axis) % per_axis, i % per_axis, (i // per_axis ** 2) % per_axis
        assert pos[i, 0] == np.float32(off + np.float32(x) * d)
        assert pos[i, 1] == np.float32(np.float32(0.3) + np.float32(y) * d)
        assert pos[i, 2] == np.float32(off + np.float32(z) * d)


def test_constants_follow_reference_literals(pbf_mod, oracle_mod):
    """POLY6 / GRAD_SPIKY go through a 6-significant-digit text round trip
    (src/Simulation.cpp:167,179-180)."""
    p = pbf_mod.load_scenario("dam_break_32k")
    poly6, grad, poly6q = oracle_mod.constants(p)
    h = float(np.float32(0.1))
    assert poly6 == np.float32(float("%.6g" % (315.0 / (64.0 * np.pi * h ** 9))))
    assert grad == np.float32(float("%.6g" % (45.0 / (np.pi * h ** 6))))
    qh = np.float32(np.float32(0.2) * np.float32(0.1))
    d = np.float32(p.h_2 - np.float32(float(qh) * float(qh)))
    assert poly6q == np.float32(float(d) ** 3)


def test_wave_position_follows_the_runner_formula(pbf_mod):
    """pbf_wave_position: (1 - cos(2 pi fmod(f t, 1)^duty)) amp (xMax - xMin) / 2
    (src/Runner.cpp:103-107)."""
    import math
    p = pbf_mod.load_scenario("dam_break_32k")
    p.waveGenAmp, p.waveGenFreq, p.waveGenDuty = 0.2, 0.7, 1.5
    for t in (0.0, 0.3, 1.1, 2.9):
        want = (1 - math.cos(2 * math.pi * math.fmod(0.7 * float(np.float32(t)), 1.0) ** 1.5)) * \
            0.2 * (p.xMax - p.xMin) / 2
        assert abs(pbf_mod.wave_position(p, t) - want) <= 1e-6 * max(1.0, abs(want))


def test_scene_keys(pbf_mod):
    """BlockDims / BlockOrigin / Jitter / Seed: read by pbf_load_scene, skipped
    silently by the parameter loader, and the bundled scenes come from them."""
    text = "SmoothLen 0.1\nSetupSpacing 0.5\nBlockDims 4 3 2\nBlockOrigin 0.1 0.2 0.3\nJitter 0.001\nSeed 7\n"
    s = pbf_mod.load_scene(text)
    assert list(s.blockDims) == [4, 3, 2] and s.seed == 7
    assert abs(s.jitter - 0.001) < 1e-9 and abs(s.blockOrigin[2] - 0.3) < 1e-7
    params = pbf_mod.load_parameters(text)
    pos = pbf_mod.scene_positions(params, s)
    want = pbf_mod.scene_block(4, 3, 2, 0.05, (0.1, 0.2, 0.3), 0.001, 7)
    assert np.array_equal(pos, want)
    with pytest.raises(pbf_mod.PbfError):
        pbf_mod.load_scene("SmoothLen 0.1\n")
    p, pos32, _ = pbf_mod.make_scene("dam_break_32k")
    assert pos32.shape == (32768, 4) and p.particleCount == 32768
