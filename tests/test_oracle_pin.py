"""The oracle against the reference's own kernels (CPU only).

The reference ships no tests or golden data, so the oracle is pinned against
the reference's kernel sources themselves: tests/golden/ holds digests of
their outputs (generated by tests/golden/make_golden.py through
oracle/clshim.hpp), and where the reference checkout is present the oracle is
also run side by side with the shimmed kernels on fresh cases.
"""
from __future__ import annotations

import hashlib
import importlib.util
import json
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"


def _make_golden():
    spec = importlib.util.spec_from_file_location("make_golden", GOLDEN / "make_golden.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _digest(a):
    return _make_golden().digest(a)


MANIFEST = json.loads((GOLDEN / "golden.json").read_text())


@pytest.mark.parametrize("case", MANIFEST["cases"], ids=[c["name"] for c in MANIFEST["cases"]])
def test_oracle_matches_reference_digests(case, pbf_mod, oracle_mod):
    mg = _make_golden()
    params, pos, vel = mg.scene(tuple(case["block"]), case["overrides"])
    p, v, pr, dbg = oracle_mod.step(params, pos, vel, case["substeps"], debug=True)
    got = {"pos": p, "vel": v, "pred": pr, "keys": dbg["keys"], "perm": dbg["perm"], "cells": dbg["cells"]}
    for k, want in case["sha256"].items():
        assert _digest(got[k]) == want, f"{case['name']}: {k} differs from the reference kernels"


def test_oracle_matches_small_case_arrays(pbf_mod, oracle_mod):
    data = np.load(GOLDEN / "small_case.npz")
    mg = _make_golden()
    case = next(c for c in MANIFEST["cases"] if c["name"] == "small_2k_2sub")
    params, pos, vel = mg.scene(tuple(case["block"]), case["overrides"])
    assert np.array_equal(pos, data["init_pos"])
    p, v, pr = oracle_mod.step(params, pos, vel, case["substeps"])
    for name, arr in (("pos", p), ("vel", v), ("pred", pr)):
        assert np.array_equal(arr.view(np.uint32), data[name].view(np.uint32)), name


def test_sort_is_stable_argsort(pbf_mod, oracle_mod):
    """The 6-pass, 5-bit reference sort equals a stable sort by key."""
    params = pbf_mod.load_scenario("dam_break_32k")
    rng = np.random.default_rng(5)
    n = 5000
    params.particleCount = n
    pred = np.zeros((n, 4), np.float32)
    pred[:, :3] = rng.uniform(0.0, 1.6, (n, 3)).astype(np.float32)
    keys, perm, cells = oracle_mod.sort(params, pred)
    raw = np.array([oracle_mod.grid_hash(int(x), int(y), int(z), params.gridBufSize)
                    for x, y, z in (pred[:, :3] / np.float32(params.h)).astype(np.int32)], np.uint32)
    order = np.argsort(raw, kind="stable")
    nk = oracle_mod.n_keys(n)
    assert np.array_equal(perm[:n], order)
    assert np.array_equal(keys[:n], raw[order])
    assert np.all(keys[n:] == 2147483646) and np.array_equal(perm[n:], np.arange(n, nk))
    # cell table: start/end (inclusive) of every occupied key, all ones elsewhere
    table = cells.reshape(-1, 2)
    occupied = np.unique(raw)
    for k in occupied[:200]:
        idx = np.nonzero(keys[:n] == k)[0]
        assert table[k, 0] == idx[0] and table[k, 1] == idx[-1]
    empty = np.setdiff1d(np.arange(params.gridBufSize), occupied)
    assert np.all(table[empty] == 0xFFFFFFFF)


needs_ref = pytest.mark.skipif(
    not __import__("oracle.oracle", fromlist=["ref_available"]).ref_available(),
    reason="the reference kernels are not available here")


@needs_ref
@pytest.mark.parametrize("seed,substeps,overrides", [
    (1, 3, {}),
    (2, 2, {"viscosityFactor": 0.05, "vorticityFactor": 0.01, "surfaceTenstionK": -0.3}),
    (3, 2, {"epsilon": 100.0, "restDensity": 5000.0}),
    (4, 1, {"gridBufSize": 1000}),  # not a power of two: the modulo path
])
def test_oracle_matches_reference_live(seed, substeps, overrides, pbf_mod, oracle_mod):
    params = pbf_mod.load_scenario("dam_break_32k")
    params.boxClamp = 0
    for k, v in overrides.items():
        setattr(params, k, v)
    dims = (12, 20, 9)
    n = dims[0] * dims[1] * dims[2]
    params.particleCount = n
    pos = pbf_mod.scene_block(*dims, 0.05, (0.3, 0.2, 0.1), 0.01, seed)
    rng = np.random.default_rng(seed)
    vel = np.zeros_like(pos)
    vel[:, :3] = rng.normal(0, 0.2, (n, 3)).astype(np.float32)
    a = oracle_mod.step(params, pos, vel, substeps)
    b = oracle_mod.ref_step(params, pos, vel, substeps)
    mg = _make_golden()
    for x, y, name in zip(a, b[:3], ("pos", "vel", "pred")):
        assert np.array_equal(mg.canonical(x).view(np.uint32), mg.canonical(y).view(np.uint32)), name


@needs_ref
def test_reference_kernels_same_bits_on_one_and_all_threads(pbf_mod, oracle_mod):
    """The shim runs work-items on several threads (applyViscosity on per-thread
    copies of the pre-pass velocities); the result must not depend on how many."""
    params = pbf_mod.load_scenario("dam_break_32k")
    dims = (14, 12, 10)
    params.particleCount = dims[0] * dims[1] * dims[2]
    pos = pbf_mod.scene_block(*dims, 0.05, (0.3, 0.2, 0.1), 0.01, 11)
    vel = np.zeros_like(pos)
    vel[:, :3] = np.random.default_rng(11).normal(0, 0.2, (len(pos), 3)).astype(np.float32)
    one = oracle_mod.ref_step(params, pos, vel, 3, threads=1)
    every = oracle_mod.ref_step(params, pos, vel, 3, threads=0)
    for a, b in zip(one, every):
        assert np.array_equal(np.ascontiguousarray(a).view(np.uint32), np.ascontiguousarray(b).view(np.uint32))


def test_fp64_oracle_close_to_fp32(pbf_mod, oracle_mod):
    """The FP64 oracle runs the same pipeline; one substep stays close."""
    params = pbf_mod.load_scenario("dam_break_32k")
    dims = (16, 16, 16)
    params.particleCount = 4096
    params.boxClamp = 0
    pos = pbf_mod.scene_block(*dims, 0.05, (0.025,) * 3, 0.005, 7)
    vel = np.zeros_like(pos)
    p32, v32, _ = oracle_mod.step(params, pos, vel, 1)
    p64, v64, _ = oracle_mod.step_f64(params, pos, vel, 1)
    assert np.max(np.abs(p32[:, :3] - p64[:, :3])) < 1e-5
    assert np.max(np.abs(v32[:, :3] - v64[:, :3])) < 5e-3


# ---- force planes (compute_delta.cl:1-42, 157-182) ----

FORCE = MANIFEST["force_planes"]


def _force_setup():
    mg = _make_golden()
    params, pos, vel = mg.force_scene()
    return mg, params, pos, vel, mg.quads_array(FORCE["quads"]), mg.force_mask(FORCE["mask"])


def test_force_planes_are_the_reference_planes():
    """golden.json holds the reference's 14 hard-coded planes as data."""
    assert len(FORCE["quads"]) == 14
    assert FORCE["quads"][7]["maskYOffset"] == 3578 and FORCE["quads"][7]["maskHeight"] == 369


def test_oracle_force_planes_match_reference_digests(pbf_mod, oracle_mod):
    mg, params, pos, vel, quads, mask = _force_setup()
    oracle_mod.set_force_planes(quads, mask)
    try:
        p, v, pr, dbg = oracle_mod.step(params, pos, vel, FORCE["substeps"], debug=True)
        p0, _, _ = oracle_mod.step(params, pos, vel, 1)
    finally:
        oracle_mod.set_force_planes(None, None)
    got = {"pos": p, "vel": v, "pred": pr, "keys": dbg["keys"], "perm": dbg["perm"], "cells": dbg["cells"]}
    for k, want in FORCE["sha256"].items():
        assert _digest(got[k]) == want, f"force planes: {k} differs from the reference kernels"
    q0, _, _ = oracle_mod.step(params, pos, vel, 1)  # without planes
    assert not np.array_equal(p0, q0), "the planes act on this scene"


@pytest.mark.skipif(not __import__("oracle.oracle", fromlist=["x"]).ref_available(),
                    reason="the reference's kernels are not available here")
def test_oracle_force_planes_match_reference_live(pbf_mod, oracle_mod):
    """Another mask (holes in the other texels) and two substeps, against the
    reference's computeDelta with its own hard-coded planes."""
    mg, params, pos, vel, quads, mask = _force_setup()
    mask = (1 - mask).astype(np.uint32)
    oracle_mod.set_force_planes(quads, mask)
    oracle_mod.ref_set_force_mask(mask)
    try:
        a = oracle_mod.step(params, pos, vel, 2)
        b = oracle_mod.ref_step(params, pos, vel, 2)
    finally:
        oracle_mod.set_force_planes(None, None)
        oracle_mod.ref_set_force_mask(None)
    for x, y, name in zip(a, b[:3], ("pos", "vel", "pred")):
        assert np.array_equal(mg.canonical(x).view(np.uint32), mg.canonical(y).view(np.uint32)), name


def test_noise_sine_accuracy(oracle_mod):
    """The planes' portable FP32 sine against the FP64 sine: a few ulp over
    the range the noise offset sees, exact at the quadrant points."""
    rng = np.random.default_rng(3)
    xs = np.concatenate([rng.uniform(-3000.0, 3000.0, 20000), rng.uniform(-4.0, 4.0, 5000)]).astype(np.float32)
    got = np.array([oracle_mod.noise_sinf(float(x)) for x in xs], np.float32)
    want = np.sin(xs.astype(np.float64))
    ulp = np.spacing(np.maximum(np.abs(want), 2.0 ** -24).astype(np.float32)).astype(np.float64)
    err = np.abs(got.astype(np.float64) - want) / ulp
    print(f"noise sine: max error {err.max():.2f} ulp, mean {err.mean():.3f}")
    assert err.max() <= 4.0
    assert oracle_mod.noise_sinf(0.0) == 0.0 and np.isnan(oracle_mod.noise_sinf(float("nan")))


def test_render_restatement_sanity(pbf_mod, oracle_mod):
    """The renderer's restatement on the reference's scene scale: the splat
    covers the block with window depths in [0, 1]; on covered pixels the
    smoothing pass lands near the splat depth; colour modes stay in range."""
    params = pbf_mod.load_scenario("dam_break_32k")
    params.h, params.h_2 = 2.0, 4.0
    pos = pbf_mod.scene_block(16, 16, 16, 0.55, (0.3, 0.3, 0.3), 0.05, 7)
    params.particleCount = len(pos)
    cam = pbf_mod.render_camera((4.4, 8.0, 30.0), (4.4, 4.0, 4.4), (0.0, 1.0, 0.0), 45.0, 96, 72, 1.0)
    splat, smooth, out = oracle_mod.render(cam, 0, params, pos)
    covered = splat[..., 1] > 0
    assert 0.05 < covered.mean() < 0.9
    d = splat[covered][:, 0]
    assert np.all((d > 0.0) & (d <= 1.0))
    ok = covered & np.isfinite(smooth[..., 0]) & (smooth[..., 0] > 0)
    assert ok.mean() > 0.5 * covered.mean()
    assert np.all(np.abs(smooth[ok][:, 0] - splat[ok][:, 0]) < 0.01)
    for mode in (1, 2):
        s, _, o = oracle_mod.render(cam, mode, params, pos)
        assert np.array_equal(s, o) and np.all((o >= 0.0) & (o <= 2.0))


def test_complete_neighbours_density(pbf_mod, oracle_mod):
    """One solver iteration, so that the density of both rules is taken at the
    same predicted positions: every particle's complete density (every circle
    plus its own W(0)) is at least its density over the reference's truncated
    sets, and larger by at least the self term."""
    params, pos, vel = pbf_mod.make_scene("dam_break_32k")
    params.simIterations = 1
    dens = {}
    for complete in (0, 1):
        p = params.copy()
        p.completeNeighbours = complete
        _, _, pr = oracle_mod.step(p, pos, vel, 1)
        dens[complete] = pr[:, 3].astype(np.float64)
    poly6, _, _ = oracle_mod.constants(params)
    self_term = poly6 * float(np.float32(params.h_2)) ** 3
    assert np.all(dens[1] - dens[0] >= 0.999 * self_term)
    print(f"mean density / rest: reference sets {dens[0].mean() / params.restDensity:.3f}, "
          f"complete {dens[1].mean() / params.restDensity:.3f}")
