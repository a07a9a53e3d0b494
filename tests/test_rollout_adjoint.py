"""The FP64 adjoint of the oracle against central finite differences (CPU).

The rollout is differentiated over a fixed neighbour structure: the sort
permutation, the friend lists and the box-clamp decisions of the recorded
FP32 forward are constants, so the function of (v0, c, g) replayed in FP64
is smooth and a central difference with step 1e-3 checks its gradient.  The
dam break is chaotic (a perturbation grows about 1.34x per substep, mostly
at wall impacts), so the check runs over 10 substeps, where the
fixed-structure function still equals the FP32 forward to a few 1e-6.

Directions are unit vectors in (v0 [3N], g [3]) space plus a component along
c scaled by 1e-6 (c itself is about 1.6e-6).
"""
from __future__ import annotations

import numpy as np
import pytest

SUBSTEPS = 10
DIRECTIONS = 64
FD_STEP = 1e-3
FD_TOL = 1e-3


@pytest.fixture(scope="module")
def rollout(pbf_mod, oracle_mod):
    params, pos, vel = pbf_mod.make_rollout_scene(16, 16, 16)
    rng = np.random.default_rng(11)
    vel[:, :3] = rng.normal(0.0, 0.05, (params.particleCount, 3)).astype(np.float32)
    R = oracle_mod.Rollout(params, pos, vel, SUBSTEPS)
    # the target: the same start run with gravity tilted 5 degrees and c = 0.03
    T = oracle_mod.Rollout(pbf_mod.rollout_target_params(params), pos, vel, SUBSTEPS)
    return params, R, T.final_by_id32().astype(np.float64)


def test_replay_matches_fp32_forward(rollout):
    params, R, _ = rollout
    _, x64 = R.replay()
    x32 = R.final_by_id32()
    err = float(np.max(np.abs(x64[:, :3] - x32[:, :3])))
    print(f"FP64 replay vs FP32 forward after {SUBSTEPS} substeps: max |dx| {err:.2e}")
    assert err < 1e-4


def test_fp64_adjoint_matches_central_differences(rollout):
    params, R, target = rollout
    n = R.n
    g0 = np.array([params.gravityX, params.gravityY, params.gravityZ], np.float64)
    c0 = float(params.viscosityFactor)
    loss, dv, dc, dg = R.grad(target)
    assert loss > 0
    rng = np.random.default_rng(5)
    v0 = R.vel0.astype(np.float64)
    rel = []
    for _ in range(DIRECTIONS):
        d = rng.normal(0.0, 1.0, 3 * n + 4)
        d /= np.linalg.norm(d)
        d_v = np.zeros((n, 4))
        d_v[:, :3] = d[:3 * n].reshape(n, 3)
        d_c = d[3 * n] * 1e-6
        d_g = d[3 * n + 1:]

        def L(s):
            return R.replay(vel0=v0 + s * d_v, gravity=g0 + s * d_g, visc=c0 + s * d_c, target=target)[0]

        fd = (L(FD_STEP) - L(-FD_STEP)) / (2 * FD_STEP)
        ad = float((dv * d_v).sum() + dc * d_c + (dg * d_g).sum())
        rel.append(abs(fd - ad) / max(abs(ad), 1e-30))
    rel = np.array(rel)
    print(f"FP64 adjoint vs central differences over {DIRECTIONS} directions: median {np.median(rel):.2e}, "
          f"max {rel.max():.2e}")
    assert rel.max() < FD_TOL


def test_fp64_adjoint_scalar_parameters(rollout):
    """dL/dc and dL/dg alone, against central differences along each."""
    params, R, target = rollout
    g0 = np.array([params.gravityX, params.gravityY, params.gravityZ], np.float64)
    c0 = float(params.viscosityFactor)
    _, _, dc, dg = R.grad(target)
    for axis in range(3):
        e = np.zeros(3)
        e[axis] = 1.0
        fd = (R.replay(gravity=g0 + FD_STEP * e, target=target)[0] -
              R.replay(gravity=g0 - FD_STEP * e, target=target)[0]) / (2 * FD_STEP)
        assert abs(fd - dg[axis]) <= FD_TOL * max(abs(dg).max(), 1e-30), (axis, fd, dg[axis])
    h = 1e-3 * c0
    fd = (R.replay(visc=c0 + h, target=target)[0] - R.replay(visc=c0 - h, target=target)[0]) / (2 * h)
    assert abs(fd - dc) <= FD_TOL * abs(dc), (fd, dc)


def test_fp32_reverse_pass_error(pbf_mod, oracle_mod, rollout):
    """The oracle's reverse pass evaluated in FP32 (serial, same formulas)
    against FP64, given the same dL/dx: the error FP32 arithmetic alone
    gives.  Most of it comes from vorticity confinement's direction
    eta/|eta|, whose derivative scales with 1/|eta|: without vorticity the
    error is an order of magnitude smaller."""
    params, R, target = rollout
    n = R.n
    _, x64 = R.replay()
    dldx = np.zeros((n, 4))
    dldx[:, :3] = 2.0 * (x64[:, :3] - target[:, :3]) / (3.0 * n)
    _, dv64, dc64, dg64 = R.grad(target)
    _, dv32, dc32, dg32 = R.grad_f32(target, dldx)
    rel = float(np.linalg.norm(dv32[:, :3] - dv64[:, :3]) / np.linalg.norm(dv64[:, :3]))
    p = params.copy()
    p.vorticityFactor = 0.0
    R0 = oracle_mod.Rollout(p, R.pos0, R.vel0, SUBSTEPS)
    _, xa = R0.replay()
    d0 = np.zeros((n, 4))
    d0[:, :3] = 2.0 * (xa[:, :3] - target[:, :3]) / (3.0 * n)
    _, a64, _, _ = R0.grad(target)
    _, a32, _, _ = R0.grad_f32(target, d0)
    rel0 = float(np.linalg.norm(a32[:, :3] - a64[:, :3]) / np.linalg.norm(a64[:, :3]))
    print(f"FP32 reverse pass vs FP64 over {SUBSTEPS} substeps: dv0 {rel:.2e} ({rel0:.2e} without vorticity), "
          f"dc {abs(dc32 - dc64) / abs(dc64):.2e}, dg {np.linalg.norm(dg32 - dg64) / np.linalg.norm(dg64):.2e}")
    assert rel < FD_TOL and rel0 < rel
