"""The CUDA differentiable rollout (pbf_rollout_forward / _backward) against
the oracle (needs a GPU).

Forward: the rollout is the plain substep pipeline, so final positions and
particle ids are bit-exact against the FP32 oracle.  Backward: the FP32
adjoint kernels scatter neighbour terms with atomics, so gradients are
compared with the FP64 adjoint of the same fixed-structure function by
relative L2 error (within twice the error of the oracle's serial FP32
reverse pass, and within GRAD_TOL), and with central differences of the FP64
replay along random directions (median within GRAD_TOL).
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SUBSTEPS = 10
GRAD_TOL = 1e-3


def _case(pbf_mod, oracle_mod, seed=11):
    params, pos, vel = pbf_mod.make_rollout_scene(16, 16, 16)
    rng = np.random.default_rng(seed)
    vel[:, :3] = rng.normal(0.0, 0.05, (params.particleCount, 3)).astype(np.float32)
    R = oracle_mod.Rollout(params, pos, vel, SUBSTEPS)
    T = oracle_mod.Rollout(pbf_mod.rollout_target_params(params), pos, vel, SUBSTEPS)
    return params, pos, vel, R, T.final_by_id32().astype(np.float64)


def _dl_dx(x_by_id, target):
    n = x_by_id.shape[0]
    g = np.zeros((n, 4), np.float64)
    g[:, :3] = 2.0 * (x_by_id[:, :3].astype(np.float64) - target[:, :3]) / (3.0 * n)
    return g.astype(np.float32)


def _rel(a, b):
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / max(np.linalg.norm(np.ravel(b)), 1e-30))


@pytest.fixture(scope="module")
def case(pbf_mod, oracle_mod):
    return _case(pbf_mod, oracle_mod)


def test_rollout_forward_bit_exact(pbf_mod, case, cuda_device):
    params, pos, vel, R, _ = case
    with pbf_mod.Simulation.create(params, pos, vel, device=cuda_device) as sim:
        sim.rollout_forward(SUBSTEPS, 4)
        got = sim.positions_by_id()
        ids = sim.read_ids()
    np.testing.assert_array_equal(ids, R.ids)
    assert np.array_equal(got[:, :3].view(np.uint32), R.final_by_id32()[:, :3].view(np.uint32))


@pytest.mark.parametrize("every", [10, 3])
def test_adjoint_matches_fp64_adjoint(pbf_mod, case, cuda_device, every):
    """Same dL/dx in, FP32 GPU adjoint against the FP64 adjoint.  dL/dx is
    taken from the FP64 replay's final positions: the loss residual
    (x - target) is about 1e-4 after a few substeps, so FP32 rounding of the
    final positions alone moves dL/dx by a few 1e-4 relative.  The bound is
    twice the error of the oracle's serial FP32 reverse pass given the same
    dL/dx (the vorticity direction eta/|eta| is what makes FP32 lose about
    3e-4 here), and GRAD_TOL."""
    params, pos, vel, R, target = case
    loss64, dv64, dc64, dg64 = R.grad(target)
    _, x64 = R.replay()
    dldx = _dl_dx(x64, target)
    _, dv32, dc32, dg32 = R.grad_f32(target, dldx.astype(np.float64))
    with pbf_mod.Simulation.create(params, pos, vel, device=cuda_device) as sim:
        sim.rollout_forward(SUBSTEPS, every)
        x_end = sim.positions_by_id()
        dv, dc, dg = sim.rollout_backward(dldx)
        after = sim.positions_by_id()
        own = sim.rollout_backward(_dl_dx(x_end, target))  # the caller's own dL/dx
    np.testing.assert_array_equal(after, x_end)  # the state is left at the end of the rollout
    ev, ec, eg = _rel(dv[:, :3], dv64[:, :3]), abs(dc - dc64) / abs(dc64), _rel(dg, dg64)
    fv, fc, fg = _rel(dv32[:, :3], dv64[:, :3]), abs(dc32 - dc64) / abs(dc64), _rel(dg32, dg64)
    print(f"checkpoint every {every}: rel err dv0 {ev:.2e}, dc {ec:.2e}, dg {eg:.2e} (serial FP32: {fv:.2e}, "
          f"{fc:.2e}, {fg:.2e}); with dL/dx from the FP32 forward: dv0 {_rel(own[0][:, :3], dv64[:, :3]):.2e}")
    for got, f32 in ((ev, fv), (ec, fc), (eg, fg)):
        assert got < max(2.0 * f32, 1e-5) and got < GRAD_TOL
    assert _rel(own[0][:, :3], dv64[:, :3]) < GRAD_TOL


def test_graph_and_eager_reverse_passes_agree(pbf_mod, case, cuda_device):
    """The reverse pass replays each segment as a captured CUDA graph (one per
    segment length and starting buffer role); without graphs it launches the
    same work eagerly.  With 10 substeps in segments of 4, 4 and 2, two graphs
    are captured and one is replayed.  A second backward replays them all.
    The adjoint's atomic sums make the last bits run-dependent, so the two are
    compared within GRAD_TOL; a wrong segment or buffer role would be off by
    far more."""
    params, pos, vel, R, target = case
    results = {}
    for graph in (True, False):
        with pbf_mod.Simulation.create(params, pos, vel, device=cuda_device) as sim:
            sim.use_graph(graph)
            sim.rollout_forward(SUBSTEPS, 4)
            dldx = _dl_dx(sim.positions_by_id(), target)
            first = sim.rollout_backward(dldx)
            second = sim.rollout_backward(dldx)
        results[graph] = (first, second)
    for (gv, gc, gg), (ev, ec, eg) in ((results[True][0], results[False][0]), (results[True][1], results[False][0])):
        dv, dc, dg = _rel(gv[:, :3], ev[:, :3]), abs(gc - ec) / abs(ec), _rel(gg, eg)
        print(f"graph vs eager reverse pass: dv0 {dv:.2e}, dc {dc:.2e}, dg {dg:.2e}")
        assert dv < GRAD_TOL and dc < GRAD_TOL and dg < GRAD_TOL


def test_adjoint_matches_central_differences(pbf_mod, case, cuda_device):
    """Directional derivatives of the GPU gradient against central
    differences (step 1e-3) of the FP64 replay on 64 random unit directions.

    Two bounds, both GRAD_TOL: the median relative error |fd - ad| / |ad|,
    and the maximum over all 64 directions of |fd - ad| / |grad L|.  The
    second is the per-direction bound: a unit direction's derivative is at
    most |grad L|, and the relative error of one direction is unbounded where
    that direction is nearly orthogonal to the gradient (|ad| -> 0), since
    the FP32 gradient's own error (about 3e-4 of its norm) does not shrink
    with ad.  The FP32 reverse pass of the oracle gives a median of 2.3e-4,
    a scaled maximum of 5.7e-6 and a largest plain relative error of 4.5e-2
    on these 64 directions."""
    params, pos, vel, R, target = case
    n = R.n
    with pbf_mod.Simulation.create(params, pos, vel, device=cuda_device) as sim:
        sim.rollout_forward(SUBSTEPS, 5)
        dv, dc, dg = sim.rollout_backward(_dl_dx(sim.positions_by_id(), target))
    g0 = np.array([params.gravityX, params.gravityY, params.gravityZ], np.float64)
    c0 = float(params.viscosityFactor)
    v0 = R.vel0.astype(np.float64)
    rng = np.random.default_rng(5)
    rel, scaled = [], []
    gnorm = float(np.sqrt((dv[:, :3].astype(np.float64) ** 2).sum() + (float(dc) * 1e-6) ** 2 +
                          (np.asarray(dg, np.float64) ** 2).sum()))
    for _ in range(64):
        d = rng.normal(0.0, 1.0, 3 * n + 4)
        d /= np.linalg.norm(d)
        d_v = np.zeros((n, 4))
        d_v[:, :3] = d[:3 * n].reshape(n, 3)
        d_c, d_g = d[3 * n] * 1e-6, d[3 * n + 1:]
        L = lambda s: R.replay(vel0=v0 + s * d_v, gravity=g0 + s * d_g, visc=c0 + s * d_c, target=target)[0]
        fd = (L(1e-3) - L(-1e-3)) / 2e-3
        ad = float((dv.astype(np.float64) * d_v).sum() + dc * d_c + (dg.astype(np.float64) * d_g).sum())
        rel.append(abs(fd - ad) / max(abs(ad), 1e-30))
        scaled.append(abs(fd - ad) / gnorm)
    rel, scaled = np.array(rel), np.array(scaled)
    print(f"GPU adjoint vs central differences: median {np.median(rel):.2e}, max {rel.max():.2e}; "
          f"|fd - ad| / |grad L|: max {scaled.max():.2e}")
    assert np.median(rel) < GRAD_TOL
    assert scaled.max() < GRAD_TOL


def test_torch_autograd_wrapper(pbf_mod, case, cuda_device):
    torch = pytest.importorskip("torch")
    import pbf_autograd
    params, pos, vel, R, target = case
    _, dv64, dc64, dg64 = R.grad(target)
    v0 = torch.tensor(vel[:, :3], requires_grad=True)
    c = torch.tensor(float(params.viscosityFactor), requires_grad=True)
    g = torch.tensor([params.gravityX, params.gravityY, params.gravityZ], requires_grad=True)
    tgt = torch.from_numpy(target[:, :3].astype(np.float32))
    with pbf_mod.Simulation.create(params, pos, vel, device=cuda_device) as sim:
        x = pbf_autograd.rollout(v0, c, g, sim, params, pos, SUBSTEPS, 5)
        loss = ((x.double() - tgt.double()) ** 2).mean()
        loss.backward()
    assert _rel(v0.grad.numpy(), dv64[:, :3]) < GRAD_TOL
    assert abs(float(c.grad) - dc64) < GRAD_TOL * abs(dc64)
    assert _rel(g.grad.numpy(), dg64) < GRAD_TOL


def test_rollout_argument_errors(pbf_mod, case, cuda_device):
    params, pos, vel, _, _ = case
    with pbf_mod.Simulation.create(params, pos, vel, device=cuda_device) as sim:
        with pytest.raises(pbf_mod.PbfError):
            sim.rollout_backward(np.zeros((params.particleCount, 4), np.float32))  # no forward yet
        with pytest.raises(pbf_mod.PbfError):
            sim.rollout_forward(0, 1)
        # the reverse pass recomputes the forward's substeps: parameters set
        # in between (here 65 solver iterations, beyond the tape's 64) are refused
        sim.rollout_forward(2, 1)
        p2 = params.copy()
        p2.simIterations = 65
        sim.set_params(p2)
        with pytest.raises(pbf_mod.PbfError, match="changed since pbf_rollout_forward"):
            sim.rollout_backward(np.zeros((params.particleCount, 4), np.float32))
        sim.set_params(params)
        sim.rollout_forward(2, 1)
        sim.rollout_backward(np.zeros((params.particleCount, 4), np.float32))
        sim.bPauseSim = True
        with pytest.raises(pbf_mod.PbfError):
            sim.rollout_forward(2, 1)  # a paused simulation has no rollout
