"""The particle-count sweep scene (double dam break) through the CUDA path:
bit-exact against the oracle at 262,144 particles for 2, 4 and 8 solver
iterations, and for one substep at 8,388,608 particles (the reference sort's
own limit, hesp.hpp:77)."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _same(a, b):
    a = a.copy(); b = b.copy()
    a[np.isnan(a)] = 0; b[np.isnan(b)] = 0
    return np.array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.mark.parametrize("iters", [2, 4, 8])
def test_double_dam_break_262k(iters, pbf_mod, oracle_mod, cuda_device):
    params, pos, vel = pbf_mod.make_double_dam_break(262144, iterations=iters)
    with pbf_mod.Simulation.create(params, pos, vel, device=cuda_device) as sim:
        sim.Step(2)
        gp, gv, gpr = sim.read_state()
    op, ov, opr = oracle_mod.step(params, pos, vel, 2)
    assert _same(gp, op) and _same(gv, ov) and _same(gpr, opr)


def test_double_dam_break_8m_one_substep(pbf_mod, oracle_mod, cuda_device):
    params, pos, vel = pbf_mod.make_double_dam_break(8388608, iterations=2)
    with pbf_mod.Simulation.create(params, pos, vel, device=cuda_device) as sim:
        sim.Step(1)
        gp, gv, gpr = sim.read_state()
    op, ov, opr = oracle_mod.step(params, pos, vel, 1)
    assert _same(gp, op) and _same(gv, ov) and _same(gpr, opr)
