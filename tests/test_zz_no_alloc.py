"""The allocation-free sort entry point (pbf_sort_state_noalloc).

Hosts that reserve all device memory up front and forbid later allocations
(real-time frame loops, engines that own the GPU memory budget) call this
variant with their own device buffers; its working memory is a fixed array
inside the library.  Its keys, permutation and cell table must equal those of
pbf_sort_state, the entry point that allocates, bit for bit (integer data:
no tolerance), on two calls in a row, the second smaller than the first so
that it runs over what the first left in the shared array.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _case(pbf, dims, grid, seed):
    params = pbf.load_scenario("dam_break_32k")
    params.gridBufSize = grid
    params.particleCount = dims[0] * dims[1] * dims[2]
    pos = pbf.scene_block(*dims, 0.05, (0.025, 0.025, 0.025), 0.005, seed)
    rng = np.random.default_rng(seed)
    pred = pos.copy()
    pred[:, :3] += rng.uniform(-0.02, 0.02, (len(pos), 3)).astype(np.float32)
    return params, pos, pred


def test_noalloc_sort_equals_allocating_entry_point(pbf_mod, cuda_device):
    import torch
    dev = torch.device("cuda", cuda_device)
    torch.cuda.set_device(dev)
    cases = [
        _case(pbf_mod, (40, 32, 40), 524288, 11),   # 51,200 particles, 3 sort passes
        _case(pbf_mod, (20, 25, 30), 8192, 12),     # 15,000 particles, 2 sort passes
    ]
    for params, pos, pred in cases:
        n = params.particleCount
        with pbf_mod.Simulation.create(params, pos, np.zeros_like(pos), device=cuda_device) as sim:
            want_keys, want_perm, want_cells = sim.sort_state(pred)
        d_pred = torch.from_numpy(pred).to(dev)
        d_keys = torch.empty(n, dtype=torch.int32, device=dev)
        d_perm = torch.empty(n, dtype=torch.int32, device=dev)
        d_cells = torch.empty(2 * params.gridBufSize, dtype=torch.int32, device=dev)
        stream = torch.cuda.current_stream(dev)
        pbf_mod.sort_state_noalloc(params, d_pred.data_ptr(), d_keys.data_ptr(), d_perm.data_ptr(),
                                   d_cells.data_ptr(), stream.cuda_stream)
        stream.synchronize()
        got_keys = d_keys.cpu().numpy().view(np.uint32)
        got_perm = d_perm.cpu().numpy().view(np.uint32)
        got_cells = d_cells.cpu().numpy().view(np.uint32)
        assert np.array_equal(got_keys, want_keys[:n]), "keys"
        assert np.array_equal(got_perm, want_perm[:n]), "permutation"
        assert np.array_equal(got_cells, want_cells), "cell table"


def test_noalloc_sort_rejects_sizes_beyond_its_array(pbf_mod, cuda_device):
    params = pbf_mod.load_scenario("dam_break_32k")
    params.particleCount = (1 << 20) + 1
    with pytest.raises(pbf_mod.PbfError) as e:
        pbf_mod.sort_state_noalloc(params, 1, 1, 1, None, None)  # rejected before any device access
    assert e.value.code == pbf_mod.PBF_ERR_INVALID
    assert "1048576" in str(e.value)
