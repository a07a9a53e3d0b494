"""The allocation-free sort entry point (pbf_sort_state_noalloc).

Hosts that reserve all device memory up front and forbid later allocations
(real-time frame loops, engines that own the GPU memory budget) call this
variant with their own device buffers; its working memory is a fixed array
inside the library.  Its keys, permutation and cell table must equal those of
pbf_sort_state, the entry point that allocates, and those of the oracle's
sort, bit for bit (integer data: no tolerance).  The calls run back to back,
largest first, so that each later call runs over what the earlier ones left
in the shared array.  The sizes cover both tile sizes of the sort (1,024-key
tiles up to 2^18 keys, 2,048-key tiles above), odd and even pass counts (an
odd count leaves the result in the array and copies it out), and the largest
accepted count, 1,048,576, where the histogram region of the array is
exactly full.
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


CASES = [
    ((128, 64, 128), 1 << 19, 13),  # 1,048,576 particles: the maximum, 2,048-key tiles, 3 passes
    ((100, 60, 50), 1 << 16, 14),   # 300,000 particles: 2,048-key tiles, 2 passes
    ((40, 32, 40), 524288, 11),     # 51,200 particles: 1,024-key tiles, 3 passes
    ((20, 25, 30), 8192, 12),       # 15,000 particles: 1,024-key tiles, 2 passes
]


def test_noalloc_sort_equals_allocating_entry_point_and_oracle(pbf_mod, oracle_mod, cuda_device):
    import torch
    dev = torch.device("cuda", cuda_device)
    torch.cuda.set_device(dev)
    for dims, grid, seed in CASES:
        params, pos, pred = _case(pbf_mod, dims, grid, seed)
        n = params.particleCount
        with pbf_mod.Simulation.create(params, pos, np.zeros_like(pos), device=cuda_device) as sim:
            want_keys, want_perm, want_cells = sim.sort_state(pred)
        o_keys, o_perm, o_cells = oracle_mod.sort(params, pred)
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
        for name, got, alloc, orc in (("keys", got_keys, want_keys[:n], o_keys[:n]),
                                      ("permutation", got_perm, want_perm[:n], o_perm[:n]),
                                      ("cell table", got_cells, want_cells, o_cells)):
            assert np.array_equal(got, alloc), f"{n} particles: {name} differ from pbf_sort_state"
            assert np.array_equal(got, orc), f"{n} particles: {name} differ from the oracle"


def test_noalloc_sort_rejects_sizes_beyond_its_array(pbf_mod, cuda_device):
    params = pbf_mod.load_scenario("dam_break_32k")
    params.particleCount = (1 << 20) + 1
    with pytest.raises(pbf_mod.PbfError) as e:
        pbf_mod.sort_state_noalloc(params, 1, 1, 1, None, None)  # rejected before any device access
    assert e.value.code == pbf_mod.PBF_ERR_INVALID
    assert "1048576" in str(e.value)


def test_noalloc_sort_rejects_misaligned_and_host_pointers(pbf_mod, cuda_device):
    """A float4 input that is not 16-byte aligned, or a host buffer, is an
    argument error reported before any work is enqueued."""
    import torch
    dev = torch.device("cuda", cuda_device)
    params, pos, pred = _case(pbf_mod, (8, 8, 8), 8192, 5)
    n = params.particleCount
    d_pred = torch.from_numpy(pred).to(dev)
    d_keys = torch.zeros(n, dtype=torch.int32, device=dev)
    d_perm = torch.zeros(n, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev)
    with pytest.raises(pbf_mod.PbfError) as e:
        pbf_mod.sort_state_noalloc(params, d_pred.data_ptr() + 4, d_keys.data_ptr(), d_perm.data_ptr(), None,
                                   stream.cuda_stream)
    assert e.value.code == pbf_mod.PBF_ERR_INVALID and "aligned" in str(e.value)
    host_keys = np.zeros(n, np.uint32)
    with pytest.raises(pbf_mod.PbfError) as e:
        pbf_mod.sort_state_noalloc(params, d_pred.data_ptr(), host_keys.ctypes.data, d_perm.data_ptr(), None,
                                   stream.cuda_stream)
    assert e.value.code == pbf_mod.PBF_ERR_INVALID and "d_keys" in str(e.value)
    stream.synchronize()
    assert not d_keys.any() and not d_perm.any(), "nothing may run after a rejected argument"
