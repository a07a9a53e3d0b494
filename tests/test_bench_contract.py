"""Host-side pieces of bench.py that need no GPU: the stage groups partition
the stage names the library reports, and the per-stage byte models cover
only reported stages."""
from __future__ import annotations

import re
import sys
from pathlib import Path

REPO = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(REPO))


def _reported_stages() -> set[str]:
    src = (REPO / "position-based-fluids_gb300" / "csrc" / "pbf_capi.cu").read_text()
    return set(re.findall(r'mark\("([A-Za-z]+)"', src))


def test_stage_groups_partition_reported_stages():
    import bench
    stages = _reported_stages()
    assert {"computeScaling", "computeDelta", "radixsort", "applyVorticity"} <= stages
    grouped = [k for ks in bench.STAGE_GROUPS.values() for k in ks]
    assert len(grouped) == len(set(grouped)), "a stage sits in two groups"
    assert set(grouped) == stages


def test_stage_byte_models_name_reported_stages():
    import bench
    stages = _reported_stages()
    assert set(bench.STAGE_BYTES) <= stages
    for model in bench.STAGE_BYTES.values():
        assert model(30.0, 27.0) > 0
