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


def test_reference_arm_prints_the_contract_line():
    """bench.py --impl reference (CPU only) prints one JSON line with the keys
    the bench contract names, timed on a bounded sample."""
    import json
    import subprocess
    run = subprocess.run([sys.executable, str(REPO / "bench.py"), "--impl", "reference", "--scene", "dam_break_32k",
                          "--steps", "2", "--warmup", "3", "--cpu-budget", "1"], capture_output=True, text=True,
                         timeout=600)
    assert run.returncode == 0, run.stderr[-2000:]
    lines = [l for l in run.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["value"] > 0 and line["higher_is_better"] is True
    for key in ("metric", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["cpu_baseline"]["kind"] in ("reference", "port") and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["value"] == line["value"]
    assert line["warmup"] == 3 and 1 <= line["steps"] <= 2  # untimed warm-up substeps, then the timed ones
