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
    assert line["warmup"] == 3 and 1 <= line["steps"] <= 2  # untimed warm-up frames, then the timed ones
    for key in ("epsilon 20000", "s_corr k 0.001", "XSPH c"):
        assert key in line["config"]["workload"], key


def test_reference_scene_leaves_the_product_library_unloaded():
    """The reference arm builds its scene through the oracle: the same
    parameters and positions as the product's scenario reader, with
    libpbf_gb300.so never mapped into the process."""
    import subprocess
    code = (
        "import sys; sys.path[:0] = [%r, %r]\n"
        "import bench\n"
        "params, pos, vel = bench.reference_scene('dam_break_32k')\n"
        "maps = open('/proc/self/maps').read()\n"
        "assert 'libpbf_gb300' not in maps, 'product library mapped'\n"
        "assert 'libpbf_oracle' in maps\n"
        "import numpy as np, pbf\n"
        "p2, pos2, _ = pbf.make_scene('dam_break_32k')\n"
        "assert bytes(params) == bytes(p2) and np.array_equal(pos.view(np.uint32), pos2.view(np.uint32))\n"
        "print('ok')\n" % (str(REPO), str(REPO / "position-based-fluids_gb300")))
    run = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert run.returncode == 0 and run.stdout.strip() == "ok", run.stderr[-2000:]


def test_survey_byte_model_sums_to_the_substep_total():
    """The per-stage byte model adds up to 444 + 56 I bytes per particle and
    substep (3 sort passes)."""
    import bench
    it = 4
    per_substep = ["predictPositions", "radixsort", "sortParticles", "updateCells", "updateVelocities",
                   "applyViscosity", "applyVorticity"]
    total = sum(bench.survey_bytes(k) for k in per_substep) + it * (bench.survey_bytes("computeScaling") +
                                                                   bench.survey_bytes("computeDelta"))
    assert total == 444.0 + 56.0 * it
    assert bench.survey_bytes("buildFriendsList") is None


def test_stage_rooflines_and_dominant_kernel():
    import bench
    stage_ms = {"computeScaling": 1.0, "computeDelta": 0.8, "buildFriendsList": 0.9, "radixsort": 0.1}
    n, it, sub = 1 << 20, 4, 2
    rows = bench.stage_rooflines(stage_ms, n, it, sub, 30.0, 26.0, 6700.0)
    assert rows["computeScaling"]["launches_per_step"] == 8 and rows["radixsort"]["launches_per_step"] == 2
    assert rows["computeScaling"]["bytes_per_launch"] == 20.0 * n
    assert "frac" not in rows["buildFriendsList"] and rows["buildFriendsList"]["frac_with_lists"] > 0
    roof = bench.dominant_roofline(stage_ms, n, it, sub, 30.0, 26.0, 6700.0, "measured")
    assert roof["kernel"] == "computeScaling"
    assert abs(roof["achieved"] - 20.0 * n / (1.0 / 8 / 1e3) / 1e9) < 1e-6
    assert roof["frac_with_lists"] > roof["frac"]
