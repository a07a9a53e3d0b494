"""The C++ facade (include/pbf_simulation.hpp) driven like the reference's
frame loop, compiled against libpbf_gb300.so by g++."""
from __future__ import annotations

import subprocess
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parent.parent
PKG = REPO / "position-based-fluids_gb300"


@pytest.fixture(scope="module")
def facade_exe(built_lib, tmp_path_factory):
    exe = tmp_path_factory.mktemp("facade") / "facade_check"
    cmd = ["g++", "-O2", "-std=c++17", "-I", str(REPO / "include"), str(REPO / "tests" / "cpp" / "facade_check.cpp"),
           "-o", str(exe), str(built_lib), f"-Wl,-rpath,{built_lib.parent}"]
    subprocess.run(cmd, check=True, capture_output=True)
    return exe


def _scene(pbf_mod, tmp_path, dims=(16, 16, 8)):
    par = (PKG / "scenarios" / "dam_break_32k.par").read_text().replace(
        "ParticleCount           32768", f"ParticleCount           {dims[0] * dims[1] * dims[2]}")
    par_file = tmp_path / "scene.par"
    par_file.write_text(par)
    pos = pbf_mod.scene_block(*dims, 0.05, (0.025,) * 3, 0.005, 20240601)
    pos_file = tmp_path / "pos.bin"
    pos.tofile(pos_file)
    return par_file, pos_file, pos


def test_facade_builds_and_reports_missing_device(facade_exe, pbf_mod, tmp_path):
    from tests.conftest import has_cuda_device
    if has_cuda_device():
        pytest.skip("a device is present; the GPU test covers the run")
    par_file, pos_file, _ = _scene(pbf_mod, tmp_path)
    r = subprocess.run([str(facade_exe), str(par_file), str(pos_file), "1", str(tmp_path / "out.bin")],
                       capture_output=True, text=True)
    assert r.returncode == 3 and "no CUDA device" in r.stderr


@pytest.mark.gpu
def test_facade_frames_match_oracle(facade_exe, pbf_mod, oracle_mod, tmp_path, cuda_device):
    par_file, pos_file, pos = _scene(pbf_mod, tmp_path)
    out = tmp_path / "out.bin"
    r = subprocess.run([str(facade_exe), str(par_file), str(pos_file), "3", str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "computeScaling" in r.stdout  # per-stage trackers reported
    got = np.fromfile(out, np.float32).reshape(2, -1, 4)
    params = pbf_mod.load_parameters(par_file.read_text())
    opos, ovel, _ = oracle_mod.step(params, pos, np.zeros_like(pos), 3 * params.subSteps)
    assert np.array_equal(got[0].view(np.uint32), opos.view(np.uint32))
    assert np.array_equal(got[1].view(np.uint32), ovel.view(np.uint32))
