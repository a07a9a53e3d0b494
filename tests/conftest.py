"""Shared test setup: import paths, the `gpu` marker, and builds.

`oracle` (the CPU checker) and `pbf` (the binding of libpbf_gb300.so) are
importable from every test.  Tests marked `gpu` need a CUDA device; the rest
run on CPU only and never launch a kernel.
"""
from __future__ import annotations

import os
import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parent.parent
PKG = REPO / "position-based-fluids_gb300"
for p in (str(REPO), str(PKG)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); run with -m gpu")


def load_pkg_build():
    """position-based-fluids_gb300/build.py as a module."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("pbf_pkg_build", PKG / "build.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="session")
def built_lib():
    """The product library, built in-tree if needed."""
    return load_pkg_build().build()


@pytest.fixture(scope="session")
def pbf_mod(built_lib):
    import pbf
    return pbf


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle
    oracle.lib()
    return oracle


def has_cuda_device() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def cuda_device():
    if not has_cuda_device():
        pytest.fail("a CUDA device is required for tests marked gpu")
    return int(os.environ.get("PBF_TEST_DEVICE", "0"))
