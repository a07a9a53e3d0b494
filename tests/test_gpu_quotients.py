"""The exact passes' division through one reciprocal (quotient_rn in
csrc/pbf_device.cuh) against IEEE division (needs a GPU).

The four neighbour passes divide three numerators by |r| and, in the
position pass, (h^2 - r^2)^3 by poly6q.  With a correctly rounded reciprocal
y = RN(1/b), Markstein's correction RN(q0 + (a - b q0) y), q0 = RN(a y), is
the correctly rounded quotient when no underflow occurs; the library uses it
only where the numerators and quotients are in that range.  Here it is
compared bit for bit with CUDA's IEEE `/` on 2^33 seeded operand pairs over
that range (|r| in [2^-60, 2^10], numerators of either sign in
[2^-100, 2^40]) and on 2^31 numerators of the constant poly6q division of the
bundled scenes.  The passes' |r| and reciprocal y (sqrt_recip_rn: Markstein's
square-root correction and one Newton-Raphson reciprocal step) are checked on
every float r^2 in [2^-100, 2^64) (the passes' r^2 lie in [2^-100, 2^20] or
are 0): |r| against sqrtf, and wherever y differs from __frcp_rn(|r|), the
quotients it gives against IEEE division for every numerator significand.
r^2 = 0 gives the NaN its callers turn into the same NaN sums as IEEE
division by 0.  Integer-exact contract: no mismatch is tolerated.
"""
from __future__ import annotations

import ctypes
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REPO = Path(__file__).resolve().parent.parent
SRC = REPO / "tests" / "cuda" / "quotient_check.cu"
OUT = REPO / "tests" / "_build"


def _lib():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    OUT.mkdir(exist_ok=True)
    so = OUT / "libquotient_check.so"
    csrc = REPO / "position-based-fluids_gb300" / "csrc"
    cmd = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "--fmad=false", "-shared",
           "-Xcompiler", "-fPIC", "-I", str(REPO / "include"), "-I", str(csrc), str(SRC), "-o", str(so)]
    run = subprocess.run(cmd, capture_output=True, text=True)
    assert run.returncode == 0, run.stderr[-3000:]
    lib = ctypes.CDLL(str(so))
    lib.quotient_check.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int, ctypes.c_float, ctypes.c_float,
                                   ctypes.POINTER(ctypes.c_ulonglong), ctypes.POINTER(ctypes.c_float)]
    lib.quotient_check.restype = ctypes.c_int
    lib.sqrt_recip_check.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(ctypes.c_ulonglong),
                                     ctypes.POINTER(ctypes.c_float)]
    lib.sqrt_recip_check.restype = ctypes.c_int
    lib.sqrt_recip_at.argtypes = [ctypes.c_float, ctypes.c_float, ctypes.POINTER(ctypes.c_float)]
    lib.sqrt_recip_at.restype = ctypes.c_int
    return lib


def _run(lib, seed, count, mode, b0=0.0, y0=0.0):
    bad = ctypes.c_ulonglong(0)
    first = (ctypes.c_float * 2)()
    assert lib.quotient_check(seed, count, mode, b0, y0, ctypes.byref(bad), first) == 0
    return bad.value, (first[0], first[1])


def test_quotient_by_distance_equals_ieee_division(cuda_device):
    lib = _lib()
    total = 0
    for seed in range(8):
        bad, first = _run(lib, seed + 1, 1 << 30, 0)
        assert bad == 0, f"{bad} mismatches, first a={first[0]!r} b={first[1]!r}"
        total += 1 << 30
    assert total == 1 << 33


def test_quotient_by_poly6q_equals_ieee_division(pbf_mod, oracle_mod, cuda_device):
    lib = _lib()
    for scene in ("dam_break_1m", "dam_break_32k"):
        params = pbf_mod.load_scenario(scene)
        _, _, poly6q = oracle_mod.constants(params)
        b0 = np.float32(poly6q)
        y0 = np.float32(1.0) / b0
        bad, first = _run(lib, 99, 1 << 31, 1, float(b0), float(y0))
        assert bad == 0, f"{scene}: {bad} mismatches, first a={first[0]!r}"


def test_sqrt_and_reciprocal_equal_ieee_on_every_float(cuda_device):
    lib = _lib()
    bad = (ctypes.c_ulonglong * 3)()
    first = (ctypes.c_float * 2)()
    # bit patterns 0x0D800000 (2^-100) up to 0x5F800000 (2^64, excluded): |r| is sqrtf(r2) for all
    # of them; where y is not __frcp_rn(|r|), quotient_rn(a, |r|, y) is a / |r| for every numerator
    assert lib.sqrt_recip_check(0x0D800000, 0x5F800000, bad, first) == 0
    assert bad[0] == 0, f"{bad[0]} square roots differ from sqrtf, first at r2={first[0]!r}"
    assert bad[2] == 0, f"{bad[2]} quotients differ from IEEE division, first at r2={first[1]!r}"
    # r2 = 0 (coincident particles without the zero-distance guard): the quotient the
    # passes form is NaN, as IEEE 0 / 0 is
    out = (ctypes.c_float * 4)()
    assert lib.sqrt_recip_at(0.0, 0.0, out) == 0
    assert np.isnan(out[0]) and np.isnan(out[2]) and np.isnan(out[3])
