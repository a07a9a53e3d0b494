"""Build recipe for libpbf_gb300.so (the CUDA kernels plus the C-ABI).

Compiles every translation unit of ``csrc/`` for sm_103a in parallel and links
the shared library in-tree, next to this file.  Flags that matter for the
arithmetic contract:

* ``--fmad=false`` on the kernel translation units: no multiply-add
  contraction, so each float operation is rounded on its own;
* IEEE division and square root (nvcc's defaults; no ``--use_fast_math``);
* ``-ffp-contract=off`` for all host code, so the constants formed on the
  host are the same on x86-64 and aarch64.

``build(checked=True)`` builds libpbf_gb300_checked.so from the same sources
with ``-DPBF_CHECK_BOUNDS``: every index the kernels read from device memory
(friend-list entries, the sort permutation, keys) is checked before use and
an out-of-range one is reported through the context's error word.  The
arithmetic is the same, so its results are identical.  ``pbf.py`` loads it
when ``PBF_CHECK_BOUNDS=1`` is set.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
REPO = PKG.parent
CSRC = PKG / "csrc"
OBJ = PKG / "_build"
LIB = PKG / "libpbf_gb300.so"
OBJ_CHECKED = PKG / "_build_checked"
LIB_CHECKED = PKG / "libpbf_gb300_checked.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
INCLUDES = ["-I", str(REPO / "include"), "-I", str(CSRC)]
HOST_FLAGS = ["-fPIC", "-ffp-contract=off", "-fno-fast-math"]

# translation unit -> extra nvcc flags
CUDA_UNITS = {
    "pbf_kernels.cu": ["--fmad=false"],
    "pbf_sort.cu": [],
    "pbf_capi.cu": ["--fmad=false"],
    "pbf_noalloc.cu": ["--fmad=false"],
    "pbf_adjoint.cu": [],
    "pbf_render.cu": ["--fmad=false"],
}
CXX_UNITS = ["params.cpp"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def _cuda_include() -> str:
    nvcc = Path(_nvcc()).resolve()
    return str(nvcc.parent.parent / "include")


def _run(cmd: list[str]) -> tuple[int, str]:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    return proc.returncode, proc.stdout + proc.stderr


def _headers() -> list[Path]:
    return sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted((REPO / "include").glob("*.h"))


def _stale(obj: Path, src: Path) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(p.stat().st_mtime > t for p in [src, *_headers(), Path(__file__)])


def compile_commands(checked: bool = False) -> list[tuple[Path, Path, list[str]]]:
    jobs = []
    out = OBJ_CHECKED if checked else OBJ
    defs = ["-DPBF_CHECK_BOUNDS"] if checked else []
    for unit, extra in CUDA_UNITS.items():
        src, obj = CSRC / unit, out / (unit + ".o")
        cmd = [_nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", *extra, *defs, *INCLUDES,
               "-Xcompiler", ",".join(HOST_FLAGS), "-c", str(src), "-o", str(obj)]
        jobs.append((src, obj, cmd))
    for unit in CXX_UNITS:
        src, obj = CSRC / unit, out / (unit + ".o")
        cmd = ["g++", "-O2", "-std=c++17", *HOST_FLAGS, *INCLUDES, "-I", _cuda_include(),
               "-c", str(src), "-o", str(obj)]
        jobs.append((src, obj, cmd))
    return jobs


def build(force: bool = False, verbose: bool = False, checked: bool = False) -> Path:
    out, lib = (OBJ_CHECKED, LIB_CHECKED) if checked else (OBJ, LIB)
    out.mkdir(exist_ok=True)
    jobs = [j for j in compile_commands(checked) if force or _stale(j[1], j[0])]
    if jobs:
        with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
            results = list(ex.map(lambda j: _run(j[2]), jobs))
        for (src, _, cmd), (rc, log) in zip(jobs, results):
            if verbose and log:
                sys.stderr.write(log)
            if rc != 0:
                sys.stderr.write(log)
                raise RuntimeError(f"compile failed: {src.name}\n{' '.join(cmd)}")
    objs = [str(o) for _, o, _ in compile_commands(checked)]
    if force or jobs or not lib.exists():
        # the library exports the C-ABI (pbf_*) and nothing of its internals
        exports = out / "exports.map"
        exports.write_text("{\n  global: pbf_*;\n  local: *;\n};\n")
        tmp = lib.with_suffix(".so.tmp")
        rc, log = _run([_nvcc(), *ARCH, "-shared", "-o", str(tmp), *objs, "-lcudart",
                        "-Xlinker", f"--version-script={exports}"])
        if rc != 0:
            sys.stderr.write(log)
            raise RuntimeError("link failed")
        os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv, checked="--checked" in sys.argv))
