"""Build recipe for the test oracle (TEST INFRASTRUCTURE ONLY).

Two libraries:

* ``oracle/_build/libpbf_oracle.so`` — the CPU restatement in
  ``pbf_oracle.cpp`` (FP32 parity oracle and FP64 error oracle).
* ``oracle/_ref/libpbf_ref.so`` — the reference's own kernel sources
  (assets/kernels/*.cl, in the order of Simulation::KernelFileList,
  src/Simulation.cpp:103-127, without logging.cl) compiled as C++ through
  ``clshim.hpp`` and driven by ``ref_driver.inc``.  The generated translation
  unit ``oracle/_ref/ref_kernels.cpp`` is written from the reference checkout
  named by ``PBF_REFERENCE_DIR`` (or ``--reference DIR``) when it is set;
  the only edit made to the kernel text is the rewrite of OpenCL vector
  literals ``(float3)(a, b, c)`` into ``make_float3(a, b, c)``.
  Where the checkout is absent but a generated unit is already there, that
  unit is compiled.

Both are compiled with ``-ffp-contract=off`` so that every floating-point
operation is rounded on its own, on x86-64 and on aarch64 alike, and with
OpenMP: the restatement runs particles in parallel, the reference's kernels
run their work-items in parallel (``ref_driver.inc``).
"""
from __future__ import annotations

import os
import re
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
REPO = HERE.parent
BUILD = HERE / "_build"
REF_OUT = HERE / "_ref"


def reference_dir() -> Path | None:
    """The reference checkout whose kernels build_ref compiles: the directory
    named by PBF_REFERENCE_DIR, or None when it is unset (the generated unit
    already under oracle/_ref, if any, is compiled instead)."""
    d = os.environ.get("PBF_REFERENCE_DIR")
    return Path(d) if d else None


ORACLE_LIB = BUILD / "libpbf_oracle.so"
REF_LIB = REF_OUT / "libpbf_ref.so"
REF_TU = REF_OUT / "ref_kernels.cpp"

# Simulation::KernelFileList (src/Simulation.cpp:105-123), logging.cl omitted.
KERNEL_FILES = [
    "hesp.hpp", "parameters.hpp", "utilities.cl", "predict_positions.cl",
    "update_cells.cl", "build_friends_list.cl", "reset_grid.cl",
    "compute_scaling.cl", "compute_delta.cl", "update_predicted.cl",
    "pack_data.cl", "update_velocities.cl", "apply_viscosity.cl",
    "apply_vorticity.cl", "radixsort.cl",
]

CXXFLAGS = ["-O2", "-std=gnu++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math"]

_VEC_LITERAL = re.compile(r"\(\s*(float|int|uint)([234])\s*\)\s*\(")


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        sys.stderr.write(proc.stdout + proc.stderr)
        raise RuntimeError(f"command failed ({proc.returncode}): {' '.join(cmd)}")


def _stale(target: Path, sources: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(s.exists() and s.stat().st_mtime > t for s in sources)


def build_oracle(force: bool = False) -> Path:
    src = HERE / "pbf_oracle.cpp"
    deps = [src, REPO / "include" / "pbf_params.h", HERE / "noise_sin.hpp"]
    if force or _stale(ORACLE_LIB, deps):
        BUILD.mkdir(exist_ok=True)
        _run(["g++", *CXXFLAGS, "-fopenmp", str(src), "-o", str(ORACLE_LIB)])
    return ORACLE_LIB


def generate_ref_tu() -> bool:
    """Write oracle/_ref/ref_kernels.cpp from the reference checkout."""
    ref = reference_dir()
    if ref is None:
        return False
    kdir = ref / "assets" / "kernels"
    if not kdir.is_dir():
        return False
    parts = [
        "// GENERATED by oracle/build.py from the reference's assets/kernels/*.cl.\n",
        "// Not part of the repository (oracle/_ref is git-ignored).\n",
        "#include <cstdio>\n#include <cstdlib>\n",
        '#include "../../include/pbf_params.h"\n',
        '#include "../clshim.hpp"\n',
        "namespace clref {\n",
    ]
    for name in KERNEL_FILES:
        text = (kdir / name).read_text()
        text = _VEC_LITERAL.sub(lambda m: f"make_{m.group(1)}{m.group(2)}(", text)
        parts.append(f"\n// ---- {name} ----\n#line 1 \"{name}\"\n{text}\n")
    parts.append("}  // namespace clref\n")
    parts.append('#include "../ref_driver.inc"\n')
    REF_OUT.mkdir(exist_ok=True)
    new = "".join(parts)
    if not REF_TU.exists() or REF_TU.read_text() != new:
        REF_TU.write_text(new)
    return True


def build_ref(force: bool = False) -> Path | None:
    """Build the shimmed reference kernels; None when no source is available."""
    generated = generate_ref_tu()
    if not generated and not REF_TU.exists():
        return None
    deps = [REF_TU, HERE / "clshim.hpp", HERE / "ref_driver.inc", HERE / "noise_sin.hpp"]
    if force or _stale(REF_LIB, deps):
        _run(["g++", *CXXFLAGS, "-fopenmp", "-fwrapv", "-w", str(REF_TU), "-o", str(REF_LIB)])
    return REF_LIB


def build(force: bool = False) -> None:
    build_oracle(force)
    build_ref(force)


if __name__ == "__main__":
    # python oracle/build.py [--force] [--reference DIR]
    if "--reference" in sys.argv:
        os.environ["PBF_REFERENCE_DIR"] = sys.argv[sys.argv.index("--reference") + 1]
    build(force="--force" in sys.argv)
    print(ORACLE_LIB, REF_LIB if REF_LIB.exists() else "(reference kernels unavailable)")
