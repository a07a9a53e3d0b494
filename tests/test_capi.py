"""The C-ABI library: it loads, exports what include/*.h declares, and fails
cleanly where no GPU is present (CPU only; no kernel is launched)."""
from __future__ import annotations

import ctypes
import re
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parent.parent


def declared_functions() -> set[str]:
    names = set()
    for h in (REPO / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names.update(re.findall(r"\b(pbf_[a-z0-9_]+)\s*\(", text))
    return names


def test_every_declared_symbol_is_exported(built_lib, pbf_mod):
    lib = ctypes.CDLL(str(built_lib))
    declared = declared_functions()
    assert declared, "no declarations found"
    missing = [n for n in sorted(declared) if not hasattr(lib, n)]
    assert not missing, f"declared but not exported: {missing}"
    assert set(pbf_mod.EXPORTED_SYMBOLS) <= declared


def test_library_exports_only_the_declared_c_abi(built_lib):
    """The dynamic symbol table holds exactly the functions include/*.h
    declares: no internal C++ function or helper leaks into a caller's
    namespace."""
    import shutil
    import subprocess
    nm = shutil.which("nm")
    if nm is None:
        pytest.skip("nm not available")
    out = subprocess.run([nm, "-D", "--defined-only", str(built_lib)], capture_output=True, text=True, check=True)
    exported = {line.split()[-1] for line in out.stdout.splitlines() if line.strip()}
    assert exported == declared_functions()


def test_build_tracks_every_header():
    """A unit is rebuilt when any header it may include changes, device
    headers (.cuh) included: an edit there must not leave stale objects."""
    from tests.conftest import load_pkg_build
    pkg_build = load_pkg_build()
    tracked = {h.name for h in pkg_build._headers()}
    csrc = REPO / "position-based-fluids_gb300" / "csrc"
    headers = {h.name for pattern in ("*.h", "*.cuh") for h in csrc.glob(pattern)}
    headers |= {h.name for h in (REPO / "include").glob("*.h")}
    assert headers and headers <= tracked, f"untracked headers: {sorted(headers - tracked)}"


def test_checked_build_exports_the_same_symbols():
    """The bounds-checked build (build.py --checked) is a drop-in for the plain
    library: built from the same sources with -DPBF_CHECK_BOUNDS into its own
    object directory, it exports every declared symbol."""
    from tests.conftest import load_pkg_build
    pkg_build = load_pkg_build()
    commands = pkg_build.compile_commands(checked=True)
    assert all("-DPBF_CHECK_BOUNDS" in cmd for src, _, cmd in commands if src.suffix == ".cu")
    assert all(obj.parent == pkg_build.OBJ_CHECKED for _, obj, _ in commands)
    lib = ctypes.CDLL(str(pkg_build.build(checked=True)))
    missing = [n for n in sorted(declared_functions()) if not hasattr(lib, n)]
    assert not missing, f"declared but not exported: {missing}"


def test_create_without_device_or_with_bad_args(pbf_mod):
    from tests.conftest import has_cuda_device
    p = pbf_mod.load_scenario("dam_break_32k")
    if not has_cuda_device():
        with pytest.raises(pbf_mod.PbfError) as e:
            pbf_mod.Simulation(p)
        assert e.value.code == pbf_mod.PBF_ERR_NO_DEVICE
    lib = pbf_mod.library()
    ctx = ctypes.c_void_p()
    assert lib.pbf_create(None, 0, ctypes.byref(ctx)) == pbf_mod.PBF_ERR_INVALID
    assert b"NULL" in lib.pbf_last_error(None)
    # calls on a NULL context are rejected, not crashed
    assert lib.pbf_step(None, 1) == pbf_mod.PBF_ERR_INVALID
    assert lib.pbf_init_cells(None) == pbf_mod.PBF_ERR_INVALID
    assert lib.pbf_destroy(None) == pbf_mod.PBF_OK
