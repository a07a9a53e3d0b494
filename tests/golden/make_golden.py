"""Generate tests/golden/ from the reference's own kernels.

Runs the reference's assets/kernels/*.cl, compiled as C++ through
oracle/clshim.hpp (oracle/build.py builds oracle/_ref from the reference
checkout), on seeded dam-break scenes and writes

* golden.json   — per case: the scene, the parameter overrides, the number of
                  substeps, and SHA-256 digests of every output array
                  (positions, velocities, predictions after the last substep;
                  sorted keys, permutation and cell table of that substep);
* small_case.npz — every output array of the smallest case in full.

The box clamp is a stage the reference does not have, so every case runs with
BoxClamp 0.  Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(REPO))
sys.path.insert(0, str(REPO / "position-based-fluids_gb300"))

import pbf  # noqa: E402
from oracle import oracle  # noqa: E402

OUT = Path(__file__).resolve().parent

# name, block dims, parameter overrides, substeps; "base" selects the
# scenario file the overrides apply to (default dam_break_32k)
CASES = [
    ("small_2k_2sub", (16, 16, 8), {}, 2),
    ("dam32k_1sub", (32, 32, 32), {}, 1),
    ("dam32k_2sub", (32, 32, 32), {}, 2),
    ("dam32k_6sub", (32, 32, 32), {}, 6),
    # hash collisions: 64 buckets, so distinct cells share a bucket and some
    # of the 27 neighbour cells map to the same bucket (double visits)
    ("collide_4k_grid64", (16, 16, 16), {"gridBufSize": 64}, 2),
    # friend-list overflow: 8 per circle drops neighbours (build_friends_list.cl:79-83)
    ("overflow_4k_cap8", (16, 16, 16), {"particlesPerCircle": 8}, 2),
    # 3 circles and 2 solver iterations, odd particle count (not a multiple of 32)
    ("circles3_iter2_odd", (17, 13, 11), {"friendsCircles": 3, "simIterations": 2}, 2),
    # larger kernel radius: more neighbours per particle
    ("wide_h_4k", (16, 16, 16), {"h": 0.13, "h_2": 0.13 * 0.13, "gridBufSize": 4096}, 1),
    # the BASELINE solver constants: violent dynamics (velocities of tens of m/s)
    ("literal_32k_8sub", (32, 32, 32), {"base": "dam_break_32k_literal"}, 8),
]
SEED = 20240601


def scene(dims, overrides):
    params = pbf.load_scenario(overrides.get("base", "dam_break_32k"))
    params.boxClamp = 0            # stages the reference does not have
    params.zeroDistanceGuard = 0
    for k, v in overrides.items():
        if k == "base":
            continue
        if k == "h_2":
            v = float(np.float32(np.float32(overrides["h"]) * np.float32(overrides["h"])))
        setattr(params, k, v)
    n = dims[0] * dims[1] * dims[2]
    params.particleCount = n
    pos = pbf.scene_block(*dims, 0.05, (0.025, 0.025, 0.025), 0.005, SEED)
    return params, pos, np.zeros_like(pos)


def canonical(a: np.ndarray) -> np.ndarray:
    """Float arrays with every NaN replaced by one bit pattern (0x7FC00000):
    NaN payloads differ between x86-64, aarch64 and the GPU."""
    a = np.ascontiguousarray(a)
    if a.dtype == np.float32:
        a = a.copy()
        a[np.isnan(a)] = np.float32("nan")
        a.view(np.uint32)[np.isnan(a)] = 0x7FC00000
    return a


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(canonical(a).tobytes()).hexdigest()


def main() -> None:
    if not oracle.ref_available():
        raise SystemExit("the reference checkout is needed to generate the golden vectors")
    manifest = {
        "generator": "tests/golden/make_golden.py",
        "source": "reference assets/kernels/*.cl compiled through oracle/clshim.hpp (oracle/_ref)",
        "scene": {"spacing": 0.05, "origin": [0.025, 0.025, 0.025], "jitter": 0.005, "seed": SEED,
                  "base_par": "dam_break_32k", "boxClamp": 0, "zeroDistanceGuard": 0},
        "cases": [],
    }
    for name, dims, overrides, substeps in CASES:
        params, pos, vel = scene(dims, overrides)
        p, v, pr, keys, perm, cells = oracle.ref_step(params, pos, vel, substeps)
        arrays = {"pos": p, "vel": v, "pred": pr, "keys": keys, "perm": perm, "cells": cells}
        manifest["cases"].append({
            "name": name, "block": list(dims), "overrides": overrides, "substeps": substeps,
            "sha256": {k: digest(a) for k, a in arrays.items()},
        })
        if name == "small_2k_2sub":
            np.savez_compressed(OUT / "small_case.npz", init_pos=pos, **arrays)
        print(f"{name}: n={params.particleCount} substeps={substeps}")
    (OUT / "golden.json").write_text(json.dumps(manifest, indent=1) + "\n")


if __name__ == "__main__":
    main()
