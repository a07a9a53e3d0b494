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
BoxClamp 0.  Run from the repository root, with PBF_REFERENCE_DIR naming the
reference checkout:  PBF_REFERENCE_DIR=<checkout> python tests/golden/make_golden.py
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
    # the benchmark's published solver constants: violent dynamics (velocities of tens of m/s)
    ("literal_32k_8sub", (32, 32, 32), {"base": "dam_break_32k_literal"}, 8),
]
SEED = 20240601

# Force planes: the reference's 14 BouncePointQuad calls are read from its
# computeDelta source and stored as data; a 4,096-particle block falls onto
# plane 7 (a floor at y = -41.65, normal +y) through a mask with holes.
FORCE_CASE = {"name": "force_planes_4k_4sub", "block": [16, 16, 16], "origin": [-62.0, -40.9, -1.0],
              "substeps": 4, "mask": {"width": 512, "height": 9262, "rule": "0 where (x // 8 + y // 4) % 3 == 0, else 1"}}


def reference_force_quads():
    """The 14 planes hard-coded in the reference (compute_delta.cl:169-182)."""
    import re
    src = (oracle._build.reference_dir() / "assets" / "kernels" / "compute_delta.cl").read_text()
    vec = r"\(float3\)\(\s*([-0-9.eE]+),\s*([-0-9.eE]+),\s*([-0-9.eE]+)\)"
    pat = re.compile(r"BouncePointQuad\(positions\[i\]\.xyz, future, " + vec + r", " + vec + r", " + vec +
                     r", surfacesMask, (\d+), (\d+), edgeOffset\)")
    quads = []
    for m in pat.finditer(src):
        v = [float(x) for x in m.groups()[:9]]
        quads.append({"B": v[0:3], "E0": v[3:6], "E1": v[6:9], "maskYOffset": int(m.group(10)),
                      "maskHeight": int(m.group(11))})
    return quads


def force_mask(spec):
    y, x = np.mgrid[0:spec["height"], 0:spec["width"]]
    return np.where((x // 8 + y // 4) % 3 == 0, 0, 1).astype(np.uint32)


def quads_array(quads):
    a = np.zeros(len(quads), oracle.QUAD_DTYPE)
    for k, q in enumerate(quads):
        a[k] = (q["B"], q["E0"], q["E1"], q["maskYOffset"], q["maskHeight"])
    return a


def force_scene():
    params = pbf.load_scenario("dam_break_32k")
    params.boxClamp = 0
    params.zeroDistanceGuard = 0
    dims = FORCE_CASE["block"]
    params.particleCount = dims[0] * dims[1] * dims[2]
    pos = pbf.scene_block(*dims, 0.05, tuple(FORCE_CASE["origin"]), 0.005, SEED)
    return params, pos, np.zeros_like(pos)


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
    if oracle._build.reference_dir() is None or not oracle.ref_available():
        raise SystemExit("set PBF_REFERENCE_DIR to the reference checkout to generate the golden vectors")
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
    quads = reference_force_quads()
    assert len(quads) == 14, len(quads)
    params, pos, vel = force_scene()
    oracle.ref_set_force_mask(force_mask(FORCE_CASE["mask"]))
    try:
        p, v, pr, keys, perm, cells = oracle.ref_step(params, pos, vel, FORCE_CASE["substeps"])
    finally:
        oracle.ref_set_force_mask(None)
    arrays = {"pos": p, "vel": v, "pred": pr, "keys": keys, "perm": perm, "cells": cells}
    manifest["force_planes"] = dict(FORCE_CASE, quads=quads, sha256={k: digest(a) for k, a in arrays.items()},
                                    source="reference assets/kernels/compute_delta.cl:169-182")
    moved = float(np.mean(np.abs(p[:, 1] - pos[:, 1]) > 0))
    print(f"{FORCE_CASE['name']}: n={params.particleCount}, min y {p[:, 1].min():.3f}, nan {int(np.isnan(p).sum())}")
    (OUT / "golden.json").write_text(json.dumps(manifest, indent=1) + "\n")


if __name__ == "__main__":
    main()
