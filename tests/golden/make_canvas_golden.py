"""Generates tests/golden/reference_canvas.npz from the reference's own Canvas.

src/voromesh/canvas.cpp and shape2d.cpp are compiled for the host by
oracle/ref_shim/build_ref.sh into oracle/_ref/libref_canvas.so; this script
drives them (RasterizeShape, then a seeded series of StampDisc calls) and
records the polygon, the stamp parameters, every edit (tile rectangle,
counts, dirty-slot list) and the full canvas state at checkpoints. Needs the
reference sources (run where they are present):

    REF=/path/to/reference bash oracle/ref_shim/build_ref.sh
    python tests/golden/make_canvas_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT / "bb-temp-testing_gb300"))
sys.path.insert(0, str(ROOT))

from oracle import oracle as orc  # noqa: E402

CASES = [
    # name, width, height, voxel, heart (cx, cy, width, segments), stamps, seed, checkpoint every
    ("heart96", 96.0, 96.0, 1.0, (48.0, 48.0, 76.8, 500), 32, 11, 8),
    ("heart_odd", 50.0, 37.0, 0.37, (25.0, 18.0, 30.0, 61), 24, 12, 8),
]


def compact(st: dict) -> dict:
    on = np.flatnonzero(st["sslot"] >= 0)
    return dict(inside=st["inside"], smask=st["smask"], vox=on.astype(np.int32), pts=st["spt"][on],
                vslots=st["sslot"][on], slots=st["slots"], free=st["free"], counts=np.asarray(st["counts"], np.int64))


def main() -> None:
    if not orc.ref_canvas_available():
        raise SystemExit("oracle/_ref/libref_canvas.so missing: run oracle/ref_shim/build_ref.sh first")
    from voromesh_gb300 import synth

    out = {}
    for name, w, h, vs, hp, nst, seed, every in CASES:
        poly = synth.heart(*hp)
        c = orc.RefCanvas(w, h, vs)
        c.rasterize(poly)
        out[f"{name}/dims"] = np.array([w, h, vs], np.float32)
        out[f"{name}/poly"] = poly
        for k, v in compact(c.state()).items():
            out[f"{name}/s0/{k}"] = v
        rng = np.random.default_rng(seed)
        stamps, edits, dirty = [], [], []
        for k in range(nst):
            cx, cy = rng.uniform(-0.1 * w, 1.1 * w), rng.uniform(-0.1 * h, 1.1 * h)
            r = rng.uniform(0.5, 0.2 * min(w, h) / vs) * vs
            ins = int(rng.integers(2))
            stamps.append((cx, cy, r, ins))
            e = c.stamp(np.float32(cx), np.float32(cy), np.float32(r), ins)
            edits.append(e.rect() + e.counts() + (len(e.dirty),))
            dirty.append(e.dirty)
            if (k + 1) % every == 0:
                for kk, v in compact(c.state()).items():
                    out[f"{name}/s{k + 1}/{kk}"] = v
        out[f"{name}/stamps"] = np.asarray(stamps, np.float32)
        out[f"{name}/edits"] = np.asarray(edits, np.int32)
        out[f"{name}/dirty"] = np.concatenate(dirty).astype(np.int32) if dirty else np.zeros(0, np.int32)
    np.savez_compressed(HERE / "reference_canvas.npz", **out)
    print("wrote", HERE / "reference_canvas.npz", sum(v.nbytes for v in out.values()), "bytes raw")


if __name__ == "__main__":
    main()
