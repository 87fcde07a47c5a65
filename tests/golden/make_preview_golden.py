"""Writes tests/golden/preview.npz from the reference's own octree queries.

Runs `oracle/_ref/wb_ref preview` (the reference's octree.cpp / shape.cpp
compiled unchanged by `make -C oracle ref`): the points of each golden cloud
put into the reference's OctStore, then OctStore::countPointsIn and
hiLoPointsIn (octree.cpp:1244-1293) of the Column (shape.cpp:245-254) of
every pixel of a few views.  Runs on the development machine only (it needs
the reference sources); the tests read the .npz.

    python tests/golden/make_preview_golden.py
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from wolkenbase_gb300 import synth  # noqa: E402

WB_REF = os.path.join(ROOT, "oracle", "_ref", "wb_ref")
CASES = ["tile20k", "utm8k", "split", "dups5k"]


def cloud_of(name):
    g = np.load(os.path.join(HERE, name + ".npz"))
    return synth.Cloud(g["xyz"].astype(np.int32), tuple(g["scale"]), tuple(g["offset"]), float(g["unit"]),
                       tuple(g["minc"]), tuple(g["maxc"]))


def views(cloud):
    d = cloud.decoded()
    lo, hi = d.min(axis=0), d.max(axis=0)
    span = max(hi[0] - lo[0], hi[1] - lo[1])
    out = []
    for k, frac in enumerate((0.02, 0.037, 0.11)):
        side = float(np.float64(span * frac))
        x0 = float(lo[0] - 0.3 * side)
        y0 = float(lo[1] + 0.25 * side)
        w = min(64, int((hi[0] - x0) / side) + 2)
        h = min(48, int((hi[1] - y0) / side) + 2)
        out.append((x0, y0, side, w, h))
    return out


def main():
    res = {}
    with tempfile.TemporaryDirectory() as tmp:
        for name in CASES:
            cloud = cloud_of(name)
            inp = os.path.join(tmp, name + ".wbxyz")
            synth.write_wbxyz(inp, cloud)
            for k, (x0, y0, side, w, h) in enumerate(views(cloud)):
                outp = os.path.join(tmp, f"{name}_{k}.bin")
                subprocess.run([WB_REF, "preview", inp, outp, repr(x0), repr(y0), repr(side), str(w), str(h)],
                               check=True, timeout=600)
                raw = np.fromfile(outp, dtype=np.dtype([("count", "<u8"), ("lo", "<f8"), ("hi", "<f8")]))
                res[f"{name}_{k}_view"] = np.array([x0, y0, side, w, h], np.float64)
                res[f"{name}_{k}_count"] = raw["count"].reshape(h, w)
                res[f"{name}_{k}_lo"] = raw["lo"].reshape(h, w)
                res[f"{name}_{k}_hi"] = raw["hi"].reshape(h, w)
    res["cases"] = np.array(CASES)
    np.savez_compressed(os.path.join(HERE, "preview.npz"), **res)
    print("wrote", len(res), "arrays")


if __name__ == "__main__":
    main()
