"""Writes tests/golden/c1_ref.npz: the reference's own serial run on the 1M-point
plain workload (1,000,000 points over 100 x 100 m, 1 mm int32 XYZ, offset 0,
seed 1; wolkenbase_gb300.synth.plain_small).

Runs oracle/_ref/wb_ref (the reference's octree / scan / classify sources,
compiled unchanged by `make -C oracle ref`) in pipeline mode: serial insertion
in input order, then scan, postscan and classify over every tile in flowsnake
order.  It takes about an hour of one core, so it runs on the development
machine only; the fixture keeps what the tests need in little room:

  xyz_sha256      digest of the int32 input, so a test knows it regenerated
                  the same cloud
  leaf_cube       every distinct leaf cube (center xyz, side), sorted
  stored_bits     per point, 1 where the record is stored (not overwritten by a
                  later identical point), bit-packed
  point_cube_sha256  digest of the (n, 4) float64 array of every point's leaf
                  cube (center xyz, side; zeros where not stored)
  cls_bits        per point, 1 where the reference wrote class 2 (ground),
                  bit-packed; cls_set_bits: 1 where it wrote any class
  tile_n          points per tile (flowsnake order)
  tile_flags      treeFlags per tile
  tile_h          hyperboloid size per tile after postscan
  timing          the reference's own stage times (seconds)

    python tests/golden/make_c1_golden.py [--raw DIR]

--raw keeps the reference's binary output in DIR and reuses it when present (default: a new
temporary directory).
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from wolkenbase_gb300 import synth  # noqa: E402


def xyz_digest(xyz):
    return hashlib.sha256(np.ascontiguousarray(xyz, dtype="<i4").tobytes()).hexdigest()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--raw", default=None)
    args = ap.parse_args()
    if not os.path.exists(O.REF_BIN):
        subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True)
    cloud = synth.plain_small(seed=1)
    raw = args.raw or tempfile.mkdtemp(prefix="c1_raw_")
    os.makedirs(raw, exist_ok=True)
    inp = os.path.join(raw, "in.wbxyz")
    out = os.path.join(raw, "ref.out")
    tim = os.path.join(raw, "timing.json")
    if not os.path.exists(out):
        synth.write_wbxyz(inp, cloud)
        r = subprocess.run([O.REF_BIN, "pipeline", inp, out, "1.0", "1.0", "0.0", "0.1", "3"], capture_output=True,
                           text=True, check=True)
        with open(tim, "w") as f:
            f.write(r.stdout.strip().splitlines()[-1])
    res = O.read_ref_output(out)
    timing = json.load(open(tim)) if os.path.exists(tim) else {}
    have = res["block"] >= 0          # records a later identical point overwrote have no block
    lc = np.where(have[:, None], res["leaf_cube"], 0.0)
    uniq = np.unique(lc[have], axis=0)
    cls = res["cls"]
    np.savez_compressed(
        os.path.join(HERE, "c1_ref.npz"),
        xyz_sha256=np.array(xyz_digest(cloud.xyz)), n=np.array(cloud.n),
        scale=np.array(cloud.scale), offset=np.array(cloud.offset), minc=np.array(cloud.minc),
        maxc=np.array(cloud.maxc), leaf_cube=uniq, stored_bits=np.packbits(have),
        point_cube_sha256=np.array(hashlib.sha256(np.ascontiguousarray(lc, dtype="<f8").tobytes()).hexdigest()),
        cls_bits=np.packbits(cls == 2), cls_set_bits=np.packbits(cls != 0),
        tile_n=res["tiles"]["n_points"].astype(np.int32), tile_flags=res["tiles"]["tree_flags"].astype(np.int8),
        tile_h=res["tiles"]["h_final"], root=np.array(list(res["root_center"]) + [res["root_side"]]),
        n_blocks=np.array(res["n_blocks"]), timing=np.array(json.dumps(timing)))
    print("c1_ref.npz written:", cloud.n, "points,", uniq.shape[0], "leaves,", timing)


if __name__ == "__main__":
    main()
