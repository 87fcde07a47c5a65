"""Writes the golden fixtures in this directory from the reference's own code.

Runs oracle/_ref/wb_ref -- the reference's octree / scan / classify / angle /
flowsnake / least-squares sources compiled unchanged by `make -C oracle ref`
-- on small seeded inputs and stores inputs and outputs as compressed .npz
files.  Needs the reference source tree (the REF environment variable, passed
on to `make -C oracle ref`) and runs on the development machine only; the
tests read the committed .npz files.

    python tests/golden/make_golden.py [NAME ...]

With names, only those fixtures are written (e.g. `negscale8k`).
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

from oracle import oracle as O  # noqa: E402
from wolkenbase_gb300 import synth  # noqa: E402

CASES = {
    # name: (builder, params, phases)
    "tile20k": (lambda: synth.density_tile(20000, 7), dict(), 3),
    "params6k": (lambda: synth.density_tile(6000, 11),
                 dict(tile_size=0.5, max_slope=1.5, thickness=0.02, min_hyp_size=0.05), 3),
    "utm8k": (lambda: synth.terrain_cloud(8000, 9.0, 9.0, 13, scale=(0.01, 0.01, 0.01),
                                          offset=(500000.0, 4500000.0, 1500.0), max_slope=1.0, steps=2.0,
                                          origin=(3.0, 5.0)), dict(), 3),
    "dups5k": (None, dict(), 3),
    "split": (None, dict(), 1),
    # x and z record integers running against the coordinates (negative scales)
    "negscale8k": (lambda: negscale_cloud(), dict(), 3),
}

SPLIT_PRIMES = [(523, 516), (541, 10), (719, 710), (727, 10), (4289, 17), (4297, 15), (5749, 18), (5779, 5762)]


def negscale_cloud():
    """A seeded tile with its x and z record integers and scales negated: the
    same decoded points, read through negative scales."""
    c = synth.density_tile(8000, 23)
    xyz = c.xyz.copy()
    xyz[:, 0] = -xyz[:, 0]
    xyz[:, 2] = -xyz[:, 2]
    return synth.Cloud(xyz, (-c.scale[0], c.scale[1], -c.scale[2]), c.offset, c.unit, c.minc, c.maxc)


def dups_cloud():
    c = synth.density_tile(5000, 17)
    rng = np.random.default_rng(170)
    pick = rng.choice(c.n, 500, replace=False)
    xyz = np.concatenate([c.xyz, c.xyz[pick]])
    perm = rng.permutation(xyz.shape[0])
    return synth.Cloud(xyz[perm], c.scale, c.offset, c.unit, c.minc, c.maxc)


def split_cloud():
    """Primitive-root lattices around the 537-point split threshold
    (the point sets of wolkentest.cpp:933-981), concatenated side by side."""
    xs, ys, zs = [], [], []
    xoff = 0
    for p, r in SPLIT_PRIMES:
        zstep = (r * r) % p
        i = np.arange(p, dtype=np.int64)
        xs.append(i + xoff)
        ys.append((i * r) % p)
        zs.append((i * zstep) % p)
        xoff += p + 7
    xyz = np.stack([np.concatenate(xs), np.concatenate(ys), np.concatenate(zs)], axis=1).astype(np.int32)
    scale = (1 / 5779, 1 / 5779, 1 / 5779)
    c = synth.Cloud(xyz, scale, (0.0, 0.0, 0.0), 1.0, (0, 0, 0), (0, 0, 0))
    d = c.decoded()
    c.minc = tuple(d.min(axis=0))
    c.maxc = tuple(d.max(axis=0))
    return c


def run_case(name, cloud, params, phases, tmp):
    res = O.run_reference(cloud, tmp, phases=phases, timeout=3600, **params)
    out = dict(xyz=cloud.xyz.astype(np.int32), scale=np.array(cloud.scale), offset=np.array(cloud.offset),
               unit=np.array(cloud.unit), minc=np.array(cloud.minc), maxc=np.array(cloud.maxc),
               phases=np.array(phases), params=np.array([params.get("tile_size", 1.0), params.get("max_slope", 1.0),
                                                         params.get("thickness", 0.0),
                                                         params.get("min_hyp_size", 0.1)]),
               block=res["block"].astype(np.int32), pos=res["pos"].astype(np.int32), cls=res["cls"],
               leaf_cube=res["leaf_cube"], tiles=res["tiles"], root=np.array(list(res["root_center"]) +
                                                                            [res["root_side"]]),
               snake=np.array(list(res["snake_center"]) + [res["snake_side"], res["spacing"]]),
               n_blocks=np.array(res["n_blocks"]))
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    print(name, res["timing"])


def primitives(tmp):
    ref = O.REF_BIN
    tab = os.path.join(tmp, "tables.bin")
    subprocess.run([ref, "tables", tab], check=True)
    t = np.fromfile(tab, "<f8")
    quad = os.path.join(tmp, "quad.bin")
    subprocess.run([ref, "quadrant", quad], check=True)
    q = np.fromfile(quad, "<f8")
    rng = np.random.default_rng(42)
    m = 15000
    y = rng.integers(-20000, 20000, m) * 0.001
    x = rng.integers(-20000, 20000, m) * 0.001
    # axis and diagonal cases, tiny and huge ratios, zeros
    ex = [(0.0, 0.0), (0.0, 1.0), (1.0, 0.0), (0.0, -1.0), (-1.0, 0.0), (1.0, 1.0), (-1.0, -1.0), (1.0, -1.0),
          (-1.0, 1.0), (1e-3, -100.0), (-1e-3, -100.0), (0.0, -5.0), (-0.0, -5.0), (3.0, 4.0), (4.0, 3.0)]
    y = np.concatenate([y, [e[0] for e in ex], rng.normal(0, 1, 5000)])
    x = np.concatenate([x, [e[1] for e in ex], rng.normal(0, 1, 5000)])
    yx = np.stack([y, x], axis=1).astype("<f8")
    fin = os.path.join(tmp, "a_in.bin")
    fout = os.path.join(tmp, "a_out.bin")
    with open(fin, "wb") as f:
        f.write(np.uint64(yx.shape[0]).tobytes())
        f.write(yx.tobytes())
    subprocess.run([ref, "atan2i", fin, fout], check=True)
    a = np.fromfile(fout, "<i4")
    snakes = {}
    for idx in range(6):
        fs = os.path.join(tmp, f"fs{idx}.bin")
        subprocess.run([ref, "flowsnake", str(idx), fs], check=True)
        snakes[f"flowsnake{idx}"] = np.fromfile(fs, "<i4").reshape(-1, 2)
    # least-squares planes of 3..200 points
    systems = []
    lsin = os.path.join(tmp, "lsq_in.bin")
    with open(lsin, "wb") as f:
        f.write(np.uint64(40).tobytes())
        for s in range(40):
            rows = int(rng.integers(3, 200))
            pts = np.stack([rng.uniform(-1, 1, rows), rng.uniform(-1, 1, rows), rng.normal(0, 1, rows)], 1)
            if s % 10 == 0:
                pts[:, 2] = 0.3 * pts[:, 0] - 0.7 * pts[:, 1] + 2.0   # exact plane
            systems.append(pts)
            f.write(np.uint64(rows).tobytes())
            f.write(pts.astype("<f8").tobytes())
    lsout = os.path.join(tmp, "lsq_out.bin")
    subprocess.run([ref, "lsq", lsin, lsout], check=True)
    sol = np.fromfile(lsout, "<f8").reshape(-1, 3)
    lens = np.array([p.shape[0] for p in systems])
    np.savez_compressed(os.path.join(HERE, "primitives.npz"), tan=t[:511], sin=t[511:1023], cos=t[1023:],
                        quadrant=q, atan_yx=yx, atan_out=a, lsq_len=lens, lsq_pts=np.concatenate(systems),
                        lsq_sol=sol, **snakes)
    print("primitives", yx.shape[0], "atan2i cases")


def main():
    if not os.path.exists(O.REF_BIN):
        subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True)
    only = set(sys.argv[1:])
    with tempfile.TemporaryDirectory() as tmp:
        if not only:
            primitives(tmp)
        for name, (builder, params, phases) in CASES.items():
            if only and name not in only:
                continue
            if name == "dups5k":
                cloud = dups_cloud()
            elif name == "split":
                cloud = split_cloud()
            else:
                cloud = builder()
            run_case(name, cloud, params, phases, tmp)


if __name__ == "__main__":
    main()
