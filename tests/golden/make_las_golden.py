"""Writes tests/golden/lasio.npz from the reference's own LAS code.

Runs oracle/_ref/wb_ref (the reference's las.cpp, angle.cpp, manygcd.cpp ...
compiled unchanged by `make -C oracle ref`) on seeded records of every point
format 0-10: LasHeader::readPoint of each record (every LasPoint field), then
LasHeader::writePoint into a file opened the way CloudOutput::openFiles opens
one (openWrite, setUnit, setScale, setVersion 1.4, setPointFormat) and
writeHeader -- for several output formats, units and scales.  Also
combineScales and joinPointFormat on a few inputs.  Runs on the development
machine only (it needs the reference sources); the tests read the .npz.

    python tests/golden/make_las_golden.py
"""
from __future__ import annotations

import os
import struct
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import las_oracle as LO  # noqa: E402

WB_REF = os.path.join(ROOT, "oracle", "_ref", "wb_ref")
FEET = 1200 / 3937   # US survey foot, metres


def records_for(fmt, n, rng):
    lay = LO.layout(fmt)
    rec = rng.integers(0, 256, size=(n, lay["len"]), dtype=np.uint8)
    xyz = np.stack([rng.integers(-2_000_000, 2_000_000, n), rng.integers(-2_000_000, 2_000_000, n),
                    rng.integers(-200_000, 200_000, n)], axis=1).astype("<i4")
    rec[:, 0:12] = xyz.view(np.uint8).reshape(n, 12)
    if fmt < 6:
        ang = rng.integers(-90, 91, n)
        ang[:8] = [-128, 127, -91, 91, 0, -1, 1, 90]
        rec[:, 16] = (ang & 0xFF).astype(np.uint8)
    else:
        ang = rng.integers(-30000, 30001, n)
        ang[:8] = [-32768, 32767, -30000, 30000, 0, -1, 1, 15000]
        rec[:, 18:20] = (ang.astype("<i2")).view(np.uint8).reshape(n, 2)
    if lay["gps"] is not None:
        gps = rng.uniform(0, 1e9, n)
        rec[:, lay["gps"]:lay["gps"] + 8] = gps.astype("<f8").view(np.uint8).reshape(n, 8)
    return rec


def las_file(path, fmt, rec, scale, offset):
    n = rec.shape[0]
    h = bytearray(375)
    h[0:4] = b"LASF"
    h[24], h[25] = 1, 4
    struct.pack_into("<HHII", h, 94, 375, 375, 0, 0)
    struct.pack_into("<BH", h, 104, fmt, LO.POINT_LENGTHS[fmt])
    struct.pack_into("<6I", h, 107, n, n, 0, 0, 0, 0)
    struct.pack_into("<3d", h, 131, *scale)
    struct.pack_into("<3d", h, 155, *offset)
    struct.pack_into("<6d", h, 179, 1e9, -1e9, 1e9, -1e9, 1e9, -1e9)
    struct.pack_into("<QQI", h, 227, 0, 0, 0)
    nn = [0] * 16
    nn[0] = nn[1] = n
    struct.pack_into("<16Q", h, 247, *nn)
    with open(path, "wb") as f:
        f.write(bytes(h))
        f.write(rec.tobytes())


def run_case(tmp, k, fmt_in, rec, scale, offset, unit, fmt_out, out_scale, lo, hi, cls, sysid):
    inp = os.path.join(tmp, f"in{k}.las")
    outp = os.path.join(tmp, f"out{k}.las")
    clsp = os.path.join(tmp, f"cls{k}.bin")
    fld = os.path.join(tmp, f"fields{k}.bin")
    las_file(inp, fmt_in, rec, scale, offset)
    cls.astype(np.uint8).tofile(clsp)
    args = [WB_REF, "lasrw", inp, outp, str(fmt_out), repr(unit), *map(repr, out_scale), *map(repr, lo), *map(repr, hi),
            clsp, fld, str(sysid)]
    subprocess.run(args, check=True, timeout=60)
    dt = np.dtype([(name, t) for name, t in LO.FIELDS])
    fields = np.fromfile(fld, dtype=dt)
    out = np.fromfile(outp, dtype=np.uint8)
    return fields, out


def main():
    rng = np.random.default_rng(2026)
    cases = {}
    k = 0
    with tempfile.TemporaryDirectory() as tmp:
        for fmt_in in range(11):
            n = 96
            rec = records_for(fmt_in, n, rng)
            scale = (0.001, 0.001, 0.001) if fmt_in % 2 == 0 else (0.01, 0.005, 0.0025)
            offset = (1000.0, 2000.0, 100.0) if fmt_in % 3 else (500000.0, 4500000.0, 1500.0)
            outs = sorted({fmt_in, 1, 3, 6, 8, 10, (fmt_in + 5) % 11})
            for j, fmt_out in enumerate(outs):
                unit = FEET if (fmt_in + j) % 4 == 0 else 1.0
                dec = LO.decode(rec, fmt_in, scale, offset, unit)
                lo = tuple(float(dec[a].min()) - 0.5 for a in "xyz")
                hi = tuple(float(dec[a].max()) + 0.5 for a in "xyz")
                out_scale = (0.0, 0.0, 0.0) if j % 3 == 2 else (0.001, 0.002, 0.0005)
                cls = rng.integers(0, 256, n)
                sysid = j % 3
                fields, out = run_case(tmp, k, fmt_in, rec, scale, offset, unit, fmt_out, out_scale, lo, hi, cls,
                                       sysid)
                cases[f"c{k}_rec"] = rec
                cases[f"c{k}_meta"] = np.array([fmt_in, fmt_out, sysid], np.int64)
                cases[f"c{k}_in"] = np.array([*scale, *offset, unit], np.float64)
                cases[f"c{k}_out"] = np.array([*out_scale, *lo, *hi], np.float64)
                cases[f"c{k}_cls"] = cls.astype(np.uint8)
                cases[f"c{k}_fields"] = fields
                cases[f"c{k}_file"] = out
                k += 1
        combine_in = [
            ([[0.001] * 3], [[0.0] * 3]),
            ([[0.01, 0.01, 0.01], [0.001, 0.001, 0.001]], [[500000.0, 4500000.0, 1500.0]] * 2),
            ([[0.01, 0.01, 0.001], [0.005, 0.02, 0.001]], [[1000.0, 2000.0, 100.0], [1500.0, 2500.0, 50.0]]),
            ([[0.003, 0.003, 0.003], [0.002, 0.002, 0.002]], [[0.3, 0.6, 0.9], [0.4, 0.8, 1.2]]),
            ([[FEET * 0.01] * 3, [FEET * 0.01] * 3], [[FEET * 1e5] * 3, [FEET * 2e5] * 3]),
        ]
        comb = []
        for s, o in combine_in:
            args = [WB_REF, "combine", str(len(s))]
            for i in range(len(s)):
                args += [repr(v) for v in s[i]] + [repr(v) for v in o[i]]
            r = subprocess.run(args, check=True, capture_output=True, text=True, timeout=60)
            comb.append([float(v) for v in r.stdout.split()])
        cases["combine_scales"] = np.array([np.array(s, np.float64).ravel().tolist() + [np.nan] * (6 - 3 * len(s))
                                            for s, _ in combine_in])
        cases["combine_offsets"] = np.array([np.array(o, np.float64).ravel().tolist() + [np.nan] * (6 - 3 * len(o))
                                             for _, o in combine_in])
        cases["combine_n"] = np.array([len(s) for s, _ in combine_in])
        cases["combine_out"] = np.array(comb)
        joins = [[1], [0, 2], [1, 2], [6, 1], [4, 2], [7, 8], [9, 3], [0], [10, 0], [5, 6]]
        jout = []
        for j in joins:
            r = subprocess.run([WB_REF, "join", *map(str, j)], check=True, capture_output=True, text=True, timeout=60)
            jout.append(int(r.stdout))
        cases["join_in"] = np.array([j + [-1] * (2 - len(j)) for j in joins])
        cases["join_out"] = np.array(jout)
    cases["n_cases"] = np.array(k)
    np.savez_compressed(os.path.join(HERE, "lasio.npz"), **cases)
    print("wrote", k, "record cases")


if __name__ == "__main__":
    main()
