"""Precision mode report: the FP32 path (tile-local FP32 coordinates,
compensated fit sums, FP64 3x3 solve, FP32 neighbour decisions) against the
exact FP64 path on the same cloud.

  flips        points whose class byte differs
  agreement    1 - flips / points
  slope_err    max over tiles of |(a, b)_fp32 - (a, b)_fp64| (and its 99.9th
               percentile: a fit of a few nearly collinear points is
               ill-conditioned in any precision)
  residual_err max over tiles of max_i |r32_i - r64_i| / max(max_i |r64_i|, q),
               where r = z - (a*x + b*y + c) is a point's fit residual and q
               the height quantum (scale * unit).  The difference of two
               planes is linear in x and y, so over the tile cylinder
               (radius R) it is at most |da|R + |db|R + |dc|; max_i |r64_i| is
               at least half the tile's untilted height range.  The ratio of
               the two bounds is reported.
  h_rel_err    max relative difference of the tiles' hyperboloid sizes
"""
from __future__ import annotations

import time

import numpy as np

from . import _lib


def compare(clf, cloud, params=None, built=False):
    """Runs scan + classify exact and in FP32 on one built context."""
    if not built:
        clf.set_precision(_lib.WB_PRECISION_EXACT)
        clf.build(cloud)
    out = {}
    res = {}
    for name, mode in (("fp64", _lib.WB_PRECISION_EXACT), ("fp32", _lib.WB_PRECISION_FP32)):
        clf.set_precision(mode)
        clf.synchronize()
        t0 = time.perf_counter()
        clf.scan(params)
        t1 = time.perf_counter()
        cls = clf.classify(params)
        t2 = time.perf_counter()
        res[name] = (cls, clf.planes(), clf.tiles())
        out[name + "_ms"] = {"scan": (t1 - t0) * 1e3, "classify": (t2 - t1) * 1e3}
    clf.set_precision(_lib.WB_PRECISION_EXACT)
    c64, p64, t64 = res["fp64"]
    c32, p32, t32 = res["fp32"]
    flips = int(np.count_nonzero(c64 != c32))
    n = int(c64.size)
    ok = (t64["n_points"] >= 3) & np.all(np.isfinite(p64), axis=1) & np.all(np.isfinite(p32), axis=1)
    d = np.abs(p32 - p64)[ok]
    R = clf.info()["spacing"] * 41.0 / 71.0
    bound = d[:, 0] * R + d[:, 1] * R + d[:, 2]
    q = abs(cloud.scale[2] * cloud.unit)
    half = np.maximum(t64["height"][ok] / 2, q)
    h64, h32 = t64["hyperboloid_size"], t32["hyperboloid_size"]
    hm = (t64["n_points"] > 0) & (h64 > 0)
    out.update({
        "points": n, "flips": flips, "agreement": 1.0 - flips / max(n, 1),
        "tiles_compared": int(ok.sum()),
        "slope_err": float(np.max(np.hypot(d[:, 0], d[:, 1]))) if len(d) else 0.0,
        "slope_err_p999": float(np.percentile(np.hypot(d[:, 0], d[:, 1]), 99.9)) if len(d) else 0.0,
        "residual_abs_err_m": float(np.max(bound)) if len(d) else 0.0,
        "residual_err": float(np.max(bound / half)) if len(d) else 0.0,
        "residual_err_p999": float(np.percentile(bound / half, 99.9)) if len(d) else 0.0,
        "h_rel_err": float(np.max(np.abs(h32[hm] - h64[hm]) / h64[hm])) if hm.any() else 0.0,
        "tree_flag_changes": int(np.count_nonzero(t64["tree_flags"] != t32["tree_flags"])),
    })
    return out
