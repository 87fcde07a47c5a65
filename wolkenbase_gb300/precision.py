"""Precision mode report: the FP32 path (tile-local FP32 coordinates,
compensated fit sums, FP64 3x3 solve, FP32 neighbour decisions) against the
exact FP64 path on the same cloud.

  flips        points whose class byte differs
  agreement    1 - flips / points
  slope_err    max over tiles of |(a, b)_fp32 - (a, b)_fp64| (and its 99.9th
               percentile: a fit of a few nearly collinear points is
               ill-conditioned in any precision)
  residual_err max over tiles of max_i |r32_i - r64_i| / max(max_i |r64_i|, q),
               where r = z - (a*x + b*y + c) is point i's fit residual under
               each mode's plane (x, y from the tile centre; the residuals of
               scanCylinder's untilting, scan.cpp:74-87) and q the height
               quantum (scale * unit); also its 99.9th percentile and the
               largest absolute difference in metres
  h_changed    tiles whose hyperboloid size differs, and h_rel_err the largest
               relative difference: the size follows integer counts of the
               points below a height threshold (scan.cpp:88-112), so a plane
               that moves by rounding can move one point across the threshold
               and change a size by a whole count -- a threshold effect, not
               an accumulated error
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
        if name == "fp32":
            rdiff, rref = clf.residuals(res["fp64"][1])
    clf.set_precision(_lib.WB_PRECISION_EXACT)
    c64, p64, t64 = res["fp64"]
    c32, p32, t32 = res["fp32"]
    flips = int(np.count_nonzero(c64 != c32))
    n = int(c64.size)
    ok = (t64["n_points"] >= 3) & np.all(np.isfinite(p64), axis=1) & np.all(np.isfinite(p32), axis=1)
    ok &= np.isfinite(rdiff) & np.isfinite(rref)
    d = np.abs(p32 - p64)[ok]
    q = abs(cloud.scale[2] * cloud.unit)
    rel = rdiff[ok] / np.maximum(rref[ok], q)
    h64, h32 = t64["hyperboloid_size"], t32["hyperboloid_size"]
    hm = (t64["n_points"] > 0) & (h64 > 0)
    out.update({
        "points": n, "flips": flips, "agreement": 1.0 - flips / max(n, 1),
        "tiles_compared": int(ok.sum()),
        "slope_err": float(np.max(np.hypot(d[:, 0], d[:, 1]))) if len(d) else 0.0,
        "slope_err_p999": float(np.percentile(np.hypot(d[:, 0], d[:, 1]), 99.9)) if len(d) else 0.0,
        "residual_abs_err_m": float(np.max(rdiff[ok])) if len(d) else 0.0,
        "residual_err": float(np.max(rel)) if len(d) else 0.0,
        "residual_err_p999": float(np.percentile(rel, 99.9)) if len(d) else 0.0,
        "h_rel_err": float(np.max(np.abs(h32[hm] - h64[hm]) / h64[hm])) if hm.any() else 0.0,
        "h_changed": int(np.count_nonzero(h32[hm] != h64[hm])),
        "tree_flag_changes": int(np.count_nonzero(t64["tree_flags"] != t32["tree_flags"])),
    })
    return out
