"""CPU restatement of the steps either side of the path, in numpy.

TEST INFRASTRUCTURE ONLY: imported by tests/ as the checker of the device
versions; the product package never imports it.

  write_classes   the class field LasHeader::writePoint writes (las.cpp:853-862):
                  formats 0-5: (classification & 31) + (flags << 5) in byte 15,
                  where the flags are what readPoint found in the top three bits
                  (las.cpp:752-754); formats 6-10: the class byte at 16 (las.cpp:771).
  split_by_class  CloudOutput::writeFiles (cloudoutput.cpp:187-231) sends every
                  point to the file of its classification; here the records of
                  each class, in input order, and the class boundaries.
  class_totals    OctBuffer::countClasses (octree.cpp:664-671) summed over the
                  blocks (threads.cpp:425-444): one count per stored point.
  survivors       OctBuffer::put (octree.cpp:620-662) keeps the last point read
                  at an exact location: for each record, the record kept.
  preview         OctStore::hiLoPointsIn / countPointsIn (octree.cpp:1244-1293) for
                  each pixel Column (shape.cpp:251-254) of a view.
"""
from __future__ import annotations

import numpy as np


def class_offset(fmt):
    return 15 if fmt < 6 else 16


def record_classes(records, fmt):
    c = records[:, class_offset(fmt)]
    return (c & 31) if fmt < 6 else c.copy()


def write_classes(records, fmt, cls):
    out = records.copy()
    off = class_offset(fmt)
    if fmt < 6:
        out[:, off] = (records[:, off] & 0xE0) | (cls.astype(np.uint8) & 31)
    else:
        out[:, off] = cls.astype(np.uint8)
    return out


def split_by_class(records, fmt):
    c = record_classes(records, fmt)
    order = np.argsort(c, kind="stable")
    offsets = np.zeros(257, np.uint64)
    offsets[1:] = np.cumsum(np.bincount(c, minlength=256))
    return records[order], offsets


def survivors(xyz):
    """For each record, the index of the last record with identical X, Y, Z."""
    n = xyz.shape[0]
    keys = np.ascontiguousarray(xyz.astype(np.int32)).view(np.dtype((np.void, 12))).ravel()
    out = np.arange(n, dtype=np.int64)
    last = {}
    for i in range(n - 1, -1, -1):
        k = keys[i].tobytes()
        if k in last:
            out[i] = last[k]
        else:
            last[k] = i
    return out


def class_totals(stored_records, cls):
    """Counts of the final class bytes of the stored (surviving) records."""
    return np.bincount(cls[stored_records].astype(np.int64), minlength=256).astype(np.uint64)


def preview(points, x0, y0, side, w, h):
    """points: (m, 3) decoded stored points.  Returns count, lo, hi per pixel (h, w)."""
    cnt = np.zeros((h, w), np.uint64)
    lo = np.full((h, w), np.inf)
    hi = np.full((h, w), -np.inf)
    half = side / 2
    px, py, pz = points[:, 0], points[:, 1], points[:, 2]
    fi = np.rint((px - x0) / side).astype(np.int64)
    fj = np.rint((py - y0) / side).astype(np.int64)
    for dj in (-1, 0, 1):
        for di in (-1, 0, 1):
            i = fi + di
            j = fj + dj
            ok = (i >= 0) & (i < w) & (j >= 0) & (j < h)
            cx = x0 + i * side
            cy = y0 + j * side
            ok &= (np.abs(cx - px) <= half) & (np.abs(cy - py) <= half)
            np.add.at(cnt, (j[ok], i[ok]), 1)
            np.minimum.at(lo, (j[ok], i[ok]), pz[ok])
            np.maximum.at(hi, (j[ok], i[ok]), pz[ok])
    return cnt, lo, hi
