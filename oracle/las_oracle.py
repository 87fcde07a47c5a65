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


# ---------------------------------------------------------------------------
# Full record decode / encode and the class-split writer
#
#   decode          LasHeader::readPoint (las.cpp:735-820): every LasPoint field
#   encode          LasHeader::writePoint (las.cpp:822-904) of decoded points
#   set_scale       LasHeader::setScale (las.cpp:636-673)
#   plan_files      CloudOutput::openFiles (cloudoutput.cpp:116-185)
#   write_output    CloudOutput::writeFiles (cloudoutput.cpp:187-231) over blocks
#   header_bytes    LasHeader::writeHeader (las.cpp:540-595)
#   file_name       the names openFiles gives (cloudoutput.cpp:27-185)
#   combine_scales  combineScales / combine1Scale (las.cpp:906-944), manygcd
#                   (manygcd.cpp:28-74), pairwisesum (manysum.cpp:120-154)
#   join_point_format  joinPointFormat (las.cpp:103-118)
# ---------------------------------------------------------------------------

POINT_LENGTHS = [20, 28, 26, 34, 57, 63, 30, 36, 38, 59, 67]
POINT_FEATURES = [0x0, 0x1, 0x2, 0x3, 0x9, 0xb, 0x101, 0x103, 0x107, 0x109, 0x10f]
MASK_GPS, MASK_RGB, MASK_NIR, MASK_WAVE = 0x7fa, 0x5ac, 0x500, 0x630
FIELDS = [("x", "<f8"), ("y", "<f8"), ("z", "<f8"), ("intensity", "<u2"), ("return_num", "<u2"),
          ("n_returns", "<u2"), ("scan_direction", "u1"), ("edge_line", "u1"), ("classification", "<u2"),
          ("class_flags", "<u2"), ("scanner_channel", "<u2"), ("user_data", "<u2"), ("scan_angle", "<i4"),
          ("point_source", "<u2"), ("gps_time", "<f8"), ("red", "<u2"), ("green", "<u2"), ("blue", "<u2"),
          ("nir", "<u2")]
CLASS_NAMES = {0: "raw", 1: "nonground", 2: "ground", 3: "lowveg", 4: "medveg", 5: "highveg", 6: "building",
               7: "lownoise", 9: "water", 10: "rail", 11: "road", 12: "overlap", 13: "wireguard", 14: "conductor",
               15: "tower", 16: "insulator", 17: "bridge", 18: "highnoise", 19: "overhead", 20: "ignground",
               21: "snow", 22: "temporal"}


def layout(fmt):
    """Offsets of the optional parts (None: absent) and the record length."""
    o = 20 if fmt < 6 else 22
    lay = {}
    for key, mask, size in (("gps", MASK_GPS, 8), ("rgb", MASK_RGB, 6), ("nir", MASK_NIR, 2), ("wave", MASK_WAVE, 29)):
        if (1 << fmt) & mask:
            lay[key] = o
            o += size
        else:
            lay[key] = None
    lay["len"] = o
    return lay


def _u16(rec, o):
    return rec[:, o].astype(np.uint32) | (rec[:, o + 1].astype(np.uint32) << 8)


def _i32(rec, o):
    return np.ascontiguousarray(rec[:, o:o + 4]).view("<i4").ravel()


def deg_to_bin(deg):
    """degtobin -> rottobin (angle.cpp:229-243): the turn fraction folded into
    [-1, 1) by modf, times 2^31, lrint, wrapped to int."""
    deg = np.asarray(deg, np.float64)
    f = 2 * np.modf(deg / 360 / 2)[0]
    f = np.where(f >= 1, f - 2, f)
    f = np.where(f < -1, f + 2, f)
    return _wrap32(np.rint(2147483648.0 * f))


def bin_to_deg(a):
    return np.asarray(a, np.float64) / 2147483648.0 * 360


def _wrap32(v):
    return (np.asarray(v).astype(np.int64) & 0xFFFFFFFF).astype(np.uint32).view(np.int32)


def decode(records, fmt, scale, offset, unit):
    """readPoint of every (n, stride) uint8 record: dict of LasPoint fields."""
    rec = np.ascontiguousarray(records, np.uint8)
    n = rec.shape[0]
    lay = layout(fmt)
    out = {}
    for k, name in enumerate("xyz"):
        out[name] = (offset[k] + scale[k] * _i32(rec, 4 * k).astype(np.float64)) * unit
    out["intensity"] = _u16(rec, 12).astype(np.uint16)
    t = rec[:, 14].astype(np.uint16)
    if fmt < 6:
        c = rec[:, 15].astype(np.uint16)
        out["return_num"] = t & 7
        out["n_returns"] = (t >> 3) & 7
        out["scan_direction"] = ((t >> 6) & 1).astype(np.uint8)
        out["edge_line"] = ((t >> 7) & 1).astype(np.uint8)
        out["class_flags"] = (c >> 5) & 7
        out["classification"] = c & 31
        out["scanner_channel"] = np.zeros(n, np.uint16)
        out["scan_angle"] = deg_to_bin(rec[:, 16].view(np.int8).astype(np.float64))
        out["user_data"] = rec[:, 17].astype(np.uint16)
        out["point_source"] = _u16(rec, 18).astype(np.uint16)
    else:
        u = rec[:, 15].astype(np.uint16)
        out["return_num"] = t & 15
        out["n_returns"] = (t >> 4) & 15
        out["class_flags"] = u & 15
        out["scanner_channel"] = (u >> 4) & 3
        out["scan_direction"] = ((u >> 6) & 1).astype(np.uint8)
        out["edge_line"] = ((u >> 7) & 1).astype(np.uint8)
        out["classification"] = rec[:, 16].astype(np.uint16)
        out["user_data"] = rec[:, 17].astype(np.uint16)
        sa = _u16(rec, 18).astype(np.uint16).view(np.int16).astype(np.float64)
        out["scan_angle"] = deg_to_bin(sa * 0.006)
        out["point_source"] = _u16(rec, 20).astype(np.uint16)
    if lay["gps"] is not None:
        out["gps_time"] = np.ascontiguousarray(rec[:, lay["gps"]:lay["gps"] + 8]).view("<f8").ravel().copy()
    else:
        out["gps_time"] = np.zeros(n)
    for k, name in enumerate(("red", "green", "blue")):
        out[name] = _u16(rec, lay["rgb"] + 2 * k).astype(np.uint16) if lay["rgb"] is not None else np.zeros(n, np.uint16)
    out["nir"] = _u16(rec, lay["nir"]).astype(np.uint16) if lay["nir"] is not None else np.zeros(n, np.uint16)
    return {name: np.asarray(out[name]).astype(dt) for name, dt in FIELDS}


def quantise(v, unit, off, scale):
    """writePoint's lrint((v/unit - off)/scale), kept as the int it is stored in."""
    return _wrap32(np.rint((np.asarray(v) / unit - off) / scale))


def encode(pts, fmt, scale, offset, unit):
    """writePoint of decoded points (dict as decode returns) -> (n, length) uint8."""
    lay = layout(fmt)
    n = len(pts["x"])
    o = np.zeros((n, lay["len"]), np.uint8)

    def put(off, v, nbytes):
        v = np.asarray(v).astype(np.int64) & ((1 << (8 * nbytes)) - 1)
        for b in range(nbytes):
            o[:, off + b] = (v >> (8 * b)) & 0xFF

    for k, name in enumerate("xyz"):
        put(4 * k, quantise(pts[name], unit, offset[k], scale[k]).astype(np.int64), 4)
    put(12, pts["intensity"], 2)
    ret = pts["return_num"].astype(np.int64)
    nret = pts["n_returns"].astype(np.int64)
    sd = pts["scan_direction"].astype(np.int64)
    el = pts["edge_line"].astype(np.int64)
    cl = pts["classification"].astype(np.int64)
    fl = pts["class_flags"].astype(np.int64)
    deg = bin_to_deg(pts["scan_angle"])
    if fmt < 6:
        put(14, (ret & 7) + ((nret & 7) << 3) + ((sd & 1) << 6) + ((el & 1) << 7), 1)
        put(15, (cl & 31) + ((fl & 7) << 5), 1)
        put(16, np.rint(deg).astype(np.int64), 1)
        put(17, pts["user_data"], 1)
        put(18, pts["point_source"], 2)
    else:
        ch = pts["scanner_channel"].astype(np.int64)
        put(14, (ret & 15) + ((nret & 15) << 4), 1)
        put(15, (fl & 15) + ((ch & 3) << 4) + ((sd & 1) << 6) + ((el & 1) << 7), 1)
        put(16, cl, 1)
        put(17, pts["user_data"], 1)
        put(18, np.rint(deg / 0.006).astype(np.int64), 2)
        put(20, pts["point_source"], 2)
    if lay["gps"] is not None:
        o[:, lay["gps"]:lay["gps"] + 8] = np.ascontiguousarray(pts["gps_time"], "<f8").view(np.uint8).reshape(n, 8)
    if lay["rgb"] is not None:
        for k, name in enumerate(("red", "green", "blue")):
            put(lay["rgb"] + 2 * k, pts[name], 2)
    if lay["nir"] is not None:
        put(lay["nir"], pts["nir"], 2)
    return o


def set_scale(lo, hi, scale, unit):
    """LasHeader::setScale on one axis -> (scale, offset) in file units."""
    min_scale = (hi - lo) / 4132485216.
    off = (lo + hi) / 2 / unit
    if scale > min_scale and np.isfinite(scale):
        sc = scale / unit
        off = float(np.rint(off / sc)) * sc
    else:
        sc = min_scale / unit
    return sc, off


def plan_files(totals, out):
    """openFiles: list of sets (class, number of files) and the digits of the
    file numbers.  Class 0 is always among the class totals (threads.cpp:430)."""
    grand = int(sum(int(t) for t in totals))
    ppf = int(out["points_per_file"])
    digits = 0
    if ppf:
        quot = (grand + ppf - 1) // ppf
        if quot:
            quot -= 1
        if not quot:
            quot += 1
        while quot:
            quot //= 10
            digits += 1
    sets = []
    if out["separate_classes"]:
        for c in range(256):
            if c == 0 or totals[c]:
                sets.append((c, (int(totals[c]) + ppf - 1) // ppf if ppf else 1))
    else:
        sets.append((0, (grand + ppf - 1) // ppf if ppf else 1))
    return sets, digits


def write_output(records, in_fmt, scale, offset, unit, cls, leaf_first, leaf_count, sidx, out):
    """writeFiles over the blocks in the order given (leaf_first/leaf_count over
    the store order sidx): each block's points of a set go to the set's file with
    the fewest points, the first on a tie.  Returns (records of all files back
    to back, list of file dicts)."""
    pts = decode(records, in_fmt, scale, offset, unit)
    cls = np.asarray(cls, np.uint8)
    stored_cls = cls[sidx]
    totals = np.bincount(stored_cls, minlength=256)
    sets, digits = plan_files(totals, out)
    set_of = np.zeros(256, np.int64)
    if out["separate_classes"]:
        for s, (c, _) in enumerate(sets):
            set_of[c] = s
    files = []
    set_files = []
    for s, (c, q) in enumerate(sets):
        set_files.append(list(range(len(files), len(files) + q)))
        for i in range(q):
            files.append({"class_id": c, "index": i, "name_digits": digits, "members": []})
    counts = [0] * len(files)
    for b in range(len(leaf_first)):
        seg = np.arange(int(leaf_first[b]), int(leaf_first[b]) + int(leaf_count[b]))
        ss = set_of[stored_cls[seg]]
        for s in range(len(sets)):
            m = seg[ss == s]
            if not len(m):
                continue
            f = min(set_files[s], key=lambda k: (counts[k], k))
            files[f]["members"].extend(m.tolist())
            counts[f] += len(m)
    esc = [set_scale(out["min_cor"][k], out["max_cor"][k], out["scale"][k], out["unit"]) for k in range(3)]
    sc = [e[0] for e in esc]
    of = [e[1] for e in esc]
    lay = layout(out["point_format"])
    chunks = []
    first = 0
    for f in files:
        pos = np.asarray(f["members"], np.int64)
        idx = sidx[pos] if len(pos) else np.zeros(0, np.int64)
        sel = {k: v[idx] for k, v in pts.items()}
        sel["classification"] = cls[idx].astype(np.uint16)
        enc = encode(sel, out["point_format"], sc, of, out["unit"]) if len(idx) else np.zeros((0, lay["len"]), np.uint8)
        chunks.append(enc)
        n_pts = [0] * 16
        n_pts[0] = len(idx)
        for r in range(1, 16):
            n_pts[r] = int(np.count_nonzero(sel["return_num"] == r))
        f.update(first=first, n_points=n_pts, scale=tuple(sc), offset=tuple(of), point_format=out["point_format"])
        if len(idx):
            q = [quantise(sel[name], out["unit"], of[k], sc[k]).astype(np.float64) for k, name in enumerate("xyz")]
            f["min"] = tuple(float(q[k].min() * sc[k] + of[k]) for k in range(3))
            f["max"] = tuple(float(q[k].max() * sc[k] + of[k]) for k in range(3))
        else:
            f["min"] = (np.inf,) * 3
            f["max"] = (-np.inf,) * 3
        f["store_positions"] = pos
        first += len(idx)
        del f["members"]
    allrec = np.concatenate(chunks) if chunks else np.zeros((0, lay["len"]), np.uint8)
    return allrec, files


def header_bytes(out, f, day, year, software="Wolkenbase 0.1.2~alpha"):
    """writeHeader of one file written by CloudOutput (version 1.4, header and
    point offset 375, no variable length records; unset fields 0)."""
    import struct
    h = bytearray(375)
    h[0:4] = b"LASF"
    h[24], h[25] = 1, 4
    sysid = b"EXTRACTION" if out["separate_classes"] else (b"MERGE" if out.get("n_input_files", 1) > 1
                                                           else b"MODIFICATION")
    h[26:26 + len(sysid)] = sysid
    sw = software.encode()[:32]
    h[58:58 + len(sw)] = sw
    struct.pack_into("<HHHII", h, 90, day, year, 375, 375, 0)
    length = POINT_LENGTHS[f["point_format"]]
    struct.pack_into("<BH", h, 104, f["point_format"], length)
    n = f["n_points"]
    legacy = all(n[i] <= 0xFFFFFFFF for i in range(6)) and all(n[i] == 0 for i in range(6, 16))
    struct.pack_into("<6I", h, 107, *[(n[i] if legacy else 0) for i in range(6)])
    struct.pack_into("<3d", h, 131, *f["scale"])
    struct.pack_into("<3d", h, 155, *f["offset"])
    struct.pack_into("<6d", h, 179, f["max"][0], f["min"][0], f["max"][1], f["min"][1], f["max"][2], f["min"][2])
    struct.pack_into("<QQI", h, 227, 0, (375 + n[0] * length) if n[0] else 0, 0)
    struct.pack_into("<16Q", h, 247, *n)
    return bytes(h)


def class_name(c):
    return CLASS_NAMES.get(c, "reserved%d" % c)


def file_name(out, f, base):
    name = base
    if out["separate_classes"]:
        name += "-" + class_name(f["class_id"])
    if out["points_per_file"]:
        name += "-"
    if f["name_digits"]:
        name += "%0*d" % (f["name_digits"], f["index"])
    return name + ".las"


def join_point_format(formats):
    allf = 0
    for f in formats:
        if 0 <= f < 11:
            allf |= POINT_FEATURES[f]
    for i, feat in enumerate(POINT_FEATURES):
        if (allf | feat) == feat:
            return i
    return None


def pairwise_sum(a):
    a = list(a)
    n = len(a)

    def tree(lo, size):
        return a[lo] if size == 1 else tree(lo, size // 2) + tree(lo + size // 2, size // 2)

    total, start = 0.0, n
    for bit in range(64):
        if (n >> bit) & 1:
            start -= 1 << bit
            total += tree(start, 1 << bit)
    return total


def many_gcd(numbers, toler, max_steps=1 << 20):
    v = [abs(float(x)) for x in numbers]

    def up():
        for i in range(len(v) - 1):
            if v[i] > v[i + 1]:
                v[i], v[i + 1] = v[i + 1], v[i]

    def down():
        for i in range(len(v) - 2, -1, -1):
            if v[i] > v[i + 1]:
                v[i], v[i + 1] = v[i + 1], v[i]

    if not v:
        return 0.0
    up()
    down()
    up()
    steps = 0
    while v and v[-1] > v[0] + toler:
        steps += 1
        if steps > max_steps:
            return None
        if v[-1] - v[-2] > toler:
            v[-1] -= v[-2]
            down()
        else:
            v.pop()
        up()
    return pairwise_sum(v) / len(v) if v else 0.0


def combine_scales(scales, offsets):
    scales = np.asarray(scales, np.float64).reshape(-1, 3)
    offsets = np.asarray(offsets, np.float64).reshape(-1, 3)
    res = []
    for k in range(3):
        s, o = scales[:, k], offsets[:, k]
        toler = min(abs(float(x)) for x in s) / 1e6
        sg, og = many_gcd(s, toler), many_gcd(o, toler)
        if sg is None or og is None:
            return None
        ret = 0.0
        with np.errstate(divide="ignore", invalid="ignore"):
            q = np.float64(og) / np.float64(sg)
            if (og > 10.5 * sg or og == 0) and abs(q - np.rint(q)) < 1e-6:
                ret = sg
        for i in range(10, 0, -1):
            for j in range(10, 0, -1):
                if abs(sg * i - og * j) < toler:
                    ret = sg / j
        res.append(ret)
    return tuple(res)
