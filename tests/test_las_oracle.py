"""The restatements of the steps either side of the path (oracle/las_oracle.py)
against the reference's own outputs: readPoint / writePoint / writeHeader /
combineScales / joinPointFormat (tests/golden/lasio.npz, written by
tests/golden/make_las_golden.py) and the preview queries countPointsIn /
hiLoPointsIn (tests/golden/preview.npz, make_preview_golden.py); and the
library's host-side writer pieces (header bytes, file names, scale
combination, format join) against the same fixtures.  No GPU."""
import os

import numpy as np
import pytest

from conftest import ROOT
from oracle import las_oracle as LO

GOLDEN = os.path.join(ROOT, "tests", "golden", "lasio.npz")
SYSID = {0: dict(separate_classes=False, n_input_files=2), 1: dict(separate_classes=False, n_input_files=1),
         2: dict(separate_classes=True, n_input_files=1)}


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


def _case(g, k):
    fmt_in, fmt_out, sysid = (int(v) for v in g[f"c{k}_meta"])
    inp = g[f"c{k}_in"]
    outp = g[f"c{k}_out"]
    return dict(rec=g[f"c{k}_rec"], fmt_in=fmt_in, fmt_out=fmt_out, sysid=sysid, scale=tuple(inp[:3]),
                offset=tuple(inp[3:6]), unit=float(inp[6]), out_scale=tuple(outp[:3]), lo=tuple(outp[3:6]),
                hi=tuple(outp[6:9]), cls=g[f"c{k}_cls"], fields=g[f"c{k}_fields"], file=g[f"c{k}_file"])


def _bits(a):
    a = np.ascontiguousarray(a)
    return a.view(np.uint64) if a.dtype == np.float64 else a


def _expected_file(c):
    """The oracle's version of the file the reference wrote for case c."""
    pts = LO.decode(c["rec"], c["fmt_in"], c["scale"], c["offset"], c["unit"])
    pts["classification"] = c["cls"].astype(np.uint16)
    es = [LO.set_scale(c["lo"][k], c["hi"][k], c["out_scale"][k], c["unit"]) for k in range(3)]
    sc, of = [e[0] for e in es], [e[1] for e in es]
    recs = LO.encode(pts, c["fmt_out"], sc, of, c["unit"])
    q = [LO.quantise(pts[a], c["unit"], of[k], sc[k]).astype(np.float64) for k, a in enumerate("xyz")]
    n_pts = [len(recs)] + [int(np.count_nonzero(pts["return_num"] == r)) for r in range(1, 16)]
    f = dict(point_format=c["fmt_out"], n_points=n_pts, scale=tuple(sc), offset=tuple(of),
             min=tuple(float(q[k].min() * sc[k] + of[k]) for k in range(3)),
             max=tuple(float(q[k].max() * sc[k] + of[k]) for k in range(3)), class_id=0, index=0, name_digits=0)
    out = dict(point_format=c["fmt_out"], points_per_file=0, unit=c["unit"], **SYSID[c["sysid"]])
    return recs, f, out


def test_decode_matches_reference(golden):
    for k in range(int(golden["n_cases"])):
        c = _case(golden, k)
        got = LO.decode(c["rec"], c["fmt_in"], c["scale"], c["offset"], c["unit"])
        for name, _ in LO.FIELDS:
            assert np.array_equal(_bits(got[name]), _bits(c["fields"][name])), (k, name)


def test_encode_and_header_match_reference(golden):
    for k in range(int(golden["n_cases"])):
        c = _case(golden, k)
        recs, f, out = _expected_file(c)
        assert np.array_equal(recs.ravel(), c["file"][375:]), k
        day, year = int(c["file"][90]) | (int(c["file"][91]) << 8), int(c["file"][92]) | (int(c["file"][93]) << 8)
        hdr = np.frombuffer(LO.header_bytes(out, f, day, year, software="Wolkenbase oracle"), np.uint8)
        assert np.array_equal(hdr, c["file"][:375]), (k, np.nonzero(hdr != c["file"][:375])[0][:8])


def test_scale_combination_and_format_join(golden):
    for i in range(len(golden["combine_n"])):
        n = int(golden["combine_n"][i])
        s = golden["combine_scales"][i][:3 * n].reshape(n, 3)
        o = golden["combine_offsets"][i][:3 * n].reshape(n, 3)
        assert LO.combine_scales(s, o) == tuple(golden["combine_out"][i]), i
    for j, want in zip(golden["join_in"], golden["join_out"]):
        assert LO.join_point_format([int(v) for v in j if v >= 0]) == int(want)


def test_writer_plan_and_names():
    """openFiles: class 0 always has a set; files per set = ceil(total / ppf)."""
    tot = np.zeros(256, np.int64)
    tot[1], tot[2] = 25, 61
    sets, digits = LO.plan_files(tot, dict(points_per_file=0, separate_classes=True))
    assert sets == [(0, 1), (1, 1), (2, 1)] and digits == 0
    sets, digits = LO.plan_files(tot, dict(points_per_file=10, separate_classes=True))
    assert sets == [(0, 0), (1, 3), (2, 7)] and digits == 1
    sets, digits = LO.plan_files(tot, dict(points_per_file=3, separate_classes=False))
    assert sets == [(0, 29)] and digits == 2
    out = dict(separate_classes=True, points_per_file=10)
    assert LO.file_name(out, dict(class_id=2, index=3, name_digits=1), "a/b") == "a/b-ground-3.las"
    assert LO.file_name(out, dict(class_id=8, index=0, name_digits=2), "x") == "x-reserved8-00.las"
    assert LO.file_name(dict(separate_classes=False, points_per_file=0), dict(class_id=0, index=0, name_digits=0),
                        "x") == "x.las"


def test_writer_balances_blocks_over_files():
    """Each block's points of a class go to that class's file with the fewest
    points (cloudoutput.cpp:196-209)."""
    rng = np.random.default_rng(5)
    n = 400
    rec = np.zeros((n, 20), np.uint8)
    rec[:, 0:12] = rng.integers(0, 1000, (n, 3)).astype("<i4").view(np.uint8).reshape(n, 12)
    cls = np.where(rng.random(n) < 0.7, 2, 1).astype(np.uint8)
    counts = [37, 50, 13, 100, 80, 120]
    first = np.concatenate([[0], np.cumsum(counts)[:-1]])
    sidx = rng.permutation(n)
    out = dict(point_format=0, separate_classes=True, points_per_file=60, unit=1.0, min_cor=(0, 0, 0),
               max_cor=(1, 1, 1), scale=(0.001, 0.001, 0.001))
    recs, files = LO.write_output(rec, 0, (1, 1, 1), (0, 0, 0), 1.0, cls, first, counts, sidx, out)
    assert sum(f["n_points"][0] for f in files) == n
    # replay the rule
    for f in files:
        assert (cls[sidx[f["store_positions"]]] == f["class_id"]).all() if f["n_points"][0] else True
    by_class = {}
    for f in files:
        by_class.setdefault(f["class_id"], []).append(f)
    for c, fs in by_class.items():
        sizes = [0] * len(fs)
        for b in range(len(counts)):
            seg = np.arange(first[b], first[b] + counts[b])
            k = int(np.count_nonzero(cls[sidx[seg]] == c))
            if not k:
                continue
            j = min(range(len(fs)), key=lambda i: (sizes[i], i))
            assert set(sidx[seg][cls[sidx[seg]] == c]) <= set(sidx[fs[j]["store_positions"]])
            sizes[j] += k


def _lib_or_skip():
    from wolkenbase_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("library not built")
    return _lib.load()


def test_library_host_pieces_match_reference(golden):
    """wb_las_header_bytes, wb_las_combine_scales, wb_las_join_point_format and
    wb_las_file_name are host code: checked here without a GPU."""
    _lib_or_skip()
    import wolkenbase_gb300 as wb
    from wolkenbase_gb300 import _lib
    for k in range(0, int(golden["n_cases"]), 3):
        c = _case(golden, k)
        _, f, out = _expected_file(c)
        day, year = int(c["file"][90]) | (int(c["file"][91]) << 8), int(c["file"][92]) | (int(c["file"][93]) << 8)
        o = wb.LasOutput(point_format=c["fmt_out"], separate_classes=out["separate_classes"],
                         n_input_files=out["n_input_files"], unit=c["unit"], creation_day=day, creation_year=year,
                         software="Wolkenbase oracle")
        cf = _lib.wb_las_file()
        cf.point_format = c["fmt_out"]
        cf.n_points[:] = f["n_points"]
        cf.scale[:] = f["scale"]
        cf.offset[:] = f["offset"]
        cf.min[:] = f["min"]
        cf.max[:] = f["max"]
        assert np.array_equal(wb.las_header_bytes(o, cf), c["file"][:375]), k
    for i in range(len(golden["combine_n"])):
        n = int(golden["combine_n"][i])
        got = wb.combine_scales(golden["combine_scales"][i][:3 * n].reshape(n, 3),
                                golden["combine_offsets"][i][:3 * n].reshape(n, 3))
        assert got == tuple(golden["combine_out"][i]), i
    for j, want in zip(golden["join_in"], golden["join_out"]):
        assert wb.join_point_format([int(v) for v in j if v >= 0]) == int(want)
    for fmt in range(11):
        assert wb.las_point_length(fmt) == LO.POINT_LENGTHS[fmt]
    o = wb.LasOutput(separate_classes=True, points_per_file=10)
    cf = _lib.wb_las_file()
    cf.class_id, cf.index, cf.name_digits = 8, 4, 2
    assert wb.las_file_name(o, cf, "out/cloud") == "out/cloud-reserved8-04.las"
    # manygcd that would never return (a zero offset beside a nonzero one) is refused
    with pytest.raises(wb.WolkenbaseError):
        wb.combine_scales([[0.01] * 3, [0.001] * 3], [[500000.0] * 3, [0.0] * 3])


def _golden_cloud(name):
    from wolkenbase_gb300 import synth
    c = np.load(os.path.join(ROOT, "tests", "golden", name + ".npz"))
    return synth.Cloud(c["xyz"].astype(np.int32), tuple(c["scale"]), tuple(c["offset"]), float(c["unit"]),
                       tuple(c["minc"]), tuple(c["maxc"]))


def test_preview_matches_reference():
    """OctStore::countPointsIn / hiLoPointsIn of every pixel Column, as the
    reference's own octree answered them (tests/golden/preview.npz)."""
    g = np.load(os.path.join(ROOT, "tests", "golden", "preview.npz"))
    for name in g["cases"]:
        cloud = _golden_cloud(str(name))
        stored = np.unique(LO.survivors(cloud.xyz))
        pts = cloud.decoded()[stored]
        for k in range(3):
            x0, y0, side, w, h = g[f"{name}_{k}_view"]
            cnt, lo, hi = LO.preview(pts, x0, y0, side, int(w), int(h))
            assert np.array_equal(cnt, g[f"{name}_{k}_count"]), (name, k)
            assert np.array_equal(lo, g[f"{name}_{k}_lo"]) and np.array_equal(hi, g[f"{name}_{k}_hi"]), (name, k)


@pytest.mark.parametrize("name", ["dups5k", "tile20k", "split"])
def test_duplicates_and_class_totals_match_reference(name):
    """OctBuffer::put's overwrites and countClasses, as the reference's own run
    recorded them in the golden fixtures: a record has no block exactly when a
    later identical point replaced it, and the class totals count the stored
    points."""
    g = np.load(os.path.join(ROOT, "tests", "golden", name + ".npz"))
    surv = LO.survivors(g["xyz"])
    replaced = surv != np.arange(len(surv))
    assert np.array_equal(g["block"] < 0, replaced)
    stored = np.flatnonzero(~replaced)
    if int(g["phases"]) >= 3:
        want = np.bincount(g["cls"][g["block"] >= 0].astype(np.int64), minlength=256)
        assert np.array_equal(LO.class_totals(stored, g["cls"]).astype(np.int64), want)
