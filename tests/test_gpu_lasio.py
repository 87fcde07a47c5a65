"""LAS decode and the class-split writer on the device, against the
reference's own readPoint / writePoint / writeHeader outputs
(tests/golden/lasio.npz) and the CPU restatement of CloudOutput
(oracle/las_oracle.py).  Byte-exact."""
import os

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(ROOT, "tests", "golden", "lasio.npz")
SYSID = {0: dict(separate_classes=False, n_input_files=2), 1: dict(separate_classes=False, n_input_files=1),
         2: dict(separate_classes=True, n_input_files=1)}


def _bits(a):
    a = np.ascontiguousarray(a)
    return a.view(np.uint64) if a.dtype == np.float64 else a


def _case(g, k):
    fmt_in, fmt_out, sysid = (int(v) for v in g[f"c{k}_meta"])
    inp, outp = g[f"c{k}_in"], g[f"c{k}_out"]
    return dict(rec=g[f"c{k}_rec"], fmt_in=fmt_in, fmt_out=fmt_out, sysid=sysid, scale=tuple(inp[:3]),
                offset=tuple(inp[3:6]), unit=float(inp[6]), out_scale=tuple(outp[:3]), lo=tuple(outp[3:6]),
                hi=tuple(outp[6:9]), cls=g[f"c{k}_cls"], fields=g[f"c{k}_fields"], file=g[f"c{k}_file"])


def _cloud_of(rec, scale, offset, unit):
    from oracle import las_oracle as LO
    from wolkenbase_gb300 import synth
    xyz = np.ascontiguousarray(rec[:, 0:12]).view("<i4").reshape(-1, 3).copy()
    d = LO.decode(rec, 0, scale, offset, unit)
    lo = tuple(float(d[a].min()) for a in "xyz")
    hi = tuple(float(d[a].max()) for a in "xyz")
    return synth.Cloud(xyz, scale, offset, unit, lo, hi)


def test_decode_matches_reference_fields(classifier):
    g = np.load(GOLDEN)
    for k in range(int(g["n_cases"])):
        c = _case(g, k)
        got = classifier.las_decode(c["rec"], c["fmt_in"], c["scale"], c["offset"], c["unit"])
        for name in c["fields"].dtype.names:
            assert np.array_equal(_bits(got[name]), _bits(c["fields"][name])), (k, name)


@pytest.mark.parametrize("fmt,pad", [(1, 0), (3, 1), (6, 2), (10, 5), (0, 4), (8, 0)])
def test_decode_large_matches_restatement(classifier, fmt, pad):
    """100k records, with padded and odd strides (byte loads)."""
    from oracle import las_oracle as LO
    n = 100_003
    stride = LO.POINT_LENGTHS[fmt] + pad
    rec = np.random.default_rng(fmt * 7 + pad).integers(0, 256, size=(n, stride), dtype=np.uint8)
    lay = LO.layout(fmt)
    if lay["gps"] is not None:   # finite GPS times
        rec[:, lay["gps"]:lay["gps"] + 8] = np.random.default_rng(1).uniform(0, 1e9, n).view(np.uint8).reshape(n, 8)
    scale, offset, unit = (0.001, 0.002, 0.0005), (500000.0, 4500000.0, 1500.0), 1200 / 3937
    got = classifier.las_decode(rec, fmt, scale, offset, unit)
    want = LO.decode(rec, fmt, scale, offset, unit)
    for name, _ in LO.FIELDS:
        assert np.array_equal(_bits(got[name]), _bits(want[name])), name


def test_writer_files_match_reference_bytes(classifier):
    """Every golden case written by wb_las_write_output: each file's records
    and header equal what the reference's writePoint / writeHeader wrote, in
    the octree's store order (for separated classes, the reference's file
    filtered by class)."""
    import wolkenbase_gb300 as wb
    from oracle import las_oracle as LO
    g = np.load(GOLDEN)
    for k in range(int(g["n_cases"])):
        c = _case(g, k)
        classifier.build(_cloud_of(c["rec"], c["scale"], c["offset"], c["unit"]))
        sidx = classifier.store_order().astype(np.int64)
        assert len(sidx) == len(c["rec"])            # distinct points: every record is stored
        day = int(c["file"][90]) | (int(c["file"][91]) << 8)
        year = int(c["file"][92]) | (int(c["file"][93]) << 8)
        o = wb.LasOutput(point_format=c["fmt_out"], unit=c["unit"], min_cor=c["lo"], max_cor=c["hi"],
                         scale=c["out_scale"], creation_day=day, creation_year=year, software="Wolkenbase oracle",
                         **SYSID[c["sysid"]])
        recs, files, cfiles = classifier.las_write_output(c["rec"], c["fmt_in"], c["scale"], c["offset"], c["unit"], o,
                                                          cls=c["cls"])
        length = LO.POINT_LENGTHS[c["fmt_out"]]
        # the reference wrote the records in input order; the writer writes them in store order
        ref = c["file"][375:].reshape(-1, length)[sidx]
        cls_stored = c["cls"][sidx]
        if not o.separate_classes:
            assert len(files) == 1
            assert np.array_equal(recs, ref), k
            assert np.array_equal(wb.las_header_bytes(o, cfiles[0]), c["file"][:375]), k
        else:
            for i, f in enumerate(files):
                sel = ref[cls_stored == f["class_id"]]
                got = recs[f["first"]:f["first"] + f["n_points"][0]]
                assert np.array_equal(got, sel), (k, f["class_id"])
                want_hdr = LO.header_bytes(dict(separate_classes=True), dict(f, point_format=c["fmt_out"]), day, year,
                                           software="Wolkenbase oracle")
                assert np.array_equal(wb.las_header_bytes(o, cfiles[i]), np.frombuffer(want_hdr, np.uint8)), k


def _attributed_records(cloud, fmt, seed):
    from oracle import las_oracle as LO
    rng = np.random.default_rng(seed)
    n = cloud.n
    rec = rng.integers(0, 256, size=(n, LO.POINT_LENGTHS[fmt]), dtype=np.uint8)
    rec[:, 0:12] = np.ascontiguousarray(cloud.xyz, "<i4").view(np.uint8).reshape(n, 12)
    lay = LO.layout(fmt)
    if lay["gps"] is not None:
        rec[:, lay["gps"]:lay["gps"] + 8] = rng.uniform(0, 1e9, n).view(np.uint8).reshape(n, 8)
    return rec


@pytest.mark.parametrize("fmt_in,fmt_out,separate,ppf", [(1, 6, True, 0), (1, 1, True, 4000), (6, 3, False, 7000),
                                                           (3, 10, True, 2500), (7, 0, False, 0)])
def test_writer_on_classified_cloud_matches_restatement(classifier, fmt_in, fmt_out, separate, ppf):
    """A classified 40k-point cloud with duplicates: files, their balance over
    the octree blocks, records and header figures equal the restatement."""
    import wolkenbase_gb300 as wb
    from oracle import las_oracle as LO
    from wolkenbase_gb300 import synth
    base = synth.density_tile(40_000, 77)
    rng = np.random.default_rng(8)
    dup = rng.choice(base.n, 800, replace=False)
    xyz = np.concatenate([base.xyz, base.xyz[dup]])
    cloud = synth.Cloud(xyz, base.scale, base.offset, base.unit, base.minc, base.maxc)
    rec = _attributed_records(cloud, fmt_in, fmt_in + 10 * fmt_out)
    cls = classifier.classify_cloud(cloud)
    _, first, count = classifier.leaves()
    sidx = classifier.store_order().astype(np.int64)
    assert classifier.info()["n_leaves"] > 20
    d = cloud.decoded()
    o = wb.LasOutput(point_format=fmt_out, separate_classes=separate, points_per_file=ppf, unit=cloud.unit,
                     min_cor=tuple(d.min(axis=0)), max_cor=tuple(d.max(axis=0)), scale=(0.001, 0.001, 0.001))
    recs, files, _ = classifier.las_write_output(rec, fmt_in, cloud.scale, cloud.offset, cloud.unit, o)
    want_recs, want_files = LO.write_output(rec, fmt_in, cloud.scale, cloud.offset, cloud.unit, cls, first, count,
                                            sidx, dict(point_format=fmt_out, separate_classes=separate,
                                                       points_per_file=ppf, unit=cloud.unit,
                                                       min_cor=o.min_cor, max_cor=o.max_cor, scale=o.scale))
    assert len(files) == len(want_files)
    for f, w in zip(files, want_files):
        for key in ("class_id", "index", "name_digits", "first", "n_points", "scale", "offset", "min", "max"):
            assert f[key] == (list(w[key]) if key == "n_points" else w[key]), key
    assert np.array_equal(recs, want_recs)


def test_write_files_to_disk(classifier, tmp_path):
    import wolkenbase_gb300 as wb
    from oracle import las_oracle as LO
    from wolkenbase_gb300 import synth
    cloud = synth.density_tile(30_000, 91)
    rec = _attributed_records(cloud, 1, 3)
    classifier.classify_cloud(cloud)
    d = cloud.decoded()
    o = wb.LasOutput(point_format=1, separate_classes=True, points_per_file=5000, unit=1.0,
                     min_cor=tuple(d.min(axis=0)), max_cor=tuple(d.max(axis=0)), scale=(0.001, 0.001, 0.001),
                     creation_day=45, creation_year=2026)
    recs, files, cfiles = classifier.las_write_output(rec, 1, cloud.scale, cloud.offset, cloud.unit, o)
    base = str(tmp_path / "cloud")
    written = classifier.las_write_files(rec, 1, cloud.scale, cloud.offset, cloud.unit, o, base)
    assert [w["n_points"] for w in written] == [f["n_points"] for f in files]
    names = set()
    for i, w in enumerate(written):
        assert w["name"] == LO.file_name(dict(separate_classes=True, points_per_file=5000), w, base)
        data = np.fromfile(w["name"], np.uint8)
        assert np.array_equal(data[:375], wb.las_header_bytes(o, cfiles[i]))
        n = w["n_points"][0]
        assert np.array_equal(data[375:].reshape(-1, 28), recs[w["first"]:w["first"] + n])
        names.add(w["name"])
    assert len(names) == len(written)
    assert sum(w["n_points"][0] for w in written) == classifier.info()["n_distinct"]
    assert not any(os.path.basename(w["name"]).startswith("cloud-raw") for w in written)   # ppf > 0: no empty raw file


@pytest.mark.parametrize("offset,unit", [((1000.0005, 2000.00025, 100.0), 1.0),       # half-unit offsets: FP64 path
                                         ((0.0, 0.0, 0.0), 1200 / 3937),                 # feet, integer path
                                         ((333.3333, -7.0, 0.1), 1.0)])
def test_writer_coordinate_paths_match_restatement(classifier, offset, unit):
    """Same scale in and out takes the integer path when the offsets allow it
    and the FP64 path otherwise; both equal writePoint's arithmetic."""
    import wolkenbase_gb300 as wb
    from oracle import las_oracle as LO
    from wolkenbase_gb300 import synth
    base = synth.density_tile(30_000, 55)
    cloud = synth.Cloud(base.xyz, base.scale, offset, unit, base.minc, base.maxc)
    d = cloud.decoded()
    cloud.minc = tuple(float(v) / unit for v in d.min(axis=0))
    cloud.maxc = tuple(float(v) / unit for v in d.max(axis=0))
    rec = _attributed_records(cloud, 1, 21)
    cls = np.random.default_rng(4).integers(1, 3, cloud.n).astype(np.uint8)
    classifier.build(cloud)
    _, first, count = classifier.leaves()
    sidx = classifier.store_order().astype(np.int64)
    scale_m = tuple(float(s) * unit for s in cloud.scale)      # the same record scale out
    o = wb.LasOutput(point_format=1, separate_classes=True, unit=unit, min_cor=tuple(d.min(axis=0)),
                     max_cor=tuple(d.max(axis=0)), scale=scale_m)
    recs, files, _ = classifier.las_write_output(rec, 1, cloud.scale, cloud.offset, unit, o, cls=cls)
    want_recs, want_files = LO.write_output(rec, 1, cloud.scale, cloud.offset, unit, cls, first, count, sidx,
                                            dict(point_format=1, separate_classes=True, points_per_file=0, unit=unit,
                                                 min_cor=o.min_cor, max_cor=o.max_cor, scale=o.scale))
    assert np.array_equal(recs, want_recs)
    for f, w in zip(files, want_files):
        assert (f["min"], f["max"], f["n_points"]) == (w["min"], w["max"], list(w["n_points"]))


def test_device_resident_decode_and_writer_equal_host_path(classifier, tmp_path):
    """Records, field arrays and output on the device give the host path's bytes."""
    import ctypes as C
    torch = pytest.importorskip("torch")
    import wolkenbase_gb300 as wb
    from wolkenbase_gb300 import _lib, synth
    cloud = synth.density_tile(50_000, 71)
    rec = _attributed_records(cloud, 3, 5)
    n = cloud.n
    cls = classifier.classify_cloud(cloud)
    d = cloud.decoded()
    o = wb.LasOutput(point_format=8, separate_classes=True, points_per_file=9000, unit=cloud.unit,
                     min_cor=tuple(d.min(axis=0)), max_cor=tuple(d.max(axis=0)), scale=(0.001, 0.001, 0.001))
    want_recs, want_files, _ = classifier.las_write_output(rec, 3, cloud.scale, cloud.offset, cloud.unit, o)
    want_fields = classifier.las_decode(rec, 3, cloud.scale, cloud.offset, cloud.unit)
    drec = torch.from_numpy(rec).cuda()
    cs = wb.cloud_struct(drec.data_ptr(), n, rec.shape[1], cloud.scale, cloud.offset, cloud.unit, cloud.minc,
                         cloud.maxc, device_resident=True)
    tdt = {C.c_double: torch.float64, C.c_uint16: torch.int16, C.c_uint8: torch.uint8, C.c_int32: torch.int32}
    fields = {name: torch.zeros(n, dtype=tdt[t], device="cuda") for name, t in _lib.LAS_POINT_FIELDS}
    pts = _lib.wb_las_points(**{name: t.data_ptr() for name, t in fields.items()})
    classifier._check(classifier.L.wb_las_decode(classifier.ctx, C.byref(cs), 3, C.byref(pts)))
    for name, _ in _lib.LAS_POINT_FIELDS:
        got = fields[name].cpu().numpy().view(want_fields[name].dtype)
        assert np.array_equal(got, want_fields[name]), name
    nd = classifier.info()["n_distinct"]
    dout = torch.zeros((nd, wb.las_point_length(8)), dtype=torch.uint8, device="cuda")
    files = (_lib.wb_las_file * 64)()
    nf = C.c_int(0)
    oc = o.c()
    classifier._check(classifier.L.wb_las_write_output(classifier.ctx, C.byref(cs), 3, None, C.byref(oc),
                                                       C.c_void_p(dout.data_ptr()), 1, files, 64, C.byref(nf)))
    assert nf.value == len(want_files)
    assert np.array_equal(dout.cpu().numpy(), want_recs)
    for i, w in enumerate(want_files):
        assert list(files[i].n_points) == w["n_points"] and files[i].first == w["first"]


def test_writer_errors(classifier, tmp_path):
    """Too little room for the files, and an unwritable destination."""
    import ctypes as C
    import wolkenbase_gb300 as wb
    from wolkenbase_gb300 import _lib, synth
    cloud = synth.density_tile(20_000, 72)
    rec = _attributed_records(cloud, 1, 6)
    classifier.classify_cloud(cloud)
    d = cloud.decoded()
    o = wb.LasOutput(point_format=1, separate_classes=True, points_per_file=1000, unit=1.0,
                     min_cor=tuple(d.min(axis=0)), max_cor=tuple(d.max(axis=0)), scale=(0.001, 0.001, 0.001))
    cs = wb.cloud_struct(rec, cloud.n, 28, cloud.scale, cloud.offset, cloud.unit, cloud.minc, cloud.maxc)
    out = np.zeros((classifier.info()["n_distinct"], 28), np.uint8)
    files = (_lib.wb_las_file * 2)()
    nf = C.c_int(0)
    oc = o.c()
    rc = classifier.L.wb_las_write_output(classifier.ctx, C.byref(cs), 1, None, C.byref(oc), out.ctypes.data, 0,
                                          files, 2, C.byref(nf))
    assert rc == _lib.WB_EINVAL and nf.value >= 20      # 20k points, 1000 per file
    with pytest.raises(wb.WolkenbaseError) as e:
        classifier.las_write_files(rec, 1, cloud.scale, cloud.offset, cloud.unit, o,
                                   str(tmp_path / "missing" / "dir" / "cloud"))
    assert e.value.code == _lib.WB_EIO
    bad = wb.LasOutput(point_format=11, unit=1.0)
    with pytest.raises(wb.WolkenbaseError) as e:
        classifier.las_write_output(rec, 1, cloud.scale, cloud.offset, cloud.unit, bad)
    assert e.value.code == _lib.WB_EINVAL


def test_written_files_census(classifier, tmp_path):
    """censusPoints (testpattern.cpp:56-123) on the files: with the GPS time of
    every record set to its index, the files hold every surviving record once
    and no overwritten duplicate."""
    import wolkenbase_gb300 as wb
    from wolkenbase_gb300 import synth
    base = synth.density_tile(40_000, 73)
    rng = np.random.default_rng(9)
    dup = rng.choice(base.n, 1500, replace=False)
    xyz = np.concatenate([base.xyz, base.xyz[dup]])
    cloud = synth.Cloud(xyz, base.scale, base.offset, base.unit, base.minc, base.maxc)
    rec = _attributed_records(cloud, 1, 10)
    rec[:, 20:28] = np.arange(cloud.n, dtype="<f8").view(np.uint8).reshape(-1, 8)
    classifier.classify_cloud(cloud)
    survivors = np.sort(classifier.store_order().astype(np.int64))
    d = cloud.decoded()
    o = wb.LasOutput(point_format=1, separate_classes=True, points_per_file=6000, unit=1.0,
                     min_cor=tuple(d.min(axis=0)), max_cor=tuple(d.max(axis=0)), scale=(0.001, 0.001, 0.001))
    written = classifier.las_write_files(rec, 1, cloud.scale, cloud.offset, cloud.unit, o, str(tmp_path / "c"))
    ids = []
    for w in written:
        data = np.fromfile(w["name"], np.uint8)[375:].reshape(-1, 28)
        ids.append(np.ascontiguousarray(data[:, 20:28]).view("<f8").ravel())
        assert w["n_points"][0] == len(data)
    ids = np.sort(np.concatenate(ids)).astype(np.int64)
    assert np.array_equal(ids, survivors)
    assert len(ids) <= cloud.n - 1500                    # every appended copy overwrote its original
    assert not np.isin(dup, ids).any()


def test_wrong_side_pointers_are_refused(classifier):
    """A host array passed as a device pointer is refused before any kernel
    reads it."""
    import ctypes as C
    import wolkenbase_gb300 as wb
    from wolkenbase_gb300 import _lib, synth
    cloud = synth.density_tile(5_000, 74)
    xyz = np.ascontiguousarray(cloud.xyz, np.int32)
    cs = wb.cloud_struct(xyz, cloud.n, 12, cloud.scale, cloud.offset, cloud.unit, cloud.minc, cloud.maxc,
                         device_resident=True)
    assert classifier.L.wb_octree_build(classifier.ctx, C.byref(cs)) == _lib.WB_EINVAL
    cls = np.zeros(cloud.n, np.uint8)
    classifier.classify_cloud(cloud)
    rec = np.zeros((cloud.n, 28), np.uint8)
    assert classifier.L.wb_las_write_classes(classifier.ctx, rec.ctypes.data, cloud.n, 28, 1, 1,
                                             cls.ctypes.data) == _lib.WB_EINVAL
    p = wb.Params().c()
    assert classifier.L.wb_classify(classifier.ctx, C.byref(p), cls.ctypes.data, 1) == _lib.WB_EINVAL
