"""The steps either side of the path on the device (class bytes into LAS
records, the class split, class totals, the duplicate report) against their
CPU restatement in oracle/las_oracle.py."""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, golden_cloud, golden_params, load_golden

pytestmark = pytest.mark.gpu


def _records(n, stride, seed):
    return np.random.default_rng(seed).integers(0, 256, size=(n, stride), dtype=np.uint8)


@pytest.mark.parametrize("fmt,stride", [(1, 28), (0, 20), (3, 34), (6, 30), (7, 36), (10, 67)])
def test_write_classes_matches_restatement(classifier, fmt, stride):
    from oracle import las_oracle as LO
    rec = _records(70_001, stride, fmt)
    cls = np.random.default_rng(99).integers(0, 256, size=rec.shape[0], dtype=np.uint8)
    got = classifier.las_write_classes(rec.copy(), fmt, cls)
    assert np.array_equal(got, LO.write_classes(rec, fmt, cls))


@pytest.mark.parametrize("fmt,stride", [(1, 28), (6, 32), (1, 29)])
def test_split_by_class_matches_restatement(classifier, fmt, stride):
    from oracle import las_oracle as LO
    rec = _records(123_457, stride, 3)
    # a realistic spread of classes: mostly 1 and 2, a few others
    c = np.random.default_rng(5).choice([0, 1, 2, 7, 31], size=rec.shape[0], p=[0.05, 0.25, 0.65, 0.03, 0.02])
    rec = LO.write_classes(rec, fmt, c.astype(np.uint8))
    out, offsets = classifier.las_split_by_class(rec, fmt)
    ref_out, ref_off = LO.split_by_class(rec, fmt)
    assert np.array_equal(offsets, ref_off)
    assert np.array_equal(out, ref_out)


def test_classify_then_write_back_and_split(classifier):
    """The classified cloud's class bytes go into format-1 records and split
    into the ground / not-ground groups of the counts the classify reports."""
    from oracle import las_oracle as LO
    from wolkenbase_gb300 import synth
    cloud = synth.density_tile(60_000, 31)
    cls = classifier.classify_cloud(cloud)
    rec = np.zeros((cloud.n, 28), np.uint8)
    rec[:, 0:12] = np.ascontiguousarray(cloud.xyz).view(np.uint8).reshape(-1, 12)
    rec[:, 15] = 0xA0   # flag bits that must survive
    got = classifier.las_write_classes(rec.copy(), 1)           # the last classify's bytes
    assert np.array_equal(got, LO.write_classes(rec, 1, cls))
    out, offsets = classifier.las_split_by_class(got, 1)
    assert offsets[3] - offsets[2] == np.count_nonzero(cls == 2)
    assert offsets[2] - offsets[1] == np.count_nonzero(cls == 1)
    assert np.array_equal(out, LO.split_by_class(got, 1)[0])


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_class_totals_and_duplicates(classifier, name):
    from oracle import las_oracle as LO
    g = load_golden(name)
    cloud = golden_cloud(g)
    import wolkenbase_gb300 as wb
    params = wb.Params(**golden_params(g))
    cls = classifier.classify_cloud(cloud, params)
    stored = classifier.store_order().astype(np.int64)
    assert np.array_equal(classifier.class_totals(), LO.class_totals(stored, cls))
    ndup, kept = classifier.duplicates(per_record=True)
    surv = LO.survivors(cloud.xyz)
    assert ndup == int(np.count_nonzero(surv != np.arange(cloud.n)))
    assert np.array_equal(kept.astype(np.int64), surv)


@pytest.mark.parametrize("side", [0.5, 0.37, 2.0])
def test_preview_matches_restatement(classifier, side):
    from oracle import las_oracle as LO
    from wolkenbase_gb300 import synth
    cloud = synth.density_tile(80_000, 41)
    classifier.build(cloud)
    stored = classifier.store_order().astype(np.int64)
    pts = cloud.decoded()[stored]
    x0, y0 = float(pts[:, 0].min()) - 1.0, float(pts[:, 1].min()) + 0.25
    w, h = 70, 41
    cnt, lo, hi = classifier.preview(x0, y0, side, w, h)
    rc, rl, rh = LO.preview(pts, x0, y0, side, w, h)
    assert np.array_equal(cnt, rc)
    assert np.array_equal(lo, rl) and np.array_equal(hi, rh)
    assert cnt.sum() > 0 and (cnt == 0).any()


def test_preview_matches_reference_goldens(classifier):
    """wb_preview against the reference's own countPointsIn / hiLoPointsIn
    (tests/golden/preview.npz, written by tests/golden/make_preview_golden.py)."""
    import os
    from conftest import ROOT
    from wolkenbase_gb300 import synth
    g = np.load(os.path.join(ROOT, "tests", "golden", "preview.npz"))
    for name in g["cases"]:
        c = np.load(os.path.join(ROOT, "tests", "golden", str(name) + ".npz"))
        cloud = synth.Cloud(c["xyz"].astype(np.int32), tuple(c["scale"]), tuple(c["offset"]), float(c["unit"]),
                            tuple(c["minc"]), tuple(c["maxc"]))
        classifier.build(cloud)
        for k in range(3):
            x0, y0, side, w, h = g[f"{name}_{k}_view"]
            cnt, lo, hi = classifier.preview(float(x0), float(y0), float(side), int(w), int(h))
            assert np.array_equal(cnt, g[f"{name}_{k}_count"]), (name, k)
            assert np.array_equal(lo, g[f"{name}_{k}_lo"]) and np.array_equal(hi, g[f"{name}_{k}_hi"]), (name, k)
