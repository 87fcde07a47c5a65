"""Precision mode (WB_PRECISION_FP32) against the exact path on UTM-like
clouds (x ~ 500 km, y ~ 4500 km, 1 cm scale, 45 degree slopes, 2 m steps).

The exact path is the one pinned to the reference; the FP32 mode may flip
labels only where a decision lies within FP32 rounding, and its fit may
differ from the FP64 fit only by rounding.  Bounds (stated here, checked on
every run): label agreement >= 99.99%, slope error < 1e-5, per-point
fit-residual difference < 1e-5 m, and for 99.9% of the tiles the per-point
residual difference within 1e-6 of the tile's largest FP64 residual.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def utm_cloud():
    from wolkenbase_gb300 import synth
    return synth.mosaic([synth.utm_block(50_000, 22.0, i, j) for i in range(3) for j in range(3)])


def test_fp32_mode_within_bounds(utm_cloud, cuda_lib_path):
    import wolkenbase_gb300 as wb
    from wolkenbase_gb300 import precision
    clf = wb.Classifier(0)
    try:
        exact_first = clf.classify_cloud(utm_cloud)
        r = precision.compare(clf, utm_cloud)
        assert r["tiles_compared"] > 1000
        assert r["agreement"] >= 0.9999, r
        assert r["slope_err"] < 1e-5, r
        assert r["residual_abs_err_m"] < 1e-5, r
        assert r["residual_err_p999"] < 1e-6, r
        assert r["h_rel_err"] < 1e-9, r
        # back in exact mode the labels are the exact ones again
        assert np.array_equal(clf.classify_cloud(utm_cloud), exact_first)
    finally:
        clf.close()


def test_fp32_mode_on_a_1mm_tile(cuda_lib_path):
    import wolkenbase_gb300 as wb
    from wolkenbase_gb300 import precision, synth
    clf = wb.Classifier(0)
    try:
        r = precision.compare(clf, synth.density_tile(300_000, 78))
        assert r["agreement"] >= 0.9999 and r["slope_err"] < 1e-6 and r["residual_err"] < 1e-6, r
    finally:
        clf.close()


def test_fp32_mode_same_tile_membership(utm_cloud, cuda_lib_path):
    """The tile gather is shared: both modes fit the same points per tile."""
    import wolkenbase_gb300 as wb
    from wolkenbase_gb300 import _lib
    clf = wb.Classifier(0)
    try:
        clf.build(utm_cloud)
        clf.scan()
        t64 = clf.tiles()
        clf.set_precision(_lib.WB_PRECISION_FP32)
        clf.scan()
        t32 = clf.tiles()
        assert np.array_equal(t64["n_points"], t32["n_points"])
        p = clf.planes()
        ok = t32["n_points"] >= 3
        assert np.isfinite(p[ok]).all()
    finally:
        clf.close()


def test_precision_mode_rejects_unknown_values(cuda_lib_path):
    import wolkenbase_gb300 as wb
    from wolkenbase_gb300 import _lib
    clf = wb.Classifier(0)
    try:
        assert clf.L.wb_set_precision(clf.ctx, 7) == _lib.WB_EINVAL
    finally:
        clf.close()


def test_tile_residuals_match_numpy(cuda_lib_path):
    """wb_tile_residuals against numpy over each tile's cylinder points
    (OctStore::pointsIn of the tile's Cylinder): against its own planes the
    difference is zero, and the largest residual matches."""
    import wolkenbase_gb300 as wb
    from wolkenbase_gb300 import synth
    cloud = synth.density_tile(30_000, 91)
    clf = wb.Classifier(0)
    try:
        clf.build(cloud)
        clf.scan()
        planes = clf.planes()
        diff, rmax = clf.residuals(planes)
        tiles = clf.tiles()
        ok = (tiles["n_points"] >= 3) & np.all(np.isfinite(planes), axis=1)
        assert ok.sum() > 100
        assert np.all(diff[ok] == 0)
        info = clf.info()
        sp, (cx0, cy0, _) = info["spacing"], info["tile_center"]
        d = cloud.decoded()
        rng = np.random.default_rng(4)
        for k in rng.choice(np.nonzero(ok)[0], 40, replace=False):
            cx = cx0 + (tiles["ex"][k] - tiles["ey"][k] / 2.0) * sp
            cy = cy0 + (tiles["ey"][k] * 0.86602540378443864676372317) * sp
            pts = clf.points_in(1, (cx, cy), sp * 41 / 71)
            assert pts.size == tiles["n_points"][k]
            a, b, c = planes[k]
            r = d[pts, 2] - (a * (d[pts, 0] - cx) + b * (d[pts, 1] - cy) + c)
            assert abs(np.abs(r).max() - rmax[k]) <= 1e-9 * max(1.0, rmax[k])
        # against shifted planes the difference is the shift where x = y = 0 is the worst case
        shifted = planes.copy()
        shifted[:, 2] += 1e-3
        diff2, _ = clf.residuals(shifted)
        assert np.allclose(diff2[ok], 1e-3, rtol=1e-9, atol=1e-12)
    finally:
        clf.close()
