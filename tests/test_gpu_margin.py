"""Decision margins (wb_classify_ex): the largest gap between a point's
hyperboloid directions minus 144 degrees.  The sign follows the label; for a
ground point (never surrounded, so every neighbour was seen) the value equals
the oracle's largest gap of the full direction set, within the FP32 direction
error of the fast pass (2 x 2048 units of the 2^31-per-turn angle, 3.4e-4
degrees) and exactly where the exact pass re-ran the point."""
import numpy as np
import pytest

from conftest import golden_cloud, golden_params, load_golden

pytestmark = pytest.mark.gpu
GAP_TOL_DEG = 2 * 2048 * 360.0 / 2**31 + 1e-5


@pytest.mark.parametrize("case", ["tile20k", "params6k", "utm8k"])
def test_margins_follow_labels_and_oracle(classifier, oracle_mod, case):
    import wolkenbase_gb300 as wb
    g = load_golden(case)
    cloud = golden_cloud(g)
    prm = golden_params(g)
    classifier.build(cloud)
    classifier.scan(wb.Params(**prm))
    cls, margin = classifier.classify_margins(wb.Params(**prm))
    assert np.array_equal(cls, classifier.classify(wb.Params(**prm)))   # same labels as wb_classify
    o = oracle_mod.run(cloud, canonical_order=True, threads=8, margins=True, **prm)
    stored = o["block"] >= 0
    decided = stored & (o["cls"] != 0)
    assert np.array_equal(np.isnan(margin[stored]), o["cls"][stored] == 0)
    assert np.all(margin[decided & (cls == 1)] < 0)
    assert np.all(margin[decided & (cls == 2)] >= 0)
    ground = decided & (cls == 2)
    idx = np.nonzero(ground)[0]
    err = np.abs(margin[idx].astype(np.float64) - o["margin"][idx])
    worst = int(idx[np.argmax(err)])
    assert err.max() <= GAP_TOL_DEG, (err.max(), worst, float(margin[worst]), float(o["margin"][worst]))
