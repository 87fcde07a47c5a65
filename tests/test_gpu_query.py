"""Octree::findBlocks and OctStore::pointsIn through the C ABI against the
oracle (octree.cpp:234-251, 1214-1242): cylinders of the tile grid and
downward hyperboloids of stored points, on a golden cloud and on a cloud
with points outside the root cube, sorted and unsorted."""
import numpy as np
import pytest

from conftest import golden_cloud, load_golden

pytestmark = pytest.mark.gpu


def _queries(cloud, seed, m=40):
    rng = np.random.default_rng(seed)
    d = cloud.decoded()
    pick = d[rng.integers(0, cloud.n, m)]
    out = []
    for k, p in enumerate(pick):
        out.append((1, (p[0] + rng.normal(0, 0.3), p[1] + rng.normal(0, 0.3)), float(rng.uniform(0.05, 2.5)), 1.0))
        out.append((2, tuple(p + np.array([0, 0, rng.uniform(0, 3)])), float(rng.uniform(0.02, 0.5)),
                    float(rng.choice([0.5, 1.0, 1.5]))))
    out.append((1, tuple(d[:, :2].mean(axis=0)), 1e6, 1.0))     # everything
    out.append((2, tuple(d.min(axis=0) - 5.0), 0.1, 1.0))         # nothing
    return out


@pytest.mark.parametrize("case", ["tile20k", "split"])
def test_points_in_and_find_blocks_match_oracle(classifier, oracle_mod, case):
    g = load_golden(case)
    cloud = golden_cloud(g)
    classifier.build(cloud)
    oracle_mod.run(cloud, canonical_order=True, phases=1, keep=True)
    try:
        for kind, v, r, s in _queries(cloud, 5):
            fb = classifier.find_blocks(kind, v, r, s)
            assert np.array_equal(fb, oracle_mod.find_blocks(kind, v, r, s)), (kind, v, r, s)
            for srt in (False, True):
                got = classifier.points_in(kind, v, r, s, sorted=srt)
                want = oracle_mod.points_in(kind, v, r, s, sorted=srt)
                assert np.array_equal(got, want), (kind, v, r, s, srt, got.size, want.size)
    finally:
        oracle_mod.reset()


def test_points_in_capacity_and_errors(classifier):
    import ctypes as C
    import wolkenbase_gb300 as wb
    from wolkenbase_gb300 import _lib, synth
    cloud = synth.density_tile(3000, 71)
    classifier.build(cloud)
    d = cloud.decoded()
    sh = classifier._shape(1, d[:, :2].mean(axis=0), 1e6, 1.0)
    n = C.c_uint64(0)
    small = np.zeros(5, np.uint32)
    rc = classifier.L.wb_points_in(classifier.ctx, C.byref(sh), 0, small.ctypes.data, 5, C.byref(n))
    assert rc == _lib.WB_EINVAL and n.value == cloud.n
    bad = classifier._shape(7, (0, 0, 0), 1.0, 1.0)
    assert classifier.L.wb_points_in(classifier.ctx, C.byref(bad), 0, None, 0, C.byref(n)) == _lib.WB_EINVAL
    assert sorted(classifier.points_in(1, d[:, :2].mean(axis=0), 1e6)) == list(range(cloud.n))
