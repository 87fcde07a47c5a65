"""Host-side logic that needs no GPU: the precision report's arithmetic (on a
stand-in context), the synthetic workloads' determinism, the LAS output
settings as the C struct sees them, and the bench's sampling helpers."""
import numpy as np
import pytest


class _FakeContext:
    """Answers the calls precision.compare makes, with fixed results per mode."""

    def __init__(self, results, spacing=1.2):
        self.results = results
        self.mode = 0
        self.spacing = spacing

    def set_precision(self, mode):
        self.mode = mode

    def build(self, cloud):
        pass

    def synchronize(self):
        pass

    def scan(self, params=None):
        pass

    def classify(self, params=None):
        return self.results[self.mode][0]

    def planes(self):
        return self.results[self.mode][1]

    def tiles(self):
        return self.results[self.mode][2]

    def info(self):
        return {"spacing": self.spacing}

    def residuals(self, ref_planes):
        """Per tile max |r32 - r64| and max |r64| of the points' residuals."""
        return np.array([2e-6, 0.0, 3e-8]), np.array([0.2, 0.0, 0.01])


def _tiles(n_points, height, h, flags):
    from wolkenbase_gb300 import TILE_DTYPE
    t = np.zeros(len(n_points), TILE_DTYPE)
    t["n_points"] = n_points
    t["height"] = height
    t["hyperboloid_size"] = h
    t["tree_flags"] = flags
    return t


def test_precision_report_arithmetic():
    from wolkenbase_gb300 import _lib, precision, synth
    cls64 = np.array([1, 2, 2, 1, 2], np.uint8)
    cls32 = np.array([1, 2, 1, 1, 2], np.uint8)
    p64 = np.array([[0.1, 0.2, 5.0], [0.0, 0.0, 1.0], [0.3, 0.1, 2.0]])
    p32 = p64 + np.array([[3e-7, -4e-7, 1e-6], [0, 0, 0], [0, 0, 0]])
    t64 = _tiles([10, 2, 7], [0.5, 0.1, 0.8], [0.4, 0.0, 1.0], [0, 0, 1])
    t32 = _tiles([10, 2, 7], [0.5, 0.1, 0.8], [0.41, 0.0, 1.0], [0, 1, 1])
    clf = _FakeContext({_lib.WB_PRECISION_EXACT: (cls64, p64, t64), _lib.WB_PRECISION_FP32: (cls32, p32, t32)})
    cloud = synth.Cloud(np.zeros((5, 3), np.int32), (0.001,) * 3, (0.0,) * 3, 1.0, (0, 0, 0), (1, 1, 1))
    r = precision.compare(clf, cloud)
    assert r["points"] == 5 and r["flips"] == 1 and r["agreement"] == pytest.approx(0.8)
    assert r["tiles_compared"] == 2                      # the 2-point tile is not a fit
    assert r["slope_err"] == pytest.approx(5e-7)
    # per-point residual differences over the residual range, per tile (tiles 0 and 2)
    assert r["residual_abs_err_m"] == pytest.approx(2e-6)
    assert r["residual_err"] == pytest.approx(max(2e-6 / 0.2, 3e-8 / 0.01))
    assert r["h_rel_err"] == pytest.approx(0.025) and r["h_changed"] == 1
    assert r["tree_flag_changes"] == 1


def test_synthetic_workloads_are_seeded():
    from wolkenbase_gb300 import synth
    a, b, c = synth.density_tile(3000, 7), synth.density_tile(3000, 7), synth.density_tile(3000, 8)
    assert np.array_equal(a.xyz, b.xyz) and not np.array_equal(a.xyz, c.xyz)
    d = a.decoded()
    assert (d.min(axis=0) >= np.array(a.minc) * a.unit - 1e-9).all()
    assert (d.max(axis=0) <= np.array(a.maxc) * a.unit + 1e-9).all()


def test_las_output_settings_reach_the_struct():
    import wolkenbase_gb300 as wb
    o = wb.LasOutput(point_format=7, separate_classes=False, n_input_files=3, points_per_file=12345,
                     unit=0.3048, min_cor=(1, 2, 3), max_cor=(4, 5, 6), scale=(0.01, 0.02, 0.03),
                     creation_day=45, creation_year=2026, software="tool 1")
    c = o.c()
    assert (c.point_format, c.separate_classes, c.n_input_files, c.points_per_file) == (7, 0, 3, 12345)
    assert (c.creation_day, c.creation_year, c.software) == (45, 2026, b"tool 1")
    assert tuple(c.min_cor) == (1, 2, 3) and tuple(c.max_cor) == (4, 5, 6) and tuple(c.scale) == (0.01, 0.02, 0.03)
    assert wb.LasOutput().c().software is None


def test_bench_tile_sample_estimate_and_single_rank_max():
    import bench
    t = bench.sample_tiles(1000, 0.01, 7)
    assert t.shape[0] == 10 and np.all(np.diff(t) > 0) and t.min() >= 0 and t.max() < 1000
    assert np.array_equal(t, bench.sample_tiles(1000, 0.01, 7))
    # build time plus the sample's scan time scaled by scanned tiles and its classify time by sampled tiles
    est = bench.oracle_estimate(2.0, {"t_scan": 0.5, "t_classify": 3.0, "n_scanned": 50}, 1000, 10)
    assert abs(est - (2.0 + 0.5 * 1000 / 50 + 3.0 * 1000 / 10)) < 1e-9
    assert bench.max_over_ranks(3.5, "cpu") == 3.5


def test_bench_oracle_baseline_parity_on_a_small_cloud():
    """The CPU baseline's parity check, run against the oracle's own full
    answers: every count agrees and the agreement is 1."""
    import bench
    from oracle import oracle as O
    from wolkenbase_gb300 import synth
    cloud = synth.density_tile(12_000, 5)
    full = O.run(cloud, canonical_order=True, threads=4)
    tiles = full["tiles"]
    gpu = {"n_leaves": full["n_leaves"], "leaves": full["leaves"], "count": full["leaf_count"].astype(np.uint32),
           "pleaf": np.maximum(full["leaf"], 0).astype(np.uint32), "cls": full["cls"],
           "tiles": {"n_points": tiles["n_points"], "tree_flags": tiles["tree_flags"], "density": tiles["density"],
                     "h_scan": tiles["h_scan"], "hyperboloid_size": tiles["h_final"], "height": tiles["height"]}}
    base, parity = bench.oracle_baseline(cloud, 4, 0.2, 3, gpu)
    assert base["value"] > 0 and base["kind"] == "port"
    assert parity["octree_exact"] and parity["sampled_tiles_exact"] == parity["sampled_tiles"]
    assert parity["sampled_labels"] > 0 and parity["agreement"] == 1.0


def test_scan_packed_pairwise_tree_groups_as_the_reference():
    """The exact scan adds the eight quantities of a 32-point chunk's four
    groups of eight with a lane exchange (pairs, quads, groups; each lane adds
    the quantities it and its partner split).  Replayed here lane by lane with
    the kernel's index rules, every group sum equals the fixed tree
    ((a0+a1)+(a2+a3))+((a4+a5)+(a6+a7)) of pairwisesum bit for bit, and lane l
    of the first eight holds quantity 4*(l&1) + 2*((l>>1)&1) + ((l>>2)&1)."""
    rng = np.random.default_rng(11)
    for _ in range(100):
        q = rng.standard_normal((32, 8)) * 10.0 ** rng.integers(-8, 9, (32, 8))
        s1 = np.zeros((32, 4))
        for r in range(4):
            give = np.array([q[l][r] if l & 1 else q[l][4 + r] for l in range(32)])
            for l in range(32):
                s1[l][r] = (q[l][4 + r] if l & 1 else q[l][r]) + give[l ^ 1]
        s2 = np.zeros((32, 2))
        for t in range(2):
            give = np.array([s1[l][t] if (l >> 1) & 1 else s1[l][2 + t] for l in range(32)])
            for l in range(32):
                s2[l][t] = (s1[l][2 + t] if (l >> 1) & 1 else s1[l][t]) + give[l ^ 2]
        give = np.array([s2[l][0] if (l >> 2) & 1 else s2[l][1] for l in range(32)])
        for l in range(32):
            g = (s2[l][1] if (l >> 2) & 1 else s2[l][0]) + give[l ^ 4]
            u, gq = 4 * (l & 1) + 2 * ((l >> 1) & 1) + ((l >> 2) & 1), l >> 3
            a = q[8 * gq:8 * gq + 8, u]
            assert g == ((a[0] + a[1]) + (a[2] + a[3])) + ((a[4] + a[5]) + (a[6] + a[7]))


def test_split_word_index_by_multiply_high_is_exact():
    """The class split finds a word's record as the high half of
    w * ceil(2^32 / words): exact while w * words < 2^32, which holds for every
    tile of 2048 records whenever the kernel takes that path."""
    for words in range(2, 4096):
        magic = ((1 << 32) + words - 1) // words
        total = 2048 * words
        if total * words >= 1 << 32:
            continue
        w = np.unique(np.concatenate([np.arange(0, min(total, 3000)), np.arange(max(0, total - 3000), total),
                                      np.arange(0, total, max(1, total // 5000))])).astype(np.uint64)
        assert np.array_equal((w * np.uint64(magic)) >> np.uint64(32), w // np.uint64(words)), words
