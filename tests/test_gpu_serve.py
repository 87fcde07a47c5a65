"""Serving and batching: the request loop (wb_server) and the fused launch.

Each job's class bytes must be identical whether the cloud is classified
alone (wb_classify_cloud on its own context) or among other jobs of uneven
size that are admitted, scanned and classified together.  The path is exact
(octree, tiles and labels), so "the same" here means byte-identical.
"""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _clouds():
    from wolkenbase_gb300 import synth
    spec = [(40_000, 901, 0.2), (3_000, 902, 0.1), (250_000, 903, 0.35), (90_000, 904, 0.05),
            (12_000, 905, 0.4), (150_000, 906, 0.2)]
    return [synth.batch_tile(n, seed, frac) for n, seed, frac in spec]


@pytest.fixture(scope="module")
def clouds_alone(cuda_lib_path):
    import wolkenbase_gb300 as wb
    clouds = _clouds()
    clf = wb.Classifier(0)
    try:
        alone = [clf.classify_cloud(c) for c in clouds]
    finally:
        clf.close()
    return clouds, alone


def test_served_results_equal_alone(clouds_alone):
    import wolkenbase_gb300 as wb
    clouds, alone = clouds_alone
    srv = wb.Server(0, prep_slots=3)
    try:
        ids = [srv.submit(c, tag=i) for i, c in enumerate(clouds)]
        for i, jid in enumerate(ids):
            cls, st = srv.result(jid)
            assert st["state"] == 4 and st["rc"] == 0 and st["tag"] == i
            assert st["n_points"] == clouds[i].n
            assert st["t_submit"] <= st["t_admit"] <= st["t_ready"] <= st["t_done"]
            assert st["batch_jobs"] >= 1
            assert np.array_equal(cls, alone[i]), f"job {i} differs from its result alone"
        s = srv.stats()
        assert s["completed"] == len(clouds) and s["failed"] == 0
        assert s["fused_jobs"] == len(clouds)
        assert s["peak_bytes"] <= s["budget"]
    finally:
        srv.close()


def test_batch_one_fused_launch_equals_alone(clouds_alone):
    import wolkenbase_gb300 as wb
    from wolkenbase_gb300 import _lib
    clouds, alone = clouds_alone
    srv = wb.Server(0, prep_slots=4, flush=_lib.WB_FLUSH_FULL)
    try:
        got = srv.classify_batch(clouds)
        for i in range(len(clouds)):
            assert np.array_equal(got[i], alone[i]), f"job {i} differs from its result alone"
        s = srv.stats()
        assert s["fused_launches"] == 1 and s["fused_jobs"] == len(clouds)
        # again, with the contexts (and their buffers) reused
        got = srv.classify_batch(clouds[::-1])
        for i in range(len(clouds)):
            assert np.array_equal(got[i], alone[len(clouds) - 1 - i])
    finally:
        srv.close()


@pytest.mark.parametrize("shape,chunk,grid_points", [(4, 1, 16.0), (3, 64, 48.0), (2, 4, 0.0), (1, 2, 24.0), (7, 8, 64.0)])
def test_fused_launch_shapes_agree(clouds_alone, shape, chunk, grid_points):
    """Kernel shape, chunk and column density change speed, never labels."""
    import wolkenbase_gb300 as wb
    from wolkenbase_gb300 import _lib
    clouds, alone = clouds_alone
    srv = wb.Server(0, prep_slots=2, flush=_lib.WB_FLUSH_FULL, shape=shape, chunk=chunk, grid_points=grid_points)
    try:
        got = srv.classify_batch(clouds[:4])
        for i in range(4):
            assert np.array_equal(got[i], alone[i])
    finally:
        srv.close()


def test_autotuner_picks_a_shape_and_keeps_labels(clouds_alone):
    import wolkenbase_gb300 as wb
    from wolkenbase_gb300 import _lib
    clouds, alone = clouds_alone
    from wolkenbase_gb300 import synth
    srv = wb.Server(0, prep_slots=3, flush=_lib.WB_FLUSH_FULL, autotune=True)
    try:
        got = srv.classify_batch(clouds)
        for i in range(len(clouds)):
            assert np.array_equal(got[i], alone[i])
        assert srv.stats()["tuned"] == 0          # no job large enough to time yet
        clouds = clouds + [synth.batch_tile(1_100_000, 909, 0.2)]
        clf = wb.Classifier(0)
        alone = alone + [clf.classify_cloud(clouds[-1])]
        clf.close()
        got = srv.classify_batch(clouds)
        for i in range(len(clouds)):
            assert np.array_equal(got[i], alone[i])
        s = srv.stats()
        assert s["tuned"] == 1 and 0 <= s["shape"] < _lib.WB_N_SHAPES
        assert s["chunk"] in (1, 2, 4, 16) and s["grid_points"] in (32, 48, 64, 96)
        assert s["tune_ms"] > 0
        got = srv.classify_batch(clouds)          # jobs prepared with the tuned column density
        for i in range(len(clouds)):
            assert np.array_equal(got[i], alone[i])
    finally:
        srv.close()


def test_classifier_tuning_keeps_labels(clouds_alone):
    import wolkenbase_gb300 as wb
    clouds, alone = clouds_alone
    clf = wb.Classifier(0)
    try:
        clf.set_tuning(shape=3, chunk=16, grid_points=24.0)
        assert clf.tuning() == {"shape": 3, "chunk": 16, "grid_points": 24.0}
        assert np.array_equal(clf.classify_cloud(clouds[2]), alone[2])
        clf.build(clouds[5])
        clf.scan()
        t = clf.autotune()
        assert 0 <= t["shape"] < 8 and t["chunk"] in (1, 2, 4, 16) and t["grid_points"] in (32, 48, 64, 96)
        assert np.array_equal(clf.classify(), alone[5])
        assert np.array_equal(clf.classify_cloud(clouds[0]), alone[0])
    finally:
        clf.close()


def test_admission_keeps_within_budget(clouds_alone):
    """With room for about two jobs at a time, every job still completes and
    the bytes held never exceed the budget."""
    import wolkenbase_gb300 as wb
    clouds, alone = clouds_alone
    budget = 2 * (300 + 12) * 250_000 + 3 * (64 << 20)
    srv = wb.Server(0, prep_slots=4, hbm_budget=budget)
    try:
        ids = [srv.submit(c) for c in clouds]
        for i, jid in enumerate(ids):
            cls, st = srv.result(jid)
            assert np.array_equal(cls, alone[i])
        s = srv.stats()
        assert s["completed"] == len(clouds)
        assert s["peak_bytes"] <= budget
    finally:
        srv.close()


def test_job_larger_than_budget_fails_alone():
    import wolkenbase_gb300 as wb
    from wolkenbase_gb300 import _lib, synth
    srv = wb.Server(0, prep_slots=1, hbm_budget=80 << 20)
    try:
        big = synth.density_tile(200_000, 907)
        small = synth.density_tile(2_000, 908)
        jb = srv.submit(big)
        js = srv.submit(small)
        st = srv.wait(jb)
        assert st["state"] == _lib.WB_JOB_FAILED and st["rc"] == _lib.WB_ENOMEM
        cls, st = srv.result(js)
        assert st["rc"] == 0
    finally:
        srv.close()


def test_cancel_queued_job(clouds_alone):
    import wolkenbase_gb300 as wb
    from wolkenbase_gb300 import _lib
    clouds, alone = clouds_alone
    srv = wb.Server(0, prep_slots=1)
    try:
        ids = [srv.submit(clouds[2]) for _ in range(3)]
        last = srv.submit(clouds[0])
        rc = srv.cancel(last)
        st = srv.wait(last)
        if rc == 0:
            assert st["state"] == _lib.WB_JOB_CANCELLED and st["rc"] == _lib.WB_ECANCELED
        else:   # it had already been admitted
            assert rc == _lib.WB_EBUSY and st["state"] == _lib.WB_JOB_DONE
        for jid in ids:
            cls, _ = srv.result(jid)
            assert np.array_equal(cls, alone[2])
        assert srv.cancel(ids[0]) in (_lib.WB_EBUSY, _lib.WB_ENOTFOUND)
    finally:
        srv.close()


def test_wait_times_out_then_completes(clouds_alone):
    import wolkenbase_gb300 as wb
    clouds, alone = clouds_alone
    srv = wb.Server(0, prep_slots=1)
    try:
        jid = srv.submit(clouds[2])
        st = srv.wait(jid, timeout=0.0)
        assert st is None or st["state"] == 4
        t = time.time()
        cls, st = srv.result(jid)
        assert time.time() - t < 60
        assert np.array_equal(cls, alone[2])
    finally:
        srv.close()
