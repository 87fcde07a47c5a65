"""Paging: a cloud whose working set is about three times the context's HBM
budget is classified with the buffers beyond the budget in pinned host memory
(used in place by the kernels), and the labels equal the unbudgeted run's."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_paged_run_equals_resident_run():
    import wolkenbase_gb300 as wb
    from wolkenbase_gb300 import _lib, synth
    cloud = synth.density_tile(1_500_000, 61)
    clf = wb.Classifier(0)
    want = clf.classify_cloud(cloud)
    want_tiles = clf.tiles()
    clf.close()
    budget = 100 * cloud.n
    tight = wb.Classifier(0, hbm_budget=budget)
    try:
        with pytest.raises(wb.WolkenbaseError) as e:
            tight.classify_cloud(cloud)          # paging off: over budget
        assert e.value.code == _lib.WB_ENOMEM
        tight.set_paging(2 << 30)
        got = tight.classify_cloud(cloud)
        st = tight.paging_stats()
        assert st["host_peak"] > 0 and st["device_bytes"] <= budget
        assert np.array_equal(got, want)
        assert np.array_equal(tight.tiles(), want_tiles)
        # classes of the paged run feed the LAS steps the same way
        assert tight.class_totals()[2] == np.count_nonzero(want[tight.store_order().astype(np.int64)] == 2)
        tight.set_paging(0)
    finally:
        tight.close()


def test_paging_host_budget_is_respected():
    import wolkenbase_gb300 as wb
    from wolkenbase_gb300 import _lib, synth
    cloud = synth.density_tile(600_000, 62)
    clf = wb.Classifier(0, hbm_budget=60 * cloud.n)
    try:
        clf.set_paging(16 << 20)                  # far too little host memory as well
        with pytest.raises(wb.WolkenbaseError) as e:
            clf.classify_cloud(cloud)
        assert e.value.code == _lib.WB_ENOMEM
        assert clf.paging_stats()["host_peak"] <= 16 << 20
    finally:
        clf.close()


def test_pinned_inputs_are_read_in_place():
    """Records and class bytes in pinned host memory are pulled by a kernel;
    the labels equal those of a pageable-buffer run (odd byte counts take the
    tail through the copy engine)."""
    import ctypes as C
    torch = pytest.importorskip("torch")
    import wolkenbase_gb300 as wb
    from wolkenbase_gb300 import synth
    cloud = synth.density_tile(300_001, 63)
    clf = wb.Classifier(0)
    try:
        want = clf.classify_cloud(cloud)
        pin = torch.from_numpy(np.ascontiguousarray(cloud.xyz)).pin_memory()
        pcls = torch.zeros(cloud.n, dtype=torch.uint8).pin_memory()
        cs = wb.cloud_struct(pin.data_ptr(), cloud.n, 12, cloud.scale, cloud.offset, cloud.unit, cloud.minc,
                             cloud.maxc)
        clf._check(clf.L.wb_classify_cloud(clf.ctx, C.byref(cs), C.byref(wb.Params().c()),
                                           C.c_void_p(pcls.data_ptr())))
        assert np.array_equal(pcls.numpy(), want)
    finally:
        clf.close()


def test_server_runs_over_budget_job_paged():
    """With a host allowance, a job above the whole HBM budget runs alone with
    paging instead of failing; the jobs around it are unaffected."""
    import wolkenbase_gb300 as wb
    from wolkenbase_gb300 import synth
    big = synth.density_tile(200_000, 907)
    small = synth.density_tile(2_000, 908)
    clf = wb.Classifier(0)
    want_big, want_small = clf.classify_cloud(big), clf.classify_cloud(small)
    clf.close()
    srv = wb.Server(0, prep_slots=2, hbm_budget=80 << 20, host_budget=1 << 30)
    try:
        ids = [srv.submit(small), srv.submit(big), srv.submit(small)]
        got = [srv.result(i) for i in ids]
        for (cls, st), want in zip(got, [want_small, want_big, want_small]):
            assert st["rc"] == 0 and np.array_equal(cls, want)
        s = srv.stats()
        assert s["completed"] == 3 and s["failed"] == 0 and s["peak_bytes"] <= 80 << 20
    finally:
        srv.close()
