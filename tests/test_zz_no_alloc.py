"""wb_octree_find_block_static: the point lookup that allocates no device memory.

It serves callers that must not call cudaMalloc/cudaFree on their query path
(a serving loop whose cudaFree would wait for every job on the device, or a
process at its HBM budget).  Its answers must equal the allocating
wb_octree_find_block on the same positions, call after call, even though all
calls share one static staging array.  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STATIC_MAX = 65536   # WB_FIND_BLOCK_STATIC_MAX in include/wolkenbase_gb300.h


def _positions(cloud, m, seed):
    rng = np.random.default_rng(seed)
    d = cloud.decoded()
    pick = d[rng.integers(0, cloud.n, m // 2)]
    lo, hi = d.min(axis=0), d.max(axis=0)
    span = hi - lo
    # random positions in and around the cloud, some outside every leaf
    rand = lo - 0.2 * span + rng.random((m - m // 2, 3)) * 1.4 * span
    return np.ascontiguousarray(np.concatenate([pick, rand]))


def _cudart():
    """The CUDA runtime the library loaded (found through this process's maps)."""
    with open("/proc/self/maps") as f:
        for line in f:
            if "libcudart.so" in line:
                return C.CDLL(line.split()[-1])
    pytest.skip("libcudart not mapped into this process")


USED_CURRENT, USED_HIGH = 7, 8      # cudaMemPoolAttrUsedMemCurrent / UsedMemHigh (driver_types.h)


def _pool_used(rt, pool):
    cur, high = C.c_uint64(0), C.c_uint64(0)
    assert rt.cudaMemPoolGetAttribute(pool, USED_CURRENT, C.byref(cur)) == 0
    assert rt.cudaMemPoolGetAttribute(pool, USED_HIGH, C.byref(high)) == 0
    return cur.value, high.value


def _reset_high(rt, pool):
    zero = C.c_uint64(0)
    assert rt.cudaMemPoolSetAttribute(pool, USED_HIGH, C.byref(zero)) == 0


def test_static_lookup_allocates_nothing():
    """The property the entry point exists for: no device memory is taken,
    neither from the context (its byte count) nor from the device's
    stream-ordered pool (its high-water mark), while the allocating lookup
    does take pool memory for its staging."""
    import wolkenbase_gb300 as wb
    from wolkenbase_gb300 import synth
    clf = wb.Classifier(0)
    try:
        cloud = synth.density_tile(20000, 62)
        clf.build(cloud)
        clf.synchronize()
        rt = _cudart()
        pool = C.c_void_p(0)
        assert rt.cudaDeviceGetDefaultMemPool(C.byref(pool), 0) == 0
        pts = _positions(cloud, STATIC_MAX, 7)
        got = np.zeros(STATIC_MAX, np.int64)
        L = clf.L
        assert L.wb_octree_find_block_static(clf.ctx, pts.ctypes.data, STATIC_MAX, got.ctypes.data) == 0  # set-up
        held0 = clf.paging_stats()["device_bytes"]
        cur0, _ = _pool_used(rt, pool)
        _reset_high(rt, pool)
        for _ in range(2):
            assert L.wb_octree_find_block_static(clf.ctx, pts.ctypes.data, STATIC_MAX, got.ctypes.data) == 0
        cur1, high1 = _pool_used(rt, pool)
        assert clf.paging_stats()["device_bytes"] == held0
        assert cur1 == cur0 and high1 == cur0, (cur0, cur1, high1)
        # the allocating lookup, by contrast, stages through the pool
        _reset_high(rt, pool)
        ref = clf.find_block(pts)
        clf.synchronize()
        _, high2 = _pool_used(rt, pool)
        assert high2 > cur0, (cur0, high2)
        assert np.array_equal(got, ref)
    finally:
        clf.close()


def test_static_lookup_matches_allocating_lookup():
    import wolkenbase_gb300 as wb
    from wolkenbase_gb300 import _lib, synth
    clf = wb.Classifier(0)
    try:
        cloud = synth.density_tile(30000, 61)
        clf.build(cloud)
        L = clf.L
        for call, m in enumerate((STATIC_MAX, 3001)):   # the second call is shorter than the first
            pts = _positions(cloud, m, 100 + call)
            ref = clf.find_block(pts)
            got = np.full(m, -7, np.int64)
            rc = L.wb_octree_find_block_static(clf.ctx, pts.ctypes.data, m, got.ctypes.data)
            assert rc == 0, L.wb_last_error(clf.ctx)
            assert np.array_equal(got, ref)
            assert (got >= 0).any() and (got == -1).any()
        # the decoded points themselves land in their own leaves
        d = np.ascontiguousarray(cloud.decoded()[:20000])
        got = np.zeros(d.shape[0], np.int64)
        assert L.wb_octree_find_block_static(clf.ctx, d.ctypes.data, d.shape[0], got.ctypes.data) == 0
        assert np.array_equal(got, clf.point_leaf()[:20000].astype(np.int64))
        # one position more than the static array holds is refused
        big = np.zeros((STATIC_MAX + 1, 3))
        out = np.zeros(STATIC_MAX + 1, np.int64)
        rc = L.wb_octree_find_block_static(clf.ctx, big.ctypes.data, STATIC_MAX + 1, out.ctypes.data)
        assert rc == _lib.WB_EINVAL
        assert b"static staging array" in L.wb_last_error(clf.ctx)
    finally:
        clf.close()
