"""Device arithmetic against the reference's golden vectors and the oracle:
integer directions (atan2i), the C library's hypot, Hyperboloid::in."""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def _lib():
    from wolkenbase_gb300 import _lib
    return _lib.load()


def gpu_atan2i(yx):
    yx = np.ascontiguousarray(yx, np.float64)
    out = np.zeros(yx.shape[0], np.int32)
    assert _lib().wb_check_atan2i(yx.ctypes.data, yx.shape[0], out.ctypes.data) == 0
    return out


def gpu_hypot(ab):
    ab = np.ascontiguousarray(ab, np.float64)
    out = np.zeros(ab.shape[0])
    assert _lib().wb_check_hypot(ab.ctypes.data, ab.shape[0], out.ctypes.data) == 0
    return out


def gpu_hyp(v, r, s, xyz):
    v = np.ascontiguousarray(v, np.float64)
    xyz = np.ascontiguousarray(xyz, np.float64)
    out = np.zeros(xyz.shape[0], np.uint8)
    assert _lib().wb_check_hyperboloid(v.ctypes.data, r, s, xyz.ctypes.data, xyz.shape[0], out.ctypes.data) == 0
    return out


def test_atan2i_golden(cuda_lib_path):
    g = load_golden("primitives")
    got = gpu_atan2i(g["atan_yx"])
    bad = np.nonzero(got != g["atan_out"])[0]
    assert bad.size == 0, (bad[:10], g["atan_yx"][bad[:10]], got[bad[:10]], g["atan_out"][bad[:10]])


def test_atan2i_random_matches_oracle(cuda_lib_path, oracle_mod):
    rng = np.random.default_rng(3)
    m = 1_000_000
    yx = np.stack([rng.integers(-30000, 30000, m) * 0.001, rng.integers(-30000, 30000, m) * 0.001], 1)
    yx[:1000, 0] = 0.0
    got = gpu_atan2i(yx)
    ref = oracle_mod.atan2i(yx[:, 0], yx[:, 1])
    bad = np.nonzero(got != ref)[0]
    assert bad.size == 0, (bad[:10], yx[bad[:10]], got[bad[:10]], ref[bad[:10]])


def test_hypot_matches_reference_libm(cuda_lib_path, oracle_mod):
    rng = np.random.default_rng(4)
    m = 1_000_000
    ab = np.stack([rng.integers(-30000, 30000, m) * 0.001, rng.integers(-30000, 30000, m) * 0.001], 1)
    big = np.stack([10.0 ** rng.uniform(-3, 7, 10000), 10.0 ** rng.uniform(-3, 7, 10000)], 1)
    ab = np.concatenate([ab, big, [[0.0, 0.0], [0.0, 3.0], [4.0, 0.0]]])
    got = gpu_hypot(ab)
    ref = oracle_mod.hypot(ab[:, 0], ab[:, 1])
    assert np.array_equal(got, ref)


def test_hyperboloid_known_and_random(cuda_lib_path, oracle_mod):
    ver = np.array([100.0, 200.0, 300.0])
    pts = np.array([(118, 176, 294), (75, 260, 275), (118, 176, 293), (75, 260, 274), (118, 176, 295),
                    (75, 260, 276)], dtype=np.float64)
    assert gpu_hyp(ver, 72.0, 1.0, pts).tolist() == [1, 1, 1, 1, 0, 0]
    rng = np.random.default_rng(5)
    m = 200_000
    xyz = ver + np.stack([rng.normal(0, 5, m), rng.normal(0, 5, m), rng.uniform(-20, 2, m)], 1)
    got = gpu_hyp(ver, 0.37, 1.0, xyz)
    L = oracle_mod.lib()
    ref = np.array([L.wbo_hyperboloid_in(ver.ctypes.data, 0.37, 1.0, np.ascontiguousarray(p).ctypes.data)
                    for p in xyz[:20000]], dtype=np.uint8)
    assert np.array_equal(got[:20000], ref)


@pytest.mark.parametrize("scale", [(0.001, 0.001), (0.01, 0.01), (0.00025, 0.0005)])
def test_fp32_direction_within_margin(cuda_lib_path, scale):
    """The classify filter's FP32 direction stays within 1000 angle units
    (2^31 per turn) of the reference's atan2i; the filter allows 2048."""
    rng = np.random.default_rng(7)
    m = 400_000
    d = rng.integers(-(1 << 20), 1 << 20, size=(m, 2)).astype(np.int32)
    small = rng.integers(-40, 41, size=(50_000, 2)).astype(np.int32)
    axes = np.array([[k, 0] for k in range(1, 200)] + [[0, k] for k in range(1, 200)] +
                    [[-k, 0] for k in range(1, 200)] + [[0, -k] for k in range(1, 200)] +
                    [[k, k] for k in range(1, 200)] + [[k, -k] for k in range(1, 200)] +
                    [[-k, k + 1] for k in range(1, 200)], np.int32)
    d = np.concatenate([d, small, axes])
    d = d[(d[:, 0] != 0) | (d[:, 1] != 0)]
    d = np.ascontiguousarray(d)
    out = np.zeros(d.shape[0], np.uint32)
    assert _lib().wb_check_dir_f32(d.ctypes.data, scale[0], scale[1], d.shape[0], out.ctypes.data) == 0
    yx = np.stack([d[:, 1] * scale[1], d[:, 0] * scale[0]], axis=1)
    ref = gpu_atan2i(yx).astype(np.int64) & 0x7fffffff
    diff = (out.astype(np.int64) - ref) & 0x7fffffff
    err = np.minimum(diff, (1 << 31) - diff)
    assert err.max() < 1000, int(err.max())
