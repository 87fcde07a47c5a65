"""Pins the CPU restatement (oracle/) to the reference's own outputs.

The golden files were written by the reference's sources compiled unchanged
(tests/golden/make_golden.py).  Every comparison here is exact.
"""
import os
import platform
import re

import numpy as np
import pytest

from conftest import GOLDEN_CASES, ROOT, golden_cloud, golden_params, load_golden


@pytest.fixture(scope="module")
def prim():
    return load_golden("primitives")


@pytest.mark.skipif(platform.machine() != "x86_64", reason="golden tables come from x86-64 long double")
def test_oracle_fill_tables_match_reference(oracle_mod, prim):
    t, s, c = oracle_mod.fill_tables()
    assert np.array_equal(t, prim["tan"])
    assert np.array_equal(s, prim["sin"])
    assert np.array_equal(c, prim["cos"])


def _header_tables():
    text = open(os.path.join(ROOT, "wolkenbase_gb300", "csrc", "angle_tables.h")).read()
    out = {}
    for name in ("kWbTan", "kWbSin", "kWbCos", "kWbQuadrantCosSin"):
        body = re.search(name + r"\[\d+\] = \{(.*?)\};", text, re.S).group(1)
        out[name] = np.array([float.fromhex(v.strip()) for v in body.split(",") if v.strip()])
    return out


def test_product_tables_match_reference(prim):
    """The GPU library's generated tables equal the reference's fillTanTables output."""
    h = _header_tables()
    assert np.array_equal(h["kWbTan"], prim["tan"])
    assert np.array_equal(h["kWbSin"], prim["sin"])
    assert np.array_equal(h["kWbCos"], prim["cos"])
    assert np.array_equal(h["kWbQuadrantCosSin"], prim["quadrant"])


def test_atan2i_matches_reference(oracle_mod, prim):
    oracle_mod.set_tables(prim["tan"], prim["sin"], prim["cos"])
    yx = prim["atan_yx"]
    got = oracle_mod.atan2i(yx[:, 0], yx[:, 1])
    assert np.array_equal(got, prim["atan_out"])
    assert oracle_mod.lib().wbo_atan2i(0.0, 0.0) == 0   # atan2i(0,0)=0 (wolkentest.cpp:140)


def test_flowsnake_matches_reference(oracle_mod, prim):
    import ctypes as C
    for idx in range(6):
        ref = prim[f"flowsnake{idx}"]
        out = np.zeros(ref.shape, np.int32)
        oracle_mod.lib().wbo_flowsnake(idx, out.ctypes.data)
        assert np.array_equal(out, ref), idx
        lo, hi = C.c_int32(), C.c_int32()
        oracle_mod.lib().wbo_flowsnake_limits(idx, C.byref(lo), C.byref(hi))
        assert hi.value - lo.value + 1 == 7 ** idx


def test_lsq_matches_reference(oracle_mod, prim):
    pts = prim["lsq_pts"]
    off = 0
    for k, n in enumerate(prim["lsq_len"]):
        sys_ = np.ascontiguousarray(pts[off:off + n])
        off += n
        out = np.zeros(3)
        oracle_mod.lib().wbo_lsq_plane(sys_.ctypes.data, n, out.ctypes.data)
        assert np.array_equal(out, prim["lsq_sol"][k]), k
        if k % 10 == 0:   # exact planes come back to rounding
            assert np.allclose(out, [0.3, -0.7, 2.0], atol=1e-9)


def test_pairwisesum_known_answers(oracle_mod):
    """pairwisesum(odd, i) == i*i for the first 32 odd numbers (wolkentest.cpp:600-616)."""
    odd = np.array([2 * i + 1 for i in range(32)], dtype=np.float64)
    for i in range(32):
        assert oracle_mod.lib().wbo_pairwisesum(odd.ctypes.data, i) == i * i


def test_hyperboloid_known_points(oracle_mod):
    """Integer-exact points on and off Hyperboloid(ver,72,1) and (ver,97,2) (wolkentest.cpp:223-246)."""
    L = oracle_mod.lib()
    ver = np.array([100.0, 200.0, 300.0])
    ins = [(118, 176, 294), (75, 260, 275), (118, 176, 293), (75, 260, 274)]
    outs = [(118, 176, 295), (75, 260, 276)]
    for p in ins:
        assert L.wbo_hyperboloid_in(ver.ctypes.data, 72.0, 1.0, np.array(p, float).ctypes.data)
    for p in outs:
        assert not L.wbo_hyperboloid_in(ver.ctypes.data, 72.0, 1.0, np.array(p, float).ctypes.data)


def test_cylinder_known_points(oracle_mod):
    """Cylinder((0,0),13) membership (wolkentest.cpp:265-279)."""
    L = oracle_mod.lib()
    c = np.array([0.0, 0.0])
    for p, exp in [((0, 0, 13), True), ((5, 12, 0), True), ((5, 13, 4), False), ((-9, -9, -3), True),
                   ((-11, -7, 2), False)]:
        assert bool(L.wbo_cylinder_in(c.ctypes.data, 13.0, np.array(p, float).ctypes.data)) == exp


@pytest.mark.parametrize("case", GOLDEN_CASES + ["negscale8k"])
def test_pipeline_matches_reference(oracle_mod, prim, case):
    """Serial block numbers, storage order, leaf cubes, tiles and classes,
    exactly (negscale8k: x and z read through negative scales)."""
    oracle_mod.set_tables(prim["tan"], prim["sin"], prim["cos"])
    g = load_golden(case)
    cloud = golden_cloud(g)
    r = oracle_mod.run(cloud, phases=int(g["phases"]), threads=4, **golden_params(g))
    assert r["n_blocks"] == int(g["n_blocks"])
    assert np.array_equal(r["block"], g["block"].astype(np.int64))
    assert np.array_equal(r["pos"], g["pos"])
    stored = r["leaf"] >= 0
    assert np.array_equal(stored, g["block"] >= 0)
    assert np.array_equal(r["leaves"][r["leaf"][stored]], g["leaf_cube"][stored])
    assert np.array_equal(np.array(list(r["root_center"]) + [r["root_side"]]), g["root"])
    assert np.array_equal(np.array(list(r["snake_center"]) + [r["snake_side"], r["spacing"]]), g["snake"])
    if int(g["phases"]) >= 2:
        for f in ("ex", "ey", "n_points", "n_ground", "tree_flags", "density", "h_scan", "h_final", "height"):
            assert np.array_equal(r["tiles"][f], g["tiles"][f]), f
    if int(g["phases"]) >= 3:
        assert np.array_equal(r["cls"], g["cls"])


def test_leaf_structure_is_insertion_order_free(oracle_mod):
    """Leaf cubes per point do not depend on the input order (only block numbers do)."""
    from wolkenbase_gb300 import synth
    c = synth.density_tile(12000, 3)
    a = oracle_mod.run(c, phases=1)
    perm = np.random.default_rng(5).permutation(c.n)
    c2 = synth.Cloud(c.xyz[perm], c.scale, c.offset, c.unit, c.minc, c.maxc)
    b = oracle_mod.run(c2, phases=1)
    cubes_a = a["leaves"][a["leaf"]]
    cubes_b = np.empty_like(cubes_a)
    cubes_b[perm] = b["leaves"][b["leaf"]]
    assert np.array_equal(cubes_a, cubes_b)
    assert a["n_leaves"] == b["n_leaves"]
