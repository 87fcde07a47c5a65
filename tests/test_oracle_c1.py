"""The oracle against the reference's own serial run on the 1M-point workload.

tests/golden/c1_ref.npz holds what oracle/_ref/wb_ref (the reference's
sources, serial insertion in input order, every tile scanned, post-scanned
and classified in flowsnake order) produced on 1,000,000 points over
100 x 100 m (1 mm, seed 1).  The oracle, with each block's points in input
order, must give the same leaf cube for every point and the same points per
tile, and at least 99.99% of the same class bytes (the serial insertion order
inside a block feeds scanCylinder's second-lowest point, scan.cpp:79-83).
"""
import hashlib
import os

import numpy as np
import pytest

from conftest import GOLDEN

LABEL_TOL = 1e-4


def test_oracle_matches_reference_on_1m_points(oracle_mod):
    from wolkenbase_gb300 import synth
    path = os.path.join(GOLDEN, "c1_ref.npz")
    g = np.load(path)
    cloud = synth.plain_small(seed=1)
    digest = hashlib.sha256(np.ascontiguousarray(cloud.xyz, dtype="<i4").tobytes()).hexdigest()
    if digest != str(g["xyz_sha256"]):
        pytest.fail("the generator gave another cloud than the one the reference ran")
    o = oracle_mod.run(cloud, canonical_order=True, threads=max(1, os.cpu_count() or 1))
    stored = o["leaf"] >= 0
    assert np.array_equal(np.unpackbits(g["stored_bits"])[:cloud.n].astype(bool), stored)
    cubes = np.where(stored[:, None], o["leaves"][np.maximum(o["leaf"], 0)], 0.0)
    assert hashlib.sha256(np.ascontiguousarray(cubes, dtype="<f8").tobytes()).hexdigest() == \
        str(g["point_cube_sha256"])
    assert np.array_equal(np.unique(o["leaves"], axis=0), g["leaf_cube"])
    assert np.array_equal(o["tiles"]["n_points"], g["tile_n"])
    assert np.array_equal(o["tiles"]["tree_flags"], g["tile_flags"].astype(np.int32))
    ref_set = np.unpackbits(g["cls_set_bits"])[:cloud.n].astype(bool)
    ref_ground = np.unpackbits(g["cls_bits"])[:cloud.n].astype(bool)
    ref_cls = np.where(ref_set, np.where(ref_ground, 2, 1), 0).astype(np.uint8)
    diff = int(np.sum((o["cls"] != ref_cls) & stored))
    assert diff <= LABEL_TOL * cloud.n, f"{diff} labels differ from the reference's serial run"
