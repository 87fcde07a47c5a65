"""ctypes wrapper for the CPU restatement (oracle/_build/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline arm of bench.py as the checker.  The product package never
imports this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_BIN = os.path.join(HERE, "_ref", "wb_ref")


class Params(C.Structure):
    _fields_ = [("tile_size", C.c_double), ("max_slope", C.c_double),
                ("thickness", C.c_double), ("min_hyp_size", C.c_double)]


class RunIO(C.Structure):
    _fields_ = [("xyz", C.POINTER(C.c_int32)), ("n", C.c_uint64),
                ("scale", C.c_double * 3), ("offset", C.c_double * 3), ("unit", C.c_double),
                ("minc", C.c_double * 3), ("maxc", C.c_double * 3),
                ("phases", C.c_int), ("canonical_order", C.c_int), ("threads", C.c_int),
                ("block", C.POINTER(C.c_int64)), ("block_pos", C.POINTER(C.c_int32)),
                ("leaf", C.POINTER(C.c_int64)), ("cls", C.POINTER(C.c_uint8)),
                ("n_blocks", C.c_uint64), ("n_leaves", C.c_uint64), ("n_tiles", C.c_uint64),
                ("root_center", C.c_double * 3), ("root_side", C.c_double),
                ("snake_center", C.c_double * 3), ("snake_side", C.c_double), ("spacing", C.c_double),
                ("snake_index", C.c_int),
                ("t_build", C.c_double), ("t_scan", C.c_double), ("t_postscan", C.c_double),
                ("t_classify", C.c_double), ("sample_tiles", C.POINTER(C.c_int64)), ("n_sample", C.c_uint64),
                ("n_scanned", C.c_uint64), ("n_sample_points", C.c_uint64), ("margin", C.POINTER(C.c_double))]


TILE_DTYPE = np.dtype([("ex", "<i4"), ("ey", "<i4"), ("n_points", "<i4"), ("n_ground", "<i4"),
                       ("tree_flags", "<i4"), ("pad", "<i4"), ("density", "<f8"), ("h_scan", "<f8"),
                       ("h_final", "<f8"), ("height", "<f8")])


def build():
    subprocess.run(["make", "-C", HERE, "oracle"], check=True, stdout=subprocess.DEVNULL)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.wbo_run.argtypes = [C.POINTER(RunIO), C.POINTER(Params)]
        L.wbo_leaves.argtypes = [C.c_void_p, C.c_void_p]
        L.wbo_tiles.argtypes = [C.c_void_p]
        L.wbo_fill_tables.argtypes = [C.c_void_p] * 3
        L.wbo_set_tables.argtypes = [C.c_void_p] * 3
        L.wbo_atan2i.argtypes = [C.c_double, C.c_double]
        L.wbo_atan2i.restype = C.c_int32
        L.wbo_atan2i_many.argtypes = [C.c_void_p, C.c_uint64, C.c_void_p]
        L.wbo_quadrant_trig.argtypes = [C.c_void_p]
        L.wbo_pairwisesum.argtypes = [C.c_void_p, C.c_uint]
        L.wbo_pairwisesum.restype = C.c_double
        L.wbo_hypot_many.argtypes = [C.c_void_p, C.c_uint64, C.c_void_p]
        L.wbo_lsq_plane.argtypes = [C.c_void_p, C.c_uint64, C.c_void_p]
        L.wbo_hyperboloid_in.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_void_p]
        L.wbo_cylinder_in.argtypes = [C.c_void_p, C.c_double, C.c_void_p]
        L.wbo_size_fit.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.wbo_flowsnake.argtypes = [C.c_int, C.c_void_p]
        L.wbo_flowsnake_limits.argtypes = [C.c_int, C.c_void_p, C.c_void_p]
        L.wbo_sample.argtypes = [C.c_void_p, C.c_uint64, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                 C.c_void_p]
        L.wbo_points_in.argtypes = [C.c_int, C.c_void_p, C.c_double, C.c_double, C.c_int, C.c_void_p, C.c_uint64]
        L.wbo_points_in.restype = C.c_int64
        L.wbo_find_blocks.argtypes = [C.c_int, C.c_void_p, C.c_double, C.c_double, C.c_void_p, C.c_uint64]
        L.wbo_find_blocks.restype = C.c_int64
        L.wbo_snake_tiles.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_double]
        L.wbo_snake_tiles.restype = C.c_int64
        _lib = L
        # The reference's atan2i tables come from x86-64 80-bit long double;
        # hosts with another long double (aarch64: 128-bit) would round a few
        # entries differently, so the oracle uses the pinned values.
        golden = os.path.join(os.path.dirname(HERE), "tests", "golden", "primitives.npz")
        if os.path.exists(golden):
            g = np.load(golden)
            set_tables(g["tan"], g["sin"], g["cos"])
    return _lib


def _ptr(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


def run(cloud, *, tile_size=1.0, max_slope=1.0, thickness=0.0, min_hyp_size=0.1,
        phases=3, canonical_order=False, threads=1, sample_tiles=None, want_leaves=True, keep=False,
        margins=False):
    """Runs the restated pipeline; returns a dict of numpy arrays and scalars.

    sample_tiles: positions in flowsnake order of the only tiles to post-scan
    and classify (the tiles their postscan reads are scanned on demand); cls is
    then written only for the points those tiles decide (their last
    containing tile in flowsnake order), 0 elsewhere.  keep: the octree stays
    for sample() calls until reset()."""
    L = lib()
    xyz = np.ascontiguousarray(cloud.xyz, dtype=np.int32)
    n = xyz.shape[0]
    block = np.full(n, -1, np.int64)
    pos = np.full(n, -1, np.int32)
    leaf = np.full(n, -1, np.int64)
    cls = np.zeros(n, np.uint8)
    io = RunIO()
    io.xyz = _ptr(xyz, C.c_int32)
    io.n = n
    io.scale[:] = cloud.scale
    io.offset[:] = cloud.offset
    io.unit = cloud.unit
    io.minc[:] = cloud.minc
    io.maxc[:] = cloud.maxc
    io.phases = phases
    io.canonical_order = int(canonical_order)
    io.threads = threads
    io.block = _ptr(block, C.c_int64)
    io.block_pos = _ptr(pos, C.c_int32)
    io.leaf = _ptr(leaf, C.c_int64)
    io.cls = _ptr(cls, C.c_uint8)
    margin = None
    if margins:
        margin = np.zeros(n, np.float64)
        io.margin = _ptr(margin, C.c_double)
    if sample_tiles is not None:
        smp = np.ascontiguousarray(sample_tiles, dtype=np.int64)
        io.sample_tiles = _ptr(smp, C.c_int64)
        io.n_sample = smp.shape[0]
    prm = Params(tile_size, max_slope, thickness, min_hyp_size)
    rc = L.wbo_run(C.byref(io), C.byref(prm))
    if rc != 0:
        raise RuntimeError(f"wbo_run failed: {rc}")
    nl = io.n_leaves
    leaves = np.zeros((nl, 4))
    counts = np.zeros(nl, np.int64)
    if want_leaves:
        L.wbo_leaves(leaves.ctypes.data, counts.ctypes.data)
    tiles = np.zeros(io.n_tiles, TILE_DTYPE)
    if phases >= 2:
        L.wbo_tiles(tiles.ctypes.data)
    out = dict(block=block, pos=pos, leaf=leaf, cls=cls, leaves=leaves, leaf_count=counts, tiles=tiles,
               n_blocks=io.n_blocks, n_leaves=nl, n_tiles=io.n_tiles,
               root_center=tuple(io.root_center), root_side=io.root_side,
               snake_center=tuple(io.snake_center), snake_side=io.snake_side, spacing=io.spacing,
               snake_index=io.snake_index,
               t_build=io.t_build, t_scan=io.t_scan, t_postscan=io.t_postscan, t_classify=io.t_classify,
               n_scanned=io.n_scanned, n_sample_points=io.n_sample_points, margin=margin)
    if not keep:
        L.wbo_reset()
    return out


def sample(tiles, n_points, threads=1):
    """Another sampled scan + classify over the octree a run(keep=True) left:
    class bytes of the points the sampled tiles decide (0 elsewhere), the
    tiles' fields, and the times."""
    L = lib()
    smp = np.ascontiguousarray(tiles, dtype=np.int64)
    cls = np.zeros(n_points, np.uint8)
    ts, tc = C.c_double(0), C.c_double(0)
    ns, npt = C.c_uint64(0), C.c_uint64(0)
    rc = L.wbo_sample(smp.ctypes.data, smp.shape[0], threads, cls.ctypes.data, C.byref(ts), C.byref(tc),
                      C.byref(ns), C.byref(npt))
    if rc != 0:
        raise RuntimeError("wbo_sample: no octree kept (run(keep=True) first)")
    return dict(cls=cls, t_scan=ts.value, t_classify=tc.value, n_scanned=ns.value, n_sample_points=npt.value)


def sample_tiles_fields(n_tiles):
    """The tile table after the last sample() (fields of tiles it did not scan are zero)."""
    tiles = np.zeros(n_tiles, TILE_DTYPE)
    lib().wbo_tiles(tiles.ctypes.data)
    return tiles


def points_in(kind, v, r, s=1.0, sorted=False):
    """OctStore::pointsIn over the octree a run(keep=True) left (input indices)."""
    L = lib()
    vv = np.ascontiguousarray(list(v) + [0.0] * (3 - len(v)), np.float64)
    n = L.wbo_points_in(kind, vv.ctypes.data, r, s, int(sorted), None, 0)
    out = np.zeros(max(n, 0), np.uint32)
    L.wbo_points_in(kind, vv.ctypes.data, r, s, int(sorted), out.ctypes.data, out.shape[0])
    return out


def find_blocks(kind, v, r, s=1.0):
    """Octree::findBlocks over the octree a run(keep=True) left (depth-first leaf indices)."""
    L = lib()
    vv = np.ascontiguousarray(list(v) + [0.0] * (3 - len(v)), np.float64)
    n = L.wbo_find_blocks(kind, vv.ctypes.data, r, s, None, 0)
    out = np.zeros(max(n, 0), np.int64)
    L.wbo_find_blocks(kind, vv.ctypes.data, r, s, out.ctypes.data, out.shape[0])
    return out


def reset():
    lib().wbo_reset()


def snake_tiles(cloud, tile_size=1.0):
    """Tiles of the flowsnake island the reference sizes for this cloud."""
    mn = np.ascontiguousarray(cloud.minc, np.float64)
    mx = np.ascontiguousarray(cloud.maxc, np.float64)
    return int(lib().wbo_snake_tiles(mn.ctypes.data, mx.ctypes.data, float(cloud.unit), float(tile_size)))


def atan2i(y, x):
    L = lib()
    yx = np.ascontiguousarray(np.stack([np.asarray(y, np.float64), np.asarray(x, np.float64)], axis=1))
    out = np.zeros(yx.shape[0], np.int32)
    L.wbo_atan2i_many(yx.ctypes.data, yx.shape[0], out.ctypes.data)
    return out


def hypot(a, b):
    ab = np.ascontiguousarray(np.stack([np.asarray(a, np.float64), np.asarray(b, np.float64)], axis=1))
    out = np.zeros(ab.shape[0])
    lib().wbo_hypot_many(ab.ctypes.data, ab.shape[0], out.ctypes.data)
    return out


def fill_tables():
    t = np.zeros(511)
    s = np.zeros(512)
    c = np.zeros(512)
    lib().wbo_fill_tables(t.ctypes.data, s.ctypes.data, c.ctypes.data)
    return t, s, c


def set_tables(t, s, c):
    t = np.ascontiguousarray(t, np.float64)
    s = np.ascontiguousarray(s, np.float64)
    c = np.ascontiguousarray(c, np.float64)
    lib().wbo_set_tables(t.ctypes.data, s.ctypes.data, c.ctypes.data)


def read_ref_output(path):
    """Parses the binary written by ``wb_ref pipeline`` (oracle/ref_driver.cpp)."""
    import struct
    d = open(path, "rb").read()
    n, nb, nt = struct.unpack_from("<3Q", d, 0)
    off = 24
    geo = np.frombuffer(d, "<f8", 8, off).copy(); off += 64
    (sp,) = struct.unpack_from("<d", d, off); off += 8
    blk = np.frombuffer(d, "<i8", n, off).copy(); off += 8 * n
    pos = np.frombuffer(d, "<i4", n, off).copy(); off += 4 * n
    cls = np.frombuffer(d, "u1", n, off).copy(); off += n
    leaf = np.frombuffer(d, "<f8", 4 * n, off).reshape(n, 4).copy(); off += 32 * n
    rec = np.dtype([("ex", "<i4"), ("ey", "<i4"), ("n_points", "<i4"), ("n_ground", "<i4"),
                    ("tree_flags", "<i4"), ("pad", "<i4"), ("density", "<f8"), ("h_scan", "<f8"),
                    ("h_final", "<f8"), ("height", "<f8")])
    tiles = np.frombuffer(d, rec, nt, off).copy()
    return dict(n=n, n_blocks=nb, n_tiles=nt, root_center=tuple(geo[:3]), root_side=geo[3],
                snake_center=tuple(geo[4:7]), snake_side=geo[7], spacing=sp,
                block=blk, pos=pos, cls=cls, leaf_cube=leaf, tiles=tiles)


def run_reference(cloud, workdir, *, tile_size=1.0, max_slope=1.0, thickness=0.0, min_hyp_size=0.1,
                  phases=3, timeout=3600):
    """Runs the reference's own sources (oracle/_ref/wb_ref) on ``cloud``."""
    from wolkenbase_gb300 import synth
    inp = os.path.join(workdir, "in.wbxyz")
    out = os.path.join(workdir, "ref.out")
    synth.write_wbxyz(inp, cloud)
    r = subprocess.run([REF_BIN, "pipeline", inp, out, repr(tile_size), repr(max_slope), repr(thickness),
                        repr(min_hyp_size), str(phases)], capture_output=True, text=True, timeout=timeout,
                       check=True)
    res = read_ref_output(out)
    import json
    res["timing"] = json.loads(r.stdout.strip().splitlines()[-1])
    return res
