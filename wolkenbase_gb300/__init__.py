"""wolkenbase_gb300: wolkenbase's ground-classification hot path on one GB300.

The compute lives in libwolkenbase_gb300.so (hand-written sm_103a CUDA behind
the C ABI of include/wolkenbase_gb300.h).  This module is the Python host
mirror of the reference's interface for that path:

  reference (phma/wolkenbase)                     here
  ---------------------------------------------   ------------------------------
  octRoot.sizeFit + octStore.put (octree.cpp)     Classifier.build(cloud)
  Octree::findBlock / findCube (octree.cpp:199)   Classifier.find_block(xyz)
  OctStore::getNumBlocks / getAll                 Classifier.leaves(), store_order()
  scanCylinder + postscanCylinder (scan.cpp)      Classifier.scan(params)
  classifyCylinder (classify.cpp:96)              Classifier.classify(params, cls)
  Tile (tile.h:27-35)                             Classifier.tiles()
  WolkenCanvas::startProcess per cloud, many      Server.submit / result, classify_batch

Errors raise WolkenbaseError carrying the C status code.
"""
from __future__ import annotations

import ctypes as C
import dataclasses

import numpy as np

from . import _lib
from ._lib import wb_cloud, wb_octree_stats, wb_params, wb_tile

__all__ = ["Params", "Classifier", "Server", "WolkenbaseError", "cloud_struct", "LasOutput", "las_point_length",
           "join_point_format", "combine_scales", "las_header_bytes", "las_file_name"]


class WolkenbaseError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{_lib.ERROR_NAMES.get(code, code)}: {msg}")
        self.code = code


@dataclasses.dataclass
class Params:
    """Classification settings with the reference's defaults (mainwindow.cpp:407-410)."""
    tile_size: float = 1.0
    max_slope: float = 1.0
    thickness: float = 0.0
    min_hyp_size: float = 0.1

    def c(self):
        return wb_params(self.tile_size, self.max_slope, self.thickness, self.min_hyp_size)


TILE_DTYPE = np.dtype([("ex", "<i4"), ("ey", "<i4"), ("n_points", "<i4"), ("n_ground", "<i4"),
                       ("tree_flags", "<i4"), ("pad", "<i4"), ("density", "<f8"), ("h_scan", "<f8"),
                       ("hyperboloid_size", "<f8"), ("height", "<f8")])


def cloud_struct(records, n, stride, scale, offset, unit, minc, maxc, device_resident=False):
    """Builds a wb_cloud for a host array (numpy) or a device pointer (int)."""
    cs = wb_cloud()
    if isinstance(records, np.ndarray):
        cs.records = records.ctypes.data
    else:
        cs.records = int(records)
    cs.n = n
    cs.stride = stride
    cs.device_resident = 1 if device_resident else 0
    cs.scale[:] = scale
    cs.offset[:] = offset
    cs.unit = unit
    cs.minc[:] = minc
    cs.maxc[:] = maxc
    return cs


class Classifier:
    """One device context: octree, point store and tile table of one cloud."""

    def __init__(self, device=0, hbm_budget=0):
        self.L = _lib.load()
        self.ctx = self.L.wb_open(device, hbm_budget)
        if not self.ctx:
            raise WolkenbaseError(_lib.WB_ECUDA, self.L.wb_last_error(None).decode())
        self._keep = None

    def close(self):
        if self.ctx:
            self.L.wb_close(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != 0:
            raise WolkenbaseError(rc, self.L.wb_last_error(self.ctx).decode())

    # -- octree / point store --
    def build(self, cloud):
        """Octree::sizeFit + OctStore::put of every point of a synth.Cloud-like object."""
        xyz = np.ascontiguousarray(cloud.xyz, dtype=np.int32)
        self._keep = xyz
        cs = cloud_struct(xyz, xyz.shape[0], 12, cloud.scale, cloud.offset, cloud.unit, cloud.minc, cloud.maxc)
        self._check(self.L.wb_octree_build(self.ctx, C.byref(cs)))
        self.synchronize()

    def build_records(self, cs):
        self._check(self.L.wb_octree_build(self.ctx, C.byref(cs)))

    def synchronize(self):
        self._check(self.L.wb_synchronize(self.ctx))

    def set_stream(self, stream_handle):
        self._check(self.L.wb_set_stream(self.ctx, C.c_void_p(stream_handle)))

    def info(self):
        s = wb_octree_stats()
        self._check(self.L.wb_octree_info(self.ctx, C.byref(s)))
        return {f: (tuple(getattr(s, f)) if f in ("root_center", "tile_center") else getattr(s, f))
                for f, _ in s._fields_ if f != "pad"}

    def leaves(self):
        """(center_side (L,4) float64, first (L,) uint32, count (L,) uint32), depth-first order."""
        L = self.info()["n_leaves"]
        cs = np.zeros((L, 4))
        first = np.zeros(L, np.uint32)
        count = np.zeros(L, np.uint32)
        self._check(self.L.wb_octree_leaves(self.ctx, cs.ctypes.data, first.ctypes.data, count.ctypes.data))
        return cs, first, count

    def point_leaf(self):
        n = self.info()["n_points"]
        out = np.zeros(n, np.uint32)
        self._check(self.L.wb_octree_point_leaf(self.ctx, out.ctypes.data))
        return out

    def store_order(self):
        nd = self.info()["n_distinct"]
        out = np.zeros(nd, np.uint32)
        self._check(self.L.wb_octree_store_order(self.ctx, out.ctypes.data))
        return out

    def find_block(self, xyz):
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        out = np.zeros(xyz.shape[0], np.int64)
        self._check(self.L.wb_octree_find_block(self.ctx, xyz.ctypes.data, xyz.shape[0], out.ctypes.data))
        return out

    @staticmethod
    def _shape(kind, v, r, s):
        sh = _lib.wb_shape()
        sh.kind = int(kind)
        vv = list(v) + [0.0] * (3 - len(v))
        sh.v[:] = vv[:3]
        sh.r = float(r)
        sh.s = float(s)
        return sh

    def find_blocks(self, kind, v, r, s=1.0):
        """Octree::findBlocks of a Cylinder (kind WB_SHAPE_CYLINDER: v = centre xy,
        r = radius) or a Hyperboloid (WB_SHAPE_HYPERBOLOID: vertex v, r, slope s):
        depth-first leaf indices."""
        sh = self._shape(kind, v, r, s)
        n = C.c_uint64(0)
        rc = self.L.wb_find_blocks(self.ctx, C.byref(sh), None, 0, C.byref(n))
        if rc not in (0, _lib.WB_EINVAL) or (rc == _lib.WB_EINVAL and n.value == 0):
            self._check(rc)
        out = np.zeros(n.value, np.int64)
        self._check(self.L.wb_find_blocks(self.ctx, C.byref(sh), out.ctypes.data, out.shape[0], C.byref(n)))
        return out

    def points_in(self, kind, v, r, s=1.0, sorted=False):
        """OctStore::pointsIn of a Cylinder or a Hyperboloid (see find_blocks):
        input record indices, blocks depth-first, store order inside a block,
        or by height when sorted."""
        sh = self._shape(kind, v, r, s)
        n = C.c_uint64(0)
        rc = self.L.wb_points_in(self.ctx, C.byref(sh), int(sorted), None, 0, C.byref(n))
        if rc not in (0, _lib.WB_EINVAL) or (rc == _lib.WB_EINVAL and n.value == 0):
            self._check(rc)
        out = np.zeros(n.value, np.uint32)
        self._check(self.L.wb_points_in(self.ctx, C.byref(sh), int(sorted), out.ctypes.data, out.shape[0],
                                        C.byref(n)))
        return out

    # -- tiles --
    def scan(self, params=None):
        p = (params or Params()).c()
        self._check(self.L.wb_scan_tiles(self.ctx, C.byref(p)))
        self.synchronize()

    def tiles(self):
        cnt = C.c_uint64(0)
        self._check(self.L.wb_tiles(self.ctx, None, 0, C.byref(cnt)))
        out = np.zeros(cnt.value, TILE_DTYPE)
        self._check(self.L.wb_tiles(self.ctx, out.ctypes.data, cnt.value, C.byref(cnt)))
        return out

    def classify(self, params=None, cls=None):
        n = self.info()["n_points"]
        if cls is None:
            cls = np.zeros(n, np.uint8)
        cls = np.ascontiguousarray(cls, dtype=np.uint8)
        p = (params or Params()).c()
        self._check(self.L.wb_classify(self.ctx, C.byref(p), cls.ctypes.data, 0))
        return cls

    def classify_margins(self, params=None, cls=None):
        """classify() plus every record's decision margin in degrees (largest
        direction gap minus 144; negative = not ground, NaN = in no tile)."""
        n = self.info()["n_points"]
        if cls is None:
            cls = np.zeros(n, np.uint8)
        cls = np.ascontiguousarray(cls, dtype=np.uint8)
        margin = np.zeros(n, np.float32)
        p = (params or Params()).c()
        self._check(self.L.wb_classify_ex(self.ctx, C.byref(p), cls.ctypes.data, 0, margin.ctypes.data))
        return cls, margin

    def classify_cloud(self, cloud, params=None, cls=None):
        """Build + scan + postscan + classify in one C call (host in, host out)."""
        xyz = np.ascontiguousarray(cloud.xyz, dtype=np.int32)
        cs = cloud_struct(xyz, xyz.shape[0], 12, cloud.scale, cloud.offset, cloud.unit, cloud.minc, cloud.maxc)
        if cls is None:
            cls = np.zeros(xyz.shape[0], np.uint8)
        p = (params or Params()).c()
        self._check(self.L.wb_classify_cloud(self.ctx, C.byref(cs), C.byref(p), cls.ctypes.data))
        return cls

    def planes(self):
        """(T, 3) least-squares planes of the last scan (z = a*x + b*y + c from the tile centre)."""
        T = self.info()["n_tiles"]
        out = np.zeros((T, 3))
        self._check(self.L.wb_tile_planes(self.ctx, out.ctypes.data, T))
        return out

    def residuals(self, ref_planes):
        """Per tile, max |r - r_ref| and max |r_ref| of the points' fit residuals
        r = z - (a*x + b*y + c) under the last scan's planes and under ref_planes."""
        ref = np.ascontiguousarray(ref_planes, dtype=np.float64)
        T = self.info()["n_tiles"]
        if ref.shape != (T, 3):
            raise ValueError("ref_planes must be (n_tiles, 3)")
        d = np.zeros(T)
        r = np.zeros(T)
        self._check(self.L.wb_tile_residuals(self.ctx, ref.ctypes.data, d.ctypes.data, r.ctypes.data))
        return d, r

    def set_paging(self, host_budget):
        """Lets buffers beyond the HBM budget live in pinned host memory (0 turns it off)."""
        self._check(self.L.wb_set_paging(self.ctx, int(host_budget)))

    def paging_stats(self):
        h, p, d = C.c_uint64(0), C.c_uint64(0), C.c_uint64(0)
        self._check(self.L.wb_paging_stats(self.ctx, C.byref(h), C.byref(p), C.byref(d)))
        return {"host_bytes": h.value, "host_peak": p.value, "device_bytes": d.value}

    def set_precision(self, mode):
        """_lib.WB_PRECISION_EXACT (bit-exact, default) or _lib.WB_PRECISION_FP32."""
        self._check(self.L.wb_set_precision(self.ctx, int(mode)))

    # -- the steps either side of the path --
    def class_totals(self):
        """Stored points per final class byte (OctStore::countClasses summed over blocks)."""
        out = np.zeros(256, np.uint64)
        self._check(self.L.wb_class_totals(self.ctx, out.ctypes.data))
        return out

    def duplicates(self, per_record=False):
        """(records replaced by a later identical point, the kept record of every record or None)."""
        nd = C.c_uint64(0)
        out = np.zeros(self.info()["n_points"], np.uint32) if per_record else None
        self._check(self.L.wb_duplicates(self.ctx, C.byref(nd), out.ctypes.data if per_record else None))
        return nd.value, out

    def las_write_classes(self, records, point_format, cls=None):
        """Writes class bytes (default: the last classify's) into (n, stride) uint8 LAS records."""
        records = np.ascontiguousarray(records, np.uint8)
        n, stride = records.shape
        ptr = None
        if cls is not None:
            cls = np.ascontiguousarray(cls, np.uint8)
            ptr = cls.ctypes.data
        self._check(self.L.wb_las_write_classes(self.ctx, records.ctypes.data, n, stride, point_format, 0, ptr))
        return records

    def las_split_by_class(self, records, point_format):
        """(records grouped by class, input order within a class; 257 class boundaries)."""
        records = np.ascontiguousarray(records, np.uint8)
        n, stride = records.shape
        out = np.empty_like(records)
        offsets = np.zeros(257, np.uint64)
        self._check(self.L.wb_las_split_by_class(self.ctx, records.ctypes.data, n, stride, point_format, 0,
                                                 out.ctypes.data, offsets.ctypes.data))
        return out, offsets

    def preview(self, x0, y0, side, w, h):
        """Per pixel of a w x h view (pixel (i, j) centred at x0 + i*side, y0 + j*side):
        (count, lowest, highest elevation) of the stored points in its column."""
        cnt = np.zeros((h, w), np.uint64)
        lo = np.zeros((h, w))
        hi = np.zeros((h, w))
        self._check(self.L.wb_preview(self.ctx, x0, y0, side, w, h, cnt.ctypes.data, lo.ctypes.data, hi.ctypes.data))
        return cnt, lo, hi

    # -- LAS records: full decode and the class-split writer --
    def las_decode(self, records, point_format, scale, offset, unit=1.0, fields=None):
        """LasHeader::readPoint of every (n, stride) uint8 record: a dict of one
        array per LasPoint field (all fields, or those named in fields)."""
        records = np.ascontiguousarray(records, np.uint8)
        n, stride = records.shape
        cs = cloud_struct(records, n, stride, scale, offset, unit, (0, 0, 0), (0, 0, 0))
        names = [f for f, _ in _lib.LAS_POINT_FIELDS if fields is None or f in fields]
        out = {f: np.zeros(n, np.dtype(t)) for f, t in _lib.LAS_POINT_FIELDS if f in names}
        pts = _lib.wb_las_points(**{f: out[f].ctypes.data for f in names})
        self._check(self.L.wb_las_decode(self.ctx, C.byref(cs), point_format, C.byref(pts)))
        return out

    def las_write_output(self, records, in_format, scale, offset, unit, output, cls=None):
        """CloudOutput::writeFiles on the device for the built (and classified)
        cloud whose (n, stride) records are given: (records of every file back
        to back as (n_distinct, length) uint8, list of file dicts)."""
        records = np.ascontiguousarray(records, np.uint8)
        n, stride = records.shape
        cs = cloud_struct(records, n, stride, scale, offset, unit, (0, 0, 0), (0, 0, 0))
        o = output.c()
        length = self.L.wb_las_point_length(o.point_format)
        out = np.zeros((self.info()["n_distinct"], length), np.uint8)
        cptr = None
        if cls is not None:
            cls = np.ascontiguousarray(cls, np.uint8)
            cptr = cls.ctypes.data
        nf = C.c_int(0)
        rc = self.L.wb_las_write_output(self.ctx, C.byref(cs), in_format, cptr, C.byref(o), out.ctypes.data, 0,
                                        None, 0, C.byref(nf))
        files = (_lib.wb_las_file * max(1, nf.value))()
        if rc == _lib.WB_EINVAL and nf.value:
            rc = self.L.wb_las_write_output(self.ctx, C.byref(cs), in_format, cptr, C.byref(o), out.ctypes.data, 0,
                                            files, nf.value, C.byref(nf))
        self._check(rc)
        return out, [_las_file_dict(files[i]) for i in range(nf.value)], files

    def las_write_files(self, records, in_format, scale, offset, unit, output, base, cls=None, max_files=4096):
        """Writes the class files (header + records) under base; returns the file dicts with their names."""
        records = np.ascontiguousarray(records, np.uint8)
        n, stride = records.shape
        cs = cloud_struct(records, n, stride, scale, offset, unit, (0, 0, 0), (0, 0, 0))
        o = output.c()
        cptr = None
        if cls is not None:
            cls = np.ascontiguousarray(cls, np.uint8)
            cptr = cls.ctypes.data
        files = (_lib.wb_las_file * max_files)()
        nf = C.c_int(0)
        self._check(self.L.wb_las_write_files(self.ctx, C.byref(cs), in_format, cptr, C.byref(o), base.encode(),
                                              files, max_files, C.byref(nf)))
        res = []
        for i in range(nf.value):
            d = _las_file_dict(files[i])
            d["name"] = las_file_name(output, files[i], base)
            res.append(d)
        return res

    # -- kernel settings (speed only; labels do not depend on them) --
    def tuning(self):
        t = _lib.wb_tuning()
        self._check(self.L.wb_get_tuning(self.ctx, C.byref(t)))
        return {"shape": t.shape, "chunk": t.chunk, "grid_points": t.grid_points}

    def set_tuning(self, shape=-1, chunk=0, grid_points=0.0):
        t = _lib.wb_tuning(shape, chunk, grid_points)
        self._check(self.L.wb_set_tuning(self.ctx, C.byref(t)))

    def autotune(self, params=None):
        """Times the classify kernel's settings on the scanned cloud and keeps the fastest."""
        p = (params or Params()).c()
        self._check(self.L.wb_autotune(self.ctx, C.byref(p)))
        return self.tuning()

    # -- profiling --
    def profile(self, enable=True):
        self._check(self.L.wb_profile(self.ctx, 1 if enable else 0))

    def launch_count(self):
        v = C.c_uint64(0)
        self._check(self.L.wb_launch_count(self.ctx, C.byref(v)))
        return v.value

    def stage_times(self):
        cnt = C.c_uint32(0)
        names = (C.c_char_p * 64)()
        ms = (C.c_float * 64)()
        self._check(self.L.wb_stage_times(self.ctx, names, ms, 64, C.byref(cnt)))
        return [(names[i].decode(), ms[i]) for i in range(cnt.value)]


@dataclasses.dataclass
class LasOutput:
    """What CloudOutput is told before openFiles (wolkencanvas.cpp:614-622)."""
    point_format: int = 6
    separate_classes: bool = True
    n_input_files: int = 1
    points_per_file: int = 0
    unit: float = 1.0
    min_cor: tuple = (0.0, 0.0, 0.0)
    max_cor: tuple = (0.0, 0.0, 0.0)
    scale: tuple = (0.0, 0.0, 0.0)
    creation_day: int = 0
    creation_year: int = 0
    software: str = None

    def c(self):
        o = _lib.wb_las_output()
        o.point_format = self.point_format
        o.separate_classes = 1 if self.separate_classes else 0
        o.n_input_files = self.n_input_files
        o.creation_day = self.creation_day
        o.creation_year = self.creation_year
        o.points_per_file = self.points_per_file
        o.unit = self.unit
        o.min_cor[:] = self.min_cor
        o.max_cor[:] = self.max_cor
        o.scale[:] = self.scale
        o.software = self.software.encode() if self.software is not None else None
        return o


def _las_file_dict(f):
    return {"class_id": f.class_id, "index": f.index, "name_digits": f.name_digits, "point_format": f.point_format,
            "first": f.first, "n_points": list(f.n_points), "scale": tuple(f.scale), "offset": tuple(f.offset),
            "min": tuple(f.min), "max": tuple(f.max)}


def las_point_length(point_format):
    return _lib.load().wb_las_point_length(point_format)


def join_point_format(formats):
    """joinPointFormat (las.cpp:103-118)."""
    arr = (C.c_int * max(1, len(formats)))(*formats)
    return _lib.load().wb_las_join_point_format(arr, len(formats))


def combine_scales(scales, offsets):
    """combineScales (las.cpp:925-944) of n files' (scale, offset) triples in metres."""
    s = np.ascontiguousarray(scales, np.float64).reshape(-1, 3)
    o = np.ascontiguousarray(offsets, np.float64).reshape(-1, 3)
    out = np.zeros(3)
    rc = _lib.load().wb_las_combine_scales(s.ctypes.data, o.ctypes.data, s.shape[0], out.ctypes.data)
    if rc:
        raise WolkenbaseError(rc, "wb_las_combine_scales")
    return tuple(out)


def las_header_bytes(output, file):
    """LasHeader::writeHeader of one output file (a wb_las_file): 375 bytes."""
    h = np.zeros(375, np.uint8)
    rc = _lib.load().wb_las_header_bytes(C.byref(output.c()), C.byref(file), h.ctypes.data)
    if rc:
        raise WolkenbaseError(rc, "wb_las_header_bytes")
    return h


def las_file_name(output, file, base):
    buf = C.create_string_buffer(4096)
    rc = _lib.load().wb_las_file_name(C.byref(output.c()), C.byref(file), base.encode(), buf, 4096)
    if rc:
        raise WolkenbaseError(rc, "wb_las_file_name")
    return buf.value.decode()


class Server:
    """Request loop over one GPU (wb_server_open): jobs arrive with wb_submit,
    are admitted by an HBM budget, built and scanned concurrently, and
    classified together by fused launches.  Results are identical to
    Classifier.classify_cloud on the same cloud."""

    def __init__(self, device=0, prep_slots=4, hbm_budget=0, flush=_lib.WB_FLUSH_EAGER, max_batch=0,
                 shape=0, chunk=0, grid_points=0.0, autotune=False, host_budget=0):
        self.L = _lib.load()
        cfg = _lib.wb_server_config(device, prep_slots, hbm_budget, flush, max_batch, shape, chunk, grid_points,
                                    1 if autotune else 0, 0, host_budget)
        self.s = self.L.wb_server_open(C.byref(cfg))
        if not self.s:
            raise WolkenbaseError(_lib.WB_ECUDA, self.L.wb_last_error(None).decode())
        self._alive = {}   # id -> arrays the job reads or writes

    def close(self):
        if self.s:
            self.L.wb_server_close(self.s)
            self.s = None
            self._alive.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _job(self, cloud, params, cls, tag):
        xyz = np.ascontiguousarray(cloud.xyz, dtype=np.int32)
        if cls is None:
            cls = np.zeros(xyz.shape[0], np.uint8)
        cls = np.ascontiguousarray(cls, dtype=np.uint8)
        j = _lib.wb_job()
        j.cloud = cloud_struct(xyz, xyz.shape[0], 12, cloud.scale, cloud.offset, cloud.unit, cloud.minc, cloud.maxc)
        j.params = (params or Params()).c()
        j.cls = cls.ctypes.data
        j.tag = tag
        return j, xyz, cls

    def submit(self, cloud, params=None, cls=None, tag=0):
        """Queues one cloud; returns the job id.  The result lands in result(id)."""
        j, xyz, cls = self._job(cloud, params, cls, tag)
        jid = self.L.wb_submit(self.s, C.byref(j))
        if jid < 0:
            raise WolkenbaseError(jid, self.L.wb_server_error(self.s).decode())
        self._alive[jid] = (xyz, cls)
        return jid

    def poll(self, jid):
        st = _lib.wb_job_status()
        rc = self.L.wb_poll(self.s, jid, C.byref(st))
        if rc:
            raise WolkenbaseError(rc, "wb_poll")
        return _status(st)

    def wait(self, jid, timeout=-1.0):
        st = _lib.wb_job_status()
        rc = self.L.wb_wait(self.s, jid, float(timeout), C.byref(st))
        if rc == _lib.WB_ETIMEDOUT:
            return None
        if rc:
            raise WolkenbaseError(rc, "wb_wait")
        return _status(st)

    def result(self, jid):
        """Waits for the job; returns (class bytes, status) and forgets the job."""
        st = self.wait(jid)
        if st["rc"]:
            raise WolkenbaseError(st["rc"], self.L.wb_server_error(self.s).decode())
        cls = self._alive.pop(jid)[1]
        self.L.wb_release(self.s, jid)
        return cls, st

    def cancel(self, jid):
        return self.L.wb_cancel(self.s, jid)

    def stats(self):
        st = _lib.wb_server_stats()
        rc = self.L.wb_server_stats_get(self.s, C.byref(st))
        if rc:
            raise WolkenbaseError(rc, "wb_server_stats_get")
        return {f: getattr(st, f) for f, _ in st._fields_ if not f.startswith("pad")}

    def classify_batch(self, clouds, params=None):
        """wb_classify_batch over a list of clouds; returns their class bytes."""
        k = len(clouds)
        jobs = (_lib.wb_job * k)()
        keep = []
        for i, cl in enumerate(clouds):
            j, xyz, cls = self._job(cl, params, None, i)
            jobs[i] = j
            keep.append((xyz, cls))
        rcs = np.zeros(k, np.int32)
        rc = self.L.wb_classify_batch(self.s, jobs, k, rcs.ctypes.data)
        if rc:
            raise WolkenbaseError(rc, self.L.wb_server_error(self.s).decode())
        return [c for _, c in keep]


def _status(st):
    return {f: getattr(st, f) for f, _ in st._fields_ if f != "pad"}
