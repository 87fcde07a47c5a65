"""Seeded synthetic LiDAR tiles shaped like the workloads the classifier is run on.

There is no public dataset for this path, so every workload is generated here:
a ground surface made of four random sinusoids plus Gaussian noise, box
buildings whose roofs and walls carry points, and vegetation points floating
above the ground.  Coordinates are quantised to int32 exactly as a LAS file
stores them (``x = offset + scale * X``), and the header min/max are the exact
decoded extremes, which is what ``LasHeader::minCorner``/``maxCorner`` feed to
``Octree::sizeFit`` and the flowsnake sizing (wolkencanvas.cpp:497-520).

The generator uses numpy's PCG64 stream, so a (config, seed) pair gives the
same integers on every machine up to libm rounding of ``sin`` in the terrain
height; golden fixtures therefore store their integer inputs alongside the
expected outputs.
"""
from __future__ import annotations

import dataclasses
import math
import struct

import numpy as np


@dataclasses.dataclass
class Cloud:
    """A quantised point cloud plus the LAS header fields the hot path reads."""

    xyz: np.ndarray            # (n, 3) int32, LAS X/Y/Z record integers
    scale: tuple               # (sx, sy, sz)
    offset: tuple              # (ox, oy, oz)
    unit: float                # LasHeader::unit (1 for metres)
    minc: tuple                # header minX, minY, minZ (file units)
    maxc: tuple                # header maxX, maxY, maxZ (file units)
    n_ground_truth: int = 0    # how many points the generator placed on the ground
    truth: np.ndarray | None = None   # per point: 2 ground, 1 building, 3 vegetation

    @property
    def n(self) -> int:
        return int(self.xyz.shape[0])

    def decoded(self) -> np.ndarray:
        """float64 coordinates exactly as LasHeader::readPoint computes them (las.cpp:808)."""
        out = np.empty(self.xyz.shape, dtype=np.float64)
        for a in range(3):
            out[:, a] = (self.offset[a] + self.scale[a] * self.xyz[:, a].astype(np.float64)) * self.unit
        return out


def _terrain_params(rng, amp, wavelen, max_slope):
    A = rng.uniform(amp[0], amp[1], 4)
    lam = rng.uniform(wavelen[0], wavelen[1], 4)
    th = rng.uniform(0.0, 2 * math.pi, 4)
    phi = rng.uniform(0.0, 2 * math.pi, 4)
    if max_slope is not None:
        # Bound the steepest possible slope, sum_k A_k*2*pi/lambda_k, by max_slope.
        bound = float(np.sum(A * 2 * math.pi / lam))
        if bound > max_slope:
            A = A * (max_slope / bound)
    return A, lam, np.stack([np.cos(th), np.sin(th)], axis=1), phi


def _ground(x, y, params, steps):
    A, lam, d, phi = params
    z = np.zeros_like(x)
    for k in range(4):
        z += A[k] * np.sin(2 * math.pi * (x * d[k, 0] + y * d[k, 1]) / lam[k] + phi[k])
    if steps:
        # Step discontinuities: terraces of height `steps` every 40 m along x+y.
        z += steps * np.floor((x + y) / 40.0)
    return z


def _in_boxes(x, y, boxes):
    """Whether each (x, y) lies inside a building footprint (|x-cx| < hx and
    |y-cy| < hy for some box).  With many boxes the points are sorted by x
    once and each box tests only its strip (a little wider than the box, so
    the same exact test decides every point)."""
    inside = np.zeros(x.shape, dtype=bool)
    if len(boxes) <= 8 or x.size < 200_000:
        for (cx, cy, hx, hy, _roof, _h) in boxes:
            inside |= (np.abs(x - cx) < hx) & (np.abs(y - cy) < hy)
        return inside
    order = np.argsort(x)
    xs = x[order]
    for (cx, cy, hx, hy, _roof, _h) in boxes:
        pad = 1e-3 + 1e-9 * abs(cx)
        idx = order[np.searchsorted(xs, cx - hx - pad, side="left"):np.searchsorted(xs, cx + hx + pad, side="right")]
        hit = (np.abs(x[idx] - cx) < hx) & (np.abs(y[idx] - cy) < hy)
        inside[idx[hit]] = True
    return inside


def _uniform_outside(rng, n, x0, y0, sx, sy, boxes):
    xs, ys = [], []
    need = n
    while need > 0:
        m = int(need * 1.25) + 64
        x = x0 + rng.random(m) * sx
        y = y0 + rng.random(m) * sy
        keep = ~_in_boxes(x, y, boxes)
        x, y = x[keep][:need], y[keep][:need]
        xs.append(x)
        ys.append(y)
        need -= x.size
    return np.concatenate(xs), np.concatenate(ys)


def _vegetation_xy(rng, n, x0, y0, sx, sy, boxes, cover):
    """Plan positions of vegetation points: uniform inside copses (discs of
    radius 4-12 m, shrunk on small tiles) that together cover about ``cover``
    of the tile, outside building footprints.  cover=None spreads them over
    the whole tile."""
    if cover is None:
        return _uniform_outside(rng, n, x0, y0, sx, sy, boxes)
    rmax = min(12.0, 0.2 * min(sx, sy))
    rmin = min(4.0, 0.5 * rmax)
    discs = []
    area = 0.0
    while area < cover * sx * sy:
        r = rng.uniform(rmin, rmax)
        discs.append((x0 + rng.random() * sx, y0 + rng.random() * sy, r))
        area += math.pi * r * r
    d = np.array(discs)
    w = d[:, 2] ** 2
    xs, ys = [], []
    need = n
    while need > 0:
        m = int(need * 1.3) + 64
        k = rng.choice(len(d), size=m, p=w / w.sum())
        rr = d[k, 2] * np.sqrt(rng.random(m))
        th = rng.random(m) * 2 * math.pi
        x = d[k, 0] + rr * np.cos(th)
        y = d[k, 1] + rr * np.sin(th)
        keep = (x >= x0) & (x < x0 + sx) & (y >= y0) & (y < y0 + sy) & ~_in_boxes(x, y, boxes)
        x, y = x[keep][:need], y[keep][:need]
        xs.append(x)
        ys.append(y)
        need -= x.size
    return np.concatenate(xs), np.concatenate(ys)


def terrain_cloud(n, size_x, size_y, seed, *, scale=(0.001, 0.001, 0.001), offset=(0.0, 0.0, 0.0),
                  nonground=0.2, amp=(0.5, 2.0), wavelen=(20.0, 80.0), noise=0.02,
                  max_slope=None, steps=0.0, origin=(0.0, 0.0), unit=1.0, shuffle=True,
                  veg_cover=0.15, terrain_seed=None) -> Cloud:
    """One tile: ground sinusoids + noise, box buildings (3-15 m) and vegetation (0.5-10 m).

    Half of the nonground points lie on building roofs and walls (uniform by
    area), half are vegetation 0.5-10 m above ground inside copses covering
    ``veg_cover`` of the tile (None: spread over the whole tile).  Points are
    shuffled into a random order unless ``shuffle`` is false.  With
    ``terrain_seed`` the ground surface comes from that seed and the points
    from ``seed``, so tiles with one terrain seed and different origins join
    into one seamless mosaic.
    """
    rng = np.random.default_rng(seed)
    params = _terrain_params(rng if terrain_seed is None else np.random.default_rng(terrain_seed), amp, wavelen,
                             max_slope)
    x0 = origin[0] + offset[0]
    y0 = origin[1] + offset[1]
    area = size_x * size_y
    n_ng = int(round(nonground * n))
    n_box = n_ng // 2
    n_veg = n_ng - n_box
    n_gnd = n - n_ng

    nb = max(1, int(round(0.1 * area / 256.0))) if n_box > 0 else 0
    # Half-sizes 4-12 m, shrunk on small tiles so buildings never cover the tile.
    hmax = min(12.0, 0.15 * min(size_x, size_y))
    hmin = min(4.0, 0.5 * hmax)
    boxes = []
    for _ in range(nb):
        hx, hy = rng.uniform(hmin, hmax, 2)
        cx = x0 + hx + rng.random() * max(size_x - 2 * hx, 0.0)
        cy = y0 + hy + rng.random() * max(size_y - 2 * hy, 0.0)
        height = rng.uniform(3.0, 15.0)
        roof = float(_ground(np.array([cx - offset[0]]), np.array([cy - offset[1]]), params, steps)[0]) + height
        boxes.append((cx, cy, hx, hy, roof, height))

    def g(x, y):
        return _ground(x - offset[0], y - offset[1], params, steps) + offset[2]

    gx, gy = _uniform_outside(rng, n_gnd, x0, y0, size_x, size_y, boxes)
    gz = g(gx, gy) + rng.normal(0.0, noise, n_gnd)

    vx, vy = _vegetation_xy(rng, n_veg, x0, y0, size_x, size_y, boxes, veg_cover)
    vz = g(vx, vy) + rng.uniform(0.5, 10.0, n_veg)

    bx = np.empty(n_box)
    by = np.empty(n_box)
    bz = np.empty(n_box)
    if n_box:
        roof_area = np.array([4 * b[2] * b[3] for b in boxes])
        wall_h = np.array([b[5] for b in boxes])
        wall_area = np.array([4 * (b[2] + b[3]) for b in boxes]) * wall_h
        w = roof_area + wall_area
        which = rng.choice(nb, size=n_box, p=w / w.sum())
        u = rng.random(n_box)
        v = rng.random(n_box)
        t = rng.random(n_box)
        on_roof = rng.random(n_box) < (roof_area / w)[which]
        cx = np.array([b[0] for b in boxes])[which]
        cy = np.array([b[1] for b in boxes])[which]
        hx = np.array([b[2] for b in boxes])[which]
        hy = np.array([b[3] for b in boxes])[which]
        rz = np.array([b[4] for b in boxes])[which] + offset[2]
        # roof points
        bx = np.where(on_roof, cx + (2 * u - 1) * hx, 0.0)
        by = np.where(on_roof, cy + (2 * v - 1) * hy, 0.0)
        # wall points: walk the perimeter
        per = 4 * (hx + hy)
        s = u * per
        wx = np.where(s < 2 * hx, cx - hx + s,
             np.where(s < 2 * hx + 2 * hy, cx + hx,
             np.where(s < 4 * hx + 2 * hy, cx + hx - (s - 2 * hx - 2 * hy), cx - hx)))
        wy = np.where(s < 2 * hx, cy - hy,
             np.where(s < 2 * hx + 2 * hy, cy - hy + (s - 2 * hx),
             np.where(s < 4 * hx + 2 * hy, cy + hy, cy + hy - (s - 4 * hx - 2 * hy))))
        bx = np.where(on_roof, bx, wx)
        by = np.where(on_roof, by, wy)
        gz_w = g(bx, by)
        bz = np.where(on_roof, rz, gz_w + t * np.maximum(rz - gz_w, 0.0))

    x = np.concatenate([gx, bx, vx])
    y = np.concatenate([gy, by, vy])
    z = np.concatenate([gz, bz, vz])
    truth = np.concatenate([np.full(n_gnd, 2, np.uint8), np.full(n_box, 1, np.uint8), np.full(n_veg, 3, np.uint8)])
    if shuffle:
        perm = rng.permutation(n)
        x, y, z, truth = x[perm], y[perm], z[perm], truth[perm]
    q = np.empty((n, 3), dtype=np.int32)
    for a, c in enumerate((x, y, z)):
        q[:, a] = np.rint((c - offset[a]) / scale[a]).astype(np.int64).clip(-2**31, 2**31 - 1)
    cl = Cloud(q, tuple(float(s) for s in scale), tuple(float(o) for o in offset), float(unit),
               (0.0, 0.0, 0.0), (0.0, 0.0, 0.0), n_gnd, truth)
    dec = cl.decoded() / unit
    if n:
        cl.minc = tuple(float(v) for v in dec.min(axis=0))
        cl.maxc = tuple(float(v) for v in dec.max(axis=0))
    return cl


# Named workloads.  Sizes follow the configurations the classifier is measured on.
def plain_small(seed=1, n=1_000_000):
    """1M points over 100 x 100 m, scale 1 mm, offset 0."""
    side = 100.0 * math.sqrt(n / 1_000_000)
    return terrain_cloud(n, side, side, seed)


def plain_scale(seed=2, n=50_000_000):
    """50M points over 700 x 700 m (about 100 pts/m^2), scale 1 mm, offset 0."""
    side = 700.0 * math.sqrt(n / 50_000_000)
    return terrain_cloud(n, side, side, seed)


def density_tile(n, seed, *, density=100.0, **kw):
    """A square tile of ``n`` points at ``density`` points per square metre."""
    side = math.sqrt(n / density)
    return terrain_cloud(n, side, side, seed, **kw)


def batch_tiles(count=256, lo=50_000, hi=5_000_000, seed0=1000):
    """Sizes and seeds of the mixed batch: log-uniform point counts, slopes to 35 degrees."""
    rng = np.random.default_rng(seed0)
    sizes = np.exp(rng.uniform(math.log(lo), math.log(hi), count)).astype(np.int64)
    frac = rng.uniform(0.05, 0.40, count)
    return [(int(sizes[i]), seed0 + i, float(frac[i])) for i in range(count)]


def batch_tile(n, seed, nonground):
    """One tile of the mixed batch: 100 pts/m^2, slopes to 35 degrees."""
    return density_tile(n, seed, nonground=nonground, max_slope=math.tan(math.radians(35.0)))


def serve_requests(count, rate=200.0, lo=10_000, hi=10_000_000, seed=5000):
    """Poisson arrivals (mean ``rate`` per second) of tile-classify requests:
    (arrival time in seconds, point count, seed), sizes log-uniform in [lo, hi]."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, count))
    sizes = np.exp(rng.uniform(math.log(lo), math.log(hi), count)).astype(np.int64)
    return [(float(t[i]), int(sizes[i]), seed + 1 + i) for i in range(count)]


def mosaic(blocks):
    """Joins tiles that share scale and offset (e.g. utm_block results) into one cloud."""
    xyz = np.concatenate([b.xyz for b in blocks])
    first = blocks[0]
    cl = Cloud(xyz, first.scale, first.offset, first.unit, (0.0, 0.0, 0.0), (0.0, 0.0, 0.0),
               sum(b.n_ground_truth for b in blocks), np.concatenate([b.truth for b in blocks]))
    cl.minc = tuple(float(min(b.minc[a] for b in blocks)) for a in range(3))
    cl.maxc = tuple(float(max(b.maxc[a] for b in blocks)) for a in range(3))
    return cl


def utm_block(n, side, bi, bj, seed=4):
    """Block (bi, bj) of the UTM-like tile, ``side`` metres square, n points."""
    return terrain_cloud(n, side, side, seed * 1000 + bi * 64 + bj, scale=(0.01, 0.01, 0.01),
                         offset=(500000.0, 4500000.0, 1500.0), max_slope=1.0, steps=2.0,
                         origin=(bi * side, bj * side), terrain_seed=seed)


def utm_tile(n=100_000_000, seed=4):
    """UTM-like offsets, 1 cm scale, slopes to 45 degrees with 2 m steps, 100 pts/m^2."""
    side = math.sqrt(n / 100.0)
    return terrain_cloud(n, side, side, seed, scale=(0.01, 0.01, 0.01),
                         offset=(500000.0, 4500000.0, 1500.0), max_slope=1.0, steps=2.0)


WBXYZ_MAGIC = b"WBXYZ1\0\0"


def write_wbxyz(path, cloud: Cloud):
    """Raw input format read by the reference driver (header + int32 xyz records)."""
    with open(path, "wb") as f:
        f.write(WBXYZ_MAGIC)
        f.write(struct.pack("<Q", cloud.n))
        f.write(struct.pack("<3d", *cloud.scale))
        f.write(struct.pack("<3d", *cloud.offset))
        f.write(struct.pack("<d", cloud.unit))
        f.write(struct.pack("<3d", *cloud.minc))
        f.write(struct.pack("<3d", *cloud.maxc))
        f.write(np.ascontiguousarray(cloud.xyz, dtype="<i4").tobytes())


def read_wbxyz(path) -> Cloud:
    with open(path, "rb") as f:
        data = f.read()
    if data[:8] != WBXYZ_MAGIC:
        raise ValueError("not a WBXYZ1 file")
    (n,) = struct.unpack_from("<Q", data, 8)
    vals = struct.unpack_from("<13d", data, 16)
    xyz = np.frombuffer(data, dtype="<i4", count=3 * n, offset=16 + 13 * 8).reshape(n, 3).copy()
    return Cloud(xyz, vals[0:3], vals[3:6], vals[6], vals[7:10], vals[10:13])
