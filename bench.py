"""Benchmark: ground-classified Mpts/s on one GB300 (whole pipeline per step).

A step is one pass of the hot path over one synthetic cloud: octree build
(decode, keys, sort, de-duplication, leaves, store order, node hierarchy),
tile scan + postscan, and per-point classification.  The default workload is
50M points over 700 x 700 m (about 100 pts/m^2), 1 mm quantisation, seeded.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

value:  points / second with the cloud already resident in HBM (device
        pointer in, device class bytes out), CUDA events on the library's
        stream, max over ranks.
e2e:    the same through wb_classify_cloud with pinned host buffers: the
        int32 XYZ and initial class-byte copies in and the class-byte copy
        out are inside the timing.
--impl reference: the reference's CPU algorithm (the oracle restatement,
        oracle/) on this machine's cores, on a bounded sample of the workload.
Multi-GPU runs are independent replicas (one cloud per rank, no collective).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "ground-classified Mpts/s on 1 GB300, served vs plain, at >=99.99% label match"
UNIT = "Mpts/s"
CLASSIFY_BYTES_PER_POINT = 13     # 12 B int32 XYZ read + 1 B class written
BUILD_BYTES_PER_POINT = 28        # 12 B read, 12 B leaf-ordered XYZ + 4 B index written


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons while the timed region runs."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def max_over_ranks(x, device):
    """The largest x over the ranks of the process group (x itself alone):
    the slowest replica sets the whole job's time."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def sample_tiles(n_tiles, frac, seed):
    k = max(1, int(round(frac * n_tiles)))
    return np.sort(np.random.default_rng(seed).choice(n_tiles, k, replace=False))


def oracle_estimate(t_build, s, n_tiles, k):
    """Seconds the oracle would take for the whole workload: its octree build
    (timed in full) plus the sampled tiles' scan and classify times scaled to
    every tile."""
    return t_build + s["t_scan"] * n_tiles / max(1, s["n_scanned"]) + s["t_classify"] * n_tiles / k


def oracle_baseline(cloud, threads, frac, seed, gpu=None):
    """The oracle (the reference's algorithm restated, oracle/) on the
    workload itself: the whole octree built by serial insertion in input
    order (timed in full, as the reference's serial driver does it), then a
    seeded sample of the tiles scanned, post-scanned and classified on every
    host thread (the tiles their postscan reads are scanned on demand).
    Throughput is the workload's points over the build time plus the sample's
    times scaled to every tile.  With the GPU's results (gpu), the same run is
    the parity check: the whole octree, the sampled tiles' fields and the
    class byte of every point those tiles decide."""
    from oracle import oracle as O
    O.build()
    T = O.snake_tiles(cloud)
    tiles = sample_tiles(T, frac, seed)
    k = tiles.shape[0]
    r = O.run(cloud, canonical_order=True, threads=threads, phases=1, keep=True, want_leaves=gpu is not None)
    try:
        s = O.sample(tiles, cloud.n, threads)
        fields = O.sample_tiles_fields(T) if gpu is not None else None
    finally:
        O.reset()
    est = oracle_estimate(r["t_build"], s, T, k)
    base = {"value": cloud.n / est / 1e6, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"the whole workload's octree (serial insertion, {r['t_build']:.1f} s) and a seeded "
                      f"{100 * k / T:.2g}% of its tiles ({k} of {T}; {s['n_sample_points']} cylinder points) scanned "
                      f"and classified on {threads} threads in {s['t_scan'] + s['t_classify']:.1f} s, scaled to "
                      "every tile"}
    if gpu is None:
        return base, None
    stored = r["leaf"] >= 0
    octree_exact = bool(gpu["n_leaves"] == r["n_leaves"] and np.array_equal(gpu["leaves"], r["leaves"])
                        and np.array_equal(gpu["count"].astype(np.int64), r["leaf_count"])
                        and np.array_equal(gpu["pleaf"][stored].astype(np.int64), r["leaf"][stored]))
    names = (("n_points", "n_points"), ("tree_flags", "tree_flags"), ("density", "density"), ("h_scan", "h_scan"),
             ("hyperboloid_size", "h_final"), ("height", "height"))
    tiles_equal = int(np.sum(np.logical_and.reduce([gpu["tiles"][f][tiles] == fields[of][tiles] for f, of in names])))
    decided = s["cls"] != 0
    nd = int(decided.sum())
    eq = int(np.sum(gpu["cls"][decided] == s["cls"][decided]))
    parity = {"against": "oracle, each block's points in input order (pinned to the reference's own sources on the "
                         "golden fixtures and on the 1M-point workload)",
              "octree_exact": octree_exact, "leaves": int(r["n_leaves"]), "sampled_tiles": k,
              "sampled_tiles_exact": tiles_equal, "sampled_labels": nd, "sampled_labels_equal": eq,
              "agreement": eq / nd if nd else None}
    return base, parity


def workload(args, rank):
    from wolkenbase_gb300 import synth
    side = 700.0 * math.sqrt(args.points / 50_000_000)
    cloud = synth.terrain_cloud(args.points, side, side, args.seed + rank)
    cfg = {"workload": f"plain_scale: {args.points} pts over {side:.0f} x {side:.0f} m, 1 mm int32 LAS XYZ, "
                       "4-sinusoid terrain + 2 cm noise, 10% buildings 3-15 m, 10% vegetation 0.5-10 m",
           "points": args.points, "area_m": [round(side, 1), round(side, 1)], "seed": args.seed,
           "params": {"tile_size": 1.0, "max_slope": 1.0, "thickness": 0.0, "min_hyp_size": 0.1},
           "l2": "inputs larger than L2 (int32 XYZ + leaf-ordered store >> 126 MB)"}
    return cloud, cfg


def las_measure(clf, cloud, n, stream, device):
    """The steps either side of the path on the classified cloud as LAS point
    format 1 records (28 bytes) resident on the device, CUDA events on the
    library's stream: wb_las_write_classes (the last classify's bytes into the
    records), wb_las_split_by_class, wb_las_decode (every LasPoint field) and
    wb_las_write_output (the class-split writer).  Algorithmic bytes: split 56 B
    per record (read once, written once); decode 90 B per record (28 read, 62
    written as field arrays); writer 61 B per stored point (record read, record
    written, store index and class byte read)."""
    import ctypes as C
    import torch
    rec = torch.zeros((n, 28), dtype=torch.uint8, device=f"cuda:{device}")
    rec[:, 0:12] = torch.from_numpy(np.ascontiguousarray(cloud.xyz).view(np.uint8).reshape(-1, 12)).to(rec.device)
    out = torch.empty_like(rec)
    offsets = np.zeros(257, np.uint64)
    L = clf.L

    def write():
        clf._check(L.wb_las_write_classes(clf.ctx, C.c_void_p(rec.data_ptr()), n, 28, 1, 1, None))

    def split():
        clf._check(L.wb_las_split_by_class(clf.ctx, C.c_void_p(rec.data_ptr()), n, 28, 1, 1,
                                           C.c_void_p(out.data_ptr()), offsets.ctypes.data))

    # LasHeader::readPoint of every record into device arrays of every LasPoint field
    from wolkenbase_gb300 import _lib
    dev = rec.device
    tdt = {C.c_double: torch.float64, C.c_uint16: torch.int16, C.c_uint8: torch.uint8, C.c_int32: torch.int32}
    fields = {name: torch.empty(n, dtype=tdt[t], device=dev) for name, t in _lib.LAS_POINT_FIELDS}
    pts = _lib.wb_las_points(**{name: t.data_ptr() for name, t in fields.items()})
    d = cloud.decoded()
    cs = _lib.wb_cloud()
    cs.records, cs.n, cs.stride, cs.device_resident = rec.data_ptr(), n, 28, 1
    cs.scale[:], cs.offset[:], cs.unit = cloud.scale, cloud.offset, cloud.unit

    def decode():
        clf._check(L.wb_las_decode(clf.ctx, C.byref(cs), 1, C.byref(pts)))

    # CloudOutput::writeFiles as the GUI runs it (separate classes, 10M points
    # per file: wolkencanvas.cpp:619), records in and files out on the device
    import wolkenbase_gb300 as wb
    o = wb.LasOutput(point_format=1, separate_classes=True, points_per_file=10_000_000, unit=cloud.unit,
                     min_cor=tuple(d.min(axis=0)), max_cor=tuple(d.max(axis=0)), scale=(0.001, 0.001, 0.001),
                     creation_day=1, creation_year=2026).c()
    nd = clf.info()["n_distinct"]
    fout = torch.empty((nd, 28), dtype=torch.uint8, device=dev)
    files = (_lib.wb_las_file * 64)()
    nfiles = C.c_int(0)

    def writer():
        clf._check(L.wb_las_write_output(clf.ctx, C.byref(cs), 1, None, C.byref(o), C.c_void_p(fout.data_ptr()), 1,
                                          files, 64, C.byref(nfiles)))

    res = {}
    for name, fn in (("write_classes", write), ("split_by_class", split), ("decode", decode), ("writer", writer)):
        fn()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(3):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        res[name] = e0.elapsed_time(e1) / 3
    peak, kind = peaks()
    gbs = 56.0 * n / (res["split_by_class"] / 1e3) / 1e9
    dec_gbs = 90.0 * n / (res["decode"] / 1e3) / 1e9
    wr_gbs = 61.0 * nd / (res["writer"] / 1e3) / 1e9
    del rec, out, fields, fout
    return {"records": n, "format": 1, "write_classes_ms": res["write_classes"],
            "split_by_class_ms": res["split_by_class"], "split_achieved_GBps": gbs, "split_frac": gbs / peak,
            "ground_records": int(offsets[3] - offsets[2]), "algorithmic_bytes_per_record": 56,
            "decode_ms": res["decode"], "decode_GBps": dec_gbs, "decode_frac": dec_gbs / peak,
            "decode_bytes_per_record": 90,
            "writer_ms": res["writer"], "writer_GBps": wr_gbs, "writer_frac": wr_gbs / peak,
            "writer_bytes_per_point": 61, "writer_files": nfiles.value,
            "writer_workload": "format 1 in and out, separate classes, 10M points per file, device-resident"}


def paging_measure(cloud, params, want_cls, device, args):
    """The same cloud through wb_classify_cloud on a context whose HBM budget
    holds about a third of its working set, paging on (buffers beyond the
    budget in pinned host memory, used in place over the CPU link): Mpts/s with
    host buffers in and out, the bytes placed on each side, and whether the
    labels equal the unpaged run's."""
    import ctypes as C
    import torch
    import wolkenbase_gb300 as wb
    n = cloud.n
    budget = int(n * 100)
    clf = wb.Classifier(device, hbm_budget=budget)
    try:
        clf.set_paging(int(n * 400))
    except wb.WolkenbaseError as e:
        clf.close()
        return {"unavailable": str(e)}
    pin_xyz = torch.from_numpy(np.ascontiguousarray(cloud.xyz)).pin_memory()
    pin_cls = torch.zeros(n, dtype=torch.uint8).pin_memory()
    cs = wb.cloud_struct(pin_xyz.data_ptr(), n, 12, cloud.scale, cloud.offset, cloud.unit, cloud.minc, cloud.maxc)

    def step():
        clf._check(clf.L.wb_classify_cloud(clf.ctx, C.byref(cs), C.byref(params.c()), C.c_void_p(pin_cls.data_ptr())))

    step()
    reps = max(1, min(args.steps, 2))
    t0 = time.perf_counter()
    for _ in range(reps):
        step()
    dt = (time.perf_counter() - t0) / reps
    st = clf.paging_stats()
    same = bool(np.array_equal(pin_cls.numpy(), want_cls))
    clf.close()
    return {"workload": "the plain workload, HBM budget 100 B per point, host memory up to 400 B per point",
            "hbm_budget": budget, "value": n / dt / 1e6, "unit": UNIT, "host_peak_bytes": st["host_peak"],
            "device_bytes": st["device_bytes"], "same_labels": same}


def _gen_tile(spec):
    from wolkenbase_gb300 import synth
    kind, n, seed, frac = spec
    if kind == "batch":
        return synth.batch_tile(n, seed, frac)
    return synth.density_tile(n, seed)


def generate(specs, procs=None):
    """Generates clouds in a spawn-started process pool (safe beside CUDA)."""
    import multiprocessing as mp
    procs = procs or min(len(specs), os.cpu_count() or 1, 32)
    if procs <= 1:
        return [_gen_tile(s) for s in specs]
    order = sorted(range(len(specs)), key=lambda i: -specs[i][1])   # big ones first
    with mp.get_context("spawn").Pool(procs) as pool:
        got = pool.map(_gen_tile, [specs[i] for i in order], chunksize=1)
    out = [None] * len(specs)
    for i, c in zip(order, got):
        out[i] = c
    return out


def _tuned(st):
    from wolkenbase_gb300 import _lib
    shapes = ["groups 8 warps/3 blocks", "groups 4/5", "groups 8/2", "points 8/3", "points 4/6", "points 4/8",
              "points 8/4", "points 2/12"]
    return {"shape": shapes[st["shape"]], "chunk": st["chunk"], "grid_points": st["grid_points"],
            "tune_ms": st["tune_ms"]}


def _pct(v, q):
    return float(np.percentile(np.asarray(v), q)) if len(v) else None


def served_form(args, device, rate=None, count=None, pool=None):
    """Poisson arrivals of tile-classify requests replayed against the plain
    per-request path (one context, one request at a time, in arrival order)
    and against the server (admission by HBM budget, overlapping scans, fused
    classify launches).  Host buffers in and out for both.  With pool < count
    the requests reuse pool generated clouds in turn (their arrival times and
    sizes follow the request stream's own seeds)."""
    import wolkenbase_gb300 as wb
    from wolkenbase_gb300 import synth
    rate = rate or args.serve_rate
    count = count or args.serve_requests
    pool = min(pool or count, count)
    reqs = synth.serve_requests(count, rate=rate, seed=args.seed + 5000)
    made = generate([("serve", n, seed, 0.0) for _, n, seed in reqs[:pool]])
    clouds = [made[i % pool] for i in range(count)]
    arrivals = [t for t, _, _ in reqs]
    pts = sum(c.n for c in clouds)

    def plain_pass(clf):
        lat = []
        t0 = time.perf_counter()
        for t, c in zip(arrivals, clouds):
            d = t0 + t - time.perf_counter()
            if d > 0:
                time.sleep(d)
            clf.classify_cloud(c)
            lat.append(time.perf_counter() - (t0 + t))
        return time.perf_counter() - t0, lat

    def served_pass(srv):
        ids = [None] * len(clouds)
        t0 = time.perf_counter()
        s0 = srv.stats()["now"]

        def feeder():
            for i, (t, c) in enumerate(zip(arrivals, clouds)):
                d = t0 + t - time.perf_counter()
                if d > 0:
                    time.sleep(d)
                ids[i] = srv.submit(c, tag=i)
        th = threading.Thread(target=feeder)
        th.start()
        th.join()
        sts = [srv.result(j)[1] for j in ids]
        lat = [st["t_done"] - (s0 + arrivals[i]) for i, st in enumerate(sts)]
        span = max(st["t_done"] for st in sts) - s0
        return span, lat, sts

    clf = wb.Classifier(device)
    big = max(clouds, key=lambda c: c.n)
    clf.classify_cloud(big)                       # buffers sized once
    plain_span, plain_lat = plain_pass(clf)
    clf.close()
    srv = wb.Server(device, prep_slots=args.serve_slots, hbm_budget=int(args.serve_budget_gb * 2**30),
                    autotune=True)
    served_pass(srv)                              # contexts sized once
    launches0 = srv.stats()["kernel_launches"]
    span, lat, sts = served_pass(srv)
    st = srv.stats()
    srv.close()
    batch = [s["batch_jobs"] for s in sts]
    return {"workload": f"{len(clouds)} requests ({pool} distinct clouds), Poisson arrivals at {rate:g}/s, sizes "
                        f"log-uniform 10k-10M points (100 pts/m^2 tiles), {args.serve_budget_gb:g} GB HBM budget",
            "offered_Mpts_s": pts / max(arrivals[-1], 1e-9) / 1e6,
            "points": pts,
            "plain": {"value": pts / plain_span / 1e6, "unit": UNIT, "p50_ms": _pct(plain_lat, 50) * 1e3,
                      "p99_ms": _pct(plain_lat, 99) * 1e3, "makespan_s": plain_span},
            "served": {"value": pts / span / 1e6, "unit": UNIT, "p50_ms": _pct(lat, 50) * 1e3,
                       "p99_ms": _pct(lat, 99) * 1e3, "makespan_s": span, "prep_slots": args.serve_slots,
                       "fused_launches": st["fused_launches"], "mean_jobs_per_launch":
                           float(np.mean(batch)), "peak_bytes": st["peak_bytes"],
                       "gpu_launches": st["kernel_launches"] - launches0, "tuned": _tuned(st)},
            "served_over_plain": (pts / span) / (pts / plain_span)}


def batched_form(args, device):
    """256 independent tiles of uneven size: sequential plain launches (one
    wb_classify_cloud per tile) against one wb_classify_batch (all tiles
    scanned concurrently, one fused graph-captured classify).  Host buffers."""
    import wolkenbase_gb300 as wb
    from wolkenbase_gb300 import _lib, synth
    specs = synth.batch_tiles(args.batch_tiles)
    clouds = generate([("batch", n, seed, frac) for n, seed, frac in specs])
    pts = sum(c.n for c in clouds)
    clf = wb.Classifier(device)
    plain_ref = [clf.classify_cloud(c) for c in clouds]          # warm-up, buffers sized
    t0 = time.perf_counter()
    for c in clouds:
        clf.classify_cloud(c)
    plain_s = time.perf_counter() - t0
    clf.close()
    srv = wb.Server(device, prep_slots=args.batch_slots, flush=_lib.WB_FLUSH_FULL, autotune=True)
    got = srv.classify_batch(clouds)                              # warm-up, contexts sized
    st0 = srv.stats()
    launches0, fused0 = st0["kernel_launches"], st0["fused_launches"]
    t0 = time.perf_counter()
    got = srv.classify_batch(clouds)
    batch_s = time.perf_counter() - t0
    st = srv.stats()
    srv.close()
    same = all(np.array_equal(a, b) for a, b in zip(plain_ref, got))
    # the FP32 precision mode on every tile of the batch against the exact path
    from wolkenbase_gb300 import precision
    clf = wb.Classifier(device)
    reps = [precision.compare(clf, c) for c in clouds]
    clf.close()
    flips = sum(r["flips"] for r in reps)
    prec = {"points": pts, "flips": flips, "agreement": 1.0 - flips / pts,
            "slope_err": max(r["slope_err"] for r in reps),
            "residual_abs_err_m": max(r["residual_abs_err_m"] for r in reps),
            "residual_err": max(r["residual_err"] for r in reps),
            "residual_err_p999_max_over_tiles_sets": max(r["residual_err_p999"] for r in reps),
            "h_changed": sum(r["h_changed"] for r in reps), "h_rel_err": max(r["h_rel_err"] for r in reps)}
    return {"workload": f"{len(clouds)} tiles, log-uniform 50k-5M points (100 pts/m^2), slopes to 35 deg, "
                        "nonground 5-40%", "precision": prec,
            "points": pts,
            "plain": {"value": pts / plain_s / 1e6, "unit": UNIT, "seconds": plain_s},
            "batched": {"value": pts / batch_s / 1e6, "unit": UNIT, "seconds": batch_s,
                        "fused_launches": st["fused_launches"] - fused0, "prep_slots": args.batch_slots,
                        "gpu_launches": st["kernel_launches"] - launches0, "tuned": _tuned(st)},
            "batched_over_plain": plain_s / batch_s, "same_labels": same}


def _gen_utm(spec):
    from wolkenbase_gb300 import synth
    n, side, bi, bj = spec
    return synth.utm_block(n, side, bi, bj)


def precision_form(args, device):
    """The 100M-point UTM-like tile (1 cm scale, offsets 500 km / 4500 km /
    1500 m, slopes to 45 degrees, 2 m steps), generated as a 4 x 4 mosaic of
    one terrain: scan + classify exact (FP64 decisions) and in the FP32
    precision mode on one built octree; flips and fit errors of the FP32 mode."""
    import multiprocessing as mp
    import wolkenbase_gb300 as wb
    from wolkenbase_gb300 import precision, synth
    nb = 4
    side = math.sqrt(args.precision_points / 100.0) / nb
    specs = [(args.precision_points // (nb * nb), side, i, j) for i in range(nb) for j in range(nb)]
    with mp.get_context("spawn").Pool(min(len(specs), os.cpu_count() or 1)) as pool:
        blocks = pool.map(_gen_utm, specs, chunksize=1)
    cloud = synth.mosaic(blocks)
    del blocks
    clf = wb.Classifier(device)
    clf.build(cloud)
    precision.compare(clf, cloud, built=True)     # warm-up
    r = precision.compare(clf, cloud, built=True)
    clf.close()
    r["workload"] = (f"{cloud.n} pts over {nb * side:.0f} x {nb * side:.0f} m, 1 cm int32, offsets (500000, 4500000, "
                     "1500) m, slopes to 45 deg + 2 m steps")
    for k in ("fp64_ms", "fp32_ms"):
        r[k + "_mpts_s"] = cloud.n / ((r[k]["scan"] + r[k]["classify"]) / 1e3) / 1e6
    return r


def run_reference(args):
    """The reference's algorithm (the oracle restatement: the reference's own
    sources are not on the GPU machine) on this machine's cores: the workload's
    whole octree built once by serial insertion, then each step scans and
    classifies another seeded sample of its tiles; a step's value is the
    workload's points over the build time plus that sample's times scaled to
    every tile."""
    rank, world, local = dist_env()
    if rank != 0:
        return
    cloud, cfg = workload(args, 0)
    threads = os.cpu_count() or 1
    from oracle import oracle as O
    O.build()
    T = O.snake_tiles(cloud)
    r = O.run(cloud, canonical_order=True, threads=threads, phases=1, keep=True, want_leaves=False)
    vals, secs = [], []
    try:
        for i in range(args.warmup + args.steps):
            tiles = sample_tiles(T, args.ref_tile_frac, args.seed + 100 + i)
            s = O.sample(tiles, cloud.n, threads)
            est = oracle_estimate(r["t_build"], s, T, tiles.shape[0])
            if i >= args.warmup:
                vals.append(cloud.n / est / 1e6)
                secs.append(s["t_scan"] + s["t_classify"])
    finally:
        O.reset()
    value = float(np.median(vals))
    k = max(1, int(round(args.ref_tile_frac * T)))
    sample = (f"the whole workload's octree (serial insertion, {r['t_build']:.1f} s, once), then per step a seeded "
              f"{100 * args.ref_tile_frac:.2g}% of its tiles ({k} of {T}) scanned and classified "
              f"({np.median(secs):.1f} s median), scaled to every tile")
    out = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": float(np.median(secs)) * 1e3,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic", "config": cfg,
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--points", type=int, default=50_000_000)
    ap.add_argument("--seed", type=int, default=2)
    ap.add_argument("--cpu-tile-frac", type=float, default=0.01,
                    help="share of the tiles the CPU baseline (and the parity check) scans and classifies")
    ap.add_argument("--ref-tile-frac", type=float, default=0.001, help="share of the tiles per reference-arm step")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-forms", action="store_true", help="skip the served and batched measurements")
    ap.add_argument("--serve-requests", type=int, default=64)
    ap.add_argument("--serve-rate", type=float, default=200.0)
    ap.add_argument("--serve-slots", type=int, default=4)
    ap.add_argument("--serve-low-rate", type=float, default=50.0, help="arrival rate of the below-capacity run")
    ap.add_argument("--serve-low-requests", type=int, default=256)
    ap.add_argument("--serve-low-pool", type=int, default=64, help="distinct clouds the below-capacity run cycles through")
    ap.add_argument("--serve-budget-gb", type=float, default=80.0)
    ap.add_argument("--batch-tiles", type=int, default=256)
    ap.add_argument("--batch-slots", type=int, default=8)
    ap.add_argument("--precision-points", type=int, default=100_000_000)
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
        return

    import torch
    import wolkenbase_gb300 as wb

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    cloud, cfg = workload(args, rank)
    n = cloud.n
    params = wb.Params()
    stream = torch.cuda.Stream()
    clf = wb.Classifier(local)
    clf.set_stream(stream.cuda_stream)

    dev_xyz = torch.from_numpy(np.ascontiguousarray(cloud.xyz)).to(f"cuda:{local}")
    dev_cls = torch.zeros(n, dtype=torch.uint8, device=f"cuda:{local}")
    cs_dev = wb.cloud_struct(dev_xyz.data_ptr(), n, 12, cloud.scale, cloud.offset, cloud.unit, cloud.minc,
                             cloud.maxc, device_resident=True)
    import ctypes as C

    def step_dev():
        rc = clf.L.wb_classify_cloud(clf.ctx, C.byref(cs_dev), C.byref(params.c()), C.c_void_p(dev_cls.data_ptr()))
        clf._check(rc)

    for _ in range(args.warmup):
        step_dev()
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    # device-resident timed region (the library's stage events off)
    launches0 = clf.launch_count()
    barrier()
    with ClockSampler(local) as clocks:
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(args.steps):
            step_dev()
        ev1.record(stream)
        barrier()
    launches = clf.launch_count() - launches0
    ms_total = max_over_ranks(ev0.elapsed_time(ev1), f"cuda:{local}")
    ms_step = ms_total / args.steps
    value = world * n / (ms_step / 1e3) / 1e6
    cls_dev = dev_cls.cpu().numpy()
    # where a step's time goes: more steps with the library's per-stage CUDA
    # events on (outside the timed region; these give the kernels' durations)
    clf.profile(True)
    stage_acc = {}
    n_prof = max(1, min(args.steps, 3))
    for _ in range(n_prof):
        step_dev()
        for name, ms in clf.stage_times():
            stage_acc[name] = stage_acc.get(name, 0.0) + ms
    clf.profile(False)

    # end-to-end through the public API with pinned host buffers
    pin_xyz = torch.from_numpy(np.ascontiguousarray(cloud.xyz)).pin_memory()
    pin_cls = torch.zeros(n, dtype=torch.uint8).pin_memory()
    cs_host = wb.cloud_struct(pin_xyz.data_ptr(), n, 12, cloud.scale, cloud.offset, cloud.unit, cloud.minc,
                              cloud.maxc, device_resident=False)

    def step_host():
        rc = clf.L.wb_classify_cloud(clf.ctx, C.byref(cs_host), C.byref(params.c()), C.c_void_p(pin_cls.data_ptr()))
        clf._check(rc)

    step_host()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step_host()
    barrier()
    e2e_s = max_over_ranks((time.perf_counter() - t0) / args.steps, f"cuda:{local}")
    e2e_value = world * n / e2e_s / 1e6
    same = bool(np.array_equal(pin_cls.numpy(), cls_dev))
    # where the end-to-end step's extra time goes: one more (untimed) host-buffer
    # step with the library's stage events on
    clf.profile(True)
    step_host()
    e2e_stages = {k: round(v, 3) for k, v in clf.stage_times()}
    clf.profile(False)

    gpu_res = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cs_, _, cnt_ = clf.leaves()
        gpu_res = {"n_leaves": clf.info()["n_leaves"], "leaves": cs_, "count": cnt_, "pleaf": clf.point_leaf(),
                   "tiles": clf.tiles(), "cls": cls_dev}
    las = las_measure(clf, cloud, n, stream, local) if rank == 0 else None
    paging = paging_measure(cloud, params, cls_dev, local, args) if rank == 0 and not args.no_forms else None
    info = clf.info()
    prec_plain = None
    if rank == 0 and not args.no_forms:
        from wolkenbase_gb300 import precision
        prec_plain = precision.compare(clf, cloud, built=True)
        prec_plain["workload"] = cfg["workload"]
    stage_ms = {k: v / n_prof for k, v in stage_acc.items()}
    dom = max((k for k in stage_ms if k not in ("upload", "cls_upload", "cls_download", "classify_exact")), key=lambda k: stage_ms[k])
    peak, peak_kind = peaks()
    nd = info["n_distinct"]
    alg_bytes = {"classify": CLASSIFY_BYTES_PER_POINT * nd}.get(dom, None)
    roof = None
    if alg_bytes:
        achieved = alg_bytes / (stage_ms[dom] / 1e3) / 1e9
        traffic = None
        tp = os.path.join(ROOT, "profiles", "traffic.json")
        if os.path.exists(tp):
            tr = json.load(open(tp)).get(dom)
            if tr:
                traffic = float(tr["bytes_per_point"]) * nd
        roof = {"kernel": dom, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
                "algorithmic_bytes": alg_bytes, "avg_ms": stage_ms[dom]}
        # The kernel is bound by instruction issue and latency, not by HBM: its
        # issue-side fraction, from the warp instructions per point of one
        # profiled launch, over the issue rate of the GPU at the sampled clock
        tr = json.load(open(tp)).get(dom) if os.path.exists(tp) else None
        if tr and tr.get("inst_per_point"):
            ck = clocks.summary() or {}
            mhz = ck.get("sm_mhz") or ck.get("sm_max_mhz") or 2070.0
            sms = torch.cuda.get_device_properties(local).multi_processor_count
            peak_inst = sms * 4 * mhz * 1e6
            ach_inst = tr["inst_per_point"] * nd / (stage_ms[dom] / 1e3)
            roof["issue"] = {"inst_per_point": tr["inst_per_point"], "achieved_Ginst_s": ach_inst / 1e9,
                             "peak_Ginst_s": peak_inst / 1e9, "frac": ach_inst / peak_inst,
                             "ncu_issue_active": tr.get("issue_active_pct", 0) / 100,
                             "ncu_warps_active": tr.get("warps_active_pct", 0) / 100,
                             "note": "warp instructions per point of the column-group fast pass (ncu, one launch "
                                     "on 4M points) x points / the classify stage's time; peak = 4 issue slots "
                                     "per SM per cycle at the sampled SM clock"}
    # the octree build proper (sizeFit + put of every point); the column grid is this path's own index
    build_ms = sum(v for k, v in stage_ms.items() if k in ("decode_key", "sort", "dedup", "leaves", "leaf_order",
                                                         "point_map", "nodes"))
    cpu = parity = None
    if gpu_res is not None:
        cpu, parity = oracle_baseline(cloud, os.cpu_count() or 1, args.cpu_tile_frac, args.seed + 7, gpu_res)
        del gpu_res
    clk = clocks.summary()
    labels = np.bincount(cls_dev, minlength=3)
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": cfg,
           "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 13 * n, "d2h_bytes_per_step": n,
                   "same_labels_as_device_run": same, "ms_per_step": e2e_s * 1e3, "stages_ms": e2e_stages},
           "gpu_launches": launches, "roofline": roof, "cpu_baseline": cpu, "clocks": clk,
           "stages_ms": {k: round(v, 3) for k, v in stage_ms.items()},
           "las": las, "paging": paging}
    clf.close()
    del dev_xyz, dev_cls, pin_xyz, pin_cls
    torch.cuda.empty_cache()
    if rank == 0 and world == 1 and not args.no_forms:
        out["served"] = served_form(args, local)
        out["served_below_capacity"] = served_form(args, local, rate=args.serve_low_rate,
                                                   count=args.serve_low_requests, pool=args.serve_low_pool)
        out["batched"] = batched_form(args, local)
        out["precision"] = precision_form(args, local)
    # compact summaries last, where a reader of the line's end finds them
    build_gbs = BUILD_BYTES_PER_POINT * n / (build_ms / 1e3) / 1e9 if build_ms else None
    out["octree"] = {"leaves": info["n_leaves"], "distinct": nd, "max_depth": info["max_depth"]}
    out["labels"] = {"ground": int(labels[2]), "not_ground": int(labels[1]), "untouched": int(labels[0])}
    out["build"] = {"ms": round(build_ms, 3), "achieved_GBps": build_gbs, "frac": build_gbs / peak if build_gbs else None,
                    "algorithmic_bytes_per_point": BUILD_BYTES_PER_POINT, "peak_GBps": peak}
    out["parity"] = parity
    if rank == 0 and world == 1 and not args.no_forms:
        # FP32 precision mode against the exact path, per workload: label
        # flips and the per-point fit residuals' difference (scan.cpp:74-87)
        keys = ("points", "flips", "agreement", "slope_err", "residual_abs_err_m", "residual_err", "h_changed",
                "h_rel_err")
        out["precision_by_config"] = {
            "plain_scale": {k: prec_plain.get(k) for k in keys} if prec_plain else None,
            "batched": {k: out["batched"]["precision"].get(k) for k in keys},
            "utm_100M": {k: out["precision"].get(k) for k in keys}}
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
