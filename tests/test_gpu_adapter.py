"""A C++ program classifies a golden cloud through the adapter on the GPU.

The cloud is written as a LAS 1.4 file (point format 1, header from
wb_las_header_bytes); the program (built here against
include/wolkenbase_gb300.hpp and the library) reads it as INTEGRATION.md's
sketch does, runs OctStore::put, scanCylinders and classifyCylinders, and
answers findBlock / findBlocks / pointsIn / getAll / countClasses queries.
Its class bytes must equal the oracle's, and its query answers the Python
mirror's, which the query tests pin to the oracle.
"""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, golden_cloud, load_golden

pytestmark = pytest.mark.gpu

PROGRAM = r"""
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <vector>
#include "wolkenbase_gb300.hpp"

struct P3 { double x, y, z; double getx() const { return x; } double gety() const { return y; } double getz() const { return z; } };

int main(int argc, char **argv)
{
  namespace wb = wolkenbase_gb300;
  try
  {
    wb::LasFileGeometry g = wb::readLasGeometry(argv[1]);
    std::vector<char> records(g.nPoints * g.pointLength);
    std::ifstream f(argv[1], std::ios::binary);
    f.seekg(g.pointOffset);
    f.read(records.data(), records.size());
    wb::OctStore store;
    store.put(wb::cloudOf(g, records.data(), 1.0));
    wb::Params p;
    wb::scanCylinders(store, p);
    std::vector<uint8_t> cls(g.nPoints, 0);
    std::vector<float> margin;
    wb::classifyCylinders(store, p, cls, &margin);
    std::ofstream o(argv[2], std::ios::binary);
    o.write((const char *)cls.data(), cls.size());
    // queries around (qx, qy, qz)
    P3 q{atof(argv[3]), atof(argv[4]), atof(argv[5])};
    int64_t b = store.findBlock(q);
    std::vector<int64_t> bl = store.findBlocks(wb::Cylinder(q.x, q.y, 1.5));
    std::vector<uint32_t> cyl = store.pointsIn(wb::Cylinder(q.x, q.y, 1.5), true);
    std::vector<uint32_t> hyp = store.pointsIn(wb::Hyperboloid(q, 0.15, 1.0));
    std::vector<uint32_t> all = store.getAll(b);
    std::map<int, size_t> cc = store.countClasses(), cb = store.countClasses(b);
    std::vector<wb_tile> tab = wb::tiles(store);
    uint64_t counts[8] = {(uint64_t)b, bl.size(), cyl.size(), hyp.size(), all.size(), store.getNumBlocks(),
                          (uint64_t)cc[2], (uint64_t)cb[2]};
    o.write((const char *)counts, sizeof counts);
    o.write((const char *)bl.data(), bl.size() * 8);
    o.write((const char *)cyl.data(), cyl.size() * 4);
    o.write((const char *)hyp.data(), hyp.size() * 4);
    o.write((const char *)all.data(), all.size() * 4);
    o.write((const char *)margin.data(), margin.size() * 4);
    uint64_t nt = tab.size();
    o.write((const char *)&nt, 8);
    return 0;
  }
  catch (const wb::Error &e)
  {
    std::fprintf(stderr, "%s (%d)\n", e.what(), e.code());
    return 3;
  }
}
"""


def _write_las(path, cloud):
    from wolkenbase_gb300 import _lib
    L = _lib.load()
    out = _lib.wb_las_output()
    out.unit = 1.0
    out.creation_day = 1
    out.creation_year = 2026
    f = _lib.wb_las_file()
    f.point_format = 1
    f.n_points[0] = f.n_points[1] = cloud.n
    d = cloud.decoded()
    for k in range(3):
        f.scale[k] = cloud.scale[k]
        f.offset[k] = cloud.offset[k]
        f.min[k] = float(d[:, k].min())
        f.max[k] = float(d[:, k].max())
    hdr = (C.c_uint8 * 375)()
    assert L.wb_las_header_bytes(C.byref(out), C.byref(f), hdr) == 0
    rec = np.zeros((cloud.n, 28), np.uint8)
    rec[:, :12] = np.ascontiguousarray(cloud.xyz, dtype="<i4").view(np.uint8).reshape(-1, 12)
    with open(path, "wb") as fh:
        fh.write(bytes(hdr))
        fh.write(rec.tobytes())


def test_cpp_program_classifies_through_the_adapter(classifier, oracle_mod, cuda_lib_path, tmp_path):
    g = load_golden("tile20k")
    cloud = golden_cloud(g)
    las = tmp_path / "cloud.las"
    _write_las(str(las), cloud)
    src = tmp_path / "client.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "client"
    libdir = os.path.dirname(cuda_lib_path)
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe),
                        "-L" + libdir, "-lwolkenbase_gb300", "-Wl,-rpath," + libdir], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    d = cloud.decoded()
    q = d[1234]
    out = tmp_path / "out.bin"
    run = subprocess.run([str(exe), str(las), str(out), repr(float(q[0])), repr(float(q[1])), repr(float(q[2]))],
                         capture_output=True, text=True, timeout=300)
    assert run.returncode == 0, run.stderr
    raw = out.read_bytes()
    n = cloud.n
    cls = np.frombuffer(raw, np.uint8, n, 0)
    o = oracle_mod.run(cloud, canonical_order=True, threads=8)
    stored = o["block"] >= 0
    assert np.array_equal(cls[stored], o["cls"][stored])
    cnt = np.frombuffer(raw, np.uint64, 8, n)
    off = n + 64
    blocks = np.frombuffer(raw, np.int64, int(cnt[1]), off); off += 8 * int(cnt[1])
    cyl = np.frombuffer(raw, np.uint32, int(cnt[2]), off); off += 4 * int(cnt[2])
    hyp = np.frombuffer(raw, np.uint32, int(cnt[3]), off); off += 4 * int(cnt[3])
    allb = np.frombuffer(raw, np.uint32, int(cnt[4]), off); off += 4 * int(cnt[4])
    margin = np.frombuffer(raw, np.float32, n, off)
    # the same queries through the Python mirror (pinned to the oracle by the query tests)
    classifier.build(cloud)
    qq = (float(q[0]), float(q[1]), float(q[2]))
    assert int(cnt[0]) == int(classifier.find_block(np.array([qq]))[0])
    assert np.array_equal(blocks, classifier.find_blocks(1, qq[:2], 1.5))
    assert np.array_equal(cyl, classifier.points_in(1, qq[:2], 1.5, sorted=True))
    assert np.array_equal(hyp, classifier.points_in(2, qq, 0.15, 1.0))
    cs, first, count = classifier.leaves()
    b = int(cnt[0])
    assert b >= 0   # a stored point lies in a leaf
    order = classifier.store_order()
    assert np.array_equal(allb, order[first[b]:first[b] + count[b]])
    assert int(cnt[5]) == len(first)
    assert int(cnt[6]) == int(np.sum(cls[order] == 2))
    assert int(cnt[7]) == int(np.sum(cls[allb] == 2))
    assert np.all((margin[stored] < 0) == (cls[stored] == 1))
