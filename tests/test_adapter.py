"""The C++ adapter (include/wolkenbase_gb300.hpp) on the CPU.

1. A C++ program built against the adapter alone: it reads back a LAS header
   the library wrote (wb_las_header_bytes) with readLasGeometry, and opening
   an OctStore on a machine without a GPU throws wolkenbase_gb300::Error.
2. With the reference's sources (WB_REFERENCE_SRC), the adapter and the
   classifyOnGpu sketch of INTEGRATION.md, verbatim, compile against the
   reference's own headers (las.h, scan.h, shape.h, eisenstein.h), with the
   adapter's templates instantiated on the reference's xyz, xy and Eisenstein.
"""
import os
import re
import subprocess

import pytest

from conftest import ROOT

PROGRAM = r"""
#include <cmath>
#include <cstdio>
#include <fstream>
#include "wolkenbase_gb300.hpp"

struct P3 { double x, y, z; double getx() const { return x; } double gety() const { return y; } double getz() const { return z; } };
struct P2 { double x, y; double getx() const { return x; } double gety() const { return y; } };

int main(int argc, char **argv)
{
  namespace wb = wolkenbase_gb300;
  wb_las_output out{};
  wb_las_file f{};
  out.unit = 1;
  out.creation_day = 1;
  out.creation_year = 2026;
  f.point_format = 1;
  f.n_points[0] = f.n_points[1] = 12345;
  for (int k = 0; k < 3; k++)
  {
    f.scale[k] = 0.001 * (k + 1);
    f.offset[k] = 1000.0 * k;
    f.min[k] = -5.0 - k;
    f.max[k] = 7.0 + k;
  }
  unsigned char hdr[375];
  if (wb_las_header_bytes(&out, &f, hdr))
    return 1;
  {
    std::ofstream o(argv[1], std::ios::binary);
    o.write((const char *)hdr, sizeof hdr);
  }
  wb::LasFileGeometry g = wb::readLasGeometry(argv[1]);
  if (g.pointFormat != 1 || g.pointLength != 28 || g.nPoints != 12345 || g.pointOffset != 375)
    return 2;
  for (int k = 0; k < 3; k++)
    if (g.scale[k] != f.scale[k] || g.offset[k] != f.offset[k] || g.minc[k] != f.min[k] || g.maxc[k] != f.max[k])
      return 3;
  wb_cloud c = wb::cloudOf(g, hdr, 0.3048);
  if (c.n != 12345 || c.stride != 28 || c.unit != 0.3048)
    return 4;
  wb::Cylinder cy(P2{1, 2}, 0.5);
  wb::Hyperboloid hy(P3{1, 2, 3}, 0.2, 1.0);
  wb::Params p(0.5, 1.5);
  if (cy.cx != 1 || hy.v[2] != 3 || p.max_slope != 1.5 || p.min_hyp_size != 0.1)
    return 5;
  try
  {
    wb::OctStore st(0, 0);
    std::printf("gpu\n");   // a GPU is present: the store opened
  }
  catch (const wb::Error &e)
  {
    std::printf("no gpu: %d\n", e.code());
  }
  return 0;
}
"""


def test_adapter_program_builds_and_runs(cuda_lib_path, tmp_path):
    src = tmp_path / "adapter.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "adapter"
    libdir = os.path.dirname(cuda_lib_path)
    r = subprocess.run(["g++", "-std=c++17", "-Wall", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe),
                        "-L" + libdir, "-lwolkenbase_gb300", "-Wl,-rpath," + libdir],
                       capture_output=True, text=True)
    if r.returncode != 0:
        pytest.fail(r.stderr)
    run = subprocess.run([str(exe), str(tmp_path / "h.las")], capture_output=True, text=True)
    assert run.returncode == 0, (run.returncode, run.stdout, run.stderr)
    out = run.stdout.strip()
    assert out == "gpu" or out.startswith("no gpu: "), out


def _integration_sketch():
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    blocks = re.findall(r"```cpp\n(.*?)```", text, re.S)
    sketch = [b for b in blocks if "bool classifyOnGpu(" in b]
    assert len(sketch) == 1
    return sketch[0]


REFERENCE_TYPES = r"""
#include "shape.h"
#include "eisenstein.h"
#include "wolkenbase_gb300.hpp"

void useReferenceTypes(wolkenbase_gb300::OctStore &st, const std::vector<wb_tile> &table)
{
  namespace wb = wolkenbase_gb300;
  xyz p(1.0, 2.0, 3.0);
  long long b = st.findBlock(p);
  std::vector<int64_t> bl = st.findBlocks(wb::Cylinder(xy(p), 0.7));
  std::vector<uint32_t> pts = st.pointsIn(wb::Hyperboloid(p, 0.2, 1.0), true);
  std::vector<uint32_t> all = st.getAll(b);
  std::map<int, size_t> cc = st.countClasses(b);
  const wb_tile *t = wb::tileAt(table, Eisenstein(1, 2));
  (void)bl; (void)pts; (void)all; (void)cc; (void)t;
}
"""


def test_adapter_and_sketch_compile_against_reference_headers(tmp_path):
    ref = os.environ.get("WB_REFERENCE_SRC", "")
    if not ref or not os.path.isfile(os.path.join(ref, "las.h")):
        pytest.skip("WB_REFERENCE_SRC does not name the reference's source tree")
    for name, code in (("sketch.cpp", _integration_sketch()), ("types.cpp", REFERENCE_TYPES)):
        src = tmp_path / name
        src.write_text(code)
        r = subprocess.run(["g++", "-std=gnu++17", "-fsyntax-only", "-D_USE_MATH_DEFINES",
                            "-I", os.path.join(ROOT, "oracle", "ref_config"), "-I", ref,
                            "-I", os.path.join(ROOT, "include"), str(src)], capture_output=True, text=True)
        assert r.returncode == 0, name + "\n" + r.stderr[-4000:]
