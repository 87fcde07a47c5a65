"""A C program links the library through the header alone (the way the
reference's C++ would) and calls the host-side entry points that need no
GPU: point lengths, format join, scale combination, file names and LAS
headers.  No GPU."""
import os
import subprocess

import pytest

from conftest import ROOT

SRC = r"""
#include <stdio.h>
#include <string.h>
#include <math.h>
#include "wolkenbase_gb300.h"

int main(void)
{
  int fmts[2] = {1, 2};
  double s[6] = {0.01, 0.01, 0.01, 0.001, 0.001, 0.001}, o[6] = {500000, 4500000, 1500, 500000, 4500000, 1500};
  double comb[3];
  wb_las_output out;
  wb_las_file f;
  char name[256];
  unsigned char hdr[375];
  if (wb_las_point_length(1) != 28 || wb_las_point_length(10) != 67 || wb_las_point_length(11) != 0)
    return 1;
  if (wb_las_join_point_format(fmts, 2) != 3)
    return 2;
  if (wb_las_combine_scales(s, o, 2, comb) || comb[0] != 0.001 || comb[2] != 0.001)
    return 3;
  memset(&out, 0, sizeof out);
  memset(&f, 0, sizeof f);
  out.separate_classes = 1;
  out.points_per_file = 1000;
  out.creation_day = 1;
  out.creation_year = 2026;
  f.class_id = 2;
  f.index = 7;
  f.name_digits = 2;
  f.point_format = 6;
  f.n_points[0] = f.n_points[1] = 10;
  for (int k = 0; k < 3; k++)
  {
    f.scale[k] = 0.001;
    f.min[k] = -1;
    f.max[k] = 1;
  }
  if (wb_las_file_name(&out, &f, "cloud", name, sizeof name) || strcmp(name, "cloud-ground-07.las"))
    return 4;
  if (wb_las_header_bytes(&out, &f, hdr) || memcmp(hdr, "LASF", 4) || hdr[24] != 1 || hdr[25] != 4 || hdr[104] != 6 ||
      strcmp((const char *)hdr + 26, "EXTRACTION"))
    return 5;
  printf("ok\n");
  return 0;
}
"""


def test_c_program_links_and_runs(cuda_lib_path, tmp_path):
    src = tmp_path / "client.c"
    src.write_text(SRC)
    exe = tmp_path / "client"
    libdir = os.path.dirname(cuda_lib_path)
    r = subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe),
                        "-L" + libdir, "-lwolkenbase_gb300", "-Wl,-rpath," + libdir, "-lm"],
                       capture_output=True, text=True)
    if r.returncode != 0:
        pytest.fail(r.stderr)
    run = subprocess.run([str(exe)], capture_output=True, text=True)
    assert run.returncode == 0 and run.stdout.strip() == "ok", (run.returncode, run.stdout, run.stderr)
