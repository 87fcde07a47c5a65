"""The ctypes mirror of every struct in include/wolkenbase_gb300.h has the C
layout: size and field offsets as gcc lays them out on this host.  No GPU."""
import ctypes as C
import os
import subprocess

import pytest

from conftest import ROOT


def _structs():
    from wolkenbase_gb300 import _lib
    return {
        "wb_params": _lib.wb_params,
        "wb_cloud": _lib.wb_cloud,
        "wb_octree_stats": _lib.wb_octree_stats,
        "wb_tile": _lib.wb_tile,
        "wb_server_config": _lib.wb_server_config,
        "wb_job": _lib.wb_job,
        "wb_job_status": _lib.wb_job_status,
        "wb_server_stats": _lib.wb_server_stats,
        "wb_las_points": _lib.wb_las_points,
        "wb_las_output": _lib.wb_las_output,
        "wb_las_file": _lib.wb_las_file,
    }


def test_struct_layouts_match_header(tmp_path):
    structs = _structs()
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "wolkenbase_gb300.h"', "int main(void) {"]
    for name, cls in structs.items():
        lines.append(f'printf("{name} size %zu\\n", sizeof({name}));')
        for f, _ in cls._fields_:
            lines.append(f'printf("{name} {f} %zu\\n", offsetof({name}, {f}));')
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    r = subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    if r.returncode != 0:
        pytest.fail(r.stderr)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {}
    for line in out:
        if line:
            a, b, v = line.split()
            got[(a, b)] = int(v)
    for name, cls in structs.items():
        assert got[(name, "size")] == C.sizeof(cls), name
        for f, _ in cls._fields_:
            assert got[(name, f)] == getattr(cls, f).offset, (name, f)
