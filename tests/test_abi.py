"""The C-ABI library builds for sm_103a, loads, and exports every entry point
include/wolkenbase_gb300.h declares.  No GPU needed: nothing is called that
touches a device."""
import ctypes
import os
import re
import subprocess

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "wolkenbase_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:[A-Za-z_][\w ]*\*?\s*)\b(wb_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("wb_open", "wb_close", "wb_octree_build", "wb_scan_tiles", "wb_classify", "wb_classify_cloud"):
        assert must in names


def test_library_exports_every_declared_symbol(cuda_lib_path):
    lib = ctypes.CDLL(cuda_lib_path)
    for name in declared_functions():
        assert hasattr(lib, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", cuda_lib_path], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (wb_\w+)", out))
    assert set(declared_functions()) <= exported


def test_python_binding_covers_header(cuda_lib_path):
    from wolkenbase_gb300 import _lib
    assert set(declared_functions()) == set(_lib.SIGNATURES)
    _lib.load()


def test_build_targets_sm_103a_only():
    from wolkenbase_gb300 import _build
    assert _build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
    assert "-fmad=false" in _build._flags("x.cu")


def test_open_without_gpu_fails_cleanly(cuda_lib_path):
    """With no device visible, wb_open returns NULL and an error string."""
    import pytest
    from wolkenbase_gb300 import _lib
    L = _lib.load()
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    ctx = L.wb_open(0, 0)
    assert not ctx
    assert L.wb_last_error(None)
