import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def cuda_lib_path():
    from wolkenbase_gb300 import _build
    return _build.build()


@pytest.fixture(scope="session")
def classifier(cuda_lib_path):
    import wolkenbase_gb300 as wb
    c = wb.Classifier(0)
    yield c
    c.close()


def load_golden(name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    return {k: d[k] for k in d.files}


def golden_cloud(g):
    from wolkenbase_gb300 import synth
    return synth.Cloud(g["xyz"], tuple(g["scale"]), tuple(g["offset"]), float(g["unit"]), tuple(g["minc"]),
                       tuple(g["maxc"]))


def golden_params(g):
    p = g["params"]
    return dict(tile_size=float(p[0]), max_slope=float(p[1]), thickness=float(p[2]), min_hyp_size=float(p[3]))


GOLDEN_CASES = ["tile20k", "params6k", "utm8k", "dups5k", "split"]
