import glob
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN_DIR = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and the built libebsdgpu.so")


def golden_names():
    """Band-detection golden cases (NLPAR, orientation and voting fixtures are separate)."""
    return sorted(n for n in (os.path.splitext(os.path.basename(p))[0]
                              for p in glob.glob(os.path.join(GOLDEN_DIR, "*.npz")))
                  if not n.startswith(("nlpar", "orient_", "vote_")))


def vote_golden_names():
    return sorted(os.path.splitext(os.path.basename(p))[0]
                  for p in glob.glob(os.path.join(GOLDEN_DIR, "vote_*.npz")))


def nlpar_golden_names():
    return sorted(os.path.splitext(os.path.basename(p))[0]
                  for p in glob.glob(os.path.join(GOLDEN_DIR, "nlpar_*.npz")))  # not nlparlam_*


def load_golden(name):
    d = np.load(os.path.join(GOLDEN_DIR, name + ".npz"))
    case = {k: d[k] for k in d.files}
    case["params"] = json.loads(str(d["params"]))
    case["name"] = name
    return case


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def built_lib():
    """Build libebsdgpu.so once per session (nvcc cross-compiles without a GPU)."""
    from pyebsdindex_gb300 import _build
    return _build.build()


@pytest.fixture(scope="session")
def cuda(built_lib):
    if not gpu_available():
        pytest.skip("no CUDA device")
    import torch
    torch.cuda.init()
    return torch.device("cuda:0")
