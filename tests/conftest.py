import glob
import importlib
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")


def golden_names(mode=None):
    """The golden tree cases (fixtures with a tree and a run; the loader fixture is not one)."""
    names = []
    for p in sorted(glob.glob(os.path.join(GOLDEN, "*.npz"))):
        z = np.load(p)
        if "mode" in z.files and (mode is None or str(z["mode"]) == mode):
            names.append(os.path.basename(p)[:-4])
    return names


def load_golden(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    d = {k: z[k] for k in z.files}
    model = importlib.import_module("168861_gb300.model")
    d["spec"] = model.TreeSpec.from_arrays(d)
    return d


@pytest.fixture(scope="session")
def pkg():
    return importlib.import_module("168861_gb300")


@pytest.fixture(scope="session")
def model():
    return importlib.import_module("168861_gb300.model")


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.build()
    return oracle.Oracle()


@pytest.fixture(scope="session")
def lib(pkg):
    """The CUDA library (built on demand; host-only entry points work without a GPU)."""
    build = importlib.import_module("168861_gb300.build")
    if not os.path.exists(build.LIB):
        build.build()
    return pkg.load()


@pytest.fixture(scope="session")
def gpu(lib):
    """Requires a visible CUDA device; the GPU tests have no fallback."""
    import torch
    if not torch.cuda.is_available():
        pytest.fail("the -m gpu tests need a CUDA device")
    return lib
