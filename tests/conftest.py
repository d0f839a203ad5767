import importlib.util
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_DIR = os.path.join(ROOT, "sparse-operator-graph-lu_gb300")
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


def load_package():
    """Import the package directory (its name is not a Python identifier) as soglu_gb300."""
    if "soglu_gb300" in sys.modules:
        return sys.modules["soglu_gb300"]
    spec = importlib.util.spec_from_file_location("soglu_gb300", os.path.join(PKG_DIR, "__init__.py"),
                                                  submodule_search_locations=[PKG_DIR])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["soglu_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


def build_native():
    spec = importlib.util.spec_from_file_location("soglu_build", os.path.join(PKG_DIR, "build.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    return b.build()


@pytest.fixture(scope="session")
def sg():
    build_native()
    return load_package()


@pytest.fixture(scope="session")
def wl(sg):
    import soglu_gb300.workloads as w
    return w


@pytest.fixture(scope="session")
def oracle():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as o
    o.build()
    return o


def golden(name):
    return np.load(os.path.join(GOLDEN, f"{name}.npz"))


# fixture cases: name -> generator call (must match tests/golden/make_golden.py)
def golden_cases(wl):
    def zdiag():
        s = wl.random_band(600, seed=11, band_frac=0.05)
        d = np.nonzero(s.rows == s.cols)[0]
        kill = d[(s.rows[d] % 97) == 3]
        keep = np.ones(s.nnz, bool)
        keep[kill] = False
        s.rows, s.cols, s.vals = s.rows[keep], s.cols[keep], s.vals[keep]
        s.b = s.b[0]
        return s

    return {
        "lap2d_8": lambda: wl.lap2d(8),
        "lap2d_32": lambda: wl.lap2d(32),
        "lap2d_128": lambda: wl.lap2d(128),
        "var3d_16": lambda: wl.varcoef3d(16),
        "cd_40": lambda: wl.convdiff2d(40, 5.0, 1.0, nrhs=1),
        "cd_17": lambda: wl.convdiff2d(17, 9.0, 4.0, nrhs=1),
        "band_3000": lambda: wl.random_band(3000, seed=5),
        "band_130": lambda: wl.random_band(130, seed=7),
        "zdiag_600": zdiag,
        "spd_lap2d_32": lambda: wl.spd_lower(wl.lap2d(32)),
        "spd_var3d_16": lambda: wl.spd_lower(wl.varcoef3d(16)),
        "spd_lap2d_8": lambda: wl.spd_lower(wl.lap2d(8)),
    }


def rhs_of(s):
    return s.b if s.b.ndim == 1 else s.b[0]


def gpu_available():
    try:
        import ctypes
        cudart = None
        for name in ("libcudart.so", "libcudart.so.13", "libcudart.so.12"):
            try:
                cudart = ctypes.CDLL(name)
                break
            except OSError:
                continue
        if cudart is None:
            return False
        n = ctypes.c_int(0)
        return cudart.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0
    except Exception:
        return False
