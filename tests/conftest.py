"""Shared fixtures.  Tests marked ``gpu`` need a CUDA device; everything else
runs on the CPU (set-up code, ABI layout, the oracle against the golden
fixtures, host-only Chebyshev routines)."""
from __future__ import annotations

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


def _has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


HAS_GPU = _has_gpu()


def pytest_collection_modifyitems(config, items):
    if HAS_GPU:
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def lib():
    from libstokes_gb300 import build as B
    B.build()
    from libstokes_gb300 import abi
    lib = abi.load()
    # report failures as Python exceptions instead of exiting the process
    lib.stokes_gpu_set_error_mode(1)
    return lib


@pytest.fixture(scope="session")
def products():
    z = np.load(os.path.join(GOLDEN, "products.npz"))
    cases = {}
    for key in z.files:
        name, field = key.split("/")
        cases.setdefault(name, {})[field] = z[key]
    return cases


@pytest.fixture(scope="session")
def nonewald():
    """Free-space cases: name -> {meta [version, rmin], pos, x, y, mat, a, slip}."""
    z = np.load(os.path.join(GOLDEN, "nonewald.npz"))
    cases = {}
    for key in z.files:
        name, field = key.split("/")
        cases.setdefault(name, {})[field] = z[key]
    return cases


def make_open_oracle(case: dict):
    from oracle.oracle import Oracle
    o = Oracle(int(case["meta"][0]), case["pos"], (1.0, 1.0, 1.0))
    if "a" in case:
        o.set_radius(case["a"])
    if "slip" in case:
        o.set_slip(case["slip"])
    o.set_misc(float(case["meta"][1]), 0, 0.0)
    return o


def make_open_system(case: dict, periodic=False):
    """An open system as stokes_init leaves it (periodic = 0, no box, no
    split); periodic=True gives the same particles in a box instead."""
    from libstokes_gb300 import System
    if periodic:
        s = System(int(case["meta"][0]), case["pos"], (30.0, 31.0, 32.0))
    else:
        s = System(int(case["meta"][0]), case["pos"], periodic=False)
    if "a" in case:
        s.set_radius(case["a"])
    if "slip" in case:
        s.set_slip(case["slip"])
    s.set_misc(float(case["meta"][1]))
    return s


@pytest.fixture(scope="session")
def setup_golden():
    return np.load(os.path.join(GOLDEN, "setup.npz"))


@pytest.fixture(scope="session")
def cheb_golden():
    return np.load(os.path.join(GOLDEN, "chebyshev.npz"))


def rel_l2(a, b) -> float:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def case_kwargs(case: dict) -> dict:
    """Decode a golden case into constructor arguments."""
    m = case["meta"]
    kw = dict(version=int(m[0]), box=(m[1], m[2], m[3]), tratio=m[4], eps=m[5],
              shear=(int(m[6]), m[7]), rmin=float(m[8]) if len(m) > 8 else 0.0,
              pos=case["pos"], a=case.get("a"), slip=case.get("slip"),
              cube=tuple(int(v) for v in case["cube"]) if "cube" in case else None)
    return kw


def make_oracle(case: dict):
    from oracle.oracle import Oracle
    kw = case_kwargs(case)
    o = Oracle(kw["version"], kw["pos"], kw["box"])
    if kw["a"] is not None:
        o.set_radius(kw["a"])
    if kw["slip"] is not None:
        o.set_slip(kw["slip"])
    o.set_split(o.xi_by_tratio(kw["tratio"]), kw["eps"])
    if kw["cube"] is not None:
        o.set_cube(*kw["cube"])
    o.set_misc(kw["rmin"], *kw["shear"])
    return o


def make_system(case: dict):
    from libstokes_gb300 import System
    kw = case_kwargs(case)
    s = System(kw["version"], kw["pos"], kw["box"], tratio=kw["tratio"], eps=kw["eps"])
    if kw["a"] is not None:
        s.set_radius(kw["a"])
    if kw["slip"] is not None:
        s.set_slip(kw["slip"])
    if kw["cube"] is not None:
        s.set_cube(*kw["cube"])
    s.set_misc(kw["rmin"], *kw["shear"])
    return s
