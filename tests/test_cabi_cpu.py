"""CPU-only checks of the C ABI: the library loads, exports every symbol that
include/*.h declares, and its host-side helpers (no GPU work) agree with the
oracle.  No compute call is made here."""
import glob
import os
import re

import numpy as np
import pytest

from oracle import bf_oracle as O

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def L():
    import build as _b  # boostfractor.jl_gb300/build.py (on sys.path via conftest)
    _b.build()
    from bfgb300 import _lib
    return _lib.lib()


def _declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(REPO, "include", "*.h")):
        txt = open(h).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        names |= set(re.findall(r"\b(bf_[a-z0-9_]+)\s*\(", txt))
    return names


def test_exports_every_declared_symbol(L):
    declared = _declared_symbols()
    assert declared, "no declarations found"
    missing = [n for n in sorted(declared) if not hasattr(L, n)]
    assert not missing, missing
    from bfgb300 import _lib
    assert set(_lib.symbols()) >= declared


def test_version(L):
    assert L.bf_version() >= 100


def test_create_without_gpu_fails_cleanly(L):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import ctypes
    h = ctypes.c_void_p()
    rc = L.bf_create(0, 0, ctypes.byref(h))
    assert rc != 0 and not h.value


def test_kspace_helper_matches_oracle(L):
    import bfgb300 as B
    for X in (O.decimal_grid(-50, 50, 100), np.array([1e-7]), np.linspace(-0.5, 0.5, 64)):
        got = B.get_kspace_coords(X)
        ref = O.get_kspace_coords(X)
        assert np.max(np.abs(got - ref) / np.maximum(1e-300, np.abs(ref).max())) < 1e-15


def test_gauss_profile_matches_golden_and_oracle(L):
    """bf_gauss_profile (host FP64) against test/runtests.jl:47 and the oracle."""
    import bfgb300 as B
    from tests.golden import reference_goldens as G
    c, co = B.SeedCoordinateSystem(), O.seed_coordinate_system()
    g = B.gauss_profile(c, z=1e-9, omega0=0.097, f=22e9)
    got = g.flatten(order="F")[3999]
    assert abs(got - G.GAUSS_4000) / abs(G.GAUSS_4000) < G.RTOL
    for z, w0, f in ((1e-9, 0.097, 22e9), (0.3, 0.05, 19e9)):
        ref = O.gauss_profile(co, z=z, omega0=w0, f=f)
        got = B.gauss_profile(c, z=z, omega0=w0, f=f)
        assert np.max(np.abs(got - ref)) / np.max(np.abs(ref)) < 1e-13


def test_seed_setup_boundaries_matches_oracle(L):
    import bfgb300 as B
    c = B.SeedCoordinateSystem()
    co = O.seed_coordinate_system()
    for kw in (dict(diskno=1), dict(diskno=3),
               dict(diskno=2, epsilon=[np.nan, 1, 24, 1, 9.4, 1], distance=[0, 1e-3, 2e-3, 3e-3, 4e-3, 0])):
        a = B.SeedSetupBoundaries(c, **kw)
        b = O.seed_setup_boundaries(co, **kw)
        assert np.allclose(a.r, b.r, rtol=1e-15) and np.allclose(a.distance, b.distance)
        assert np.array_equal(np.signbit(a.eps.imag), np.signbit(b.eps.imag))
    with pytest.raises(ValueError):
        B.SeedSetupBoundaries(c, diskno=1, distance=[0, 1, 0])


def test_workloads_are_seeded():
    from bfgb300 import workloads as W
    a, b = W.config2_cheerleader(), W.config2_cheerleader()
    assert np.array_equal(a["distance"], b["distance"]) and len(a["freqs"]) == 256
    assert len(a["distance"]) == 42 and a["nmax"] == 400
    assert np.all((a["distance"][1:-1:2] >= 7.5e-3) & (a["distance"][1:-1:2] <= 8.5e-3))
    X = W.symmetric_grid(128)
    assert np.array_equal(X, -X[::-1]) and X[0] == -0.5 and X[-1] == 0.5
