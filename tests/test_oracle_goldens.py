"""Pins the CPU oracle against every golden vector of the reference test
suite (test/runtests.jl) at the reference's tolerance, and against the
reference's own 1D model (src/Analytical1D.py, committed fixture)."""
import math
import os

import numpy as np
import pytest

from oracle import bf_oracle as O
from tests.golden import reference_goldens as G

HERE = os.path.dirname(os.path.abspath(__file__))
DISKR = 0.15
DEPS = np.arange(0, 3 * math.pi, 1.0)          # test/runtests.jl:57 (0:1.:3pi)


def _isapprox(a, b, rtol=G.RTOL):
    a = np.asarray(a); b = np.asarray(b)
    return np.linalg.norm((a - b).ravel()) <= rtol * max(np.linalg.norm(a.ravel()), np.linalg.norm(b.ravel()))


def _distance(deps):
    return np.array([0.0, math.pi * 3e-2 / (2 * math.pi), deps * 1e-2 / (2 * math.pi), 0.0])


@pytest.fixture(scope="module")
def coords():
    return O.seed_coordinate_system()          # X = Y = -0.5:0.01:0.5


def _eps_stack():
    return np.array([np.nan, 1, 9, 1], dtype=complex), np.array([0.0, 0.15, 0.15 / math.sqrt(9), 0.0]) * 1e-2


def test_grid_and_kspace(coords):
    assert len(coords.X) == 101 and coords.X[50] == 0.0 and coords.X[0] == -0.5
    # dk = 2pi / (2 max X) (src/boost_fractor.jl:43), not 2pi/(N dx)
    assert math.isclose(coords.kX[1] - coords.kX[0], 2 * math.pi, rel_tol=1e-12)
    assert np.allclose(coords.kX, -coords.kX[::-1], rtol=0, atol=1e-12)


def test_gauss_and_match(coords):
    g = O.gauss_profile(coords, z=1e-9, omega0=0.097, f=22e9)
    assert _isapprox(g.flatten(order="F")[3999], G.GAUSS_4000)           # :47
    dx = 0.0001 * math.floor(10000.0 * (coords.X[1] - coords.X[0]))
    m = O.unnormalized_match(g, 3 * g, dx=dx, dy=dx)
    assert _isapprox(m, G.MATCH)                                         # :52


def test_seed_setup_boundaries_defaults(coords):
    sb = O.seed_setup_boundaries(coords, diskno=1)
    assert np.allclose(sb.distance, [0, 8e-3, 1e-3, 0])
    assert np.isnan(sb.eps[0].real) and sb.eps[2] == 9
    assert np.signbit(sb.eps[1].imag)                                    # real eps -> re - 0.0im
    assert np.allclose(sb.r, [1, -0.5, 0.5])                             # Fresnel, r1 = 1
    with pytest.raises(ValueError):
        O.seed_setup_boundaries(coords, diskno=1, distance=[0, 1, 0])


def test_cheerleader_golden(coords):
    sb = O.seed_setup_boundaries(coords, diskno=1)                       # :38
    out = []
    for d in DEPS:
        sb.distance = _distance(d)                                       # :65
        E = O.cheerleader(0, 100, sb, coords, prop=O.propagator, f=10e9, diskR=DISKR)
        out.append(np.sum(np.abs(E) ** 2) * 0.01 * 0.01 / (math.pi * DISKR ** 2))
    assert _isapprox(out, G.CHEERLEADER_BETA2)                           # :211


def test_dancer_golden(coords):
    eps, dist = _eps_stack()
    sb = O.seed_setup_boundaries(coords, diskno=1, distance=dist, epsilon=eps)
    out = []
    for d in DEPS:
        sb.distance = _distance(d)
        E = O.dancer(0, 200, sb, coords, prop=O.propagator1d, f=10e9, diskR=DISKR)
        out.append(np.sum(np.abs(E) ** 2) * 0.01 * 0.01 / (math.pi * DISKR ** 2))
    assert _isapprox(out, G.DANCER_BETA2)                                # :214


def test_transformer_modes_propmat_traceback(coords):
    eps, dist = _eps_stack()
    sb = O.seed_setup_boundaries(coords, diskno=1, distance=dist, epsilon=eps)
    modes = O.seed_modes(coords, ThreeDim=True, Mmax=10, Lmax=0, diskR=DISKR)
    out = []
    for d in DEPS:
        sb.distance = _distance(d)
        b = O.transformer(sb, coords, modes, prop=O.propagator, f=10e9, diskR=DISKR)
        out.append(np.sum(np.abs(b) ** 2))
    assert _isapprox(out, G.TRANSFORMER_BETA2)                           # :217
    fld = O.modes2field(O.field2modes(None, coords, modes, diskR=DISKR), coords, modes)
    assert _isapprox(fld.flatten(order="F")[4999], G.MODES_FIELD_5000)   # :168
    # transformer() replaced eps NaN by 1e30 in place (src/boost_fractor_transformer.jl:289)
    assert sb.eps[0] == 1e30
    pm = O.calc_propagation_matrices(sb, coords, modes)
    assert _isapprox(pm[0][3, 5], G.PROPMAT_1_4_6)                       # :171

    c1 = O.seed_coordinate_system(X=np.array([1e-7]), Y=np.array([1e-7]))
    sb1 = O.seed_setup_boundaries(c1, diskno=1, distance=dist, epsilon=eps)
    m1 = O.seed_modes(c1, ThreeDim=False, Mmax=1, Lmax=0, diskR=DISKR)
    res = []
    for d in DEPS:
        sb1.distance = _distance(d)
        res.append(O.transformer(sb1, c1, m1, prop=O.propagator1d, f=10e9, diskR=DISKR)[0])
    ff = O.transformer_trace_back(res[4], 0, sb1, c1, m1, prop=O.propagator1d, f=10e9)
    assert _isapprox(ff[:, :, 0], np.array(G.TRACE_BACK))                # :221


def test_transformer_1d_vs_reference_analytical1d():
    """The reference's own 1D model (src/Analytical1D.py:79-131) vs the oracle 1D transformer."""
    d = np.load(os.path.join(HERE, "golden", "analytical1d.npz"))
    c1 = O.seed_coordinate_system(X=np.array([1e-7]), Y=np.array([1e-7]))
    m1 = O.seed_modes(c1, ThreeDim=False)
    for k in range(int(d["ncases"])):
        nd, eps_d, spac, freqs, gold = int(d[f"nd_{k}"]), float(d[f"eps_{k}"]), d[f"spacings_{k}"], d[f"freqs_{k}"], d[f"beta2_{k}"]
        dist, eps = [0.0], [np.nan]
        for i in range(nd):
            dist += [spac[i], 1e-3]
            eps += [1.0, eps_d]
        dist += [0.0]; eps += [1.0]
        got = []
        for f in freqs:
            sb = O.seed_setup_boundaries(c1, diskno=nd, distance=np.array(dist), epsilon=np.array(eps, dtype=complex))
            got.append(abs(O.transformer(sb, c1, m1, prop=O.propagator1d, f=f)[0]) ** 2)
        # mirror modelled as eps=1e20 there and 1e30 here: agreement ~1e-8
        assert np.allclose(got, gold, rtol=1e-6), k
