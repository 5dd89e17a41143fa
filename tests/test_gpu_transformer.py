"""GPU parity of the transformer path (mode basis, propagation matrices,
transfer-matrix chain, FP64 boundary solve) against the CPU oracle and the
reference's golden vectors.

Tolerances: FP64 path 1e-10 relative; mixed path 1e-4 relative in beta^2.
"""
import math
import os

import numpy as np
import pytest

from oracle import bf_oracle as O
from tests.golden import reference_goldens as G

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
FP64_TOL = 1e-10
MIXED_BETA2_TOL = 1e-4
DEPS = np.arange(0, 3 * math.pi, 1.0)


@pytest.fixture(scope="module")
def B():
    import build as _b
    _b.build()
    import bfgb300
    return bfgb300


def rel(a, b):
    a = np.asarray(a); b = np.asarray(b)
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


def _dist(d):
    return np.array([0.0, math.pi * 3e-2 / (2 * math.pi), d * 1e-2 / (2 * math.pi), 0.0])


def test_modes_match_oracle(B):
    from bfgb300 import workloads as W
    X = W.symmetric_grid(48)
    cb = B.SeedCoordinateSystem(X=X, Y=X)
    co = O.seed_coordinate_system(X=X, Y=X)
    mb = B.SeedModes(cb, ThreeDim=True, Mmax=4, Lmax=2, diskR=0.15)
    mo = O.seed_modes(co, ThreeDim=True, Mmax=4, Lmax=2, diskR=0.15)
    assert rel(mb.mode_patterns, mo.mode_patterns) < 1e-12
    assert rel(mb.mode_kt, mo.mode_kt) < 1e-13


def test_transformer_goldens_on_gpu(B):
    """test/runtests.jl:122-171,217 through the GPU (FP64 path)."""
    c = B.SeedCoordinateSystem()
    eps = np.array([np.nan, 1, 9, 1], dtype=complex)
    sb = B.SeedSetupBoundaries(c, diskno=1, distance=np.array([0, 0.15, 0.05, 0]) * 1e-2, epsilon=eps)
    modes = B.SeedModes(c, ThreeDim=True, Mmax=10, Lmax=0, diskR=0.15)
    out = []
    for d in DEPS:
        sb.distance = _dist(d)
        b = B.transformer(sb, c, modes, prop=B.propagator, f=10e9, diskR=0.15)
        out.append(np.sum(np.abs(b) ** 2))
    assert rel(out, G.TRANSFORMER_BETA2) < G.RTOL
    fld = B.modes2field(B.field2modes(None, c, modes, diskR=0.15), c, modes)
    assert abs(fld.flatten(order="F")[4999] - G.MODES_FIELD_5000) / abs(G.MODES_FIELD_5000) < G.RTOL
    assert sb.eps[0] == 1e30                     # mutated like the reference (:289)
    pm = B.calc_propagation_matrices(sb, c, modes)
    assert abs(pm[0][3, 5] - G.PROPMAT_1_4_6) / abs(G.PROPMAT_1_4_6) < G.RTOL


def test_trace_back_golden_on_gpu(B):
    """test/runtests.jl:196-207,221: 1D transformer over the Deps scan, then
    transformer_trace_back of the 5th solution, through the GPU."""
    eps = np.array([np.nan, 1, 9, 1], dtype=complex)
    c1 = B.SeedCoordinateSystem(X=np.array([1e-7]), Y=np.array([1e-7]))
    sb1 = B.SeedSetupBoundaries(c1, diskno=1, distance=_dist(0.0), epsilon=eps)
    m1 = B.SeedModes(c1, ThreeDim=False, Mmax=1, Lmax=0, diskR=0.15)
    res = []
    for d in DEPS:
        sb1.distance = _dist(d)
        res.append(B.transformer(sb1, c1, m1, prop=B.propagator1D, f=10e9, diskR=0.15))
    ff = B.transformer_trace_back(res[4], 0, sb1, c1, m1, prop=B.propagator1D, f=10e9)
    assert rel(ff[:, :, 0], np.array(G.TRACE_BACK)) < G.RTOL


@pytest.mark.parametrize("axion", [False, True])
def test_trace_back_3d_vs_oracle(B, axion):
    """transformer_trace_back (transformer.jl:372-421) with L = 1 modes, tilted
    disks and surface maps: FP64 within 1e-10 of the oracle, mixed within 1e-4."""
    distance, eps, tx, ty, X, s = _stack(2, 40, seed=13, surf=True)
    kw = dict(diskno=2, distance=distance, epsilon=eps, relative_tilt_x=tx, relative_tilt_y=ty,
              relative_surfaces=s)
    cb, co = B.SeedCoordinateSystem(X=X, Y=X), O.seed_coordinate_system(X=X, Y=X)
    mb = B.SeedModes(cb, ThreeDim=True, Mmax=3, Lmax=1, diskR=0.15)
    mo = O.seed_modes(co, ThreeDim=True, Mmax=3, Lmax=1, diskR=0.15)
    nm = mo.nm
    rng = np.random.default_rng(14)
    refl = rng.standard_normal(nm) + 1j * rng.standard_normal(nm)
    inp = rng.standard_normal(nm) + 1j * rng.standard_normal(nm)
    sbo = O.seed_setup_boundaries(co, **kw)
    sbo.eps[0] = 1e30          # a boundary set the transformer already mutated (transformer.jl:289)
    ref = O.transformer_trace_back(refl, inp, sbo, co, mo, inlcudes_axion=axion, f=20.1e9)
    sbb = B.SeedSetupBoundaries(cb, **kw)
    sbb.eps[0] = 1e30
    got = B.transformer_trace_back(refl, inp, sbb, cb, mb, inlcudes_axion=axion, f=20.1e9)
    assert got.shape == ref.shape == (len(distance), 2, nm)
    assert rel(got, ref) < FP64_TOL
    got32 = B.transformer_trace_back(refl, inp, sbb, cb, mb, inlcudes_axion=axion, f=20.1e9, precision="mixed")
    assert rel(got32, ref) < 1e-4


def _stack(ndisk, n, seed, tilt_air=False, surf=False):
    from bfgb300 import workloads as W
    rng = np.random.default_rng(seed)
    nd = 2 * ndisk + 2
    tx = np.zeros(nd); ty = np.zeros(nd)
    for k in range(ndisk):
        tx[2 + 2 * k] = rng.uniform(-5e-4, 5e-4)
        ty[2 + 2 * k] = rng.uniform(-5e-4, 5e-4)
    if tilt_air:
        tx[1] = 3e-4
    distance, eps, tx, ty = W.booster(ndisk, rng.uniform(7.5e-3, 8.5e-3, ndisk), tilt_x=tx, tilt_y=ty)
    X = W.symmetric_grid(n)
    s = None
    if surf:
        s = np.zeros((nd, n, n))
        for k in range(ndisk):
            s[2 + 2 * k] = 1e-5 * rng.standard_normal((n, n))
    return distance, eps, tx, ty, X, s


@pytest.mark.parametrize("n,ndisk,M,L,tilt_air,surf", [(32, 1, 4, 0, False, False), (48, 2, 3, 1, False, True),
                                                       (32, 2, 3, 0, True, False)])
def test_transformer_fp64_vs_oracle(B, n, ndisk, M, L, tilt_air, surf):
    distance, eps, tx, ty, X, s = _stack(ndisk, n, seed=n + M, tilt_air=tilt_air, surf=surf)
    kw = dict(diskno=ndisk, distance=distance, epsilon=eps, relative_tilt_x=tx, relative_tilt_y=ty)
    if s is not None:
        kw["relative_surfaces"] = s
    cb, co = B.SeedCoordinateSystem(X=X, Y=X), O.seed_coordinate_system(X=X, Y=X)
    mb = B.SeedModes(cb, ThreeDim=True, Mmax=M, Lmax=L, diskR=0.15)
    mo = O.seed_modes(co, ThreeDim=True, Mmax=M, Lmax=L, diskR=0.15)
    for f in (19.6e9, 20.4e9):
        sbb, sbo = B.SeedSetupBoundaries(cb, **kw), O.seed_setup_boundaries(co, **kw)
        rng = np.random.default_rng(1)
        refl_in = rng.standard_normal(mb.nm) + 1j * rng.standard_normal(mb.nm)
        ref_b, ref_r = O.transformer(sbo, co, mo, f=f, reflect=refl_in)
        got_b, got_r = B.transformer(sbb, cb, mb, f=f, reflect=refl_in)
        assert rel(got_b, ref_b) < FP64_TOL and rel(got_r, ref_r) < FP64_TOL
        pmo = O.calc_propagation_matrices(sbo, co, mo, f=f)
        pmb = B.calc_propagation_matrices(sbb, cb, mb, f=f)
        for j in range(1, len(pmo)):
            assert rel(pmb[j], pmo[j]) < FP64_TOL, j


def test_transformer_batched_mixed_and_injected(B):
    distance, eps, tx, ty, X, s = _stack(3, 64, seed=7, surf=True)
    kw = dict(diskno=3, distance=distance, epsilon=eps, relative_tilt_x=tx, relative_tilt_y=ty,
              relative_surfaces=s)
    cb, co = B.SeedCoordinateSystem(X=X, Y=X), O.seed_coordinate_system(X=X, Y=X)
    mb = B.SeedModes(cb, ThreeDim=True, Mmax=6, Lmax=0, diskR=0.15)
    mo = O.seed_modes(co, ThreeDim=True, Mmax=6, Lmax=0, diskR=0.15)
    freqs = np.linspace(19.5e9, 20.5e9, 5)
    b64 = B.transformer(B.SeedSetupBoundaries(cb, **kw), cb, mb, f=freqs)
    b32 = B.transformer(B.SeedSetupBoundaries(cb, **kw), cb, mb, f=freqs, precision="mixed")
    for k, f in enumerate(freqs):
        ref = O.transformer(O.seed_setup_boundaries(co, **kw), co, mo, f=f)
        assert rel(b64[k], ref) < FP64_TOL
        r2 = np.sum(np.abs(ref) ** 2)
        assert abs(np.sum(np.abs(b32[k]) ** 2) - r2) / r2 < MIXED_BETA2_TOL
    # injected matrices (transformer.jl:335-337) give the same boost
    sbo = O.seed_setup_boundaries(co, **kw)
    sbo.eps[0] = 1e30
    pm = O.calc_propagation_matrices(sbo, co, mo, f=freqs[2])
    got = B.transformer(B.SeedSetupBoundaries(cb, **kw), cb, mb, f=freqs[2], propagation_matrices=pm)
    assert rel(got, O.transformer(O.seed_setup_boundaries(co, **kw), co, mo, f=freqs[2], propagation_matrices=pm)) < FP64_TOL


@pytest.mark.parametrize("prec", ["mixed", "mixed-simt"])
@pytest.mark.parametrize("M,L,n", [(5, 2, 32), (8, 2, 64)])
def test_transformer_mixed_mid_mode_counts(B, M, L, n, prec):
    """Mixed path at 25 and 40 modes: the register-resident complex64 inverses
    (padded to 32 and 64; the 32-pixel case has propagation matrices of
    condition ~100, so pivoting matters) and the real-row pixel-class GEMM, on
    the tensor cores (mixed) and on the SIMT pipes (mixed-simt).  beta^2
    within 1e-4 of the oracle."""
    distance, eps, tx, ty, X, s = _stack(2, n, seed=M, surf=True)
    kw = dict(diskno=2, distance=distance, epsilon=eps, relative_tilt_x=tx, relative_tilt_y=ty,
              relative_surfaces=s)
    cb, co = B.SeedCoordinateSystem(X=X, Y=X), O.seed_coordinate_system(X=X, Y=X)
    mb = B.SeedModes(cb, ThreeDim=True, Mmax=M, Lmax=L, diskR=0.15)
    mo = O.seed_modes(co, ThreeDim=True, Mmax=M, Lmax=L, diskR=0.15)
    assert mb.nm == M * (2 * L + 1)
    freqs = np.array([19.6e9, 20.3e9])
    b32 = B.transformer(B.SeedSetupBoundaries(cb, **kw), cb, mb, f=freqs, precision=prec)
    for k, f in enumerate(freqs):
        ref = O.transformer(O.seed_setup_boundaries(co, **kw), co, mo, f=f)
        r2 = np.sum(np.abs(ref) ** 2)
        assert abs(np.sum(np.abs(b32[k]) ** 2) - r2) / r2 < MIXED_BETA2_TOL
        assert rel(b32[k], ref) < 1e-3


@pytest.mark.parametrize("prec", ["mixed", "mixed-simt"])
@pytest.mark.parametrize("cut", [0.15, 0.3])
def test_transformer_mixed_modes_inside_and_beyond_mask(B, cut, prec):
    """Laguerre-Gauss pattern_input cut at r <= 0.15 m (inside the 0.15 m disk
    mask: the k-space overlaps are Hermitian in the mode pair and the mixed
    path runs their upper triangle as real rows, on the tensor cores) and at
    r <= 0.3 m (non-zero outside the mask: the full complex overlap GEMM on the
    SIMT pipes).  Mixed beta^2 within 1e-4 of the oracle either way."""
    from bfgb300 import workloads as W
    distance, eps, tx, ty, _, _ = _stack(3, 64, seed=53, tilt_air=True)
    X = W.symmetric_grid(64, width=0.4)
    pats, kt = W.lg_modes(X, X, 20, 0.05, cut)
    kw = dict(diskno=3, distance=distance, epsilon=eps, relative_tilt_x=tx, relative_tilt_y=ty)
    cb, co = B.SeedCoordinateSystem(X=X, Y=X), O.seed_coordinate_system(X=X, Y=X)
    mb = B.SeedModes(cb, ThreeDim=True, Mmax=20, Lmax=0, diskR=0.15, pattern_input=pats, kT_arr=kt)
    mo = O.seed_modes(co, ThreeDim=True, Mmax=20, Lmax=0, diskR=0.15, pattern_input=pats, kT_arr=kt)
    outside = (X[:, None] ** 2 + X[None, :] ** 2) >= 0.15 ** 2
    assert np.any(np.abs(pats[:, 0, :, :, 0][:, outside]) > 0) == (cut > 0.15)
    freqs = np.array([19.4e9, 20.7e9])
    b32 = B.transformer(B.SeedSetupBoundaries(cb, **kw), cb, mb, f=freqs, precision=prec)
    for k, f in enumerate(freqs):
        ref = O.transformer(O.seed_setup_boundaries(co, **kw), co, mo, f=f)
        r2 = np.sum(np.abs(ref) ** 2)
        assert abs(np.sum(np.abs(b32[k]) ** 2) - r2) / r2 < MIXED_BETA2_TOL


def test_transformer_lg_pattern_input_vs_oracle(B):
    """Laguerre-Gauss modes through pattern_input/kT_arr (transformer.jl:46,
    :99-104) on a reduced stack with surface maps: FP64 boost within 1e-10,
    mixed beta^2 within 1e-4."""
    from bfgb300 import workloads as W
    distance, eps, tx, ty, _, _ = _stack(4, 64, seed=41)
    X = W.symmetric_grid(64, width=0.4)
    rng = np.random.default_rng(42)
    nd = len(distance)
    s = np.zeros((nd, 64, 64))
    s[2:nd - 1:2] = W.surface_roughness(X, X, 4, rng)
    pats, kt = W.lg_modes(X, X, 16, 0.03, 0.15)
    kw = dict(diskno=4, distance=distance, epsilon=eps, relative_tilt_x=tx, relative_tilt_y=ty,
              relative_surfaces=s)
    cb, co = B.SeedCoordinateSystem(X=X, Y=X), O.seed_coordinate_system(X=X, Y=X)
    mb = B.SeedModes(cb, ThreeDim=True, Mmax=16, Lmax=0, diskR=0.15, pattern_input=pats, kT_arr=kt)
    mo = O.seed_modes(co, ThreeDim=True, Mmax=16, Lmax=0, diskR=0.15, pattern_input=pats, kT_arr=kt)
    freqs = np.array([19.2e9, 20.0e9, 20.9e9])
    b64 = B.transformer(B.SeedSetupBoundaries(cb, **kw), cb, mb, f=freqs)
    b32 = B.transformer(B.SeedSetupBoundaries(cb, **kw), cb, mb, f=freqs, precision="mixed")
    for k, f in enumerate(freqs):
        ref = O.transformer(O.seed_setup_boundaries(co, **kw), co, mo, f=f)
        assert rel(b64[k], ref) < FP64_TOL
        r2 = np.sum(np.abs(ref) ** 2)
        assert abs(np.sum(np.abs(b32[k]) ** 2) - r2) / r2 < MIXED_BETA2_TOL


def test_transformer_full_size_lg_vs_oracle_fixture(B):
    """The full transformer workload (20 disks with surface maps, 64
    Laguerre-Gauss modes, 256x256) at three of its frequencies against the
    oracle's boost stored by tests/golden/make_c3_fixture.py: FP64 within 1e-10,
    mixed beta^2 within 1e-4 (tensor-core and SIMT overlap GEMMs)."""
    import os
    from bfgb300 import workloads as W
    fx = np.load(os.path.join(os.path.dirname(__file__), "golden", "c3_lg_oracle.npz"))
    w = W.config3_transformer()
    assert np.array_equal(w["freqs"][fx["freq_index"]], fx["freqs"])
    c = B.SeedCoordinateSystem(X=w["X"], Y=w["Y"])
    kw = dict(diskno=(len(w["distance"]) - 2) // 2, distance=w["distance"], epsilon=w["eps"],
              relative_tilt_x=w["relative_tilt_x"], relative_tilt_y=w["relative_tilt_y"],
              relative_surfaces=w["relative_surfaces"])
    m = B.SeedModes(c, ThreeDim=True, Mmax=w["M"], Lmax=w["L"], diskR=w["diskR"],
                    pattern_input=w["pattern_input"], kT_arr=w["kT_arr"])
    b64 = B.transformer(B.SeedSetupBoundaries(c, **kw), c, m, f=fx["freqs"], diskR=w["diskR"])
    b32 = B.transformer(B.SeedSetupBoundaries(c, **kw), c, m, f=fx["freqs"], diskR=w["diskR"], precision="mixed")
    bs = B.transformer(B.SeedSetupBoundaries(c, **kw), c, m, f=fx["freqs"], diskR=w["diskR"],
                       precision="mixed-simt")
    for k in range(len(fx["freqs"])):
        assert rel(b64[k], fx["boost"][k]) < FP64_TOL
        assert abs(np.sum(np.abs(b32[k]) ** 2) - fx["beta2"][k]) / fx["beta2"][k] < MIXED_BETA2_TOL
        assert abs(np.sum(np.abs(bs[k]) ** 2) - fx["beta2"][k]) / fx["beta2"][k] < MIXED_BETA2_TOL


def _lg_reduced(B):
    from bfgb300 import workloads as W
    distance, eps, tx, ty, _, _ = _stack(4, 64, seed=41)
    X = W.symmetric_grid(64, width=0.4)
    rng = np.random.default_rng(42)
    nd = len(distance)
    s = np.zeros((nd, 64, 64))
    s[2:nd - 1:2] = W.surface_roughness(X, X, 4, rng)
    pats, kt = W.lg_modes(X, X, 16, 0.03, 0.15)
    kw = dict(diskno=4, distance=distance, epsilon=eps, relative_tilt_x=tx, relative_tilt_y=ty,
              relative_surfaces=s)
    cb = B.SeedCoordinateSystem(X=X, Y=X)
    mb = B.SeedModes(cb, ThreeDim=True, Mmax=16, Lmax=0, diskR=0.15, pattern_input=pats, kT_arr=kt)
    return cb, mb, kw


def test_tf32_propagation_matrices_vs_fp64(B):
    """BF_PREC_TF32: the overlap GEMMs on the tensor cores (split TF32).  Every
    propagation matrix within 1e-4 (relative, Frobenius) of the FP64 path; a
    layout or descriptor error would show as O(1)."""
    cb, mb, kw = _lg_reduced(B)
    freqs = np.array([19.3e9, 20.6e9])
    p64 = B.calc_propagation_matrices(B.SeedSetupBoundaries(cb, **kw), cb, mb, f=freqs)
    p32 = B.calc_propagation_matrices(B.SeedSetupBoundaries(cb, **kw), cb, mb, f=freqs, precision="tf32")
    for f in range(len(freqs)):
        for j in range(1, len(kw["distance"])):
            assert rel(p32[f][j], p64[f][j]) < 1e-4, (f, j)


def test_tf32_transformer_full_size_vs_oracle_fixture(B):
    """BF_PREC_TF32 on the full transformer workload: the overlap GEMMs on the
    tensor cores (accumulator drained every 32 K-elements, operands less their
    centre value) keep beta^2 within the 1e-4 bar of the oracle."""
    import os
    from bfgb300 import workloads as W
    fx = np.load(os.path.join(os.path.dirname(__file__), "golden", "c3_lg_oracle.npz"))
    w = W.config3_transformer()
    c = B.SeedCoordinateSystem(X=w["X"], Y=w["Y"])
    kw = dict(diskno=(len(w["distance"]) - 2) // 2, distance=w["distance"], epsilon=w["eps"],
              relative_tilt_x=w["relative_tilt_x"], relative_tilt_y=w["relative_tilt_y"],
              relative_surfaces=w["relative_surfaces"])
    m = B.SeedModes(c, ThreeDim=True, Mmax=w["M"], Lmax=w["L"], diskR=w["diskR"],
                    pattern_input=w["pattern_input"], kT_arr=w["kT_arr"])
    b = B.transformer(B.SeedSetupBoundaries(c, **kw), c, m, f=fx["freqs"], diskR=w["diskR"], precision="tf32")
    for k in range(len(fx["freqs"])):
        assert abs(np.sum(np.abs(b[k]) ** 2) - fx["beta2"][k]) / fx["beta2"][k] < MIXED_BETA2_TOL


def test_tf32_bounded_wait_times_out(B):
    """The tensor-core GEMM's mbarrier waits are bounded: with the operand
    copies withheld (a test hook; nothing is read or written that a normal
    launch would not touch), the MMA warp's wait runs out after ~2 s, the
    solve returns BF_ERR_TIMEOUT, and the next solve on the same handle is
    correct again."""
    from bfgb300 import _lib
    cb, mb, kw = _lg_reduced(B)
    freqs = np.array([19.7e9])
    ok = B.calc_propagation_matrices(B.SeedSetupBoundaries(cb, **kw), cb, mb, f=freqs, precision="tf32")
    L = _lib.lib()
    L.bf_test_tc_withhold_loads(1)
    try:
        with pytest.raises(B.BFError) as e:
            B.calc_propagation_matrices(B.SeedSetupBoundaries(cb, **kw), cb, mb, f=freqs, precision="tf32")
    finally:
        L.bf_test_tc_withhold_loads(0)
    assert e.value.code == _lib.BF_ERR_TIMEOUT
    again = B.calc_propagation_matrices(B.SeedSetupBoundaries(cb, **kw), cb, mb, f=freqs, precision="tf32")
    for j in range(1, len(kw["distance"])):
        assert np.array_equal(again[0][j], ok[0][j])


def test_tf32_rejected_by_bounce_solvers(B):
    from bfgb300 import _lib
    cb, _, kw = _lg_reduced(B)
    st = B.Stack(B.SeedSetupBoundaries(cb, **kw), cb, 0.15)
    with pytest.raises(B.BFError) as e:
        st.cheerleader(np.array([20e9]), nmax=5, precision="tf32")
    assert e.value.code == _lib.BF_ERR_INVALID
    st.close()


def test_unnormalized_match_golden_and_batch(B):
    """unnormalized_match (beam_coupling.jl:13-15) on the GPU: the golden of
    test/runtests.jl:52, and a batch of fields against the oracle."""
    c, co = B.SeedCoordinateSystem(), O.seed_coordinate_system()
    g = B.gauss_profile(c, z=1e-9, omega0=0.097, f=22e9)
    dx = 0.0001 * math.floor(10000.0 * (c.X[1] - c.X[0]))
    m = B.unnormalized_match(g, 3 * g, dx=dx, dy=dx)
    assert abs(m - G.MATCH) / abs(G.MATCH) < G.RTOL
    rng = np.random.default_rng(3)
    E = rng.standard_normal((5,) + g.shape) + 1j * rng.standard_normal((5,) + g.shape)
    got = B.unnormalized_match(E, g, dx=0.01, dy=0.02)
    ref = np.array([O.unnormalized_match(e, g, dx=0.01, dy=0.02) for e in E])
    assert rel(got, ref) < 1e-12


@pytest.mark.parametrize("precision,tol", [("fp64", FP64_TOL), ("mixed", MIXED_BETA2_TOL)])
def test_transformer_coupled_vs_oracle(B, precision, tol):
    """The antenna coupling fused into the transformer output: |sum conj(boost)
    * antenna|^2 per frequency (transformer_optim_utilities.jl:137), with the
    antenna's mode coefficients from field2modes(gauss_profile)."""
    distance, eps, tx, ty, X, s = _stack(2, 48, seed=23, surf=True)
    kw = dict(diskno=2, distance=distance, epsilon=eps, relative_tilt_x=tx, relative_tilt_y=ty,
              relative_surfaces=s)
    cb, co = B.SeedCoordinateSystem(X=X, Y=X), O.seed_coordinate_system(X=X, Y=X)
    mb = B.SeedModes(cb, ThreeDim=True, Mmax=4, Lmax=1, diskR=0.15)
    mo = O.seed_modes(co, ThreeDim=True, Mmax=4, Lmax=1, diskR=0.15)
    ant = O.field2modes(O.gauss_profile(co, z=0.2, omega0=0.05, f=20e9), co, mo, diskR=0.15)
    freqs = np.array([19.4e9, 20.0e9, 20.7e9])
    cpl, b2 = B.transformer_coupled(B.SeedSetupBoundaries(cb, **kw), cb, mb, ant, f=freqs, precision=precision)
    for k, f in enumerate(freqs):
        boost = O.transformer(O.seed_setup_boundaries(co, **kw), co, mo, f=f)
        ref = abs(np.sum(np.conj(boost) * ant)) ** 2
        assert abs(cpl[k] - ref) / ref < tol
        r2 = np.sum(np.abs(boost) ** 2)
        assert abs(b2[k] - r2) / r2 < tol


def test_1d_batch_vs_oracle(B):
    """bf_transformer_1d_batch: 24 spacing configurations of a 5-disk booster x
    9 frequencies in one launch against the oracle's 1D transformer
    (propagator1D, ThreeDim=false) at the FP64 bar."""
    from bfgb300 import workloads as W
    rng = np.random.default_rng(31)
    distance, eps, _, _ = W.booster(5, rng.uniform(7e-3, 9e-3, 5), eps_disk=9.4)
    confs = np.array([W.optimiser_step(distance, rng, sigma=1e-4) for _ in range(24)])
    freqs = np.linspace(18.5e9, 21.5e9, 9)
    boost, beta2 = B.transformer_1d_batch(confs, eps, freqs)
    c1 = O.seed_coordinate_system(X=np.array([1e-7]), Y=np.array([1e-7]))
    m1 = O.seed_modes(c1, ThreeDim=False)
    for c in range(0, 24, 5):
        for k, f in enumerate(freqs):
            sb = O.seed_setup_boundaries(c1, diskno=5, distance=confs[c], epsilon=eps.copy())
            ref = O.transformer(sb, c1, m1, f=f, prop=O.propagator1d)[0]
            assert abs(boost[c, k] - ref) / abs(ref) < FP64_TOL
            assert abs(beta2[c, k] - abs(ref) ** 2) / abs(ref) ** 2 < FP64_TOL


def test_1d_batch_vs_analytical1d(B):
    """The reference's own 1D model (src/Analytical1D.py) through the batched entry point."""
    d = np.load(os.path.join(HERE, "golden", "analytical1d.npz"))
    for k in range(int(d["ncases"])):
        nd, eps_d, spac, freqs, gold = int(d[f"nd_{k}"]), float(d[f"eps_{k}"]), d[f"spacings_{k}"], d[f"freqs_{k}"], d[f"beta2_{k}"]
        dist, eps = [0.0], [np.nan]
        for i in range(nd):
            dist += [spac[i], 1e-3]
            eps += [1.0, eps_d]
        dist += [0.0]; eps += [1.0]
        _, b2 = B.transformer_1d_batch(np.array([dist]), np.array(eps, dtype=complex), freqs)
        assert np.allclose(b2[0], gold, rtol=1e-6), k


def test_transformer_1d_vs_analytical1d(B):
    d = np.load(os.path.join(HERE, "golden", "analytical1d.npz"))
    c1 = B.SeedCoordinateSystem(X=np.array([1e-7]), Y=np.array([1e-7]))
    m1 = B.SeedModes(c1, ThreeDim=False)
    for k in range(int(d["ncases"])):
        nd, eps_d, spac, freqs, gold = int(d[f"nd_{k}"]), float(d[f"eps_{k}"]), d[f"spacings_{k}"], d[f"freqs_{k}"], d[f"beta2_{k}"]
        dist, eps = [0.0], [np.nan]
        for i in range(nd):
            dist += [spac[i], 1e-3]
            eps += [1.0, eps_d]
        dist += [0.0]; eps += [1.0]
        sb = B.SeedSetupBoundaries(c1, diskno=nd, distance=np.array(dist), epsilon=np.array(eps, dtype=complex))
        got = np.abs(B.transformer(sb, c1, m1, f=freqs, prop=B.propagator1D)[:, 0]) ** 2
        assert np.allclose(got, gold, rtol=1e-6), k


@pytest.mark.parametrize("M,precision", [(6, "fp64"), (6, "mixed"), (20, "fp64"), (20, "mixed")])
def test_singular_propagation_matrix_raises(B, M, precision):
    """An injected propagation matrix with a zero row is exactly singular: the
    reference's inv raises SingularException (transformer.jl:247); here the
    call returns BF_ERR_SINGULAR (SingularError) naming the frequency.  M = 6
    runs the warp inverses, M = 20 the CTA (FP64) and register (complex64)
    inverses.  A following regular solve on the same handle is unaffected."""
    distance, eps, tx, ty, X, s = _stack(2, 32, seed=3, surf=False)
    kw = dict(diskno=2, distance=distance, epsilon=eps, relative_tilt_x=tx, relative_tilt_y=ty)
    cb, co = B.SeedCoordinateSystem(X=X, Y=X), O.seed_coordinate_system(X=X, Y=X)
    mb = B.SeedModes(cb, ThreeDim=True, Mmax=M, Lmax=0, diskR=0.15)
    mo = O.seed_modes(co, ThreeDim=True, Mmax=M, Lmax=0, diskR=0.15)
    f = 20.1e9
    sbo = O.seed_setup_boundaries(co, **kw)
    sbo.eps[0] = 1e30
    pm = O.calc_propagation_matrices(sbo, co, mo, f=f)
    bad = [p.copy() for p in pm]
    bad[3][1, :] = 0.0
    with pytest.raises(B.SingularError, match="SingularException"):
        B.transformer(B.SeedSetupBoundaries(cb, **kw), cb, mb, f=f, propagation_matrices=bad,
                      precision=precision)
    # the flag does not outlive the call: the regular matrices solve without an error
    got = B.transformer(B.SeedSetupBoundaries(cb, **kw), cb, mb, f=f, propagation_matrices=pm, precision=precision)
    if M == 6:
        # (20 Bessel modes on 32 x 32 pixels make an ill-conditioned chain, whose
        # values mean nothing: only the error path is checked there)
        ref = O.transformer(O.seed_setup_boundaries(co, **kw), co, mo, f=f, propagation_matrices=pm)
        if precision == "fp64":
            assert rel(got, ref) < FP64_TOL
        else:
            r2 = np.sum(np.abs(ref) ** 2)
            assert abs(np.sum(np.abs(got) ** 2) - r2) / r2 < MIXED_BETA2_TOL


def _alone(B, st, modes, freqs, precision):
    from bfgb300 import _lib
    nf, nm = len(freqs), modes.nm
    boost = np.empty((nf, nm), dtype=np.complex128)
    b2 = np.empty(nf)
    st.h.check(_lib.lib().bf_transformer(st.h.ptr, st._s, modes._m, nf, _lib.ptr(freqs), _lib.BF_PROP_3D,
                                         B._prec(precision), None, None, None, 0,
                                         _lib.ptr(boost.view(np.float64)), None, _lib.ptr(b2)))
    return boost, b2


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_transformer_group_equals_alone(B, prec):
    """A group solve of three stacks that differ only in their air gaps (one
    step of three optimisers) gives every stack its own solve's result: FP64
    within 1e-12, mixed beta^2 within 1e-4; the FP64 group also matches the
    oracle.  A stack with other permittivities is refused."""
    from bfgb300 import workloads as W, _lib
    distance, eps, tx, ty, _, _ = _stack(4, 64, seed=61)
    X = W.symmetric_grid(64, width=0.4)
    pats, kt = W.lg_modes(X, X, 12, 0.03, 0.15)
    cb, co = B.SeedCoordinateSystem(X=X, Y=X), O.seed_coordinate_system(X=X, Y=X)
    mb = B.SeedModes(cb, ThreeDim=True, Mmax=12, Lmax=0, diskR=0.15, pattern_input=pats, kT_arr=kt)
    freqs = np.array([19.4e9, 20.05e9, 20.6e9])
    rng = np.random.default_rng(62)
    kws, stacks = [], []
    for r in range(3):
        d = np.array(distance)
        d[1:-1:2] += rng.normal(0.0, 2e-4, len(d[1:-1:2]))
        kw = dict(diskno=4, distance=d, epsilon=eps, relative_tilt_x=tx, relative_tilt_y=ty)
        kws.append(kw)
        stacks.append(B.Stack(B.SeedSetupBoundaries(cb, **kw), cb, 0.15, handle=mb.h))
    b2g, bg = B.transformer_group(stacks, mb, freqs, precision=prec, want_boost=True)
    for r, st in enumerate(stacks):
        boost, b2 = _alone(B, st, mb, freqs, prec)
        if prec == "fp64":
            assert rel(bg[r], boost) < 1e-12
        assert np.max(np.abs(b2g[r] - b2) / b2) < (1e-12 if prec == "fp64" else MIXED_BETA2_TOL)
    if prec == "fp64":
        mo = O.seed_modes(co, ThreeDim=True, Mmax=12, Lmax=0, diskR=0.15, pattern_input=pats, kT_arr=kt)
        ref = O.transformer(O.seed_setup_boundaries(co, **kws[1]), co, mo, f=freqs[2])
        assert rel(bg[1][2], ref) < FP64_TOL
    other = np.array(eps)
    other[2] = 9.4
    odd = B.Stack(B.SeedSetupBoundaries(cb, diskno=4, distance=distance, epsilon=other, relative_tilt_x=tx,
                                        relative_tilt_y=ty), cb, 0.15, handle=mb.h)
    with pytest.raises(B.BFError) as e:
        B.transformer_group([stacks[0], odd], mb, freqs, precision=prec)
    assert e.value.code == _lib.BF_ERR_INVALID
    for st in stacks + [odd]:
        st.close()
