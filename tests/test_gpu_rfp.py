"""GPU parity of the recursive-Fourier-propagation path against the CPU oracle.

Tolerances: FP64 path 1e-10 relative (the stated bar for the plain FP64
solve; measured agreement is ~1e-13); mixed path 1e-4 relative in beta^2.
"""
import math

import numpy as np
import pytest

from oracle import bf_oracle as O
from tests.golden import reference_goldens as G

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10
MIXED_BETA2_TOL = 1e-4


@pytest.fixture(scope="module")
def B():
    import build as _b
    _b.build()
    import bfgb300
    return bfgb300


def rel(a, b):
    a = np.asarray(a); b = np.asarray(b)
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


def coords_pair(B, X, Y=None):
    Y = X if Y is None else Y
    return B.SeedCoordinateSystem(X=X, Y=Y), O.seed_coordinate_system(X=X, Y=Y)


def bdry_pair(B, cb, co, distance, eps, tx=None, ty=None, surf=None):
    nd = len(distance)
    tx = np.zeros(nd) if tx is None else tx
    ty = np.zeros(nd) if ty is None else ty
    kw = dict(diskno=(nd - 2) // 2, distance=np.array(distance, dtype=float),
              epsilon=np.array(eps, dtype=complex), relative_tilt_x=tx, relative_tilt_y=ty)
    if surf is not None:
        kw["relative_surfaces"] = surf
    return B.SeedSetupBoundaries(cb, **kw), O.seed_setup_boundaries(co, **kw)


# ---------------------------------------------------------------- per-op ----
@pytest.mark.parametrize("n", [16, 64, 101])
@pytest.mark.parametrize("kind", ["propagator", "propagatorNoTilts", "propagatorMomentumSpace", "propagator1D"])
def test_propagate_fp64_vs_oracle(B, n, kind):
    from bfgb300 import workloads as W
    X = W.symmetric_grid(n)
    cb, co = coords_pair(B, X)
    rng = np.random.default_rng(n)
    E = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    surf = 1e-5 * rng.standard_normal((n, n))
    # permittivities as the solvers pass them: real eps as re - 0.0im (src/boost_fractor.jl:98),
    # so evanescent bins (reached on the 101-point grid) decay
    eps = complex(24.0 if kind != "propagatorMomentumSpace" else 1.0, -0.0)
    args = (0.0081, 0.15, eps, 3e-4, -2e-4, surf, O.wavelength(20e9))
    oracle_fn = {"propagator": O.propagator, "propagatorNoTilts": O.propagator_notilts,
                 "propagatorMomentumSpace": O.propagator_momentum_space, "propagator1D": O.propagator1d}[kind]
    ref = oracle_fn(E, *args, co)
    got = getattr(B, kind)(E, *args, cb)
    assert rel(got, ref) < 1e-12


@pytest.mark.parametrize("n", [32, 128])
def test_propagate_mixed_vs_oracle(B, n):
    from bfgb300 import workloads as W
    X = W.symmetric_grid(n)
    cb, co = coords_pair(B, X)
    rng = np.random.default_rng(7)
    E = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    args = (0.008, 0.15, 1.0, 0.0, 0.0, np.zeros((n, n)), O.wavelength(20e9))
    ref = O.propagator(E, *args, co)
    got = B.propagator(E, *args, cb, precision="mixed")
    assert rel(got, ref) < 1e-5


# ------------------------------------------------------ reference goldens ----
DEPS = np.arange(0, 3 * math.pi, 1.0)


def _dist(d):
    return np.array([0.0, math.pi * 3e-2 / (2 * math.pi), d * 1e-2 / (2 * math.pi), 0.0])


def test_cheerleader_golden_on_gpu(B):
    """test/runtests.jl:31-74,211 through the GPU (101x101: exact full-grid mode)."""
    c = B.SeedCoordinateSystem()
    sb = B.SeedSetupBoundaries(c, diskno=1)
    out = []
    for d in DEPS:
        sb.distance = _dist(d)
        E = B.cheerleader(0, 100, sb, c, prop=B.propagator, f=10e9, diskR=0.15)
        out.append(B.boost_factor(E, c, 0.15))
    assert rel(out, G.CHEERLEADER_BETA2) < G.RTOL


def test_dancer_golden_on_gpu(B):
    """test/runtests.jl:80-116,214 (propagator1D on the 101x101 grid)."""
    c = B.SeedCoordinateSystem()
    sb = B.SeedSetupBoundaries(c, diskno=1, distance=np.array([0, 0.15, 0.05, 0]) * 1e-2,
                               epsilon=np.array([np.nan, 1, 9, 1], dtype=complex))
    out = []
    for d in DEPS:
        sb.distance = _dist(d)
        E = B.dancer(0, 200, sb, c, prop=B.propagator1D, f=10e9, diskR=0.15)
        out.append(B.boost_factor(E, c, 0.15))
    assert rel(out, G.DANCER_BETA2) < G.RTOL


# ------------------------------------------------------ fused (pruned) path --
def _stack_case(n, ndisk, seed, tilts=True, surfaces=False):
    from bfgb300 import workloads as W
    rng = np.random.default_rng(seed)
    gaps = rng.uniform(7.5e-3, 8.5e-3, ndisk)
    nd = 2 * ndisk + 2
    tx = np.zeros(nd); ty = np.zeros(nd)
    if tilts:
        for k in range(ndisk):
            tx[2 + 2 * k] = rng.uniform(-5e-4, 5e-4)
            ty[2 + 2 * k] = rng.uniform(-5e-4, 5e-4)
    distance, eps, tx, ty = W.booster(ndisk, gaps, tilt_x=tx, tilt_y=ty)
    X = W.symmetric_grid(n)
    surf = None
    if surfaces:
        surf = np.zeros((nd, n, n))
        for k in range(ndisk):
            surf[2 + 2 * k] = 1e-5 * rng.standard_normal((n, n))
    return distance, eps, tx, ty, X, surf


@pytest.mark.parametrize("n,ndisk,surfaces", [(32, 1, False), (64, 2, True), (64, 5, False)])
def test_cheerleader_fused_fp64_vs_oracle(B, n, ndisk, surfaces):
    distance, eps, tx, ty, X, surf = _stack_case(n, ndisk, seed=n + ndisk, surfaces=surfaces)
    cb, co = coords_pair(B, X)
    sbb, sbo = bdry_pair(B, cb, co, distance, eps, tx, ty, surf)
    nmax = 30
    for f in (19.7e9, 20.3e9):
        refL, refR = O.cheerleader(0, nmax, sbo, co, f=f, diskR=0.15, returnboth=True)
        gotL, gotR = B.cheerleader(0, nmax, sbb, cb, f=f, diskR=0.15, returnboth=True)
        assert rel(gotR, refR) < FP64_TOL
        assert rel(gotL, refL) < FP64_TOL


def test_dancer_config1_fp64_vs_oracle(B):
    """Configuration 1: dancer, mirror + 1 disk, 64x64, 20 GHz, 201 bounces, complex128."""
    from bfgb300 import workloads as W
    w = W.config1_dancer()
    cb, co = coords_pair(B, w["X"])
    sbb, sbo = bdry_pair(B, cb, co, w["distance"], w["eps"])
    ref = O.dancer(0, w["nmax"], sbo, co, f=20e9, diskR=w["diskR"])
    got = B.dancer(0, w["nmax"], sbb, cb, f=20e9, diskR=w["diskR"])
    assert rel(got, ref) < FP64_TOL
    b_ref, b_got = O.boost_factor_rfp(ref, co, 0.15), B.boost_factor(got, cb, 0.15)
    assert abs(b_got - b_ref) / b_ref < FP64_TOL


@pytest.mark.parametrize("n,ndisk", [(64, 3), (128, 2), (256, 2)])
def test_cheerleader_mixed_beta2(B, n, ndisk):
    distance, eps, tx, ty, X, surf = _stack_case(n, ndisk, seed=3 * n + ndisk)
    cb, co = coords_pair(B, X)
    sbb, sbo = bdry_pair(B, cb, co, distance, eps, tx, ty)
    freqs = np.array([19.6e9, 20.0e9, 20.4e9])
    nmax = 60
    st = B.Stack(sbb, cb, 0.15)
    _, _, b_mixed = st.cheerleader(freqs, nmax=nmax, precision="mixed")
    _, _, b_fp64 = st.cheerleader(freqs, nmax=nmax, precision="fp64")
    for k, f in enumerate(freqs):
        ref = O.boost_factor_rfp(O.cheerleader(0, nmax, sbo, co, f=f, diskR=0.15), co, 0.15)
        assert abs(b_fp64[k] - ref) / ref < FP64_TOL
        assert abs(b_mixed[k] - ref) / ref < MIXED_BETA2_TOL
    st.close()


def test_batch_equals_single(B):
    distance, eps, tx, ty, X, _ = _stack_case(64, 3, seed=11)
    cb, co = coords_pair(B, X)
    sbb, _ = bdry_pair(B, cb, co, distance, eps, tx, ty)
    st = B.Stack(sbb, cb, 0.15)
    freqs = np.linspace(19.5e9, 20.5e9, 7)
    for prec in ("fp64", "mixed"):
        Rb, _, bb = st.cheerleader(freqs, nmax=20, precision=prec)
        for k in (0, 3, 6):
            R1, _, b1 = st.cheerleader(freqs[k:k + 1], nmax=20, precision=prec)
            assert np.array_equal(R1[0], Rb[k]) and b1[0] == bb[k]
    st.close()


def test_fused_batch_equals_split_single(B):
    """A batch large enough for the fused stage kernel (steps x frequencies >=
    SMs) and the same frequencies solved one at a time (split-phase stages)
    run the same per-pixel arithmetic: identical results."""
    distance, eps, tx, ty, X, _ = _stack_case(128, 3, seed=17)
    cb, co = coords_pair(B, X)
    sbb, _ = bdry_pair(B, cb, co, distance, eps, tx, ty)
    st = B.Stack(sbb, cb, 0.15)
    freqs = np.linspace(19.5e9, 20.5e9, 160)
    try:
        for prec in ("mixed", "fp64"):
            Rb, _, bb = st.cheerleader(freqs, nmax=12, precision=prec)
            for k in (0, 77, 159):
                R1, _, b1 = st.cheerleader(freqs[k:k + 1], nmax=12, precision=prec)
                assert np.array_equal(R1[0], Rb[k]) and b1[0] == bb[k], (prec, k)
    finally:
        st.close()


def test_stage_graph_replay(B):
    """Repeated solves with the same launch sequence are captured into a CUDA
    graph (second solve) and replayed (third on): bit-identical to the plain
    launches, and a replay after an optimiser step (set_distance) equals a
    fresh stack's solve at the new distances."""
    distance, eps, tx, ty, X, _ = _stack_case(64, 3, seed=21)
    cb, co = coords_pair(B, X)
    sbb, _ = bdry_pair(B, cb, co, distance, eps, tx, ty)
    st = B.Stack(sbb, cb, 0.15)
    freqs = np.linspace(19.6e9, 20.4e9, 5)
    try:
        for prec in ("mixed", "fp64"):
            runs = [st.cheerleader(freqs, nmax=25, precision=prec) for _ in range(4)]
            for R, L, b in runs[1:]:
                assert np.array_equal(R, runs[0][0]) and np.array_equal(b, runs[0][2])
        replays, launches = st.graph_stats()
        assert replays >= 4 and launches > 0
        d2 = np.array(distance, dtype=float)
        d2[1:-1:2] += 7e-6
        st.set_distance(d2)
        R2, _, b2 = st.cheerleader(freqs, nmax=25, precision="fp64")
        assert st.graph_stats()[0] == replays + 1
        sb_new, _ = bdry_pair(B, cb, co, d2, eps, tx, ty)
        fresh = B.Stack(sb_new, cb, 0.15)
        Rf, _, bf = fresh.cheerleader(freqs, nmax=25, precision="fp64")
        fresh.close()
        assert np.array_equal(R2, Rf) and np.array_equal(b2, bf)
    finally:
        st.close()


@pytest.mark.parametrize("n", [300, 512])
def test_grids_beyond_the_fused_kernel(B, n):
    """Grids the fused kernel does not take (above 256, or not a power of two
    above 256) run the exact full-grid path: FP64 parity with the oracle."""
    distance, eps, tx, ty, X, _ = _stack_case(n, 1, seed=n)
    cb, co = coords_pair(B, X)
    sbb, sbo = bdry_pair(B, cb, co, distance, eps, tx, ty)
    refL, refR = O.cheerleader(0, 3, sbo, co, f=20.1e9, diskR=0.15, returnboth=True)
    gotL, gotR = B.cheerleader(0, 3, sbb, cb, f=20.1e9, diskR=0.15, returnboth=True)
    assert rel(gotR, refR) < FP64_TOL
    assert rel(gotL, refL) < FP64_TOL


# ------------------------------------------------- exact full-grid mode -----
def test_amin_nonzero_and_dancer_per_bounce(B):
    distance, eps, tx, ty, X, _ = _stack_case(32, 1, seed=5)
    cb, co = coords_pair(B, X)
    sbb, sbo = bdry_pair(B, cb, co, distance, eps, tx, ty)
    ref = O.cheerleader(0.5, 40, sbo, co, f=20e9, diskR=0.15)
    got = B.cheerleader(0.5, 40, sbb, cb, f=20e9, diskR=0.15)
    assert rel(got, ref) < FP64_TOL
    ref = O.dancer(0, 15, sbo, co, f=20e9, diskR=0.15, returnsum=False, immediatesum=False)
    got = B.dancer(0, 15, sbb, cb, f=20e9, diskR=0.15, returnsum=False, immediatesum=False)
    assert rel(got, ref) < FP64_TOL
    ref = O.dancer(0, 15, sbo, co, f=20e9, diskR=0.15, returnsum=True, immediatesum=False)
    got = B.dancer(0, 15, sbb, cb, f=20e9, diskR=0.15, returnsum=True, immediatesum=False)
    assert rel(got, ref) < FP64_TOL


def test_emit_and_reflect(B):
    distance, eps, tx, ty, X, _ = _stack_case(32, 2, seed=9)
    cb, co = coords_pair(B, X)
    sbb, sbo = bdry_pair(B, cb, co, distance, eps, tx, ty)
    rng = np.random.default_rng(4)
    nd = len(distance)
    emit = rng.standard_normal((nd, 2, 32, 32)) + 1j * rng.standard_normal((nd, 2, 32, 32))
    refl = rng.standard_normal((32, 32)) + 0j
    for kw in (dict(emit=emit), dict(reflect=refl)):
        ref = O.cheerleader(0, 25, sbo, co, f=20e9, diskR=0.15, returnboth=True, **kw)
        got = B.cheerleader(0, 25, sbb, cb, f=20e9, diskR=0.15, returnboth=True, **kw)
        assert rel(got[0], ref[0]) < FP64_TOL and rel(got[1], ref[1]) < FP64_TOL
    ref = O.dancer(0, 25, sbo, co, f=20e9, diskR=0.15, reflect=refl)
    got = B.dancer(0, 25, sbb, cb, f=20e9, diskR=0.15, reflect=refl)
    assert rel(got, ref) < FP64_TOL


def test_1d_solvers_vs_oracle(B):
    distance, eps, tx, ty, X, _ = _stack_case(8, 4, seed=2, tilts=False)
    cb, co = coords_pair(B, X)
    sbb, sbo = bdry_pair(B, cb, co, distance, eps, tx, ty)
    ref = O.cheerleader(0, 300, sbo, co, f=20e9, prop=O.propagator1d, diskR=0.15)
    got = B.cheerleader(0, 300, sbb, cb, f=20e9, prop=B.propagator1D, diskR=0.15)
    assert rel(got, ref) < 1e-12
    ref = O.dancer(0.2, 300, sbo, co, f=20e9, prop=O.propagator1d, diskR=0.15)
    got = B.dancer(0.2, 300, sbb, cb, f=20e9, prop=B.propagator1D, diskR=0.15)
    assert rel(got, ref) < 1e-12


def test_invalid_arguments_raise(B):
    c = B.SeedCoordinateSystem(X=np.linspace(-0.5, 0.5, 16), Y=np.linspace(-0.5, 0.5, 16))
    sb = B.SeedSetupBoundaries(c, diskno=1)
    sb.distance[1] = np.nan
    with pytest.raises(B.BFError) as e:
        B.cheerleader(0, 5, sb, c, f=20e9)
    assert e.value.code == 1
    sb = B.SeedSetupBoundaries(c, diskno=1)
    with pytest.raises(B.BFError):
        B.cheerleader(0, 5, sb, c, f=-1.0)
    h = B.Handle(0, hbm_budget_bytes=2048)
    with pytest.raises(B.BFError) as e:
        B.cheerleader(0, 5, sb, c, f=20e9, handle=h)
    assert e.value.code == 2
    h.close()


def test_cheerleader_full_size_vs_oracle_fixture(B):
    """The full 20-disk cheerleader workload (128x128, per-disk tilts, 401
    bounces) at four of its 256 frequencies, one of them the spectrum's
    maximum, against the oracle's exit fields stored by
    tests/golden/make_c2_fixture.py: FP64 exit field within 1e-10, mixed
    beta^2 within 1e-4 (src/boost_fractor_recurprop.jl:226-363)."""
    import os
    from bfgb300 import workloads as W
    fx = np.load(os.path.join(os.path.dirname(__file__), "golden", "c2_cheerleader_oracle.npz"))
    w = W.config2_cheerleader()
    assert np.array_equal(w["freqs"][fx["freq_index"]], fx["freqs"])
    c = B.SeedCoordinateSystem(X=w["X"], Y=w["Y"])
    sb = B.SeedSetupBoundaries(c, diskno=(len(w["distance"]) - 2) // 2, distance=w["distance"],
                               epsilon=w["eps"], relative_tilt_x=w["relative_tilt_x"],
                               relative_tilt_y=w["relative_tilt_y"])
    st = B.Stack(sb, c, w["diskR"])
    R64, _, b64 = st.cheerleader(fx["freqs"], nmax=w["nmax"], precision="fp64")
    _, _, b32 = st.cheerleader(fx["freqs"], nmax=w["nmax"], precision="mixed")
    st.close()
    for k in range(len(fx["freqs"])):
        assert rel(R64[k], fx["exit_field"][k]) < FP64_TOL
        assert abs(b64[k] - fx["beta2"][k]) / fx["beta2"][k] < FP64_TOL
        assert abs(b32[k] - fx["beta2"][k]) / fx["beta2"][k] < MIXED_BETA2_TOL


@pytest.mark.parametrize("n,ndisk,nf", [(128, 3, 48), (256, 2, 24)])
def test_fused_variants_agree_bit_for_bit(B, n, ndisk, nf):
    """The fused stage kernel's variants (the rule, separate slots, joint
    slots, 512 threads at 256x256 complex64, and at 128x128 complex64 the lean
    ones: shared twiddles and two-half exchanges, joint at 320 threads or
    separate at 3 CTAs per SM, and both with phasor rows staged by cp.async,
    and separate slots with 160 threads at 3 CTAs per SM with staged rows)
    give identical results, so the autotuner's
    choice never changes a result; the autotuner logs a decision for the
    shape."""
    from bfgb300 import _lib
    L = _lib.lib()
    distance, eps, tx, ty, X, _ = _stack_case(n, ndisk, seed=23)
    cb, co = coords_pair(B, X)
    sbb, _ = bdry_pair(B, cb, co, distance, eps, tx, ty)
    st = B.Stack(sbb, cb, 0.15)
    freqs = np.linspace(19.5e9, 20.5e9, nf)
    try:
        for prec in ("mixed", "fp64"):
            ref = None
            for v in range(9):
                L.bf_test_force_fused_variant(v)
                R, _, b2 = st.cheerleader(freqs, nmax=10, precision=prec)
                if ref is None:
                    ref = (R, b2)
                else:
                    assert np.array_equal(R, ref[0]) and np.array_equal(b2, ref[1]), (prec, v)
            L.bf_test_force_fused_variant(-1)
            R, _, b2 = st.cheerleader(freqs, nmax=10, precision=prec)   # tuned
            assert np.array_equal(R, ref[0]) and np.array_equal(b2, ref[1])
        assert any(f"N={n}" in line for line in B.autotune_report())
    finally:
        L.bf_test_force_fused_variant(-1)
        st.close()
