"""Propagation-matrix grid with interpolation (bf_pgrid_*), the optimiser
helper of examples/transformer_optim_utilities.jl:11-91.

The interpolation is a natural cubic spline along the gap spacing (second
derivative zero at the end knots); scipy's CubicSpline(bc_type="natural") is the
same spline and serves as the check.  Tolerances: FP64 path 1e-10 (knots,
interpolation against the oracle's grid values), 1e-12 where the same matrices
go through two GPU paths.
"""
import numpy as np
import pytest

from oracle import bf_oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def B():
    import build as _b
    _b.build()
    import bfgb300
    return bfgb300


def rel(a, b):
    a = np.asarray(a); b = np.asarray(b)
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


def setup(B):
    from bfgb300 import workloads as W
    rng = np.random.default_rng(61)
    distance, eps, tx, ty = W.booster(2, rng.uniform(7.5e-3, 8.5e-3, 2))
    tx[2] = 2e-4
    X = W.symmetric_grid(32)
    kw = dict(diskno=2, distance=distance, epsilon=eps, relative_tilt_x=tx, relative_tilt_y=ty)
    cb, co = B.SeedCoordinateSystem(X=X, Y=X), O.seed_coordinate_system(X=X, Y=X)
    mb = B.SeedModes(cb, ThreeDim=True, Mmax=3, Lmax=1, diskR=0.15)
    mo = O.seed_modes(co, ThreeDim=True, Mmax=3, Lmax=1, diskR=0.15)
    grid = np.linspace(-3e-4, 3e-4, 7)
    freqs = np.array([19.6e9, 20.3e9])
    return kw, cb, co, mb, mo, grid, freqs


def shifted(kw, shift_per_disk, last=0.0):
    d = np.array(kw["distance"], dtype=float)
    for k, sh in enumerate(shift_per_disk):
        d[1 + 2 * k] += sh
    d[-1] += last
    return dict(kw, distance=d)


def test_pgrid_knots_and_spline_vs_oracle(B):
    """The device grid and its spline against the oracle's
    calc_propagation_matrices_grid + construct_prop_matrix_interpolation +
    interpolate_prop_matrix, at knots, between them and in the half cells
    beyond the end spacings (the OnCell domain)."""
    kw, cb, co, mb, mo, grid, freqs = setup(B)
    pg = B.PGrid(B.SeedSetupBoundaries(cb, **kw), cb, mb, freqs, grid)
    try:
        nd = len(kw["distance"])
        sb = O.seed_setup_boundaries(co, **kw)
        ref = O.calc_propagation_matrices_grid(sb, co, mo, grid, freqs)
        ref[0] = 0.0   # the mirror (NaN permittivity, as the reference leaves it) is not compared
        itp = O.construct_prop_matrix_interpolation(ref, grid)
        step = grid[1] - grid[0]
        assert np.allclose(pg.bounds, itp.bounds, rtol=0, atol=1e-15)
        rng = np.random.default_rng(62)
        for shifts in ([grid[2], grid[5]], [grid[0], grid[-1]], [grid[0] - 0.4 * step, grid[-1] + 0.45 * step],
                       [grid[0] - 0.5 * step, grid[-1] + 0.5 * step], list(rng.uniform(grid[0], grid[-1], 2)),
                       list(rng.uniform(*itp.bounds, 2))):
            got = pg.matrices(np.array(shifts))
            want = O.interpolate_prop_matrix(itp, shifts)
            for f in range(len(freqs)):
                for j in range(1, nd):
                    assert rel(got[f, j], want[j][f]) < 1e-10, (shifts, f, j)
    finally:
        pg.close()


def test_pgrid_transformer_matches_injected_and_direct(B):
    kw, cb, co, mb, mo, grid, freqs = setup(B)
    pg = B.PGrid(B.SeedSetupBoundaries(cb, **kw), cb, mb, freqs, grid)
    try:
        sh = np.array([1.3e-4, -2.2e-4])
        boost, beta2 = pg.transformer(sh)
        pm = pg.matrices(sh)
        for f, fr in enumerate(freqs):
            inj = B.transformer(B.SeedSetupBoundaries(cb, **kw), cb, mb, f=fr, propagation_matrices=pm[f])
            assert rel(boost[f], inj) < 1e-12
            assert abs(beta2[f] - np.sum(np.abs(inj) ** 2)) / np.sum(np.abs(inj) ** 2) < 1e-12
        # at knots the grid is exact: compare with a direct solve of the moved stack
        sh = np.array([grid[1], grid[4]])
        boost, _ = pg.transformer(sh)
        for f, fr in enumerate(freqs):
            direct = B.transformer(B.SeedSetupBoundaries(cb, **shifted(kw, sh)), cb, mb, f=fr)
            assert rel(boost[f], direct) < 1e-10
    finally:
        pg.close()


def test_pgrid_rejects_shift_outside_grid(B):
    kw, cb, co, mb, mo, grid, freqs = setup(B)
    pg = B.PGrid(B.SeedSetupBoundaries(cb, **kw), cb, mb, freqs, grid)
    try:
        with pytest.raises(B.BFError) as e:
            pg.matrices(np.array([0.0, grid[-1] + 0.51 * (grid[1] - grid[0])]))
        assert e.value.code == 1
    finally:
        pg.close()


def test_pgrid_mixed_within_bar(B):
    """A grid built at BF_PREC_MIXED (complex64 matrices, double-float chain)
    gives beta^2 within 1e-4 of the FP64 grid at the same shifts."""
    kw, cb, co, mb, mo, grid, freqs = setup(B)
    p64 = B.PGrid(B.SeedSetupBoundaries(cb, **kw), cb, mb, freqs, grid)
    p32 = B.PGrid(B.SeedSetupBoundaries(cb, **kw), cb, mb, freqs, grid, precision="mixed")
    try:
        for sh in (np.array([1.3e-4, -2.2e-4]), np.array([grid[3], grid[6]])):
            _, b64 = p64.transformer(sh)
            _, b32 = p32.transformer(sh)
            assert np.max(np.abs(b32 - b64) / b64) < 1e-4
    finally:
        p64.close()
        p32.close()


def test_pgrid_requests_through_the_server(B):
    """Grid steps queued on the serving engine (solver "pgrid", the shifts in
    distance) run in submission order and equal PGrid.transformer."""
    kw, cb, co, mb, mo, grid, freqs = setup(B)
    pg = B.PGrid(B.SeedSetupBoundaries(cb, **kw), cb, mb, freqs, grid, precision="mixed")
    try:
        rng = np.random.default_rng(31)
        shifts = [rng.uniform(grid[0], grid[-1], 2) for _ in range(5)]
        ref = [pg.transformer(sh) for sh in shifts]
        srv = B.Server(n_workers=2)
        try:
            ids = [srv.submit(None, freqs, "pgrid", distance=sh, pgrid=pg, want_boost=True) for sh in shifts]
            res = [srv.wait(i, timeout_ms=120000) for i in ids]
            for r, (bo, b2) in zip(res, ref):
                assert np.max(np.abs(r["beta2"] - b2) / np.abs(b2)) < 1e-12
                assert rel(r["boost"], bo) < 1e-12
            for a, b in zip(res, res[1:]):
                assert b["t_start"] >= a["t_done"]
            with pytest.raises(B.BFError):
                srv.submit(None, freqs[:1], "pgrid", distance=shifts[0], pgrid=pg)
        finally:
            srv.close()
    finally:
        pg.close()


def test_pgrid_cost_vs_oracle(B):
    """calc_boostfactor_cost on the device (coupled power fused after the
    solve, p-norm and soft box penalty on the host) against the oracle's,
    inside the box, in the soft-penalty band and outside the hard bounds."""
    kw, cb, co, mb, mo, grid, freqs = setup(B)
    pg = B.PGrid(B.SeedSetupBoundaries(cb, **kw), cb, mb, freqs, grid)
    try:
        sb = O.seed_setup_boundaries(co, **kw)
        ref = O.calc_propagation_matrices_grid(sb, co, mo, grid, freqs)
        itp = O.construct_prop_matrix_interpolation(ref, grid)
        rng = np.random.default_rng(64)
        m_reflect = rng.standard_normal(mo.nm) + 1j * rng.standard_normal(mo.nm)
        lo, hi = itp.bounds
        depth = 0.05 * (hi - lo)
        for sh in ([1.3e-4, -2.2e-4], [hi - 0.4 * depth, -1e-4], [lo + 0.3 * depth, 0.0], [0.0, hi + 1e-9]):
            sb_c = O.seed_setup_boundaries(co, **kw)
            want = O.calc_boostfactor_cost(sh, itp, freqs, sb_c, co, mo, m_reflect)
            got = B.calc_boostfactor_cost(np.array(sh), pg, freqs, None, cb, mb, m_reflect)
            if want == 1000.0:
                assert got == 1000.0
            else:
                assert abs(got - want) < 1e-10 * abs(want), (sh, got, want)
        cost, cpl = pg.cost(np.array([1.3e-4, -2.2e-4]), m_reflect)
        boost, _ = pg.transformer(np.array([1.3e-4, -2.2e-4]))
        assert rel(cpl, np.abs(boost.conj() @ m_reflect) ** 2) < 1e-13
    finally:
        pg.close()


def test_optimiser_utility_mirrors_vs_oracle(B):
    """The reference-named mirrors: calc_propagation_matrices_grid ->
    construct_prop_matrix_interpolation -> interpolate_prop_matrix ->
    calc_boostfactor_modes, against the oracle's (1e-10, FP64)."""
    kw, cb, co, mb, mo, grid, freqs = setup(B)
    itp = B.construct_prop_matrix_interpolation(
        B.calc_propagation_matrices_grid(B.SeedSetupBoundaries(cb, **kw), cb, mb, grid, freqs), grid)
    try:
        sbo = O.seed_setup_boundaries(co, **kw)
        ref_grid = O.calc_propagation_matrices_grid(sbo, co, mo, grid, freqs)
        ref_grid[0] = 0.0   # the mirror (NaN permittivity) is not compared
        oitp = O.construct_prop_matrix_interpolation(ref_grid, grid)
        sh = [0.7e-4, -2.6e-4]
        pm = B.interpolate_prop_matrix(itp, np.array(sh))
        opm = O.interpolate_prop_matrix(oitp, sh)
        nd = len(kw["distance"])
        assert pm.shape == (nd, len(freqs), mo.nm, mo.nm)
        for r in range(1, nd):
            for f in range(len(freqs)):
                assert rel(pm[r, f], opm[r][f]) < 1e-10
        # the transformer on per-frequency injected matrices (the mirror's own grid values)
        E = B.calc_boostfactor_modes(B.SeedSetupBoundaries(cb, **kw), cb, mb, freqs, pm)
        assert E.shape == (1, mo.nm, len(freqs))
        opm_own = [[pm[r, f] for f in range(len(freqs))] for r in range(nd)]
        Eo = O.calc_boostfactor_modes(O.seed_setup_boundaries(co, **kw), co, mo, freqs, opm_own)
        assert rel(E, Eo) < 1e-10
    finally:
        itp.close()


def test_pgrid_tilt_grids_vs_oracle(B):
    """calc_propagation_matrices_grid with tilt grids: the whole (region,
    frequency, spacing, tilt_x, tilt_y) array against the oracle's, and the
    interpolation at the tilt grids' first points, as the reference's
    interpolate_prop_matrix evaluates it (itp(r, f, shift, 1, 1, ...))."""
    kw, cb, co, mb, mo, grid, freqs = setup(B)
    grid = grid[::2]
    txg, tyg = np.array([1e-4, -2e-4]), np.array([0.0, 3e-4])
    pg = B.calc_propagation_matrices_grid(B.SeedSetupBoundaries(cb, **kw), cb, mb, grid, freqs,
                                          tilt_x_grid=txg, tilt_y_grid=tyg)
    try:
        nd = len(kw["distance"])
        sb = O.seed_setup_boundaries(co, **kw)
        ref = O.calc_propagation_matrices_grid(sb, co, mo, grid, freqs, tilt_x_grid=txg, tilt_y_grid=tyg)
        got = pg.array()
        assert got.shape == ref.shape
        assert rel(got[1:], ref[1:]) < 1e-10   # the mirror (NaN permittivity) is not compared
        ref0 = ref[:, :, :, 0, 0].copy()
        ref0[0] = 0.0
        itp = O.construct_prop_matrix_interpolation(ref0, grid)
        shifts = [0.5 * (grid[0] + grid[1]), grid[2]]
        m = pg.matrices(np.array(shifts))
        want = O.interpolate_prop_matrix(itp, shifts)
        for f in range(len(freqs)):
            for j in range(1, nd):
                assert rel(m[f, j], want[j][f]) < 1e-10, (f, j)
    finally:
        pg.close()
