"""FP64 CPU restatement of the reference boost-factor solvers (TEST ORACLE).

TEST INFRASTRUCTURE ONLY -- imported by tests/, __graft_entry__.smoke() and
the CPU-baseline leg of bench.py, never by the product package.

Every function cites the reference file:line it restates (paths relative to
the BoostFractor.jl project).  Arrays keep the reference's index semantics
with 0-based numpy indexing: a field is ``E[x, y]``, a region stack is
``fields[region, x, y]``, ``emit[region, dir, x, y]`` with dir 0 = right-
moving and 1 = left-moving.  Third-party arithmetic used by the reference
(FFTW.jl, LinearAlgebra/LAPACK, SpecialFunctions, FunctionZeros; versions
unpinned in Project.toml) is restated with numpy.fft (pocketfft),
numpy.linalg and scipy.special.

Parity pinning: tests/test_oracle_goldens.py reproduces every golden vector
of test/runtests.jl at the reference's tolerance.
"""
from __future__ import annotations

import copy
import math
from fractions import Fraction

import numpy as np
from scipy import special

SPEED_OF_LIGHT = 299792458.0


# --------------------------------------------------------------------------
# Geometry (src/boost_fractor.jl:16-108)
# --------------------------------------------------------------------------
def wavelength(frequency):
    """src/boost_fractor.jl:16-19."""
    return SPEED_OF_LIGHT / frequency


class CoordinateSystem:
    """src/boost_fractor.jl:21-28 (X, Y real space; kX, kY k space)."""

    def __init__(self, X, Y, kX, kY):
        self.X = np.asarray(X, dtype=np.float64)
        self.Y = np.asarray(Y, dtype=np.float64)
        self.kX = np.asarray(kX, dtype=np.float64)
        self.kY = np.asarray(kY, dtype=np.float64)


def julia_float_range(start, step, n):
    """Elements of a Julia Float64 range start:step:... of length n.

    Julia evaluates range elements in twice precision and rounds once; the
    exact rational evaluation below gives the same correctly rounded values.
    """
    fs, fd = Fraction(start), Fraction(step)
    return np.array([float(fs + i * fd) for i in range(n)], dtype=np.float64)


def decimal_grid(lo_num, hi_num, den):
    """Julia `lo/den : 1/den : hi/den` (e.g. -0.5:0.01:0.5): exact decimals."""
    return np.array([i / den for i in range(lo_num, hi_num + 1)], dtype=np.float64)


def get_kspace_coords(real_coords):
    """src/boost_fractor.jl:42-47: dk = 2pi/(2 max X), symmetric range."""
    real_coords = np.asarray(real_coords, dtype=np.float64)
    n = len(real_coords)
    min_k = 2 * math.pi / (np.max(real_coords) * 2)
    max_k = min_k * (n - 1) / 2
    return julia_float_range(-max_k, min_k, n)


def seed_coordinate_system(X=None, Y=None):
    """src/boost_fractor.jl:30-34 (default X = Y = -0.5:0.01:0.5)."""
    if X is None:
        X = decimal_grid(-50, 50, 100)
    if Y is None:
        Y = decimal_grid(-50, 50, 100)
    X = np.asarray(X, dtype=np.float64)
    Y = np.asarray(Y, dtype=np.float64)
    return CoordinateSystem(X, Y, get_kspace_coords(X), get_kspace_coords(Y))


def _cast_real_eps(eps):
    """Real eps -> real(eps) - 0.0im (src/boost_fractor.jl:98, :140)."""
    eps = np.array(eps, dtype=np.complex128)
    eps.imag[eps.imag == 0.0] = -0.0
    return eps


def _neg_zero_if_real(z):
    z = complex(z)
    if z.imag == 0.0:
        return complex(z.real, -0.0)
    return z


class SetupBoundaries:
    """src/boost_fractor.jl:63-71."""

    def __init__(self, distance, r, eps, relative_tilt_x, relative_tilt_y, relative_surfaces):
        self.distance = np.array(distance, dtype=np.float64)
        self.r = np.array(r, dtype=np.complex128)
        self.eps = np.array(eps, dtype=np.complex128)
        self.relative_tilt_x = np.array(relative_tilt_x, dtype=np.float64)
        self.relative_tilt_y = np.array(relative_tilt_y, dtype=np.float64)
        self.relative_surfaces = np.array(relative_surfaces, dtype=np.complex128)


def seed_setup_boundaries(coords, diskno=3, distance=None, epsilon=None,
                          relative_tilt_x=None, relative_tilt_y=None,
                          relative_surfaces=None):
    """src/boost_fractor.jl:83-108 (defaults, Fresnel r, dimension check)."""
    nd_default = 2 * diskno + 2
    if relative_tilt_x is None:
        relative_tilt_x = np.zeros(nd_default)
    if relative_tilt_y is None:
        relative_tilt_y = np.zeros(nd_default)
    if relative_surfaces is None:
        relative_surfaces = np.zeros((nd_default, len(coords.X), len(coords.Y)))
    if distance is None:
        distance = [0.0] + [8e-3 if x % 2 == 1 else 1e-3 for x in range(1, 2 * diskno + 1)] + [0.0]
    if epsilon is None:
        epsilon = [np.nan] + [1.0 if x % 2 == 1 else 9.0 for x in range(1, 2 * diskno + 1)] + [1.0]
    eps = _cast_real_eps(epsilon)
    refl = [complex(1.0)]
    for i in range(2, len(eps)):
        a, b = np.sqrt(eps[i - 1]), np.sqrt(eps[i])
        refl.append((a - b) / (a + b))
    relative_surfaces = np.asarray(relative_surfaces)
    ok = (len(distance) == len(refl) + 1 == len(eps) == len(relative_tilt_x)
          == len(relative_tilt_y) == relative_surfaces.shape[0])
    if not ok:
        raise ValueError("DimensionMismatch: the arrays in your SetupBoundaries objects don't fit together!")
    return SetupBoundaries(distance, refl, eps, relative_tilt_x, relative_tilt_y, relative_surfaces)


# --------------------------------------------------------------------------
# Propagators (src/boost_fractor.jl:137-227)
# --------------------------------------------------------------------------
def jl_fftshift(a):
    """FFTW.fftshift = circshift by div(size, 2) along every axis."""
    return np.roll(a, tuple(s // 2 for s in a.shape), axis=tuple(range(a.ndim)))


def jl_ifftshift(a):
    """FFTW.ifftshift = circshift by -div(size, 2) along every axis."""
    return np.roll(a, tuple(-(s // 2) for s in a.shape), axis=tuple(range(a.ndim)))


def disk_mask_strict(coords, diskR):
    """abs(x^2 + y^2) < diskR^2 (src/boost_fractor.jl:159)."""
    X, Y = coords.X, coords.Y
    return np.abs(X[:, None] ** 2 + Y[None, :] ** 2) < diskR ** 2


def k0_of(eps, lam):
    """k0 = 2pi/lambda * sqrt(eps) with Julia's Real*Complex (keeps the sign of a zero imag)."""
    s = np.sqrt(np.complex128(eps))
    c = 2 * math.pi / lam
    return np.complex128(complex(c * s.real, c * s.imag))


def kz_matrix(k0, coords):
    """sqrt(k0^2 - Kx^2 - Ky^2) with the reference's -0.0im branch (:171-172)."""
    k0 = np.complex128(k0)
    k0sq = k0 * k0
    KX = coords.kX[:, None] ** 2
    KY = coords.kY[None, :] ** 2
    re = (k0sq.real - KX) - KY
    return np.sqrt(_complex_with_imag(re, k0sq.imag))


def _complex_with_imag(re, imag_scalar):
    out = np.empty(re.shape, dtype=np.complex128)
    out.real = re
    out.imag = imag_scalar  # keeps the sign of a zero imaginary part
    return out


def phasor_matrix(eps, dz, lam, coords):
    """exp(-1im * k_prop * dz) in fftshifted (natural kX, kY) order (:171-174)."""
    kz = kz_matrix(k0_of(eps, lam), coords)
    return np.exp(-1j * kz * dz)


def tilt_surface_map(eps, tilt_x, tilt_y, surface, lam, coords):
    """exp(-i k0 tx x) exp(-i k0 ty y) * exp(-i k0 surface) (:145-147)."""
    eps = _neg_zero_if_real(eps)
    k0 = k0_of(eps, lam)
    X, Y = coords.X, coords.Y
    tilt = np.exp(-1j * k0 * tilt_x * X)[:, None] * np.exp(-1j * k0 * tilt_y * Y)[None, :]
    return tilt * np.exp(-1j * k0 * np.asarray(surface))


def propagator_notilts(E0, dz, diskR, eps, tilt_x, tilt_y, surface, lam, coords):
    """propagatorNoTilts (src/boost_fractor.jl:157-179)."""
    E = np.array(E0, dtype=np.complex128) * disk_mask_strict(coords, diskR)
    E = jl_fftshift(np.fft.fft2(E))
    E = E * phasor_matrix(eps, dz, lam, coords)
    E = np.fft.ifft2(jl_ifftshift(E))
    return E


def propagator(E0, dz, diskR, eps, tilt_x, tilt_y, surface, lam, coords):
    """propagator = propagatorNoTilts + tilt + surface (src/boost_fractor.jl:137-149)."""
    eps = _neg_zero_if_real(eps)
    E = propagator_notilts(E0, dz, diskR, eps, tilt_x, tilt_y, surface, lam, coords)
    return E * tilt_surface_map(eps, tilt_x, tilt_y, surface, lam, coords)


def propagator_momentum_space(E0, dz, diskR, eps, tilt_x, tilt_y, surface, lam, coords):
    """propagatorMomentumSpace (src/boost_fractor.jl:187-210)."""
    k0 = k0_of(eps, lam)
    E = np.array(E0, dtype=np.complex128) * np.exp(-1j * kz_matrix(k0, coords) * dz)
    E = np.fft.ifft2(jl_ifftshift(E))
    E = E * disk_mask_strict(coords, diskR)
    if tilt_x != 0 or tilt_y != 0:
        X, Y = coords.X, coords.Y
        E = E * (np.exp(-1j * k0 * tilt_x * X)[:, None] * np.exp(-1j * k0 * tilt_y * Y)[None, :])
    return jl_fftshift(np.fft.fft2(E))


def propagator1d(E0, dz, diskR, eps, tilt_x, tilt_y, surface, lam, coords):
    """propagator1D (src/boost_fractor.jl:218-227): scalar phase only."""
    k0 = k0_of(eps, lam)
    return np.asarray(E0, dtype=np.complex128) * np.exp(-1j * k0 * dz)


# --------------------------------------------------------------------------
# Recursive Fourier propagation (src/boost_fractor_recurprop.jl)
# --------------------------------------------------------------------------
def dance_intro(bdry, coords, bfield=None, velocity_x=0.0, f=10e9, diskR=0.1):
    """Axion-induced initial fields per gap (src/boost_fractor_recurprop.jl:153-201)."""
    nreg = len(bdry.distance)
    nx, ny = len(coords.X), len(coords.Y)
    out = np.zeros((nreg, 2, nx, ny), dtype=np.complex128)
    X, Y = coords.X, coords.Y
    if bfield is None:
        inside = ~((X[:, None] ** 2 + Y[None, :] ** 2) > diskR ** 2)
        bfield = np.broadcast_to(inside.astype(np.float64), (nreg + 1, nx, ny))
    bfield = np.asarray(bfield, dtype=np.complex128)
    if velocity_x != 0:
        lam = wavelength(f)
        ma = 2 * math.pi / lam
        bfield = bfield * np.exp(-1j * ma * (-velocity_x) * X)[None, :, None]
    eps = bdry.eps
    for n in range(nreg):
        if n == 0:
            ax_r = -1.0 if bdry.r[0] == 1 else 0.0
        else:
            ei, em = eps[n - 1], eps[n]
            den = ei * np.sqrt(em) + em * np.sqrt(ei)
            ax_r = np.sqrt(em) * (1 - ei / em) / den
        ei = eps[n]
        em = 1.0 if n == nreg - 1 else eps[n + 1]
        den = ei * np.sqrt(em) + em * np.sqrt(ei)
        ax_l = np.sqrt(ei) * (1 - em / ei) / den
        out[n, 0] = ax_r * bfield[n]
        out[n, 1] = ax_l * bfield[n + 1]
    return out


def dancer(amin, nmax, sbdry, coords, f=10.0e9, prop=propagator, emit=None, reflect=None,
           diskR=0.1, returnsum=True, immediatesum=True):
    """Legacy bounce loop, 2 fields per region (src/boost_fractor_recurprop.jl:25-146)."""
    bdry = copy.deepcopy(sbdry)
    bdry.eps = bdry.eps[1:]
    bdry.distance = bdry.distance[1:]
    bdry.relative_tilt_x = bdry.relative_tilt_x[1:]
    bdry.relative_tilt_y = bdry.relative_tilt_y[1:]
    bdry.relative_surfaces = bdry.relative_surfaces[1:]
    bdry.r = np.append(bdry.r, 0.0)
    nreg = len(bdry.distance)
    nx, ny = len(coords.X), len(coords.Y)
    rm, lm = 0, 1
    fields = np.zeros((nreg, 2, nx, ny), dtype=np.complex128)
    eout = np.zeros((nx, ny, 1 if immediatesum else nmax + 1), dtype=np.complex128)
    if reflect is None:
        fields = dance_intro(bdry, coords, diskR=diskR) if emit is None else np.array(emit, dtype=np.complex128)
    else:
        fields[nreg - 1, lm] = reflect
    lam = wavelength(f)
    nb = len(bdry.r)

    def p(j, E):
        return prop(E, bdry.distance[j], diskR, bdry.eps[j], bdry.relative_tilt_x[j],
                    bdry.relative_tilt_y[j], bdry.relative_surfaces[j], lam, coords)

    n, a = 0, 1.0
    while n <= nmax and a >= amin:
        for i in range(nb):
            if i > 0:
                fields[i - 1, rm] = p(i - 1, fields[i - 1, rm])
            if i < nb - 1:
                fields[i, lm] = p(i, fields[i, lm])
            r = bdry.r[i]
            if i == 0:
                fields[i, lm] *= -r
            elif i == nb - 1:
                if immediatesum:
                    eout[:, :, 0] += (1 + r) * fields[i - 1, rm]
                else:
                    eout[:, :, n] = (1 + r) * fields[i - 1, rm]
                fields[i - 1, rm] *= r
            else:
                arrived_left = fields[i - 1, rm].copy()
                fields[i - 1, rm] = r * fields[i - 1, rm] + (1 - r) * fields[i, lm]
                fields[i, lm] = -r * fields[i, lm] + (1 + r) * arrived_left
        rm, lm = lm, rm
        if amin != 0:
            a = np.max(np.abs(fields))
        n += 1
    if returnsum:
        return np.sum(eout[:, :, ::-1], axis=2)
    return eout


def cheerleader(amin, nmax, bdry, coords, f=10.0e9, prop=propagator, emit=None, reflect=None,
                diskR=0.1, returnboth=False):
    """Current bounce loop, one field per region (src/boost_fractor_recurprop.jl:226-363)."""
    lam = wavelength(f)
    nd = len(bdry.distance)
    nx, ny = len(coords.X), len(coords.Y)
    r_l = -bdry.r
    r_r = bdry.r
    t_l = 1 - bdry.r
    t_r = 1 + bdry.r
    if reflect is None:
        if emit is None:
            emit = np.zeros((nd, 2, nx, ny), dtype=np.complex128)
            bc = copy.deepcopy(bdry)
            bc.distance = bc.distance[1:]
            bc.eps = bc.eps[1:]
            emit[1:] = dance_intro(bc, coords, diskR=diskR)
    else:
        emit = np.zeros((nd, 2, nx, ny), dtype=np.complex128)
        emit[nd - 1, 1] = reflect
    emit = np.asarray(emit, dtype=np.complex128)

    def p(j, E):
        return prop(E, bdry.distance[j], diskR, bdry.eps[j], bdry.relative_tilt_x[j],
                    bdry.relative_tilt_y[j], bdry.relative_surfaces[j], lam, coords)

    fields = emit[:, 0].copy()
    for i in range(1, nd - 1):                       # :281-287
        fields[i] = p(i, fields[i])
        fields[i + 1] += t_r[i] * fields[i]
        fields[i] *= r_r[i]
    fields[: nd - 1] += emit[: nd - 1, 1]            # :290
    i = nd - 2                                       # :295-300
    fields[i] += t_l[i] * emit[i + 1, 1]
    fields[i + 1] += r_l[i] * emit[i + 1, 1]

    n, a = 0, 1.0
    while n <= nmax and a >= amin:                   # :306
        i = 0                                        # :310-321
        fields[i + 1] = p(i + 1, fields[i + 1])
        fields[i] += t_l[i] * fields[i + 1]
        fields[i + 1] *= r_l[i]
        for i in range(1, nd - 2):                   # :324-335
            fields[i] = p(i, fields[i])
            fields[i + 1] = p(i + 1, fields[i + 1])
            nxt = fields[i + 1].copy()
            fields[i + 1] = r_l[i] * fields[i + 1] + t_r[i] * fields[i]
            fields[i] = r_r[i] * fields[i] + t_l[i] * nxt
        i = nd - 2                                   # :337-345
        fields[i] = p(i, fields[i])
        fields[i + 1] += t_r[i] * fields[i]
        fields[i] *= r_r[i]
        if amin != 0:
            a = np.max(np.abs(fields))
        n += 1
    if returnboth:
        return fields[0], fields[nd - 1]
    return fields[nd - 1]


def boost_factor_rfp(E, coords, diskR):
    """beta^2 = sum|E|^2 dx dy / (pi R^2) (test/runtests.jl:74; docs 3d_algorithms.md:33)."""
    dx = coords.X[1] - coords.X[0] if len(coords.X) > 1 else 1.0
    dy = coords.Y[1] - coords.Y[0] if len(coords.Y) > 1 else 1.0
    return float(np.sum(np.abs(E) ** 2) * dx * dy / (math.pi * diskR ** 2))


# --------------------------------------------------------------------------
# Transformer (src/boost_fractor_transformer.jl)
# --------------------------------------------------------------------------
class Modes:
    """src/boost_fractor_transformer.jl:31-38."""

    def __init__(self, M, L, mode_patterns, mode_kt):
        self.M = M
        self.L = L
        self.mode_patterns = mode_patterns     # (M, 2L+1, nx, ny, dims)
        self.mode_kt = mode_kt                 # (M, 2L+1)
        nm = M * (2 * L + 1)
        self.id = np.eye(nm, dtype=np.complex128)
        self.zeromatrix = np.zeros((nm, nm), dtype=np.complex128)

    @property
    def nm(self):
        return self.M * (2 * self.L + 1)

    def flat(self, dim=0):
        """Patterns as (nm, nx, ny) in the reference's (m-1)(2L+1)+l+L+1 order."""
        M, L = self.M, self.L
        return np.stack([self.mode_patterns[m, l + L, :, :, dim]
                         for m in range(M) for l in range(-L, L + 1)])


def besselj_zero(nu, m):
    """FunctionZeros.besselj_zero(nu, m): m-th positive zero of J_nu (integer nu)."""
    return float(special.jn_zeros(int(nu), int(m))[-1])


def mode(m, l, L, coords, diskR=0.15, pattern_input=None, kT_arr=None):
    """Bessel disk mode (src/boost_fractor_transformer.jl:88-107); m is 1-based."""
    X, Y = coords.X, coords.Y
    RR = np.sqrt(X[:, None] ** 2 + Y[None, :] ** 2)
    XX, YY = np.broadcast_arrays(X[:, None], Y[None, :])
    Phi = np.arctan2(YY, XX)
    kr = besselj_zero(abs(l), m) / diskR
    kt = complex(kr)
    if pattern_input is None:
        pattern = special.jv(l, kr * RR) * np.exp(-1j * l * Phi)
        pattern[RR > diskR] *= 0
        pattern = pattern / np.sqrt(np.sum(np.abs(pattern) ** 2))
        pattern = pattern[:, :, None]
    else:
        pattern = np.asarray(pattern_input)[m - 1, l + L]
        if kT_arr is None:
            raise ValueError("you have to define kTs as well when putting in an input pattern")
        kt = complex(np.asarray(kT_arr)[m - 1, l + L])
    return kt, pattern


def seed_modes(coords, ThreeDim=False, Mmax=1, Lmax=0, diskR=0.15, pattern_input=None, kT_arr=None):
    """src/boost_fractor_transformer.jl:46-69."""
    nx, ny = len(coords.X), len(coords.Y)
    if ThreeDim:
        M, L = Mmax, Lmax
        dims = 1 if pattern_input is None else np.asarray(pattern_input).shape[-1]
        patterns = np.zeros((M, 2 * L + 1, nx, ny, dims), dtype=np.complex128)
        kt = np.zeros((M, 2 * L + 1), dtype=np.complex128)
        for m in range(1, M + 1):
            for l in range(-L, L + 1):
                kt[m - 1, l + L], patterns[m - 1, l + L] = mode(
                    m, l, L, coords, diskR=diskR, pattern_input=pattern_input, kT_arr=kT_arr)
    else:
        M, L = 1, 0
        patterns = np.ones((1, 1, nx, ny, 1), dtype=np.complex128)
        kt = np.zeros((1, 1), dtype=np.complex128)
    return Modes(M, L, patterns, kt)


def axion_induced_modes(coords, modes, B=None, velocity_x=0.0, diskR=0.15, f=20e9):
    """Mode coefficients of the normalised axion-induced field (:115-151)."""
    nx, ny = len(coords.X), len(coords.Y)
    dims = modes.mode_patterns.shape[4]
    if B is None:
        B = np.zeros((nx, ny, dims), dtype=np.complex128)
        if dims == 1:
            B[:, :, 0] = 1.0
        elif dims == 3:
            B[:, :, 1] = 1.0
    B = np.array(B, dtype=np.complex128)
    if B.ndim == 2:
        B = B[:, :, None]
    X, Y = coords.X, coords.Y
    if velocity_x != 0:
        lam = wavelength(f)
        ma = 2 * math.pi / lam
        B = B * np.exp(-1j * ma * (-velocity_x) * X)[:, None, None]
    B = B * (np.sqrt(X[:, None] ** 2 + Y[None, :] ** 2) <= diskR)[:, :, None]
    B = B / np.sqrt(np.sum(np.abs(B) ** 2))
    out = np.zeros(modes.nm, dtype=np.complex128)
    L = modes.L
    for m in range(modes.M):
        for l in range(-L, L + 1):
            out[m * (2 * L + 1) + l + L] = np.sum(np.conj(modes.mode_patterns[m, l + L]) * B)
    return out


def field2modes(pattern, coords, modes, diskR=0.15):
    """src/boost_fractor_transformer.jl:156."""
    return axion_induced_modes(coords, modes, B=pattern, diskR=diskR)


def modes2field(mode_coeffs, coords, modes):
    """src/boost_fractor_transformer.jl:161-167."""
    nx, ny = len(coords.X), len(coords.Y)
    dims = modes.mode_patterns.shape[4]
    res = np.zeros((nx, ny, dims), dtype=np.complex128)
    L = modes.L
    for m in range(modes.M):
        for l in range(-L, L + 1):
            res += mode_coeffs[m * (2 * L + 1) + l + L] * modes.mode_patterns[m, l + L]
    return res


def propagation_matrix(dz, diskR, eps, tilt_x, tilt_y, surface, lam, coords, modes,
                       is_air=None, onlydiagonal=False, prop=propagator):
    """Mode-mixing matrix of one region (src/boost_fractor_transformer.jl:174-227)."""
    eps = complex(eps)
    if is_air is None:
        is_air = (eps.real == 1)
    nm = modes.nm
    L = modes.L
    dims = modes.mode_patterns.shape[4]
    mat = np.zeros((nm, nm), dtype=np.complex128)
    k0 = k0_of(eps, lam)
    X, Y = coords.X, coords.Y
    if is_air:
        def propfunc(x):
            return prop(x.copy(), dz, diskR, eps, tilt_x, tilt_y, surface, lam, coords)
    else:
        tmap = (np.exp(-1j * k0 * tilt_x * X)[:, None] * np.exp(-1j * k0 * tilt_y * Y)[None, :]) \
            * np.exp(-1j * k0 * np.asarray(surface))

        def propfunc(x):
            return x * tmap
    pats = modes.mode_patterns
    for mp in range(modes.M):
        for lp in range(-L, L + 1):
            col = mp * (2 * L + 1) + lp + L
            for d in range(dims):
                propagated = propfunc(pats[mp, lp + L, :, :, d])
                if onlydiagonal:
                    mat[col, col] += np.sum(np.conj(pats[mp, lp + L, :, :, d]) * propagated)
                else:
                    for m in range(modes.M):
                        for l in range(-L, L + 1):
                            row = m * (2 * L + 1) + l + L
                            mat[row, col] += np.sum(np.conj(pats[m, l + L, :, :, d]) * propagated)
    if not is_air:
        diag = np.zeros(nm, dtype=np.complex128)
        for m in range(modes.M):
            for l in range(-L, L + 1):
                kt = np.complex128(modes.mode_kt[m, l + L])
                kz = np.sqrt(k0 * k0 - kt * kt)
                diag[m * (2 * L + 1) + l + L] = np.exp(-1j * kz * dz)
        mat = diag[:, None] * mat
    return mat


def calc_propagation_matrices(bdry, coords, modes, f=10.0e9, prop=propagator, diskR=0.15):
    """src/boost_fractor_transformer.jl:274-280."""
    lam = wavelength(f)
    return [propagation_matrix(bdry.distance[i], diskR, bdry.eps[i], bdry.relative_tilt_x[i],
                               bdry.relative_tilt_y[i], bdry.relative_surfaces[i], lam, coords,
                               modes, prop=prop)
            for i in range(len(bdry.eps))]


def get_boundary_matrix(n_left, n_right, diffprop, modes):
    """G * blockdiag(P, inv(P)) (src/boost_fractor_transformer.jl:238-252)."""
    I, Z = modes.id, modes.zeromatrix
    G = (1.0 / (2 * n_right)) * np.block([[(n_right + n_left) * I, (n_right - n_left) * I],
                                           [(n_right - n_left) * I, (n_right + n_left) * I]])
    return G @ np.block([[diffprop, Z], [Z, np.linalg.inv(diffprop)]])


def axion_S_factor(n1, n0):
    """src/boost_fractor_transformer.jl:266-268."""
    return (1.0 / n1 ** 2 - 1.0 / n0 ** 2) / 2


def axion_contrib(T, n1, n0, initial, modes):
    """src/boost_fractor_transformer.jl:258-261."""
    nm = modes.nm
    return axion_S_factor(n1, n0) * (T[nm:, :nm] @ initial + T[nm:, nm:] @ initial)


def transformer(bdry, coords, modes, f=10.0e9, velocity_x=0.0, prop=propagator,
                propagation_matrices=None, diskR=0.15, emit=None, reflect=None):
    """Transfer-matrix mode matching (src/boost_fractor_transformer.jl:285-359).

    Like the reference, NaN permittivities of ``bdry`` are replaced by 1e30 in
    place (:289).
    """
    if emit is None:
        emit = axion_induced_modes(coords, modes, B=None, velocity_x=velocity_x, diskR=diskR, f=f)
    bdry.eps[np.isnan(bdry.eps)] = 1e30
    nm = modes.nm
    T = np.block([[modes.id, modes.zeromatrix], [modes.zeromatrix, modes.id]])
    lam = wavelength(f)
    initial = np.asarray(emit, dtype=np.complex128)
    axion_beam = np.zeros(nm, dtype=np.complex128)
    nreg = len(bdry.eps)

    def idx(s):  # 1-based s -> 0-based region index (Nregions - s + 1) - 1
        return nreg - s

    for s in range(nreg - 1, 0, -1):
        axion_beam += axion_contrib(T, np.sqrt(bdry.eps[idx(s + 1)]), np.sqrt(bdry.eps[idx(s)]), initial, modes)
        j = idx(s)
        if propagation_matrices is None or len(propagation_matrices) == 0:
            diffprop = propagation_matrix(bdry.distance[j], diskR, bdry.eps[j], bdry.relative_tilt_x[j],
                                          bdry.relative_tilt_y[j], bdry.relative_surfaces[j], lam,
                                          coords, modes, prop=prop)
        else:
            diffprop = propagation_matrices[j]
        T = T @ get_boundary_matrix(np.sqrt(bdry.eps[j]), np.sqrt(bdry.eps[idx(s + 1)]), diffprop, modes)
    T22 = T[nm:, nm:]
    boost = -np.linalg.solve(T22, axion_beam)
    if reflect is None:
        return boost
    refl = -np.linalg.solve(T22, T[nm:, :nm] @ np.asarray(reflect, dtype=np.complex128))
    return boost, refl


def transformer_trace_back(reflected_beam, input_beam, bdry, coords, modes, inlcudes_axion=False,
                           f=10.0e9, velocity_x=0.0, prop=propagator, propagation_matrices=None,
                           diskR=0.15, emit=None):
    """Per-region mode amplitudes (src/boost_fractor_transformer.jl:372-421).

    The reference stores each region's solution vector vcat(R, L) (length
    2 nm) into the (2, nm) slice fields_regions[i, :, :] (:401, :419), which
    Julia fills in column-major order: element k lands at (k % 2, k // 2).
    That fill is kept here (a Fortran-order reshape); for nm = 1 it is the
    plain (R, L) pair.  vcat(input_beam, reflected_beam) must have 2 nm
    elements, as in the reference (a DimensionMismatch there otherwise)."""
    if emit is None:
        nx, ny = len(coords.X), len(coords.Y)
        emit = axion_induced_modes(coords, modes, B=np.ones((nx, ny)), diskR=diskR)
    nm = modes.nm
    lam = wavelength(f)
    nreg = len(bdry.eps)
    out = np.zeros((nreg, 2, nm), dtype=np.complex128)
    emit = np.atleast_1d(np.asarray(emit, dtype=np.complex128))
    both = np.concatenate([emit, emit])
    sol = np.concatenate([np.atleast_1d(input_beam), np.atleast_1d(reflected_beam)]).astype(np.complex128)
    if len(sol) != 2 * nm:
        raise ValueError("vcat(input_beam, reflected_beam) must have 2 nm elements")

    def idx(s):
        return nreg - s

    out[idx(1)] = sol.reshape((2, nm), order="F")
    for s in range(1, nreg):
        j = idx(s)
        if propagation_matrices is None:
            diffprop = propagation_matrix(bdry.distance[j], diskR, bdry.eps[j], bdry.relative_tilt_x[j],
                                          bdry.relative_tilt_y[j], bdry.relative_surfaces[j], lam,
                                          coords, modes, prop=prop)
        else:
            diffprop = propagation_matrices[j]
        Gb = get_boundary_matrix(np.sqrt(bdry.eps[j]), np.sqrt(bdry.eps[idx(s + 1)]), diffprop, modes)
        sol = Gb @ sol
        if inlcudes_axion:
            sol = sol + axion_S_factor(np.sqrt(bdry.eps[idx(s + 1)]), np.sqrt(bdry.eps[j])) * both
        out[idx(s + 1)] = sol.reshape((2, nm), order="F")
    return out


# --------------------------------------------------------------------------
# Beam utilities (src/beam_gaussian.jl, src/beam_coupling.jl)
# --------------------------------------------------------------------------
def gauss_profile(coords, z=1e-9, omega0=0.1, f=10e9):
    """src/beam_gaussian.jl:24-37."""
    X, Y = coords.X, coords.Y
    radius = np.sqrt(X[:, None] ** 2 + Y[None, :] ** 2)
    lam = wavelength(f)
    k = 2 * math.pi / lam
    zR = math.pi * omega0 ** 2 / lam
    omega = omega0 * math.sqrt(1 + (z / zR) ** 2)
    Rz = z * (1 + (zR / z) ** 2)
    psi = math.atan(z / zR)
    return omega0 / omega * np.exp(-radius ** 2 / omega ** 2) * \
        np.exp(-1j * (k * z + k * radius ** 2 / (2 * Rz) - psi))


def unnormalized_match(Eout, Eantenna, dx=0.01, dy=0.01):
    """src/beam_coupling.jl:13-15."""
    return np.sum(np.asarray(Eout) * np.conj(Eantenna)) * dx * dy


# --------------------------------------------------------------------------
# Optimiser utilities (examples/transformer_optim_utilities.jl)
# --------------------------------------------------------------------------
def calc_propagation_matrices_grid(sbdry, coords, modes, spacing_grid, frequencies, prop=propagator, diskR=0.15,
                                   tilt_x_grid=None, tilt_y_grid=None):
    """examples/transformer_optim_utilities.jl:10-50.

    Returns [region, frequency, spacing, nm, nm], or with tilt grids the
    reference's [region, frequency, spacing, tilt_x, tilt_y, nm, nm].  The
    gaps are the regions 1, 3, ..., nd-1 (0-based; the reference's ind_gap =
    2:2:n_region, the exit region included); they move by spacing_grid[s] and
    tilt by tilt_x_grid[tx], tilt_y_grid[ty] on top of their own tilts
    (:40-43); the mirror and the disks (ind_solid) are computed once per
    frequency.  The reference splits the setup into a gap setup and a solid
    setup; a region's matrix depends only on that region's parameters, so
    shifting the gaps of one copy of the setup gives the same matrices.
    """
    nd = len(sbdry.distance)
    gaps = np.arange(1, nd, 2)
    nm = modes.M * (2 * modes.L + 1)
    sg = np.asarray(spacing_grid, dtype=float)
    tilts = tilt_x_grid is not None or tilt_y_grid is not None
    txg = np.atleast_1d(np.asarray(0.0 if tilt_x_grid is None else tilt_x_grid, dtype=float))
    tyg = np.atleast_1d(np.asarray(0.0 if tilt_y_grid is None else tilt_y_grid, dtype=float))
    out = np.empty((nd, len(frequencies), len(sg), len(txg), len(tyg), nm, nm), dtype=complex)
    for f, fr in enumerate(frequencies):
        solid = calc_propagation_matrices(sbdry, coords, modes, f=fr, prop=prop, diskR=diskR)
        for s, sp in enumerate(sg):
            for a, tx in enumerate(txg):
                for b, ty in enumerate(tyg):
                    sb = copy.deepcopy(sbdry)
                    sb.distance = np.array(sbdry.distance, dtype=float)
                    sb.distance[gaps] += sp
                    sb.relative_tilt_x = np.array(sbdry.relative_tilt_x, dtype=float)
                    sb.relative_tilt_y = np.array(sbdry.relative_tilt_y, dtype=float)
                    sb.relative_tilt_x[gaps] += tx
                    sb.relative_tilt_y[gaps] += ty
                    pm = calc_propagation_matrices(sb, coords, modes, f=fr, prop=prop, diskR=diskR)
                    for r in range(nd):
                        out[r, f, s, a, b] = pm[r] if r % 2 == 1 else solid[r]
    return out if tilts else out[:, :, :, 0, 0]


class SpacingSpline:
    """construct_prop_matrix_interpolation (utilities :56-73): cubic B-spline
    along the spacing axis, Interpolations.jl BSpline(Cubic(Natural(OnCell()))).

    Interpolations.jl (an unpinned dependency of the example, not vendored)
    documents Natural (= Line) as a zero second derivative at the boundary, and
    OnCell as placing that boundary at the cell edges, half a grid step beyond
    the first and last point, where the interpolation's domain ends too.
    Restated from that definition: with knot coordinates u = 1..n and
    coefficients c_0..c_{n+1},
        s(u) = sum_k c_k B3(u - k),   s(j) = y_j (j = 1..n),
        s''(1/2) = s''(n + 1/2) = 0,
    the end segments' polynomials extended over the half cells; the
    (n+2) x (n+2) system is solved densely with numpy.linalg.solve.
    """

    def __init__(self, grid, spacing_grid):
        sg = np.asarray(spacing_grid, dtype=float)
        self.first, self.step, self.n = sg[0], sg[1] - sg[0], len(sg)
        n = self.n
        A = np.zeros((n + 2, n + 2))

        def d2_row(i, t):   # s''(i + t) from the four coefficients c_{i-1..i+2}
            row = np.zeros(n + 2)
            row[i - 1:i + 2] += (1 - t) * np.array([1.0, -2.0, 1.0])
            row[i:i + 3] += t * np.array([1.0, -2.0, 1.0])
            return row

        A[0] = d2_row(1, -0.5)
        for j in range(1, n + 1):
            A[j, j - 1:j + 2] = np.array([1.0, 4.0, 1.0]) / 6.0
        A[n + 1] = d2_row(n - 1, 1.5)
        y = np.moveaxis(np.asarray(grid), 2, 0)            # spacing axis first
        rhs = np.zeros((n + 2,) + y.shape[1:], dtype=complex)
        rhs[1:n + 1] = y
        self.coef = np.linalg.solve(A, rhs.reshape(n + 2, -1)).reshape(rhs.shape)

    @property
    def bounds(self):
        """Interpolations.bounds(itp)[3]: half a step beyond the end spacings."""
        return (self.first - 0.5 * self.step, self.first + (self.n - 0.5) * self.step)

    def __call__(self, r, f, shift):
        lo, hi = self.bounds
        if not (lo <= shift <= hi):
            raise IndexError("shift outside the interpolation bounds")
        u = 1.0 + (shift - self.first) / self.step
        i = min(max(int(math.floor(u)), 1), self.n - 1)
        t = u - i
        w = np.array([(1 - t) ** 3, 3 * t ** 3 - 6 * t ** 2 + 4, -3 * t ** 3 + 3 * t ** 2 + 3 * t + 1, t ** 3]) / 6.0
        return np.tensordot(w, self.coef[i - 1:i + 3, r, f], axes=1)


def construct_prop_matrix_interpolation(prop_matrix_grid, spacing_grid):
    """utilities :56-73."""
    return SpacingSpline(prop_matrix_grid, spacing_grid)


def interpolate_prop_matrix(itp, dist_shift):
    """utilities :78-91: matrices [region][frequency] at the per-disk shifts;
    solids and the exit region take shift 0 (:84)."""
    nd = itp.coef.shape[1]
    nf = itp.coef.shape[2]
    shift_all = [0.0 if (r % 2 == 0 or r == nd - 1) else dist_shift[(r - 1) // 2] for r in range(nd)]
    return [[itp(r, f, shift_all[r]) for f in range(nf)] for r in range(nd)]


def calc_boostfactor_modes(sbdry, coords, modes, frequencies, prop_matrices_set, prop=propagator, diskR=0.15):
    """utilities :99-110: EoutModes0[0, mode, frequency]."""
    nm = modes.M * (2 * modes.L + 1)
    out = np.empty((1, nm, len(frequencies)), dtype=complex)
    for f, fr in enumerate(frequencies):
        out[0, :, f] = transformer(sbdry, coords, modes, prop=prop, diskR=diskR, f=fr,
                                   propagation_matrices=[prop_matrices_set[r][f] for r in range(len(prop_matrices_set))])
    return out


def soft_box_penalty(shift, bound_hard):
    """utilities :150-160."""
    depth = (bound_hard[1] - bound_hard[0]) * 0.05
    l_soft, u_soft = bound_hard[0] + depth, bound_hard[1] - depth
    ext = np.concatenate([np.asarray(shift, dtype=float), [np.sum(shift)]])
    excess = max(np.max(ext) - u_soft, -(np.min(ext) - l_soft), 0.0)
    return 1.0 - (excess / depth) ** 6


def p_norm(X, p):
    """utilities :211-215."""
    X = np.asarray(X, dtype=float)
    mag = np.max(X)
    return mag * (np.sum((X / mag) ** p) / len(X)) ** (1.0 / p)


def calc_boostfactor_cost(dist_shift, itp, frequencies, sbdry, coords, modes, m_reflect, prop=propagator,
                          diskR=0.15):
    """utilities :130-144."""
    lo, hi = itp.bounds
    if any(not (lo < s < hi) for s in dist_shift):
        return 1000.0
    penalty = soft_box_penalty(dist_shift, (lo, hi))
    pm = interpolate_prop_matrix(itp, dist_shift)
    Eout = calc_boostfactor_modes(sbdry, coords, modes, frequencies, pm, prop=prop, diskR=diskR)
    cpld = np.abs(np.sum(np.conj(Eout[0]) * np.asarray(m_reflect)[:, None], axis=0)) ** 2
    return -p_norm(cpld, -20) * penalty
