"""Seeded synthetic disk stacks for the benchmark configurations.

No public dataset is involved: every input is generated from a numpy
``default_rng(seed)``.  Each function returns a dict with the reference's
geometry arrays (``distance``, ``eps``, ``relative_tilt_x/y``,
``relative_surfaces`` or None), the grid ``X``/``Y``, ``diskR``, the
frequencies and the solver settings.
"""
import numpy as np


def symmetric_grid(n, width=1.0):
    """n points from -width/2 to +width/2, exactly antisymmetric in floating point."""
    i = np.arange(n, dtype=np.float64)
    return width * (2 * i - (n - 1)) / (2.0 * (n - 1)) if n > 1 else np.zeros(1)


def booster(ndisk, gaps, eps_disk=24.0, thickness=1e-3, tilt_x=None, tilt_y=None):
    """Mirror + ndisk disks: regions [mirror, gap1, disk1, ..., gapN, diskN, exit]."""
    nd = 2 * ndisk + 2
    distance = np.zeros(nd)
    eps = np.ones(nd, dtype=np.complex128)
    eps[0] = np.nan
    for k in range(ndisk):
        distance[1 + 2 * k] = gaps[k]
        distance[2 + 2 * k] = thickness
        eps[2 + 2 * k] = eps_disk
    tx = np.zeros(nd) if tilt_x is None else np.asarray(tilt_x, dtype=np.float64)
    ty = np.zeros(nd) if tilt_y is None else np.asarray(tilt_y, dtype=np.float64)
    return distance, eps, tx, ty


def config1_dancer():
    """Plain dancer, complex128: mirror + 1 disk (eps 24, 1 mm, R 0.15 m, gap 8 mm),
    64x64 grid over 1 m, 20 GHz, homogeneous emission, nmax = 200 (201 bounces)."""
    distance, eps, tx, ty = booster(1, [8e-3])
    X = symmetric_grid(64)
    return dict(name="dancer-1disk-64", solver="dancer", distance=distance, eps=eps,
                relative_tilt_x=tx, relative_tilt_y=ty, relative_surfaces=None, X=X, Y=X.copy(),
                diskR=0.15, freqs=np.array([20e9]), nmax=200, precision="fp64")


def config2_cheerleader(seed=2, n=128, ndisk=20, nf=256, nmax=400, f_lo=19.5e9, f_hi=20.5e9):
    """20-disk booster, cheerleader: 128x128 over 1 m, R 0.15 m, eps 24, 1 mm disks,
    gaps U(7.5, 8.5) mm, per-disk tilts U(-0.5, 0.5) mrad (air regions untilted),
    256 frequencies 19.5-20.5 GHz, 400 bounces (nmax = 400), mixed precision."""
    rng = np.random.default_rng(seed)
    gaps = rng.uniform(7.5e-3, 8.5e-3, ndisk)
    nd = 2 * ndisk + 2
    tx = np.zeros(nd)
    ty = np.zeros(nd)
    for k in range(ndisk):
        tx[2 + 2 * k] = rng.uniform(-0.5e-3, 0.5e-3)
        ty[2 + 2 * k] = rng.uniform(-0.5e-3, 0.5e-3)
    distance, eps, tx, ty = booster(ndisk, gaps, tilt_x=tx, tilt_y=ty)
    X = symmetric_grid(n)
    return dict(name=f"cheerleader-{ndisk}disk-{n}", solver="cheerleader", distance=distance,
                eps=eps, relative_tilt_x=tx, relative_tilt_y=ty, relative_surfaces=None, X=X,
                Y=X.copy(), diskR=0.15, freqs=np.linspace(f_lo, f_hi, nf), nmax=nmax,
                precision="mixed")


def surface_roughness(X, Y, ngaps, rng, mag=1e-5, trunc=1e-4, xi=0.02, diskR=0.15):
    """Gaussian random surface maps, the recipe of the reference's optimiser
    utilities (examples/transformer_optim_utilities.jl:166-195): white noise of
    rms `mag`, 2D convolution with exp(-(x^2+y^2)/(2 xi^2)) cropped to the grid,
    renormalised to rms `mag`, clipped at +-trunc, zero outside r > diskR."""
    from scipy.signal import fftconvolve
    n = len(X)
    init = mag * rng.standard_normal((ngaps, len(X), len(Y)))
    g = np.exp(-(X[:, None] ** 2 + Y[None, :] ** 2) / (2 * xi ** 2))
    lo, hi = int(np.floor(n / 2)) - 1, int(np.floor(n * 1.5)) - 1
    for i in range(ngaps):
        init[i] = fftconvolve(init[i], g, mode="full")[lo:hi, lo:hi]
    init /= np.sqrt(np.sum(init ** 2, axis=(1, 2)) / (len(X) * len(Y)))[:, None, None]
    init *= mag
    np.clip(init, -trunc, trunc, out=init)
    init *= ((X[:, None] ** 2 + Y[None, :] ** 2) <= diskR ** 2)[None]
    return init


def lg_orders(n_modes):
    """(p, l) of the n_modes lowest-order Laguerre-Gauss modes, ordered by the
    order N = 2p + |l|, then by l (-N, -N+2, ..., N)."""
    out = []
    N = 0
    while len(out) < n_modes:
        for l in range(-N, N + 1, 2):
            out.append(((N - abs(l)) // 2, l))
        N += 1
    return out[:n_modes]


def lg_modes(X, Y, n_modes=64, waist=0.03, diskR=0.15):
    """Laguerre-Gauss modes LG_p^l(r) e^{-i l phi} at the waist, as the
    reference's `pattern_input` and `kT_arr` of SeedModes
    (src/boost_fractor_transformer.jl:46, :99-104): patterns (n_modes, 1, nx,
    ny, 1) cut to r <= diskR and normalised to sum |pattern|^2 = 1, and the
    paraxial transverse wavenumber kT = 2 sqrt(N + 1) / waist of each mode
    (the Gouy phase (N + 1) z / z_R written as kz = sqrt(k^2 - kT^2) to first
    order), N = 2p + |l|.

    With the 3 cm waist every one of the 64 lowest orders (N <= 10) lies
    inside the 0.15 m disk and propagates in air above 10 GHz (kT <= 221 rad/m),
    so the transfer-matrix chain through a 20-disk stack stays well conditioned.
    """
    from scipy.special import eval_genlaguerre
    X = np.asarray(X, dtype=np.float64)
    Y = np.asarray(Y, dtype=np.float64)
    RR = np.sqrt(X[:, None] ** 2 + Y[None, :] ** 2)
    Phi = np.arctan2(np.broadcast_to(Y[None, :], RR.shape), np.broadcast_to(X[:, None], RR.shape))
    u = 2.0 * RR ** 2 / waist ** 2
    orders = lg_orders(n_modes)
    pats = np.zeros((n_modes, 1, len(X), len(Y), 1), dtype=np.complex128)
    kt = np.zeros((n_modes, 1), dtype=np.complex128)
    for i, (p, l) in enumerate(orders):
        a = abs(l)
        field = u ** (a / 2.0) * eval_genlaguerre(p, a, u) * np.exp(-u / 2.0) * np.exp(-1j * l * Phi)
        field[RR > diskR] = 0.0
        pats[i, 0, :, :, 0] = field / np.sqrt(np.sum(np.abs(field) ** 2))
        kt[i, 0] = 2.0 * np.sqrt(2 * p + a + 1.0) / waist
    return pats, kt


def config3_transformer(seed=3, n=256, ndisk=20, nf=1024, modes=64, f_lo=19e9, f_hi=21e9, waist=0.03):
    """Transformer mode matching: the 20-disk geometry of the cheerleader
    workload on a 256x256 grid, per-disk surface maps (GRF, rms 10 um,
    correlation length 2 cm), 64 Laguerre-Gauss modes (the 64 lowest orders,
    waist 3 cm, given as pattern_input with M=64, L=0), 1024 frequencies
    19-21 GHz."""
    w = config2_cheerleader(seed=seed, n=n, ndisk=ndisk, nf=nf, f_lo=f_lo, f_hi=f_hi)
    rng = np.random.default_rng(seed + 1000)
    nd = len(w["distance"])
    surf = np.zeros((nd, n, n))
    surf[2:nd - 1:2] = surface_roughness(w["X"], w["Y"], ndisk, rng)
    pats, kt = lg_modes(w["X"], w["Y"], modes, waist, w["diskR"])
    w.update(name=f"transformer-{ndisk}disk-{n}-{modes}LGmodes", solver="transformer", relative_surfaces=surf,
             M=modes, L=0, pattern_input=pats, kT_arr=kt)
    return w


def fresnel_r(eps):
    """SeedSetupBoundaries' reflectivities (src/boost_fractor.jl:98-103), numpy form."""
    e = np.array(eps, dtype=np.complex128)
    e.imag[e.imag == 0.0] = -0.0
    r = [1.0 + 0j]
    for i in range(2, len(e)):
        a, b = np.sqrt(e[i - 1]), np.sqrt(e[i])
        r.append((a - b) / (a + b))
    return np.array(r, dtype=np.complex128)


def config4_uneven(seed=4, count=4096, nmax=100, modes=16, waist=0.03):
    """Uneven batch: `count` seeded disk stacks, disk count U{5..80}, grid
    N in {64, 128, 256} over 1 m, frequency count U{64..1024} in 19.5-20.5 GHz,
    gaps U(6, 10) mm, eps in {9.4, 24}, 1 mm disks, half dancer (nmax + 1
    bounces, mixed precision) and half transformer (`modes` Laguerre-Gauss
    modes of waist 3 cm, mixed precision).  Returns a list of request dicts;
    the stacks are untilted and flat."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        ndisk = int(rng.integers(5, 81))
        n = int(rng.choice([64, 128, 256]))
        nf = int(rng.integers(64, 1025))
        eps_disk = float(rng.choice([9.4, 24.0]))
        solver = "dancer" if rng.random() < 0.5 else "transformer"
        gaps = rng.uniform(6e-3, 10e-3, ndisk)
        distance, eps, tx, ty = booster(ndisk, gaps, eps_disk=eps_disk)
        out.append(dict(name=f"c4-{k}", solver=solver, ndisk=ndisk, n=n, nf=nf, distance=distance, eps=eps,
                        relative_tilt_x=tx, relative_tilt_y=ty, X=symmetric_grid(n), diskR=0.15,
                        freqs=np.linspace(19.5e9, 20.5e9, nf), nmax=nmax, M=modes, waist=waist,
                        precision="mixed"))
    return out


def optimiser_step(distance, rng, sigma=10e-6):
    """One disk-position optimiser step: every gap (regions 1, 3, ..., nd-3)
    moves by N(0, sigma)."""
    d = np.array(distance, dtype=np.float64)
    d[1:-1:2] += rng.normal(0.0, sigma, len(d[1:-1:2]))
    return d
