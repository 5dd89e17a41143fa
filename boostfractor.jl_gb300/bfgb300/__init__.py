"""Python mirror of BoostFractor.jl's public API on the GB300 C ABI.

Same names, keyword arguments and array semantics as the reference module
(src/BoostFractor.jl:5-20): ``SeedCoordinateSystem``, ``SeedSetupBoundaries``,
``propagator`` & co. (the ``prop=`` plug-ins), ``cheerleader``, ``dancer``.
Arrays follow the reference's index order with 0-based numpy indexing
(``E[x, y]``, ``relative_surfaces[region, x, y]``, ``emit[region, dir, x, y]``);
they are handed to the C ABI in Julia's column-major memory layout.

Extensions over the reference signatures (all keyword-only, with defaults that
keep the reference behaviour):
  * ``f`` may be an array: the frequencies are solved as one batch and the
    outputs gain a leading frequency axis;
  * ``precision``: ``"fp64"`` (default, complex128 everywhere) or ``"mixed"``
    (complex64 fields, FP64 phase arguments and exit accumulation);
  * ``handle``: a :class:`Handle` (one per host thread; a default one is made).
"""
import ctypes
import math
import atexit
import threading
import weakref

import numpy as np

from . import _lib
from ._lib import BFError, SingularError

__all__ = [
    "CoordinateSystem", "SeedCoordinateSystem", "SetupBoundaries", "SeedSetupBoundaries",
    "wavelength", "propagator", "propagatorNoTilts", "propagatorMomentumSpace", "propagator1D",
    "cheerleader", "dancer", "Handle", "Stack", "boost_factor", "BFError", "SingularError", "transformer_group",
    "autotune", "autotune_report",
    "Modes", "SeedModes", "axion_induced_modes", "field2modes", "modes2field",
    "calc_propagation_matrices", "transformer", "transformer_trace_back", "Server",
    "gauss_profile", "unnormalized_match", "transformer_coupled", "transformer_1d_batch",
    "PGrid",
]

SPEED_OF_LIGHT = 299792458.0


def wavelength(frequency):
    """src/boost_fractor.jl:16-19."""
    return SPEED_OF_LIGHT / frequency


# --------------------------------------------------------------------------
# handle
# --------------------------------------------------------------------------
class Handle:
    """One CUDA stream + device allocations (bf_create / bf_destroy)."""

    def __init__(self, device=0, hbm_budget_bytes=0):
        L = _lib.lib()
        h = _lib._vp()
        rc = L.bf_create(int(device), int(hbm_budget_bytes), _lib.ctypes.byref(h))
        if rc != _lib.BF_OK:
            raise BFError(rc, "bf_create failed (no usable CUDA device?)")
        self._h = h
        self.device = device

    @property
    def ptr(self):
        return self._h

    def check(self, rc):
        if rc != _lib.BF_OK:
            msg = _lib.lib().bf_last_error(self._h)
            cls = SingularError if rc == _lib.BF_ERR_SINGULAR else BFError
            raise cls(rc, msg.decode() if msg else "")

    def device_bytes(self):
        return int(_lib.lib().bf_device_bytes(self._h))

    def set_stream(self, cuda_stream_ptr):
        """Run on a caller's cudaStream_t (integer handle; 0 = the handle's own stream)."""
        self.check(_lib.lib().bf_set_stream(self._h, _lib._vp(int(cuda_stream_ptr) or None)))

    def set_profiling(self, enable=True):
        self.check(_lib.lib().bf_set_profiling(self._h, int(bool(enable))))

    def last_profile(self):
        """dict of the last solve's device profile (see bf_last_profile)."""
        out = np.zeros(8)
        self.check(_lib.lib().bf_last_profile(self._h, _lib.ptr(out)))
        keys = ["solve_ms", "stages_ms", "tables_ms", "exits_ms", "stage_launches", "launches",
                "propagations", "nfreq"]
        return dict(zip(keys, out.tolist()))

    def close(self):
        if self._h:
            _lib.lib().bf_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_tls = threading.local()


def default_handle():
    h = getattr(_tls, "handle", None)
    if h is None:
        h = Handle(0)
        _tls.handle = h
    return h


# --------------------------------------------------------------------------
# geometry (src/boost_fractor.jl:16-108)
# --------------------------------------------------------------------------
class CoordinateSystem:
    """src/boost_fractor.jl:21-28."""

    def __init__(self, X, Y, kX, kY):
        self.X = np.ascontiguousarray(X, dtype=np.float64)
        self.Y = np.ascontiguousarray(Y, dtype=np.float64)
        self.kX = np.ascontiguousarray(kX, dtype=np.float64)
        self.kY = np.ascontiguousarray(kY, dtype=np.float64)


def get_kspace_coords(real_coords):
    """src/boost_fractor.jl:42-47 (evaluated by the C ABI's host helper)."""
    x = np.ascontiguousarray(real_coords, dtype=np.float64)
    out = np.empty_like(x)
    rc = _lib.lib().bf_get_kspace_coords(len(x), _lib.ptr(x), _lib.ptr(out))
    if rc != _lib.BF_OK:
        raise BFError(rc, "get_kspace_coords")
    return out


def SeedCoordinateSystem(X=None, Y=None):
    """src/boost_fractor.jl:30-34; default X = Y = -0.5:0.01:0.5."""
    if X is None:
        X = np.array([i / 100 for i in range(-50, 51)])
    if Y is None:
        Y = np.array([i / 100 for i in range(-50, 51)])
    X = np.asarray(X, dtype=np.float64)
    Y = np.asarray(Y, dtype=np.float64)
    return CoordinateSystem(X, Y, get_kspace_coords(X), get_kspace_coords(Y))


class SetupBoundaries:
    """src/boost_fractor.jl:63-71."""

    def __init__(self, distance, r, eps, relative_tilt_x, relative_tilt_y, relative_surfaces):
        self.distance = np.array(distance, dtype=np.float64)
        self.r = np.array(r, dtype=np.complex128)
        self.eps = np.array(eps, dtype=np.complex128)
        self.relative_tilt_x = np.array(relative_tilt_x, dtype=np.float64)
        self.relative_tilt_y = np.array(relative_tilt_y, dtype=np.float64)
        self.relative_surfaces = np.array(relative_surfaces, dtype=np.complex128)


def _eps_cast(eps):
    eps = np.array(eps, dtype=np.complex128)
    eps.imag[eps.imag == 0.0] = -0.0
    return eps


def SeedSetupBoundaries(coords, diskno=3, distance=None, epsilon=None, relative_tilt_x=None,
                        relative_tilt_y=None, relative_surfaces=None):
    """src/boost_fractor.jl:83-108 (defaults, Fresnel r, dimension check)."""
    nd0 = 2 * diskno + 2
    if relative_tilt_x is None:
        relative_tilt_x = np.zeros(nd0)
    if relative_tilt_y is None:
        relative_tilt_y = np.zeros(nd0)
    if relative_surfaces is None:
        relative_surfaces = np.zeros((nd0, len(coords.X), len(coords.Y)))
    if distance is None:
        distance = [0.0] + [8e-3 if x % 2 == 1 else 1e-3 for x in range(1, 2 * diskno + 1)] + [0.0]
    if epsilon is None:
        epsilon = [np.nan] + [1.0 if x % 2 == 1 else 9.0 for x in range(1, 2 * diskno + 1)] + [1.0]
    eps = _eps_cast(epsilon)
    r = np.zeros(len(eps) - 1, dtype=np.complex128)
    if len(eps) >= 2:
        e = np.ascontiguousarray(eps)
        rc = _lib.lib().bf_fresnel_reflectivities(len(e), _lib.ptr(e.view(np.float64)),
                                                  _lib.ptr(r.view(np.float64)))
        if rc != _lib.BF_OK:
            raise BFError(rc, "fresnel")
    relative_surfaces = np.asarray(relative_surfaces)
    if not (len(distance) == len(r) + 1 == len(eps) == len(relative_tilt_x) == len(relative_tilt_y)
            == relative_surfaces.shape[0]):
        raise ValueError("DimensionMismatch: the arrays in your SetupBoundaries objects don't fit together!")
    return SetupBoundaries(distance, r, eps, relative_tilt_x, relative_tilt_y, relative_surfaces)


# --------------------------------------------------------------------------
# propagators: the prop= plug-ins (src/boost_fractor.jl:137-227)
# --------------------------------------------------------------------------
_PREC = {"fp64": _lib.BF_PREC_FP64, "mixed": _lib.BF_PREC_MIXED, "tf32": _lib.BF_PREC_TF32,
         "mixed-simt": _lib.BF_PREC_MIXED_SIMT}


def _prec(p):
    if isinstance(p, int):
        return p
    return _PREC[p]


class _Propagator:
    def __init__(self, kind, name):
        self.kind = kind
        self.__name__ = name

    def __call__(self, E0, dz, diskR, eps, tilt_x, tilt_y, surface, lam, coords, precision="fp64",
                 handle=None):
        h = handle or default_handle()
        E = np.asfortranarray(np.array(E0, dtype=np.complex128))
        nx, ny = E.shape
        surf = None
        if surface is not None:
            s = np.asarray(surface)
            if np.any(s != 0):
                surf = np.asfortranarray(np.broadcast_to(s, (nx, ny)).astype(np.complex128))
        eps = complex(eps)
        h.check(_lib.lib().bf_propagate(
            h.ptr, self.kind, _prec(precision), _lib.ptr(_fbuf(E)), nx, ny,
            _lib.ptr(coords.X), _lib.ptr(coords.Y), _lib.ptr(coords.kX), _lib.ptr(coords.kY),
            float(dz), float(diskR), eps.real, eps.imag, float(tilt_x), float(tilt_y),
            _lib.ptr(None if surf is None else _fbuf(surf)), float(lam)))
        return E

    def __repr__(self):
        return self.__name__


def _fbuf(a):
    """float64 view (shared memory) of an F-contiguous complex array, in Julia memory order."""
    assert a.flags.f_contiguous
    return a.T.view(np.float64).reshape(-1)


propagator = _Propagator(_lib.BF_PROP_3D, "propagator")
propagatorNoTilts = _Propagator(_lib.BF_PROP_NOTILTS, "propagatorNoTilts")
propagatorMomentumSpace = _Propagator(_lib.BF_PROP_MOMENTUM, "propagatorMomentumSpace")
propagator1D = _Propagator(_lib.BF_PROP_1D, "propagator1D")


def _prop_kind(prop):
    if isinstance(prop, _Propagator):
        return prop.kind
    if isinstance(prop, int):
        return prop
    raise ValueError("prop must be one of propagator, propagatorNoTilts, propagatorMomentumSpace, "
                     "propagator1D (a custom Python propagator cannot run on the GPU path)")


# --------------------------------------------------------------------------
# resident stacks and the solvers
# --------------------------------------------------------------------------
def _fcplx(a, shape):
    """complex128 array in Julia column-major layout, as a float64 buffer."""
    a = np.asfortranarray(np.broadcast_to(np.asarray(a, dtype=np.complex128), shape))
    return a, _fbuf(a)


class Stack:
    """A SetupBoundaries + CoordinateSystem resident on the device (bf_stack_create)."""

    def __init__(self, bdry, coords, diskR, handle=None):
        self.h = handle or default_handle()
        self.coords = coords
        self.diskR = float(diskR)
        nd = len(bdry.distance)
        nx, ny = len(coords.X), len(coords.Y)
        self.nd, self.nx, self.ny = nd, nx, ny
        self._keep = []
        dist = np.ascontiguousarray(bdry.distance, dtype=np.float64)
        r = np.ascontiguousarray(bdry.r, dtype=np.complex128)
        eps = np.ascontiguousarray(bdry.eps, dtype=np.complex128)
        tx = np.ascontiguousarray(bdry.relative_tilt_x, dtype=np.float64)
        ty = np.ascontiguousarray(bdry.relative_tilt_y, dtype=np.float64)
        surf = np.asarray(bdry.relative_surfaces)
        sbuf = None
        if surf is not None and surf.size and np.any(surf != 0):
            sarr, sbuf = _fcplx(surf, (nd, nx, ny))
            self._keep.append(sarr)
        s = _lib._vp()
        self.h.check(_lib.lib().bf_stack_create(
            self.h.ptr, nd, _lib.ptr(dist), _lib.ptr(r.view(np.float64)), _lib.ptr(eps.view(np.float64)),
            _lib.ptr(tx), _lib.ptr(ty), _lib.ptr(sbuf), nx, ny, _lib.ptr(coords.X), _lib.ptr(coords.Y),
            _lib.ptr(coords.kX), _lib.ptr(coords.kY), self.diskR, _lib.ctypes.byref(s)))
        self._s = s

    def set_distance(self, distance):
        d = np.ascontiguousarray(distance, dtype=np.float64)
        self.h.check(_lib.lib().bf_stack_set_distance(self.h.ptr, self._s, _lib.ptr(d)))

    def graph_stats(self):
        """(solves replayed from the captured stage graph, kernels in it)."""
        r, n = _lib._ull(), _lib._ull()
        self.h.check(_lib.lib().bf_stack_graph_stats(self._s, ctypes.byref(r), ctypes.byref(n)))
        return r.value, n.value

    def beta2_scale(self):
        X, Y = self.coords.X, self.coords.Y
        dx = X[1] - X[0] if len(X) > 1 else 1.0
        dy = Y[1] - Y[0] if len(Y) > 1 else 1.0
        return dx * dy / (math.pi * self.diskR ** 2)

    def cheerleader(self, freqs, amin=0.0, nmax=100, prop=None, emit=None, reflect=None,
                    returnboth=False, precision="fp64", beta2_scale=None, out_device=None):
        """Batched cheerleader; returns (right[nf, nx, ny], left or None, beta2[nf])."""
        freqs = np.ascontiguousarray(np.atleast_1d(freqs), dtype=np.float64)
        nf = len(freqs)
        nx, ny, nd = self.nx, self.ny, self.nd
        kind = _prop_kind(prop or propagator)
        ebuf = rbuf = None
        if emit is not None:
            earr, ebuf = _fcplx(emit, (nd, 2, nx, ny))
        if reflect is not None:
            rarr, rbuf = _fcplx(reflect, (nx, ny))
        right = np.empty((nf, ny, nx), dtype=np.complex128)
        left = np.empty((nf, ny, nx), dtype=np.complex128) if returnboth else None
        beta2 = np.empty(nf, dtype=np.float64)
        scale = self.beta2_scale() if beta2_scale is None else beta2_scale
        self.h.check(_lib.lib().bf_stack_cheerleader(
            self.h.ptr, self._s, nf, _lib.ptr(freqs), float(amin), int(nmax), kind, _prec(precision),
            _lib.ptr(ebuf), _lib.ptr(rbuf), int(bool(returnboth)), float(scale), 0,
            _lib.ptr(right.view(np.float64)), _lib.ptr(None if left is None else left.view(np.float64)),
            _lib.ptr(beta2)))
        return right.transpose(0, 2, 1), (None if left is None else left.transpose(0, 2, 1)), beta2

    def cheerleader_device(self, freqs, out_right_ptr, out_beta2_ptr, nmax=100, prop=None,
                           precision="mixed", out_left_ptr=None, beta2_scale=None):
        """Batched cheerleader with outputs left in device memory (raw device pointers:
        out_right [nf][ny][nx] complex128, out_beta2 [nf] float64)."""
        freqs = np.ascontiguousarray(np.atleast_1d(freqs), dtype=np.float64)
        scale = self.beta2_scale() if beta2_scale is None else beta2_scale
        P = _lib.ctypes.POINTER(_lib.ctypes.c_double)
        cast = lambda v: None if v is None else _lib.ctypes.cast(_lib.ctypes.c_void_p(int(v)), P)
        self.h.check(_lib.lib().bf_stack_cheerleader(
            self.h.ptr, self._s, len(freqs), _lib.ptr(freqs), 0.0, int(nmax),
            _prop_kind(prop or propagator), _prec(precision), None, None,
            int(out_left_ptr is not None), float(scale), _lib.BF_OUT_DEVICE,
            cast(out_right_ptr), cast(out_left_ptr), cast(out_beta2_ptr)))

    def dancer(self, freqs, amin=0.0, nmax=200, prop=None, emit=None, reflect=None, returnsum=True,
               immediatesum=True, precision="fp64", beta2_scale=None):
        """Batched dancer; returns (Eout, beta2[nf]); Eout is [nf, nx, ny] or [nf, nx, ny, nmax+1]."""
        freqs = np.ascontiguousarray(np.atleast_1d(freqs), dtype=np.float64)
        nf = len(freqs)
        nx, ny, nd = self.nx, self.ny, self.nd
        kind = _prop_kind(prop or propagator)
        ebuf = rbuf = None
        if emit is not None:
            earr, ebuf = _fcplx(emit, (nd - 1, 2, nx, ny))
        if reflect is not None:
            rarr, rbuf = _fcplx(reflect, (nx, ny))
        if returnsum or immediatesum:
            out = np.empty((nf, ny, nx), dtype=np.complex128)
        else:
            out = np.empty((nf, nmax + 1, ny, nx), dtype=np.complex128)
        beta2 = np.empty(nf, dtype=np.float64)
        scale = self.beta2_scale() if beta2_scale is None else beta2_scale
        self.h.check(_lib.lib().bf_stack_dancer(
            self.h.ptr, self._s, nf, _lib.ptr(freqs), float(amin), int(nmax), kind, _prec(precision),
            _lib.ptr(ebuf), _lib.ptr(rbuf), int(bool(returnsum)), int(bool(immediatesum)), float(scale), 0,
            _lib.ptr(out.view(np.float64)), _lib.ptr(beta2)))
        if out.ndim == 3:
            return out.transpose(0, 2, 1), beta2
        return out.transpose(0, 3, 2, 1), beta2

    def close(self):
        """bf_stack_destroy; refused (BFError) while a server still has
        requests on the stack, which then stays open."""
        if getattr(self, "_s", None) and self.h._h:
            self.h.check(_lib.lib().bf_stack_destroy(self.h.ptr, self._s))
        self._s = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _maybe_scalar(f, arr):
    return arr[0] if np.ndim(f) == 0 else arr


def cheerleader(amin, nmax, bdry, coords, f=10.0e9, prop=propagator, emit=None, reflect=None,
                diskR=0.1, returnboth=False, precision="fp64", handle=None):
    """src/boost_fractor_recurprop.jl:226-363 on the GPU."""
    st = Stack(bdry, coords, diskR, handle=handle)
    try:
        right, left, _ = st.cheerleader(f, amin=amin, nmax=nmax, prop=prop, emit=emit, reflect=reflect,
                                        returnboth=returnboth, precision=precision)
    finally:
        st.close()
    if returnboth:
        return _maybe_scalar(f, left), _maybe_scalar(f, right)
    return _maybe_scalar(f, right)


def dancer(amin, nmax, sbdry, coords, f=10.0e9, prop=propagator, emit=None, reflect=None, diskR=0.1,
           returnsum=True, immediatesum=True, precision="fp64", handle=None):
    """src/boost_fractor_recurprop.jl:25-146 on the GPU."""
    st = Stack(sbdry, coords, diskR, handle=handle)
    try:
        out, _ = st.dancer(f, amin=amin, nmax=nmax, prop=prop, emit=emit, reflect=reflect,
                           returnsum=returnsum, immediatesum=immediatesum, precision=precision)
    finally:
        st.close()
    return _maybe_scalar(f, out)


def boost_factor(E, coords, diskR):
    """beta^2 = sum|E|^2 dx dy / (pi diskR^2) (test/runtests.jl:74)."""
    X, Y = coords.X, coords.Y
    dx = X[1] - X[0] if len(X) > 1 else 1.0
    dy = Y[1] - Y[0] if len(Y) > 1 else 1.0
    return float(np.sum(np.abs(E) ** 2) * dx * dy / (math.pi * diskR ** 2))


# --------------------------------------------------------------------------
# transformer (src/boost_fractor_transformer.jl)
# --------------------------------------------------------------------------
class Modes:
    """Resident mode basis (bf_modes_create); mirrors the reference's Modes
    (src/boost_fractor_transformer.jl:31-38): M, L, mode_patterns, mode_kt."""

    def __init__(self, coords, ThreeDim=False, Mmax=1, Lmax=0, diskR=0.15, pattern_input=None,
                 kT_arr=None, handle=None):
        self.h = handle or default_handle()
        self.coords = coords
        nx, ny = len(coords.X), len(coords.Y)
        self.nx, self.ny = nx, ny
        pbuf = kbuf = None
        if pattern_input is not None:
            parr, pbuf = _fcplx(pattern_input, (Mmax, 2 * Lmax + 1, nx, ny, 1))
            self._p = parr
        if kT_arr is not None:
            karr, kbuf = _fcplx(kT_arr, (Mmax, 2 * Lmax + 1))
            self._k = karr
        m = _lib._vp()
        self.h.check(_lib.lib().bf_modes_create(
            self.h.ptr, nx, ny, _lib.ptr(coords.X), _lib.ptr(coords.Y), int(bool(ThreeDim)), int(Mmax),
            int(Lmax), float(diskR), _lib.ptr(pbuf), _lib.ptr(kbuf), _lib.ctypes.byref(m)))
        self._m = m
        self.M, self.L = (int(Mmax), int(Lmax)) if ThreeDim else (1, 0)
        self.nm = self.M * (2 * self.L + 1)

    @property
    def mode_patterns(self):
        out = np.empty((1, ny := self.ny, self.nx, 2 * self.L + 1, self.M), dtype=np.complex128)
        n = _lib.ctypes.c_int()
        self.h.check(_lib.lib().bf_modes_get(self.h.ptr, self._m, _lib.ctypes.byref(n),
                                             _lib.ptr(out.view(np.float64)), None))
        return out.transpose(4, 3, 2, 1, 0)

    @property
    def mode_kt(self):
        out = np.empty((2 * self.L + 1, self.M), dtype=np.complex128)
        self.h.check(_lib.lib().bf_modes_get(self.h.ptr, self._m, None, None, _lib.ptr(out.view(np.float64))))
        return out.T

    def close(self):
        """bf_modes_destroy; refused (BFError) while a server still has
        requests on the basis, which then stays open."""
        if getattr(self, "_m", None) and self.h._h:
            self.h.check(_lib.lib().bf_modes_destroy(self.h.ptr, self._m))
        self._m = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def SeedModes(coords, ThreeDim=False, Mmax=1, Lmax=0, diskR=0.15, pattern_input=None, kT_arr=None,
              handle=None):
    """src/boost_fractor_transformer.jl:46-69."""
    return Modes(coords, ThreeDim=ThreeDim, Mmax=Mmax, Lmax=Lmax, diskR=diskR,
                 pattern_input=pattern_input, kT_arr=kT_arr, handle=handle)


def axion_induced_modes(coords, modes, B=None, velocity_x=0.0, diskR=0.15, f=20e9):
    """src/boost_fractor_transformer.jl:115-151."""
    bbuf = None
    if B is not None:
        B = np.asarray(B)
        if B.ndim == 3:
            B = B[:, :, 0]
        barr, bbuf = _fcplx(B, (modes.nx, modes.ny))
    out = np.empty(modes.nm, dtype=np.complex128)
    modes.h.check(_lib.lib().bf_axion_induced_modes(modes.h.ptr, modes._m, _lib.ptr(bbuf), float(velocity_x),
                                                    float(diskR), float(f), _lib.ptr(out.view(np.float64))))
    return out


def field2modes(pattern, coords, modes, diskR=0.15):
    """src/boost_fractor_transformer.jl:156."""
    return axion_induced_modes(coords, modes, B=pattern, diskR=diskR)


def modes2field(mode_coeffs, coords, modes):
    """src/boost_fractor_transformer.jl:161-167; returns (nx, ny, 1)."""
    c = np.ascontiguousarray(mode_coeffs, dtype=np.complex128)
    out = np.empty((modes.ny, modes.nx), dtype=np.complex128)
    modes.h.check(_lib.lib().bf_modes2field(modes.h.ptr, modes._m, _lib.ptr(c.view(np.float64)),
                                            _lib.ptr(out.view(np.float64))))
    return out.T[:, :, None]


def autotune(enable=True):
    """Switch the autotuner on or off (bf_autotune); returns the previous setting."""
    return bool(_lib.lib().bf_autotune(1 if enable else 0))


def autotune_report():
    """The autotuner's decisions so far, one string per tuned shape."""
    L = _lib.lib()
    n = L.bf_autotune_report(None, 0)
    buf = ctypes.create_string_buffer(n + 1)
    L.bf_autotune_report(buf, n + 1)
    return [l for l in buf.value.decode().split("\n") if l]


def transformer_group(stacks, modes, freqs, prop=propagator, precision="mixed", want_boost=False):
    """transformer (default emission) for several resident stacks at once that
    differ only in their untilted air-gap distances (bf_transformer_group):
    one solve for all (stack, frequency) pairs.  Returns beta2 [nreq, nf]
    (and boost [nreq, nf, nm] with want_boost)."""
    freqs = np.ascontiguousarray(np.atleast_1d(freqs), dtype=np.float64)
    nreq, nf, nm = len(stacks), len(freqs), modes.nm
    arr = (_lib._vp * nreq)(*[st._s for st in stacks])
    beta2 = np.empty((nreq, nf))
    boost = np.empty((nreq, nf, nm), dtype=np.complex128) if want_boost else None
    h = stacks[0].h
    h.check(_lib.lib().bf_transformer_group(h.ptr, nreq, arr, modes._m, nf, _lib.ptr(freqs), _prop_kind(prop),
                                            _prec(precision),
                                            _lib.ptr(None if boost is None else boost.view(np.float64)),
                                            _lib.ptr(beta2)))
    return (beta2, boost) if want_boost else beta2


def calc_propagation_matrices(bdry, coords, modes, f=10.0e9, prop=propagator, diskR=0.15, precision="fp64"):
    """src/boost_fractor_transformer.jl:274-280: list of (nm, nm) matrices per region
    (array [nf, nd, nm, nm] when f is an array)."""
    freqs = np.ascontiguousarray(np.atleast_1d(f), dtype=np.float64)
    st = Stack(bdry, coords, diskR, handle=modes.h)
    try:
        nd, nm, nf = st.nd, modes.nm, len(freqs)
        out = np.empty((nf, nd, nm, nm), dtype=np.complex128)
        st.h.check(_lib.lib().bf_calc_propagation_matrices(
            st.h.ptr, st._s, modes._m, nf, _lib.ptr(freqs), _prop_kind(prop), _prec(precision),
            _lib.ptr(out.view(np.float64))))
    finally:
        st.close()
    out = out.transpose(0, 1, 3, 2)   # Julia column-major matrices -> [row, col]
    if np.ndim(f) == 0:
        return [out[0, j] for j in range(out.shape[1])]
    return out


def transformer(bdry, coords, modes, f=10.0e9, velocity_x=0.0, prop=propagator, propagation_matrices=None,
                diskR=0.15, emit=None, reflect=None, precision="fp64"):
    """src/boost_fractor_transformer.jl:285-359 on the GPU.  Like the reference,
    NaN permittivities of ``bdry`` are replaced by 1e30 in place (:289)."""
    freqs = np.ascontiguousarray(np.atleast_1d(f), dtype=np.float64)
    nf = len(freqs)
    if emit is None and velocity_x != 0:
        emit = axion_induced_modes(coords, modes, B=None, velocity_x=velocity_x, diskR=diskR, f=freqs[0])
    bdry.eps[np.isnan(bdry.eps)] = 1e30
    st = Stack(bdry, coords, diskR, handle=modes.h)
    try:
        nm, nd = modes.nm, st.nd
        ebuf = rbuf = pbuf = None
        if emit is not None:
            e = np.ascontiguousarray(emit, dtype=np.complex128).reshape(nm)
            ebuf = e.view(np.float64)
        if reflect is not None:
            r = np.ascontiguousarray(reflect, dtype=np.complex128).reshape(nm)
            rbuf = r.view(np.float64)
        per_freq = 0
        if propagation_matrices is not None and len(propagation_matrices):
            pmat = np.asarray(propagation_matrices, dtype=np.complex128)
            if pmat.ndim == 3:
                pmat = pmat[None]
            per_freq = int(pmat.shape[0] == nf and nf > 1)
            pm = np.ascontiguousarray(pmat.transpose(0, 1, 3, 2))   # [.., row, col] -> Julia column-major
            pbuf = pm.view(np.float64)
        boost = np.empty((nf, nm), dtype=np.complex128)
        refl = np.empty((nf, nm), dtype=np.complex128) if reflect is not None else None
        beta2 = np.empty(nf, dtype=np.float64)
        st.h.check(_lib.lib().bf_transformer(
            st.h.ptr, st._s, modes._m, nf, _lib.ptr(freqs), _prop_kind(prop), _prec(precision), _lib.ptr(ebuf),
            _lib.ptr(rbuf), _lib.ptr(pbuf), per_freq, _lib.ptr(boost.view(np.float64)),
            _lib.ptr(None if refl is None else refl.view(np.float64)), _lib.ptr(beta2)))
    finally:
        st.close()
    if np.ndim(f) == 0:
        boost = boost[0]
        refl = None if refl is None else refl[0]
    if reflect is None:
        return boost
    return boost, refl


def transformer_trace_back(reflected_beam, input_beam, bdry, coords, modes, inlcudes_axion=False, f=10.0e9,
                           velocity_x=0, prop=propagator, propagation_matrices=None, diskR=0.15, emit=None,
                           precision="fp64"):
    """src/boost_fractor_transformer.jl:372-421 on the GPU: the (nd, 2, nm)
    array of per-region mode amplitudes (a leading frequency axis when f is an
    array).  vcat(input_beam, reflected_beam) must have 2 nm elements, as in
    the reference; each region's vector fills its (2, nm) slice in
    column-major order, as the reference's slice assignment does.  The
    keyword `inlcudes_axion` keeps the reference's spelling."""
    freqs = np.ascontiguousarray(np.atleast_1d(f), dtype=np.float64)
    nf, nm = len(freqs), modes.nm
    inp = np.atleast_1d(np.asarray(input_beam, dtype=np.complex128))
    ref = np.atleast_1d(np.asarray(reflected_beam, dtype=np.complex128))
    if inp.size + ref.size != 2 * nm or inp.size != nm:
        raise ValueError(f"vcat(input_beam, reflected_beam) needs {nm} + {nm} elements")
    inp = np.ascontiguousarray(inp.reshape(nm))
    ref = np.ascontiguousarray(ref.reshape(nm))
    st = Stack(bdry, coords, diskR, handle=modes.h)
    try:
        nd = st.nd
        ebuf = pbuf = None
        if emit is not None:
            ebuf = np.ascontiguousarray(emit, dtype=np.complex128).reshape(nm).view(np.float64)
        per_freq = 0
        if propagation_matrices is not None and len(propagation_matrices):
            pmat = np.asarray(propagation_matrices, dtype=np.complex128)
            if pmat.ndim == 3:
                pmat = pmat[None]
            per_freq = int(pmat.shape[0] == nf and nf > 1)
            pbuf = np.ascontiguousarray(pmat.transpose(0, 1, 3, 2)).view(np.float64)
        out = np.empty((nf, nm, 2, nd), dtype=np.complex128)   # column-major (nd, 2, nm) per frequency
        st.h.check(_lib.lib().bf_transformer_trace_back(
            st.h.ptr, st._s, modes._m, nf, _lib.ptr(freqs), _prop_kind(prop), _prec(precision),
            _lib.ptr(ref.view(np.float64)), _lib.ptr(inp.view(np.float64)), 0, int(bool(inlcudes_axion)),
            _lib.ptr(ebuf), _lib.ptr(pbuf), per_freq, _lib.ptr(out.view(np.float64))))
    finally:
        st.close()
    out = out.transpose(0, 3, 2, 1)
    return out[0] if np.ndim(f) == 0 else out


def gauss_profile(coords, z=0.000000001, omega0=0.1, f=10e9):
    """src/beam_gaussian.jl:24-37: normalised 2D Gaussian beam (nx, ny) at distance
    z from its waist (FP64, host)."""
    X = np.ascontiguousarray(coords.X, dtype=np.float64)
    Y = np.ascontiguousarray(coords.Y, dtype=np.float64)
    out = np.empty((len(Y), len(X)), dtype=np.complex128)
    rc = _lib.lib().bf_gauss_profile(len(X), len(Y), _lib.ptr(X), _lib.ptr(Y), float(z), float(omega0), float(f),
                                     _lib.ptr(out.view(np.float64)))
    if rc != _lib.BF_OK:
        raise BFError(rc, "gauss_profile: bad arguments")
    return out.T.copy()


def unnormalized_match(Eout, Eantenna, dx=0.01, dy=0.01, handle=None):
    """src/beam_coupling.jl:13-15 on the GPU: sum(Eout .* conj(Eantenna)) dx dy.
    Eout may carry a leading batch axis (nb, nx, ny); one value per field."""
    h = handle or default_handle()
    A = np.asfortranarray(np.asarray(Eantenna, dtype=np.complex128))
    E = np.asarray(Eout, dtype=np.complex128)
    batched = E.ndim == A.ndim + 1
    Eb = E if batched else E[None]
    nb, npix = Eb.shape[0], A.size
    ebuf = np.ascontiguousarray(np.stack([np.asfortranarray(e).T for e in Eb])).view(np.float64).reshape(-1)
    abuf = np.ascontiguousarray(A.T).view(np.float64).reshape(-1)
    out = np.empty(nb, dtype=np.complex128)
    h.check(_lib.lib().bf_unnormalized_match(h.ptr, nb, npix, _lib.ptr(ebuf), _lib.ptr(abuf), float(dx), float(dy),
                                             0, _lib.ptr(out.view(np.float64))))
    return out if batched else out[0]


def transformer_coupled(bdry, coords, modes, antenna, f=10.0e9, prop=propagator, propagation_matrices=None,
                        diskR=0.15, emit=None, precision="fp64"):
    """The transformer with the antenna coupling fused into its output: per
    frequency |sum_m conj(boost_m) antenna_m|^2, antenna = the antenna's mode
    coefficients (the coupled power of examples/transformer_optim_utilities.jl:137).
    Returns (coupled, beta2), arrays over f (scalars for a scalar f)."""
    freqs = np.ascontiguousarray(np.atleast_1d(f), dtype=np.float64)
    nf, nm = len(freqs), modes.nm
    bdry.eps[np.isnan(bdry.eps)] = 1e30
    ant = np.ascontiguousarray(antenna, dtype=np.complex128).reshape(nm)
    st = Stack(bdry, coords, diskR, handle=modes.h)
    try:
        ebuf = pbuf = None
        if emit is not None:
            ebuf = np.ascontiguousarray(emit, dtype=np.complex128).reshape(nm).view(np.float64)
        per_freq = 0
        if propagation_matrices is not None and len(propagation_matrices):
            pmat = np.asarray(propagation_matrices, dtype=np.complex128)
            if pmat.ndim == 3:
                pmat = pmat[None]
            per_freq = int(pmat.shape[0] == nf and nf > 1)
            pbuf = np.ascontiguousarray(pmat.transpose(0, 1, 3, 2)).view(np.float64)
        cpl = np.empty(nf)
        b2 = np.empty(nf)
        st.h.check(_lib.lib().bf_transformer_coupled(
            st.h.ptr, st._s, modes._m, nf, _lib.ptr(freqs), _prop_kind(prop), _prec(precision), _lib.ptr(ebuf),
            _lib.ptr(ant.view(np.float64)), _lib.ptr(pbuf), per_freq, _lib.ptr(cpl), _lib.ptr(b2)))
    finally:
        st.close()
    if np.ndim(f) == 0:
        return float(cpl[0]), float(b2[0])
    return cpl, b2


def transformer_1d_batch(distances, eps, freqs, emit=None, handle=None):
    """The 1D transformer (propagator1D, one 1D mode) for many spacing
    configurations at once: distances (nconf, nd), eps (nd,) shared, freqs (nf,).
    Returns (boost, beta2), both (nconf, nf)."""
    h = handle or default_handle()
    d = np.ascontiguousarray(np.atleast_2d(distances), dtype=np.float64)
    nconf, nd = d.shape
    e = np.ascontiguousarray(eps, dtype=np.complex128).reshape(nd)
    fr = np.ascontiguousarray(np.atleast_1d(freqs), dtype=np.float64)
    em = None if emit is None else np.array([complex(emit)], dtype=np.complex128)
    boost = np.empty((nconf, len(fr)), dtype=np.complex128)
    beta2 = np.empty((nconf, len(fr)))
    h.check(_lib.lib().bf_transformer_1d_batch(
        h.ptr, nconf, nd, _lib.ptr(d), _lib.ptr(e.view(np.float64)), len(fr), _lib.ptr(fr),
        _lib.ptr(None if em is None else em.view(np.float64)), _lib.ptr(boost.view(np.float64)), _lib.ptr(beta2)))
    return boost, beta2


def _shift_gaps(bdry, spacing=0.0, tilt_x=0.0, tilt_y=0.0):
    """A copy of bdry whose air gaps (the reference's regions 2, 4, ..., n_region)
    are `spacing` longer and tilted by (tilt_x, tilt_y) more
    (examples/transformer_optim_utilities.jl:22-24, 40-43)."""
    b = SetupBoundaries(bdry.distance, bdry.r, bdry.eps, bdry.relative_tilt_x, bdry.relative_tilt_y,
                        bdry.relative_surfaces)
    b.distance[1::2] += spacing
    b.relative_tilt_x[1::2] += tilt_x
    b.relative_tilt_y[1::2] += tilt_y
    return b


class PGrid:
    """Propagation matrices on a grid of gap spacings, resident on the device,
    with spline interpolation (examples/transformer_optim_utilities.jl:11-91).
    spacing_grid is an evenly spaced sequence (the reference's range).  With
    tilt grids the interpolation runs at their first points, as the
    reference's interpolate_prop_matrix does (itp(r, f, shift, 1, 1, ...));
    array() gives the whole (region, frequency, spacing, tilt_x, tilt_y,
    mode, mode) array of calc_propagation_matrices_grid."""

    def __init__(self, bdry, coords, modes, frequencies, spacing_grid, prop=propagator, diskR=0.15,
                 precision="fp64", tilt_x_grid=0.0, tilt_y_grid=0.0):
        sg = np.asarray(spacing_grid, dtype=np.float64)
        if sg.ndim != 1 or len(sg) < 2 or not np.allclose(np.diff(sg), sg[1] - sg[0], rtol=1e-9, atol=0):
            raise ValueError("spacing_grid must be an evenly spaced sequence of at least 2 values")
        self.tilt_x_grid = np.atleast_1d(np.asarray(tilt_x_grid, dtype=np.float64))
        self.tilt_y_grid = np.atleast_1d(np.asarray(tilt_y_grid, dtype=np.float64))
        self.spacing_grid = sg
        self._source = (bdry, coords, prop, diskR, precision)
        self.h = modes.h
        self.modes = modes
        self.freqs = np.ascontiguousarray(np.atleast_1d(frequencies), dtype=np.float64)
        base = bdry
        if self.tilt_x_grid[0] != 0.0 or self.tilt_y_grid[0] != 0.0:
            base = _shift_gaps(bdry, 0.0, self.tilt_x_grid[0], self.tilt_y_grid[0])
        self.stack = Stack(base, coords, diskR, handle=self.h)
        self.nd, self.nm = self.stack.nd, modes.nm
        self.spacing_first, self.spacing_step = float(sg[0]), float(sg[1] - sg[0])
        self.spacing_last = self.spacing_first + (len(sg) - 1) * self.spacing_step
        g = _lib._vp()
        self.h.check(_lib.lib().bf_pgrid_create(self.h.ptr, self.stack._s, modes._m, len(self.freqs),
                                                _lib.ptr(self.freqs), len(sg), float(sg[0]), float(sg[1] - sg[0]),
                                                _prop_kind(prop), _prec(precision), ctypes.byref(g)))
        self._g = g

    def matrices(self, dist_shift):
        """interpolate_prop_matrix: [nf][nd] (nm, nm) matrices as an array."""
        sh = np.ascontiguousarray(dist_shift, dtype=np.float64)
        out = np.empty((len(self.freqs), self.nd, self.nm, self.nm), dtype=np.complex128)
        self.h.check(_lib.lib().bf_pgrid_matrices(self.h.ptr, self._g, _lib.ptr(sh), _lib.ptr(out.view(np.float64))))
        return out.transpose(0, 1, 3, 2).copy()

    def transformer(self, dist_shift, emit=None):
        """calc_boostfactor_modes on the interpolated matrices: (boost [nf, nm], beta2 [nf])."""
        sh = np.ascontiguousarray(dist_shift, dtype=np.float64)
        eb = None if emit is None else np.ascontiguousarray(emit, dtype=np.complex128).reshape(self.nm)
        boost = np.empty((len(self.freqs), self.nm), dtype=np.complex128)
        beta2 = np.empty(len(self.freqs))
        self.h.check(_lib.lib().bf_pgrid_transformer(self.h.ptr, self._g, _lib.ptr(sh),
                                                     _lib.ptr(None if eb is None else eb.view(np.float64)),
                                                     _lib.ptr(boost.view(np.float64)), _lib.ptr(beta2)))
        return boost, beta2

    def array(self):
        """calc_propagation_matrices_grid's array [region, frequency, spacing,
        tilt_x, tilt_y, mode, mode]: the matrices of every grid point, the air
        gaps at their shifted spacing and tilts (computed on the device, one
        geometry at a time)."""
        bdry, coords, prop, diskR, precision = self._source
        out = np.empty((self.nd, len(self.freqs), len(self.spacing_grid), len(self.tilt_x_grid),
                        len(self.tilt_y_grid), self.nm, self.nm), dtype=np.complex128)
        for si, sp in enumerate(self.spacing_grid):
            for a, tx in enumerate(self.tilt_x_grid):
                for b, ty in enumerate(self.tilt_y_grid):
                    m = calc_propagation_matrices(_shift_gaps(bdry, sp, tx, ty), coords, self.modes, f=self.freqs,
                                                  prop=prop, diskR=diskR, precision=precision)
                    out[:, :, si, a, b] = m.transpose(1, 0, 2, 3)
        return out

    @property
    def bounds(self):
        """The spacing axis' bounds, Interpolations.bounds(itp)[3] of the
        reference's OnCell interpolation: half a step beyond the end spacings."""
        return (self.spacing_first - 0.5 * self.spacing_step, self.spacing_last + 0.5 * self.spacing_step)

    def cost(self, dist_shift, m_reflect, p=-20.0):
        """calc_boostfactor_cost (utilities :130-144): (cost, coupled power per
        frequency, or None on the hard out-of-bounds penalty)."""
        sh = np.ascontiguousarray(dist_shift, dtype=np.float64)
        mr = np.ascontiguousarray(m_reflect, dtype=np.complex128).reshape(self.nm)
        c = np.zeros(1)
        cpl = np.full(len(self.freqs), np.nan)
        self.h.check(_lib.lib().bf_pgrid_cost(self.h.ptr, self._g, _lib.ptr(sh), _lib.ptr(mr.view(np.float64)),
                                              float(p), _lib.ptr(c), _lib.ptr(cpl)))
        return float(c[0]), (None if np.isnan(cpl).all() else cpl)

    def close(self):
        if getattr(self, "_g", None) and self.h._h:
            _lib.lib().bf_pgrid_destroy(self.h.ptr, self._g)
        self._g = None
        if getattr(self, "stack", None) is not None:
            self.stack.close()
            self.stack = None


_SOLVERS = {"cheerleader": _lib.BF_SOLVER_CHEERLEADER, "dancer": _lib.BF_SOLVER_DANCER,
            "transformer": _lib.BF_SOLVER_TRANSFORMER, "pgrid": _lib.BF_SOLVER_PGRID}


def calc_propagation_matrices_grid(sbdry, coords, modes, spacing_grid, frequencies, tilt_x_grid=0, tilt_y_grid=0,
                                   prop=propagator, diskR=0.15, precision="fp64"):
    """examples/transformer_optim_utilities.jl:10-50: the grid of propagation
    matrices over gap spacings (and gap tilts) x frequencies, kept on the
    device as a PGrid; PGrid.array() gives the reference's 7-D array."""
    return PGrid(sbdry, coords, modes, frequencies, spacing_grid, prop=prop, diskR=diskR, precision=precision,
                 tilt_x_grid=tilt_x_grid, tilt_y_grid=tilt_y_grid)


def construct_prop_matrix_interpolation(prop_matrix_grid, spacing_grid=None):
    """utilities :56-73.  The PGrid is prefiltered for its cubic B-spline when it
    is built, so it is its own interpolation object."""
    if not isinstance(prop_matrix_grid, PGrid):
        raise TypeError("expects the PGrid of calc_propagation_matrices_grid")
    return prop_matrix_grid


def interpolate_prop_matrix(itp, dist_shift):
    """utilities :78-91: [region, frequency, nm, nm] matrices at the shifts."""
    return itp.matrices(dist_shift).transpose(1, 0, 2, 3).copy()


def calc_boostfactor_modes(sbdry, coords, modes, frequencies, prop_matrices_set, prop=propagator, diskR=0.15,
                           precision="fp64"):
    """utilities :99-110: EoutModes0[1, mode, frequency] of the transformer on
    per-frequency matrices prop_matrices_set[region, frequency] (one batched
    solve)."""
    pm = np.asarray(prop_matrices_set, dtype=np.complex128)
    fr = np.atleast_1d(np.asarray(frequencies, dtype=np.float64))
    boost = transformer(sbdry, coords, modes, f=fr, prop=prop, diskR=diskR,
                        propagation_matrices=pm.transpose(1, 0, 2, 3), precision=precision)
    return np.asarray(boost).T[None, :, :]


def calc_boostfactor_cost(dist_shift, itp, frequencies, sbdry, coords, modes, m_reflect, prop=propagator, diskR=0.15):
    """utilities :130-144 on the device: -p_norm(coupled power, -20) x the soft
    box penalty, 1000.0 outside the interpolation bounds.  sbdry, coords, modes,
    prop and diskR are those the grid was built with."""
    fr = np.atleast_1d(np.asarray(frequencies, dtype=np.float64))
    if fr.shape != itp.freqs.shape or np.any(fr != itp.freqs):
        raise ValueError("frequencies must be the grid's")
    return itp.cost(dist_shift, m_reflect, p=-20.0)[0]


_live_servers = weakref.WeakSet()


@atexit.register
def _close_servers():
    """At interpreter exit, servers close (finishing their running solves)
    before the stacks and mode bases they serve are collected."""
    for srv in list(_live_servers):
        try:
            srv.close()
        except Exception:
            pass


class Server:
    """A request loop over resident stacks (bf_server_create / bf_submit /
    bf_wait).  Requests on different stacks run concurrently on ``n_workers``
    streams, admitted by device footprint against ``hbm_budget_bytes``
    (0 = the device's free memory).  ``dry_run`` schedules without device
    work (a request takes ``nmax`` microseconds and holds ``footprint_bytes``),
    for exercising the scheduler without a GPU.  ``reserve_hbm`` maps the
    budget into the device pool at creation (BF_SERVER_RESERVE_HBM)."""

    def __init__(self, device=0, hbm_budget_bytes=0, n_workers=4, dry_run=False, reserve_hbm=False):
        L = _lib.lib()
        p = _lib._vp()
        flags = (_lib.BF_SERVER_DRYRUN if dry_run else 0) | (_lib.BF_SERVER_RESERVE_HBM if reserve_hbm else 0)
        rc = L.bf_server_create(int(device), int(hbm_budget_bytes), int(n_workers), flags, ctypes.byref(p))
        if rc != _lib.BF_OK:
            raise BFError(rc, "bf_server_create failed")
        self._p = p
        self._live = {}   # id -> (request struct, freqs, outputs): kept alive until completion
        _live_servers.add(self)

    def _check(self, rc):
        if rc != _lib.BF_OK:
            msg = _lib.lib().bf_server_last_error(self._p)
            raise BFError(rc, msg.decode() if msg else "")

    def submit(self, stack, freqs, solver="cheerleader", modes=None, distance=None, nmax=400, prop=None,
               precision="mixed", beta2_scale=0.0, want_boost=False, footprint_bytes=0, pgrid=None, lane=0):
        """Queue one solve; returns its id.  ``stack`` is a Stack (or, dry-run, any
        non-zero integer token), ``distance`` the stack's new region distances.
        solver="pgrid": ``pgrid`` is a PGrid, ``stack`` may be None (the grid's),
        ``freqs`` the grid's frequencies and ``distance`` the per-disk shifts.
        lane=1 marks an interactive request (see set_latency_lane)."""
        if pgrid is not None:
            stack = pgrid.stack if stack is None else stack
            modes = None
        fr = np.ascontiguousarray(np.atleast_1d(freqs), dtype=np.float64)
        nm = pgrid.nm if pgrid is not None else (modes.nm if modes is not None else 0)
        b2 = np.empty(len(fr))
        boost = np.empty((len(fr), nm), dtype=np.complex128) if want_boost and nm else None
        dist = None if distance is None else np.ascontiguousarray(distance, dtype=np.float64)
        q = _lib.BFRequest()
        q.solver = _SOLVERS[solver] if isinstance(solver, str) else int(solver)
        q.stack = stack._s if isinstance(stack, Stack) else _lib._vp(int(stack))
        q.modes = modes._m if modes is not None else None
        q.nf = len(fr)
        q.freqs = _lib.ptr(fr)
        q.distance = _lib.ptr(dist)
        q.nmax = int(nmax)
        q.prop_kind = _prop_kind(prop if prop is not None else propagator)
        q.precision = _prec(precision)
        q.beta2_scale = float(beta2_scale)
        q.out_beta2 = _lib.ptr(b2)
        q.out_boost = _lib.ptr(None if boost is None else boost.view(np.float64))
        q.footprint_bytes = int(footprint_bytes)
        q.pgrid = pgrid._g if pgrid is not None else None
        q.lane = int(lane)
        rid = _lib._ull()
        self._check(_lib.lib().bf_submit(self._p, ctypes.byref(q), ctypes.byref(rid)))
        self._live[rid.value] = (q, fr, dist, b2, boost)
        return rid.value

    def _result(self, rid, st, t):
        _, _, _, b2, boost = self._live.pop(rid)
        if st.value != _lib.BF_OK:
            msg = _lib.lib().bf_server_last_error(self._p)
            raise BFError(st.value, msg.decode() if msg else "")
        return {"beta2": b2, "boost": boost, "t_submit": t[0], "t_start": t[1], "t_done": t[2]}

    def wait(self, rid, timeout_ms=-1):
        """Result dict of request ``rid`` (beta2, boost, times); TimeoutError if it
        is still pending after ``timeout_ms``."""
        st = _lib._c_int()
        t = np.zeros(3)
        rc = _lib.lib().bf_wait(self._p, rid, int(timeout_ms), ctypes.byref(st), _lib.ptr(t))
        if rc == _lib.BF_ERR_TIMEOUT:
            raise TimeoutError(f"request {rid} still pending")
        self._check(rc)
        return self._result(rid, st, t)

    def poll(self, rid):
        """None while pending, else the result dict."""
        st = _lib._c_int()
        t = np.zeros(3)
        self._check(_lib.lib().bf_poll(self._p, rid, ctypes.byref(st), _lib.ptr(t)))
        if st.value == _lib.BF_PENDING:
            return None
        return self._result(rid, st, t)

    def stats(self, solver=None):
        out = np.zeros(10)
        k = -1 if solver is None else (_SOLVERS[solver] if isinstance(solver, str) else int(solver))
        self._check(_lib.lib().bf_server_stats(self._p, k, _lib.ptr(out)))
        keys = ["completed", "failed", "freq_points", "p50_ms", "p99_ms", "mean_ms", "max_ms", "wall_s",
                "batched", "evictions"]
        return dict(zip(keys, out.tolist()))

    def set_latency_lane(self, n_lane):
        """Reserve the last n_lane workers, on high-priority streams, for
        requests submitted with lane=1 (before the first submit)."""
        self._check(_lib.lib().bf_server_set_latency_lane(self._p, int(n_lane)))

    def reset_stats(self):
        """Start a new statistics window (after warm-up requests)."""
        self._check(_lib.lib().bf_server_reset_stats(self._p))

    def close(self):
        if getattr(self, "_p", None):
            _lib.lib().bf_server_destroy(self._p)
            self._p = None
            self._live.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
