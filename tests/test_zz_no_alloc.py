"""bf_propagate_noalloc (static device scratch, no allocation) against the
oracle's propagators and against bf_propagate.

The file name sorts last so that the suite also runs these tests after every
other GPU test of the session (the static scratch then holds whatever earlier
calls left in it); they pass run alone as well.

Tolerance: 1e-12 relative, the per-op FP64 propagator bar of the other GPU
tests, against the oracle (src/boost_fractor.jl:137-227 restated in numpy)
and against bf_propagate (the same kernels in the same order).
"""
import numpy as np
import pytest

from oracle import bf_oracle as O

pytestmark = pytest.mark.gpu

TOL = 1e-12
KINDS = ["propagator", "propagatorNoTilts", "propagatorMomentumSpace", "propagator1D"]


@pytest.fixture(scope="module")
def env():
    import torch
    import build as _b
    _b.build()
    import bfgb300 as B
    from bfgb300 import _lib
    h = B.Handle(0)
    h.set_stream(torch.cuda.current_stream().cuda_stream)
    yield B, _lib, h, torch
    h.close()


def last_error(L, h):
    return L.lib().bf_last_error(h.ptr).decode()


def rel(a, b):
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


def to_device(torch, E):
    """(nx, ny) complex128 -> device float64 buffer in column-major (Julia) order."""
    flat = np.ascontiguousarray(np.asfortranarray(E).T).view(np.float64).reshape(-1)
    return torch.from_numpy(flat.copy()).to("cuda")


def from_device(torch, t, nx, ny):
    torch.cuda.synchronize()
    return t.cpu().numpy().view(np.complex128).reshape(ny, nx).T.copy()


ORACLE = {"propagator": O.propagator, "propagatorNoTilts": O.propagator_notilts,
          "propagatorMomentumSpace": O.propagator_momentum_space, "propagator1D": O.propagator1d}


def geometry(B, nx, seed, ny=None):
    from bfgb300 import workloads as W
    ny = nx if ny is None else ny
    X, Y = W.symmetric_grid(nx), W.symmetric_grid(ny)
    c = B.SeedCoordinateSystem(X=X, Y=Y)
    rng = np.random.default_rng(seed)
    E = rng.standard_normal((nx, ny)) + 1j * rng.standard_normal((nx, ny))
    surf = 1e-5 * rng.standard_normal((nx, ny))
    return c, E, surf


def call_noalloc(B, L, h, kind, t, nx, c, dz, eps, tx, ty, surf, lam, ny=None):
    ny = nx if ny is None else ny
    sbuf = None
    if surf is not None:
        s = np.asfortranarray(np.asarray(surf, dtype=np.complex128))
        sbuf = np.ascontiguousarray(s.T).view(np.float64).reshape(-1)
    sp = L.ptr(sbuf)
    return L.lib().bf_propagate_noalloc(
        h.ptr, getattr(B, kind).kind, t.data_ptr(), nx, ny, L.ptr(c.X), L.ptr(c.Y), L.ptr(c.kX), L.ptr(c.kY),
        float(dz), 0.15, eps.real, eps.imag, float(tx), float(ty), sp, float(lam))


@pytest.mark.parametrize("nx,ny", [(64, 64), (101, 101), (64, 101), (256, 256)])
@pytest.mark.parametrize("kind", KINDS)
def test_noalloc_matches_oracle_and_propagate(env, kind, nx, ny):
    """Square, non-square (an x/y swap in the mask or the scratch offsets would
    show) and the largest grid the scratch holds (256 x 256 fills it)."""
    B, L, h, torch = env
    c, E, surf = geometry(B, nx, 11 * nx + ny, ny)
    eps = complex(24.0 if kind != "propagatorMomentumSpace" else 1.0, -0.0)
    lam = O.wavelength(20e9)
    co = O.seed_coordinate_system(X=c.X, Y=c.Y)
    want = ORACLE[kind](E, 0.0081, 0.15, eps, 3e-4, -2e-4, surf, lam, co)
    ref = getattr(B, kind)(E, 0.0081, 0.15, eps, 3e-4, -2e-4, surf, lam, c, handle=h)
    t = to_device(torch, E)
    torch.cuda.synchronize()
    assert call_noalloc(B, L, h, kind, t, nx, c, 0.0081, eps, 3e-4, -2e-4, surf, lam, ny) == L.BF_OK
    got = from_device(torch, t, nx, ny)
    assert rel(got, want) < TOL
    assert rel(got, ref) < TOL


@pytest.mark.parametrize("kind", ["propagator", "propagatorMomentumSpace"])
def test_noalloc_two_calls_in_a_row(env, kind):
    """Two back-to-back calls on one stream: the second reuses the scratch the
    first filled (first with a surface map, then without, other dz and eps)."""
    B, L, h, torch = env
    n = 64
    c, E, surf = geometry(B, n, 5)
    co = O.seed_coordinate_system(X=c.X, Y=c.Y)
    lam = O.wavelength(19.5e9)
    e1 = complex(24.0, -0.0) if kind == "propagator" else complex(1.0, -0.0)
    e2 = complex(1.0, -0.0)
    want = ORACLE[kind](E, 0.0079, 0.15, e1, 2e-4, 1e-4, surf, lam, co)
    want = ORACLE[kind](want, 0.0122, 0.15, e2, 0.0, 0.0, np.zeros((n, n)), lam, co)
    ref = getattr(B, kind)(E, 0.0079, 0.15, e1, 2e-4, 1e-4, surf, lam, c, handle=h)
    ref = getattr(B, kind)(ref, 0.0122, 0.15, e2, 0.0, 0.0, None, lam, c, handle=h)
    t = to_device(torch, E)
    torch.cuda.synchronize()
    assert call_noalloc(B, L, h, kind, t, n, c, 0.0079, e1, 2e-4, 1e-4, surf, lam) == L.BF_OK
    assert call_noalloc(B, L, h, kind, t, n, c, 0.0122, e2, 0.0, 0.0, None, lam) == L.BF_OK
    got = from_device(torch, t, n, n)
    assert rel(got, want) < TOL
    assert rel(got, ref) < TOL


def test_noalloc_allocates_nothing(env):
    """100 calls leave the device's free memory and the handle's device bytes
    unchanged (after one call that has done the per-device set-up)."""
    B, L, h, torch = env
    n = 128
    c, E, surf = geometry(B, n, 9)
    lam = O.wavelength(20.3e9)
    t = to_device(torch, E)
    eps = complex(24.0, -0.0)
    assert call_noalloc(B, L, h, "propagator", t, n, c, 0.008, eps, 1e-4, 1e-4, surf, lam) == L.BF_OK
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    held0 = h.device_bytes()
    for k in range(100):
        kind = KINDS[k % len(KINDS)]
        e = eps if kind != "propagatorMomentumSpace" else complex(1.0, -0.0)
        assert call_noalloc(B, L, h, kind, t, n, c, 0.008, e, 1e-4, 1e-4, surf, lam) == L.BF_OK
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert h.device_bytes() == held0


def test_noalloc_rejects_grid_beyond_limit(env):
    B, L, h, torch = env
    n = L.BF_NOALLOC_MAX_N + 1
    c, E, _ = geometry(B, n, 1)
    t = to_device(torch, E)
    torch.cuda.synchronize()
    rc = call_noalloc(B, L, h, "propagator", t, n, c, 0.008, complex(1.0, -0.0), 0.0, 0.0, None, 0.015)
    assert rc == L.BF_ERR_INVALID
    assert str(L.BF_NOALLOC_MAX_N) in last_error(L, h)


def test_noalloc_rejects_host_pointer(env):
    B, L, h, torch = env
    n = 16
    c, E, _ = geometry(B, n, 2)
    host = torch.from_numpy(np.ascontiguousarray(np.asfortranarray(E).T).view(np.float64).reshape(-1).copy())
    rc = call_noalloc(B, L, h, "propagator", host, n, c, 0.008, complex(1.0, -0.0), 0.0, 0.0, None, 0.015)
    assert rc == L.BF_ERR_INVALID
    assert "device memory" in last_error(L, h)
