"""Serving engine on the GPU: every request's result is the same alone and in
a mix of concurrent requests of other sizes and solvers.

Tolerance: 1e-12 relative in beta^2.  A request runs the same kernels on the
same inputs whether it is alone or shares the device, and the kernels are
deterministic, so the results are expected to be identical.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12


@pytest.fixture(scope="module")
def B():
    import build as _b
    _b.build()
    import bfgb300
    return bfgb300


def stack(B, h, n, ndisk, seed, width=1.0):
    from bfgb300 import workloads as W
    rng = np.random.default_rng(seed)
    nd = 2 * ndisk + 2
    tx = np.zeros(nd)
    ty = np.zeros(nd)
    for k in range(ndisk):
        tx[2 + 2 * k] = rng.uniform(-5e-4, 5e-4)
        ty[2 + 2 * k] = rng.uniform(-5e-4, 5e-4)
    distance, eps, tx, ty = W.booster(ndisk, rng.uniform(7.5e-3, 8.5e-3, ndisk), tilt_x=tx, tilt_y=ty)
    X = W.symmetric_grid(n, width)
    c = B.SeedCoordinateSystem(X=X, Y=X)
    sb = B.SeedSetupBoundaries(c, diskno=ndisk, distance=distance, epsilon=eps, relative_tilt_x=tx,
                               relative_tilt_y=ty)
    sb.eps[np.isnan(sb.eps)] = 1e30
    return B.Stack(sb, c, 0.15, handle=h), c, distance


def transformer_alone(B, h, st, modes, freqs, precision):
    from bfgb300 import _lib
    fr = np.ascontiguousarray(freqs, dtype=np.float64)
    b2 = np.empty(len(fr))
    h.check(_lib.lib().bf_transformer(h.ptr, st._s, modes._m, len(fr), _lib.ptr(fr), _lib.BF_PROP_3D,
                                      B._prec(precision), None, None, None, 0, None, None, _lib.ptr(b2)))
    return b2


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b)) / np.abs(np.asarray(b))))


def test_results_alone_and_in_the_mix(B):
    h = B.Handle(0)
    s_cheer, _, _ = stack(B, h, 64, 3, 1)
    s_dance, _, _ = stack(B, h, 32, 2, 2)
    s_tf, c_tf, _ = stack(B, h, 48, 2, 3)
    modes = B.SeedModes(c_tf, ThreeDim=True, Mmax=4, Lmax=1, diskR=0.15, handle=h)
    fa = np.linspace(19.6e9, 20.4e9, 24)
    fb = np.linspace(19.8e9, 20.2e9, 5)
    fc = np.linspace(19.5e9, 20.5e9, 9)
    alone = {
        "cheer_a": s_cheer.cheerleader(fa, nmax=40, precision="mixed")[2],
        "cheer_b": s_cheer.cheerleader(fb, nmax=40, precision="mixed")[2],
        "dance": s_dance.dancer(fb, nmax=30, precision="fp64")[1],
        "tf_mixed": transformer_alone(B, h, s_tf, modes, fc, "mixed"),
        "tf_fp64": transformer_alone(B, h, s_tf, modes, fc, "fp64"),
    }
    srv = B.Server(n_workers=3)
    try:
        ids = []
        for rep in range(3):
            ids.append(("cheer_a", srv.submit(s_cheer, fa, "cheerleader", nmax=40, precision="mixed")))
            ids.append(("tf_mixed", srv.submit(s_tf, fc, "transformer", modes=modes, precision="mixed")))
            ids.append(("dance", srv.submit(s_dance, fb, "dancer", nmax=30, precision="fp64")))
            ids.append(("cheer_b", srv.submit(s_cheer, fb, "cheerleader", nmax=40, precision="mixed")))
            ids.append(("tf_fp64", srv.submit(s_tf, fc, "transformer", modes=modes, precision="fp64")))
        for key, rid in ids:
            r = srv.wait(rid, timeout_ms=120000)
            assert rel(r["beta2"], alone[key]) < TOL, key
        st = srv.stats()
        assert st["completed"] == len(ids) and st["failed"] == 0
    finally:
        srv.close()
        modes.close()
        for s in (s_cheer, s_dance, s_tf):
            s.close()
        h.close()


def test_latency_lane_results_equal_alone(B):
    """With a latency lane (one of three workers, high-priority stream) and
    the budget mapped into the pool at creation, transformer steps in the lane
    and bounce-loop solves on the normal workers (whose persistent GEMM is
    capped) give the same beta^2 as alone."""
    h = B.Handle(0)
    s_cheer, _, _ = stack(B, h, 64, 3, 11)
    s_tf, c_tf, _ = stack(B, h, 48, 2, 13)
    modes = B.SeedModes(c_tf, ThreeDim=True, Mmax=4, Lmax=1, diskR=0.15, handle=h)
    fa = np.linspace(19.6e9, 20.4e9, 24)
    fc = np.linspace(19.5e9, 20.5e9, 9)
    alone = {"cheer": s_cheer.cheerleader(fa, nmax=40, precision="mixed")[2],
             "tf_mixed": transformer_alone(B, h, s_tf, modes, fc, "mixed"),
             "tf_fp64": transformer_alone(B, h, s_tf, modes, fc, "fp64")}
    srv = B.Server(hbm_budget_bytes=8 << 30, n_workers=3, reserve_hbm=True)
    try:
        srv.set_latency_lane(1)
        ids = []
        for rep in range(3):
            ids.append(("cheer", srv.submit(s_cheer, fa, "cheerleader", nmax=40, precision="mixed")))
            ids.append(("tf_mixed", srv.submit(s_tf, fc, "transformer", modes=modes, precision="mixed", lane=1)))
            ids.append(("tf_fp64", srv.submit(s_tf, fc, "transformer", modes=modes, precision="fp64", lane=1)))
        for key, rid in ids:
            r = srv.wait(rid, timeout_ms=120000)
            assert rel(r["beta2"], alone[key]) < TOL, key
        assert srv.stats()["failed"] == 0
    finally:
        srv.close()
        modes.close()
        for s in (s_cheer, s_tf):
            s.close()
        h.close()


def test_optimiser_gap_steps_in_submission_order(B):
    """A client moves the disks every step (bf_request.distance): the queued
    steps run in order on the resident stack and match set_distance + solve."""
    h = B.Handle(0)
    s_ref, _, d0 = stack(B, h, 64, 3, 7)
    s_srv, _, _ = stack(B, h, 64, 3, 7)
    rng = np.random.default_rng(8)
    steps = []
    d = d0.copy()
    for _ in range(4):
        d = d.copy()
        d[1:-1:2] += rng.normal(0.0, 10e-6, len(d[1:-1:2]))
        steps.append(d)
    freqs = np.linspace(19.7e9, 20.3e9, 16)
    ref = []
    for d in steps:
        s_ref.set_distance(d)
        ref.append(s_ref.cheerleader(freqs, nmax=40, precision="mixed")[2])
    srv = B.Server(n_workers=2)
    try:
        ids = [srv.submit(s_srv, freqs, "cheerleader", distance=d, nmax=40, precision="mixed") for d in steps]
        res = [srv.wait(i, timeout_ms=120000) for i in ids]
        for r, b2 in zip(res, ref):
            assert rel(r["beta2"], b2) < TOL
        for a, b in zip(res, res[1:]):
            assert b["t_start"] >= a["t_done"]
    finally:
        srv.close()
        s_ref.close()
        s_srv.close()
        h.close()


def test_optimiser_steps_of_several_stacks_share_one_solve(B):
    """Transformer steps of six optimisers of one booster design (same mode
    basis, grid and disks, different gaps) queued together are solved as one
    group (bf_transformer_group); each result matches the stack solved alone
    at the same gaps: mixed beta^2 within 1e-4, FP64 within 1e-12."""
    from bfgb300 import workloads as W
    h = B.Handle(0)
    s_busy, _, _ = stack(B, h, 64, 3, 40)
    base, c, d0 = stack(B, h, 48, 3, 41)
    pats, kt = W.lg_modes(c.X, c.Y, 6, 0.03, 0.15)
    modes = B.SeedModes(c, ThreeDim=True, Mmax=6, Lmax=0, diskR=0.15, pattern_input=pats, kT_arr=kt, handle=h)
    rng = np.random.default_rng(42)
    stacks, dists = [], []
    for k in range(6):
        st, _, _ = stack(B, h, 48, 3, 41)
        d = d0.copy()
        d[1:-1:2] += rng.normal(0.0, 50e-6, len(d[1:-1:2]))
        stacks.append(st)
        dists.append(d)
    freqs = np.linspace(19.6e9, 20.4e9, 12)
    srv = B.Server(n_workers=1)
    try:
        for prec, tol in (("mixed", 1e-4), ("fp64", TOL)):
            busy = srv.submit(s_busy, np.linspace(19.6e9, 20.4e9, 64), "cheerleader", nmax=200, precision="mixed")
            ids = [srv.submit(st, freqs, "transformer", modes=modes, distance=d, precision=prec)
                   for st, d in zip(stacks, dists)]
            srv.wait(busy, timeout_ms=120000)
            res = [srv.wait(i, timeout_ms=120000) for i in ids]
            assert len({r["t_start"] for r in res}) == 1   # one solve
            for d, r in zip(dists, res):
                base.set_distance(d)
                alone = transformer_alone(B, h, base, modes, freqs, prec)
                assert rel(r["beta2"], alone) < tol
        assert srv.stats("transformer")["batched"] >= 10
    finally:
        srv.close()
        modes.close()
        for s in stacks + [base, s_busy]:
            s.close()
        h.close()


def test_server_keeps_its_stacks_alive(B):
    """A stack or mode basis with requests still queued or running on a
    server cannot be destroyed (BF_ERR_INVALID, the objects stay open); after
    the server is closed they can."""
    from bfgb300 import _lib, workloads as W
    h = B.Handle(0)
    st, c, _ = stack(B, h, 64, 3, 50)
    pats, kt = W.lg_modes(c.X, c.Y, 4, 0.03, 0.15)
    modes = B.SeedModes(c, ThreeDim=True, Mmax=4, Lmax=0, diskR=0.15, pattern_input=pats, kT_arr=kt, handle=h)
    srv = B.Server(n_workers=1)
    try:
        a = srv.submit(st, np.linspace(19.6e9, 20.4e9, 64), "cheerleader", nmax=200, precision="mixed")
        b = srv.submit(st, np.linspace(19.6e9, 20.4e9, 8), "transformer", modes=modes, distance=None,
                       precision="mixed")
        with pytest.raises(B.BFError) as e:
            st.close()
        assert e.value.code == _lib.BF_ERR_INVALID and st._s is not None
        with pytest.raises(B.BFError):
            modes.close()
        srv.wait(a, timeout_ms=120000)
        srv.wait(b, timeout_ms=120000)
    finally:
        srv.close()
    modes.close()
    st.close()
    h.close()
