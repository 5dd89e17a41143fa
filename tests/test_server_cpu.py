"""The serving engine's scheduler (bf_server_*), exercised without a GPU.

In dry-run mode a request "runs" for nmax microseconds and holds
footprint_bytes of device memory, so admission, ordering, batching, overlap
and timeouts are observable from the returned submit/start/done times.
Stacks are opaque tokens here.
"""
import time

import numpy as np
import pytest

MB = 1 << 20


@pytest.fixture
def B():
    import build as _b
    _b.build()
    import bfgb300
    return bfgb300


def times(r):
    return r["t_submit"], r["t_start"], r["t_done"]


def test_all_requests_complete_with_outputs(B):
    srv = B.Server(hbm_budget_bytes=1 << 40, n_workers=3, dry_run=True)
    try:
        ids = [srv.submit(0x1000 + 16 * (k % 5), np.linspace(1e10, 2e10, 7), nmax=2000, footprint_bytes=MB)
               for k in range(20)]
        res = [srv.wait(i, timeout_ms=20000) for i in ids]
        assert all(r["beta2"].shape == (7,) and np.all(r["beta2"] == 0.0) for r in res)
        st = srv.stats()
        assert st["completed"] == 20 and st["failed"] == 0 and st["freq_points"] == 140
        assert st["p99_ms"] >= st["p50_ms"] > 0.0
        with pytest.raises(B.BFError):   # a reported id is released
            srv.poll(ids[0])
    finally:
        srv.close()


def test_one_stack_runs_in_submission_order(B):
    srv = B.Server(hbm_budget_bytes=1 << 40, n_workers=4, dry_run=True)
    try:
        # distance changes keep the requests from joining one batch
        ids = [srv.submit(0x2000, [1e10], nmax=3000, distance=[0.0], footprint_bytes=MB) for _ in range(5)]
        res = [srv.wait(i, timeout_ms=20000) for i in ids]
        for a, b in zip(res, res[1:]):
            assert b["t_start"] >= a["t_done"]
        assert srv.stats()["batched"] == 0
    finally:
        srv.close()


def test_queued_requests_on_a_stack_join_one_batch(B):
    srv = B.Server(hbm_budget_bytes=1 << 40, n_workers=2, dry_run=True)
    try:
        first = srv.submit(0x3000, [1e10], nmax=50000, footprint_bytes=MB)
        time.sleep(0.01)   # the first one is running; the next three queue behind it
        rest = [srv.submit(0x3000, [1e10, 1.1e10], nmax=1000, footprint_bytes=MB) for _ in range(3)]
        r0 = srv.wait(first, timeout_ms=20000)
        rr = [srv.wait(i, timeout_ms=20000) for i in rest]
        assert all(r["t_start"] >= r0["t_done"] for r in rr)
        assert len({r["t_start"] for r in rr}) == 1          # one solve
        assert srv.stats()["batched"] == 2
    finally:
        srv.close()


def test_requests_on_different_stacks_overlap(B):
    srv = B.Server(hbm_budget_bytes=1 << 40, n_workers=4, dry_run=True)
    try:
        t0 = time.perf_counter()
        ids = [srv.submit(0x4000 + 16 * k, [1e10], nmax=100000, footprint_bytes=MB) for k in range(4)]
        res = [srv.wait(i, timeout_ms=20000) for i in ids]
        wall = time.perf_counter() - t0
        assert wall < 0.35            # 4 x 0.1 s of work on 4 workers
        starts = sorted(r["t_start"] for r in res)
        assert starts[-1] < min(r["t_done"] for r in res)   # all four were running together
    finally:
        srv.close()


def test_admission_by_footprint_and_eviction(B):
    # 100 MB budget, 60 MB requests on three stacks: at most one runs or stays resident at a time
    srv = B.Server(hbm_budget_bytes=100 * MB, n_workers=3, dry_run=True)
    try:
        ids = [srv.submit(0x5000 + 16 * k, [1e10], nmax=20000, footprint_bytes=60 * MB) for k in range(3)]
        res = sorted((srv.wait(i, timeout_ms=20000) for i in ids), key=lambda r: r["t_start"])
        for a, b in zip(res, res[1:]):
            assert b["t_start"] >= a["t_done"]
        assert srv.stats()["evictions"] >= 2
    finally:
        srv.close()


def test_request_beyond_budget_is_refused(B):
    srv = B.Server(hbm_budget_bytes=100 * MB, n_workers=1, dry_run=True)
    try:
        with pytest.raises(B.BFError) as e:
            srv.submit(0x6000, [1e10], nmax=10, footprint_bytes=200 * MB)
        assert e.value.code == 2   # BF_ERR_NOMEM
        with pytest.raises(B.BFError):
            srv.submit(0x6000, [-1.0], nmax=10, footprint_bytes=MB)   # invalid frequency
    finally:
        srv.close()


def test_wait_times_out_then_completes(B):
    srv = B.Server(hbm_budget_bytes=1 << 40, n_workers=1, dry_run=True)
    try:
        rid = srv.submit(0x7000, [1e10], nmax=300000, footprint_bytes=MB)
        with pytest.raises(TimeoutError):
            srv.wait(rid, timeout_ms=20)
        assert srv.poll(rid) is None or True   # may still be pending; the id stays valid
        r = srv.wait(rid, timeout_ms=20000)
        assert r["t_done"] - r["t_start"] >= 0.29
    finally:
        srv.close()


def test_close_cancels_queued_requests(B):
    srv = B.Server(hbm_budget_bytes=1 << 40, n_workers=1, dry_run=True)
    srv.submit(0x8000, [1e10], nmax=100000, footprint_bytes=MB)
    for _ in range(5):
        srv.submit(0x8000, [1e10], nmax=100000, distance=[0.0], footprint_bytes=MB)
    t0 = time.perf_counter()
    srv.close()
    assert time.perf_counter() - t0 < 0.5   # only the running one is waited for


def test_transformer_steps_of_different_stacks_form_one_group(B):
    """Queued transformer requests on different stacks with the same mode
    basis and frequencies join one group solve (one start time); a second
    request on a stack already in the group waits for it."""
    import ctypes
    import types
    modes = types.SimpleNamespace(_m=ctypes.c_void_p(0x9990), nm=1)
    srv = B.Server(hbm_budget_bytes=1 << 40, n_workers=1, dry_run=True)
    try:
        busy = srv.submit(0xA000, [1e10], nmax=50000, footprint_bytes=MB)
        time.sleep(0.01)   # the worker is busy; the group queues behind it
        f = [1e10, 1.1e10]
        grp = [srv.submit(0xB000 + 16 * k, f, "transformer", modes=modes, nmax=1000, distance=[0.0],
                          footprint_bytes=MB) for k in range(5)]
        again = srv.submit(0xB000, f, "transformer", modes=modes, nmax=1000, distance=[0.0], footprint_bytes=MB)
        r0 = srv.wait(busy, timeout_ms=20000)
        rg = [srv.wait(i, timeout_ms=20000) for i in grp]
        ra = srv.wait(again, timeout_ms=20000)
        assert len({r["t_start"] for r in rg}) == 1 and rg[0]["t_start"] >= r0["t_done"]
        assert ra["t_start"] >= rg[0]["t_done"]
        assert srv.stats("transformer")["batched"] == 4
    finally:
        srv.close()


def test_transformer_stack_runs_on_any_free_worker(B):
    """A transformer stack keeps no workspace bound to one worker's stream, so
    its next step starts on whichever worker is free: after each step, a long
    bounce-loop request occupies one of the two workers, and the step that
    follows starts at once on the other (a stack pinned to the worker that ran
    it would wait, in about half of the trials, for the long request)."""
    import ctypes
    import types
    modes = types.SimpleNamespace(_m=ctypes.c_void_p(0x9990), nm=1)
    srv = B.Server(hbm_budget_bytes=1 << 40, n_workers=2, dry_run=True)
    try:
        f = [1e10]
        for trial in range(8):
            r = srv.wait(srv.submit(0xC000, f, "transformer", modes=modes, nmax=1000, distance=[0.0],
                                    footprint_bytes=MB), timeout_ms=20000)
            long_id = srv.submit(0xD000 + 16 * trial, f, nmax=150000, footprint_bytes=MB)
            time.sleep(0.01)   # one worker has taken the long request
            r = srv.wait(srv.submit(0xC000, f, "transformer", modes=modes, nmax=1000, distance=[0.0],
                                    footprint_bytes=MB), timeout_ms=20000)
            rl = srv.wait(long_id, timeout_ms=20000)
            assert r["t_done"] < rl["t_done"], trial
    finally:
        srv.close()


def test_reset_stats_starts_a_new_window(B):
    srv = B.Server(hbm_budget_bytes=1 << 40, n_workers=2, dry_run=True)
    try:
        for i in [srv.submit(0xE000 + 16 * k, [1e10, 2e10], nmax=1000, footprint_bytes=MB) for k in range(3)]:
            srv.wait(i, timeout_ms=20000)
        assert srv.stats()["completed"] == 3
        srv.reset_stats()
        s = srv.stats()
        assert s["completed"] == 0 and s["freq_points"] == 0 and s["p99_ms"] == 0 and s["wall_s"] == 0
        srv.wait(srv.submit(0xE000, [1e10], nmax=1000, footprint_bytes=MB), timeout_ms=20000)
        s = srv.stats()
        assert s["completed"] == 1 and s["freq_points"] == 1
    finally:
        srv.close()


def test_latency_lane_workers_take_only_lane_requests(B):
    """With one of two workers reserved for lane 1, a second long normal
    request waits for the first (the lane worker does not take it), while a
    lane-1 request starts at once on the reserved worker; a second lane-1
    request waits for the lane worker even while the normal worker is idle."""
    srv = B.Server(hbm_budget_bytes=1 << 40, n_workers=2, dry_run=True)
    try:
        srv.set_latency_lane(1)
        with pytest.raises(Exception):
            srv.set_latency_lane(1)   # once only
        first = srv.submit(0xF000, [1e10], nmax=100000, footprint_bytes=MB)
        time.sleep(0.01)
        second = srv.submit(0xF010, [1e10], nmax=100000, footprint_bytes=MB)
        fast = srv.submit(0xF020, [1e10], nmax=1000, footprint_bytes=MB, lane=1)
        rf, r1, r2 = (srv.wait(i, timeout_ms=20000) for i in (fast, first, second))
        assert r2["t_start"] >= r1["t_done"]
        assert rf["t_done"] < r1["t_done"]
        # the normal worker is idle now; two lane requests run one after the other
        l1 = srv.submit(0xF030, [1e10], nmax=50000, footprint_bytes=MB, lane=1)
        l2 = srv.submit(0xF040, [1e10], nmax=50000, footprint_bytes=MB, lane=1)
        a1, a2 = srv.wait(l1, timeout_ms=20000), srv.wait(l2, timeout_ms=20000)
        assert a2["t_start"] >= a1["t_done"]
    finally:
        srv.close()


def test_latency_lane_needs_a_normal_worker_and_a_valid_lane(B):
    srv = B.Server(hbm_budget_bytes=1 << 40, n_workers=2, dry_run=True)
    try:
        with pytest.raises(Exception):
            srv.set_latency_lane(2)
        with pytest.raises(Exception):
            srv.submit(0xF100, [1e10], nmax=10, footprint_bytes=MB, lane=2)
    finally:
        srv.close()


def test_latency_lane_keeps_an_eighth_of_the_budget(B):
    """With a latency lane, normal requests are admitted within 7/8 of the
    budget: one that needs more is refused at submit, and while a normal
    request holds 7/8, a lane request still starts at once."""
    srv = B.Server(hbm_budget_bytes=800 * MB, n_workers=3, dry_run=True)
    try:
        srv.set_latency_lane(1)
        with pytest.raises(Exception):
            srv.submit(0xF200, [1e10], nmax=10, footprint_bytes=750 * MB)   # > 700 MB
        big = srv.submit(0xF210, [1e10], nmax=100000, footprint_bytes=700 * MB)
        time.sleep(0.01)
        other = srv.submit(0xF220, [1e10], nmax=1000, footprint_bytes=50 * MB)   # waits for memory
        fast = srv.submit(0xF230, [1e10], nmax=1000, footprint_bytes=50 * MB, lane=1)
        rb, ro, rf = (srv.wait(i, timeout_ms=20000) for i in (big, other, fast))
        assert rf["t_done"] < rb["t_done"]
        assert ro["t_start"] >= rb["t_done"]
    finally:
        srv.close()


def test_stack_changes_lane(B):
    """A bounce-loop stack whose workspace lives on a normal worker runs a
    lane-1 request on the lane worker (and back): a home worker of the other
    lane class does not hold the request."""
    srv = B.Server(hbm_budget_bytes=1 << 40, n_workers=2, dry_run=True)
    try:
        srv.set_latency_lane(1)
        for lane in (0, 1, 0, 1):
            r = srv.wait(srv.submit(0xF300, [1e10], nmax=1000, footprint_bytes=MB, lane=lane), timeout_ms=5000)
            assert r["t_done"] >= r["t_start"]
    finally:
        srv.close()
