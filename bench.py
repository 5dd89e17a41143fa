"""Benchmark: beta^2 frequency-points/s of the batched cheerleader solve.

Workload (one "step"): one 20-disk booster request -- cheerleader, 128x128
grid over 1 m, eps 24, 1 mm disks, gaps U(7.5, 8.5) mm, per-disk tilts
U(-0.5, 0.5) mrad, 256 frequencies 19.5-20.5 GHz solved as one batch, 401
bounce iterations (nmax = 400), complex64 fields with FP64 phase arguments and
FP64 exit accumulation.  Seeded synthetic geometry (no dataset exists).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  Under torchrun every rank solves its own
request (weak scaling, no collective on the data path).
"""
import argparse
import json
import math
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(REPO, "boostfractor.jl_gb300")
for _p in (REPO, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "beta2 freq-points/s (cheerleader, 20 disks, 128x128, 256 freqs, 401 bounces; <=1e-4 rel err vs FP64)"
UNIT = "freq-points/s"


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def slowest_rank_ms(ms_local):
    """Max over ranks of a rank's timed-region milliseconds (identity for one
    process).  The reduction runs on the device for NCCL, on the host for gloo."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(ms_local)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(ms_local)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(ms_total_max, steps, nf, world_size):
    """Whole-job freq-points/s of `world_size` replicas, each solving one
    nf-frequency request per step, timed by the slowest rank."""
    return nf * world_size / (ms_total_max / steps / 1000.0)


def workload(rank=0, **over):
    from bfgb300 import workloads as W
    w = W.config2_cheerleader(seed=2 + rank, **over)
    return w


# --------------------------------------------------------------------------
# CPU baseline: the FP64 oracle (numpy) on a bounded sample
# --------------------------------------------------------------------------
def _cpu_worker(args):
    w, f, nmax_s = args
    sys.path.insert(0, REPO)
    from oracle import bf_oracle as O  # the CPU baseline leg may run the oracle
    co = O.seed_coordinate_system(X=w["X"], Y=w["Y"])
    sb = O.seed_setup_boundaries(co, diskno=(len(w["distance"]) - 2) // 2, distance=w["distance"],
                                 epsilon=w["eps"], relative_tilt_x=w["relative_tilt_x"],
                                 relative_tilt_y=w["relative_tilt_y"])
    t = time.perf_counter()
    E = O.cheerleader(0, nmax_s, sb, co, f=f, diskR=w["diskR"])
    dt = time.perf_counter() - t
    return dt, float(np.sum(np.abs(E) ** 2))


def cpu_sample(pool, w, freqs, nmax_s):
    """One bounded sample of the request on the host cores: the oracle's
    cheerleader for each of `freqs` (one frequency per pool process) with
    nmax_s + 1 bounces.  Returns (wall seconds, per-process solve seconds)."""
    t0 = time.perf_counter()
    res = pool.map(_cpu_worker, [(w, float(f), nmax_s) for f in freqs])
    return time.perf_counter() - t0, [r[0] for r in res]


def sample_freqs(w, P, step=0):
    """P of the request's frequencies, evenly spread, shifted by `step` so
    that successive samples cover different frequencies."""
    nf = len(w["freqs"])
    idx = (np.linspace(0, nf - 1, P).astype(int) + step) % nf
    return w["freqs"][idx]


def cpu_baseline(w, workers=None):
    """The oracle on `workers` host cores (spawned processes, one frequency
    each) for the whole bounce count of the request: freq-points/s = workers
    / the slowest process's solve time (process start-up excluded)."""
    P = workers or os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    with ctx.Pool(P) as pool:
        pool.map(_cpu_worker, [(w, float(w["freqs"][0]), 0)] * P)   # start-up and imports
        wall, per = cpu_sample(pool, w, sample_freqs(w, P), w["nmax"])
    return dict(value=P / max(per), unit=UNIT, cores=P, kind="port",
                sample=f"FP64 numpy oracle cheerleader, {P} of the {len(w['freqs'])} frequencies at the full "
                       f"{w['nmax'] + 1} bounces ({P} spawned processes, one per core); sample wall {wall:.1f}s")


def _cpu_tf_worker(fi):
    """The oracle's transformer at the full transformer workload for frequency
    index fi (the workload is regenerated from its seed in the process)."""
    sys.path.insert(0, REPO)
    sys.path.insert(0, os.path.join(REPO, "boostfractor.jl_gb300"))
    from oracle import bf_oracle as O  # the CPU baseline leg may run the oracle
    from bfgb300 import workloads as W
    w = W.config3_transformer()
    t = time.perf_counter()
    c = O.seed_coordinate_system(X=w["X"], Y=w["Y"])
    m = O.seed_modes(c, ThreeDim=True, Mmax=w["M"], Lmax=w["L"], diskR=w["diskR"],
                     pattern_input=w["pattern_input"], kT_arr=w["kT_arr"])
    sb = O.seed_setup_boundaries(c, diskno=(len(w["distance"]) - 2) // 2, distance=w["distance"],
                                 epsilon=w["eps"].copy(), relative_tilt_x=w["relative_tilt_x"],
                                 relative_tilt_y=w["relative_tilt_y"], relative_surfaces=w["relative_surfaces"])
    b = O.transformer(sb, c, m, f=float(w["freqs"][fi]), diskR=w["diskR"])
    return time.perf_counter() - t, float(np.sum(np.abs(b) ** 2))


def cpu_baseline_transformer(nf, workers=None):
    """The oracle's transformer on `workers` host cores, one frequency each
    (spawned processes), at the full size; freq-points/s = workers / slowest."""
    P = workers or os.cpu_count() or 1
    idx = [int(i) for i in np.linspace(0, nf - 1, P).astype(int)]
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(P) as pool:
        res = pool.map(_cpu_tf_worker, idx)
    wall = time.perf_counter() - t0
    per_point = max(r[0] for r in res)
    return dict(value=P / per_point, unit=UNIT, cores=P, kind="port",
                sample=f"FP64 numpy oracle transformer, {P} of the {nf} frequencies at full size "
                       f"({P} spawned processes, one per core, mode set-up included); pool wall {wall:.1f}s")


# --------------------------------------------------------------------------
# clocks during the timed region
# --------------------------------------------------------------------------
class ClockSampler:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def simt_peaks():
    """FP32 / FP64 / TF32 rates measured on this machine's GB300 with hand-written
    FFMA/DFMA probes and a cuBLAS TF32 GEMM (profiles/simt_peaks.json), or None."""
    p = os.path.join(REPO, "profiles", "simt_peaks.json")
    if os.path.exists(p):
        try:
            return json.load(open(p))
        except Exception:
            return None
    return None


def measured_tf32_peak():
    """Dense TF32 tensor peak: the measured cuBLAS TF32 GEMM rate, else half the
    measured bf16 GEMM rate (burst)."""
    sp = simt_peaks()
    if sp and sp.get("tf32_cublas_tflops"):
        return float(sp["tf32_cublas_tflops"]), "measured (cuBLAS TF32 GEMM, profiles/simt_peaks.json)"
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["bf16_tflops"]) / 2.0, "half of measured bf16"
    return 1900.0 / 2.0, "half of fallback bf16"


def ncu_traffic():
    """DRAM bytes per propagation of the fused stage kernel from the committed ncu summary."""
    p = os.path.join(REPO, "profiles", "fused_stage_ncu.json")
    if os.path.exists(p):
        try:
            return float(json.load(open(p))["dram_bytes_per_propagation"])
        except Exception:
            return None
    return None


# --------------------------------------------------------------------------
# our implementation
# --------------------------------------------------------------------------
def run_ours(args):
    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    else:
        torch.cuda.set_device(0)
    dev = torch.cuda.current_device()
    import build as _b
    _b.build()
    import bfgb300 as B

    over = {}
    if args.nf:
        over["nf"] = args.nf
    if args.nmax is not None:
        over["nmax"] = args.nmax
    w = workload(rank, **over)
    nf, nmax = len(w["freqs"]), w["nmax"]
    if args.fused_variant is not None:
        from bfgb300 import _lib
        _lib.lib().bf_test_force_fused_variant(args.fused_variant)
    h = B.Handle(dev)
    stream = torch.cuda.current_stream()
    h.set_stream(stream.cuda_stream)
    c = B.SeedCoordinateSystem(X=w["X"], Y=w["Y"])
    sb = B.SeedSetupBoundaries(c, diskno=(len(w["distance"]) - 2) // 2, distance=w["distance"],
                               epsilon=w["eps"], relative_tilt_x=w["relative_tilt_x"],
                               relative_tilt_y=w["relative_tilt_y"])
    st = B.Stack(sb, c, w["diskR"], handle=h)
    npix = len(w["X"]) * len(w["Y"])
    out_right = torch.empty((nf, npix * 2), dtype=torch.float64, device="cuda")
    out_beta2 = torch.empty((nf,), dtype=torch.float64, device="cuda")

    def step():
        st.cheerleader_device(w["freqs"], out_right.data_ptr(), out_beta2.data_ptr(), nmax=nmax,
                              precision="mixed")

    for _ in range(max(args.warmup, 0)):
        step()
    torch.cuda.synchronize()

    # accuracy of the mixed path vs the FP64 GPU path on a subset of frequencies
    sub = np.unique(np.linspace(0, nf - 1, min(nf, 16)).astype(int))
    b_mixed = out_beta2.cpu().numpy()[sub]
    _, _, b_fp64 = st.cheerleader(w["freqs"][sub], nmax=nmax, precision="fp64")
    errs = np.abs(b_mixed - b_fp64) / np.abs(b_fp64)
    rel_err = float(np.max(errs))
    rel_err_med = float(np.median(errs))
    # the same batch's beta^2 against the oracle at the fixture's frequencies
    # (tests/golden/make_c2_fixture.py: the oracle's cheerleader at full size)
    vs_oracle = None
    fxp = os.path.join(REPO, "tests", "golden", "c2_cheerleader_oracle.npz")
    if os.path.exists(fxp) and nf == 256 and nmax == 400 and rank == 0:
        fx = np.load(fxp)
        if np.array_equal(w["freqs"][fx["freq_index"]], fx["freqs"]):
            bm = out_beta2.cpu().numpy()[fx["freq_index"]]
            e = np.abs(bm - fx["beta2"]) / np.abs(fx["beta2"])
            vs_oracle = {"max": float(np.max(e)), "freq_index": [int(i) for i in fx["freq_index"]],
                         "per_freq": [float(x) for x in e]}
    # the plain FP64 single-stack path (one frequency per solve)
    t0 = time.perf_counter()
    st.cheerleader(w["freqs"][:1], nmax=nmax, precision="fp64")
    torch.cuda.synchronize()
    fp64_single = 1.0 / (time.perf_counter() - t0)

    # ---- timed region
    h.set_profiling(True)
    clocks = ClockSampler(dev if ws == 1 else local)
    clocks.start()
    time.sleep(0.4)
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    stage_ms, launches, stage_launches, props = 0.0, 0, 0, 0
    e0.record(stream)
    for _ in range(args.steps):
        step()
        p = h.last_profile()
        stage_ms += p["stages_ms"]
        launches += int(p["launches"])
        stage_launches += int(p["stage_launches"])
        props += int(p["propagations"])
    e1.record(stream)
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    ms_total = e0.elapsed_time(e1)
    clk = clocks.stop()
    h.set_profiling(False)
    ms_total = slowest_rank_ms(ms_total)
    ms_step = ms_total / args.steps
    value = replica_value(ms_total, args.steps, nf, ws)

    # roofline of the fused stage kernel (bytes per propagation: read + write of
    # the complex64 field, 2*N^2*8)
    N = len(w["X"])
    alg_bytes_per_prop = 2 * N * N * 8
    achieved = alg_bytes_per_prop * props / (stage_ms / 1000.0) / 1e9
    peak, peak_kind = measured_peaks()
    tr = ncu_traffic()
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_source": peak_kind,
            "traffic": None if tr is None else tr * props / stage_launches,
            "kernel": "k_fused_stage", "launch_avg_ms": stage_ms / max(stage_launches, 1),
            "alg_bytes_per_launch": alg_bytes_per_prop * props / max(stage_launches, 1),
            "fft_gflops": props * (2 * N + 2 * 38) * 5 * N * math.log2(N) / (stage_ms / 1000.0) / 1e9}

    # ---- end to end through the one-shot C ABI call with host buffers
    import ctypes
    from bfgb300 import _lib
    L = _lib.lib()
    r = B.workloads.fresnel_r(w["eps"])
    host_in = dict(distance=np.ascontiguousarray(w["distance"]), r=np.ascontiguousarray(r),
                   eps=np.ascontiguousarray(w["eps"]), tx=np.ascontiguousarray(w["relative_tilt_x"]),
                   ty=np.ascontiguousarray(w["relative_tilt_y"]), X=c.X, Y=c.Y, kX=c.kX, kY=c.kY,
                   freqs=np.ascontiguousarray(w["freqs"]))
    pin = {k: torch.from_numpy(v.view(np.float64) if v.dtype == np.complex128 else v).pin_memory()
           for k, v in host_in.items()}
    out_host = torch.empty((nf, npix * 2), dtype=torch.float64).pin_memory()
    b2_host = torch.empty((nf,), dtype=torch.float64).pin_memory()
    P = lambda t: ctypes.cast(ctypes.c_void_p(t.data_ptr()), ctypes.POINTER(ctypes.c_double))
    scale = st.beta2_scale()

    def e2e_step():
        h.check(L.bf_cheerleader(h.ptr, len(w["distance"]), P(pin["distance"]), P(pin["r"]), P(pin["eps"]),
                                 P(pin["tx"]), P(pin["ty"]), None, len(c.X), len(c.Y), P(pin["X"]),
                                 P(pin["Y"]), P(pin["kX"]), P(pin["kY"]), w["diskR"], nf, P(pin["freqs"]),
                                 0.0, nmax, _lib.BF_PROP_3D, _lib.BF_PREC_MIXED, None, None, 0, scale,
                                 P(out_host), None, P(b2_host)))

    e2e_step()
    torch.cuda.synchronize()
    ke = max(1, min(args.steps, 3))
    t0 = time.perf_counter()
    for _ in range(ke):
        e2e_step()
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / ke
    h2d = int(sum(t.numel() * t.element_size() for t in pin.values()))
    d2h = int(out_host.numel() * 8 + b2_host.numel() * 8)
    b2_e2e = b2_host.numpy().copy()

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "c64 (fields, FFTs), f64 (phase kz*dz, exit accumulation)",
        "data": "synthetic (seeded geometry, no dataset)",
        "config": c2_config(w),
        "beta2_rel_err_vs_fp64": rel_err,
        "beta2_rel_err_vs_fp64_median": rel_err_med,
        "beta2_checked_freqs": int(len(sub)),
        "beta2_rel_err_vs_oracle": vs_oracle,
        "plain_fp64_single_freqpts_per_s": fp64_single,
        "gpu_launches": launches,
        "roofline": roof,
        "e2e": {"value": nf / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "path": "bf_cheerleader (one-shot C ABI, pinned host buffers; stack upload, tables, solve, D2H)"},
        "clocks": clk,
        # the fused-stage variant per stage shape (autotuner decisions, or the forced one)
        "fused_variant": (f"forced {args.fused_variant}" if args.fused_variant is not None
                          else [ln for ln in B.autotune_report() if ln.startswith("fused")]),
    }
    if ws == 1 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(w)
    assert np.all(np.isfinite(b2_e2e))
    if rank == 0:
        print(json.dumps(line), flush=True)
    st.close()
    h.close()
    if ws > 1:
        torch.distributed.destroy_process_group()


def run_transformer(args):
    """Transformer mode-matching arm: 20 disks with surface maps, 64
    Laguerre-Gauss modes on a 256x256 grid, 1024 frequencies per request (one
    request per step)."""
    import torch
    torch.cuda.set_device(0)
    import build as _b
    _b.build()
    import bfgb300 as B
    from bfgb300 import workloads as W
    over = {}
    if args.nf:
        over["nf"] = args.nf
    w = W.config3_transformer(**over)
    nf = len(w["freqs"])
    h = B.Handle(0)
    stream = torch.cuda.current_stream()
    h.set_stream(stream.cuda_stream)
    c = B.SeedCoordinateSystem(X=w["X"], Y=w["Y"])
    kw = dict(diskno=(len(w["distance"]) - 2) // 2, distance=w["distance"], epsilon=w["eps"],
              relative_tilt_x=w["relative_tilt_x"], relative_tilt_y=w["relative_tilt_y"],
              relative_surfaces=w["relative_surfaces"])
    t0 = time.perf_counter()
    modes = B.SeedModes(c, ThreeDim=True, Mmax=w["M"], Lmax=w["L"], diskR=w["diskR"],
                        pattern_input=w["pattern_input"], kT_arr=w["kT_arr"], handle=h)
    t_modes = time.perf_counter() - t0
    sb = B.SeedSetupBoundaries(c, **kw)
    sb.eps[np.isnan(sb.eps)] = 1e30
    st = B.Stack(sb, c, w["diskR"], handle=h)
    from bfgb300 import _lib
    L = _lib.lib()
    nm = modes.nm
    boost = np.empty((nf, nm), dtype=np.complex128)
    beta2 = np.empty(nf)

    def solve(freqs, prec, out_b, out_b2):
        fr = np.ascontiguousarray(freqs)
        h.check(L.bf_transformer(h.ptr, st._s, modes._m, len(fr), _lib.ptr(fr), _lib.BF_PROP_3D,
                                 B._prec(prec), None, None, None, 0, _lib.ptr(out_b.view(np.float64)), None,
                                 _lib.ptr(out_b2)))

    t0 = time.perf_counter()
    solve(w["freqs"], "mixed", boost, beta2)          # builds the resident k-space overlaps
    t_setup = time.perf_counter() - t0
    for _ in range(max(args.warmup - 1, 0)):
        solve(w["freqs"], "mixed", boost, beta2)
    sub = np.unique(np.linspace(0, nf - 1, min(nf, 16)).astype(int))
    b64 = np.empty((len(sub), nm), dtype=np.complex128)
    b2_64 = np.empty(len(sub))
    t0 = time.perf_counter()
    solve(w["freqs"][sub], "fp64", b64, b2_64)
    t_fp64 = time.perf_counter() - t0
    errs = np.abs(beta2[sub] - b2_64) / np.abs(b2_64)
    h.set_profiling(True)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    gemm_ms, gemm_fl, launches, kern_ms, kern_n = 0.0, 0.0, 0, 0.0, 0
    e0.record(stream)
    for _ in range(args.steps):
        solve(w["freqs"], "mixed", boost, beta2)
        p = h.last_profile()
        gemm_ms += p["stages_ms"]           # the propagation-matrix phase
        kern_ms += p["exits_ms"]            # slot 3: the class-GEMM kernels alone
        kern_n += int(p["stage_launches"])  # slot 4: class-GEMM launches
        gemm_fl += p["propagations"]        # slot 6: their executed flops
        launches += int(p["launches"])
    e1.record(stream)
    torch.cuda.synchronize()
    h.set_profiling(False)
    ms = e0.elapsed_time(e1) / args.steps
    # the same request with the overlap GEMMs on the FP32 SIMT pipes
    # (BF_PREC_MIXED_SIMT): its first call builds the FP32 real rows of W and V
    b2_simt = np.empty(nf)
    for _ in range(max(args.warmup, 1)):
        solve(w["freqs"], "mixed-simt", boost, b2_simt)
    errs_simt = np.abs(b2_simt[sub] - b2_64) / np.abs(b2_64)
    h.set_profiling(True)
    torch.cuda.synchronize()
    simt_ms, simt_fl = 0.0, 0.0
    e0.record(stream)
    for _ in range(args.steps):
        solve(w["freqs"], "mixed-simt", boost, b2_simt)
        p = h.last_profile()
        simt_ms += p["stages_ms"]
        simt_fl += p["propagations"]
    e1.record(stream)
    torch.cuda.synchronize()
    h.set_profiling(False)
    ms_simt = e0.elapsed_time(e1) / args.steps
    tf32_peak, tf32_src = measured_tf32_peak()
    # executed MMA work of the tensor-core class GEMMs (three MMAs, hi*hi,
    # hi*lo, lo*hi, per product of the real-row GEMMs, counted by the library)
    # over the GEMM kernels' own CUDA-event time
    tc_tensor = gemm_fl / (kern_ms / 1000.0) / 1e12
    N = len(w["X"])
    sp = simt_peaks()
    if sp and sp.get("fp32_ffma_tflops"):
        peak_fp32, fp32_src = float(sp["fp32_ffma_tflops"]), "measured (FFMA probe, profiles/simt_peaks.json)"
    else:
        peak_fp32, fp32_src = 152 * 128 * 2 * 2.07e9 / 1e12, "nominal (152 SMs x 128 lanes x 2 x 2.07 GHz)"
    line = {"metric": f"beta2 freq-points/s (transformer, 20 disks + surface maps, {nm} LG modes, {N}x{N}, {nf} freqs)",
            "value": nf / (ms / 1000.0), "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "split-TF32 overlap GEMMs on tcgen05 (FP32 register sums of 32-deep tensor-core blocks), "
                     "c64 propagation matrices and inverses, double-float chain, f64 phases and boundary solve",
            "data": "synthetic (seeded geometry and surface maps)",
            "config": {"workload": w["name"] + f"-{nf}f", "grid": N, "modes": nm, "freqs": nf},
            "beta2_rel_err_vs_fp64": float(np.max(errs)), "beta2_rel_err_vs_fp64_median": float(np.median(errs)),
            "plain_fp64_freqpts_per_s": len(sub) / t_fp64,
            "setup_s": {"modes_host": t_modes, "first_solve_with_overlaps": t_setup},
            "gpu_launches": launches,
            "cpu_baseline": (None if args.no_cpu or args.nf else cpu_baseline_transformer(nf)),
            # the work of the direct formulation (overlap GEMMs over all pixels
            # 8 nm^2 Npix per region and frequency, air-region mode FFTs, chain,
            # inverses: ~104 GFLOP per freq-point here) at the split-TF32 rate
            # (measured TF32 / 3); the Parseval/orbit folding executes far less
            "alg_roofline": {"gflop_per_freq_point": 104.0, "peak_tflops": tf32_peak / 3.0,
                             "freqpts_per_s": tf32_peak / 3.0 * 1e3 / 104.0,
                             "frac": (nf / (ms / 1000.0)) / (tf32_peak / 3.0 * 1e3 / 104.0),
                             "executed_mma_tflop_per_request": gemm_fl / args.steps / 1e12},
            "roofline": {"bound": "tensor", "achieved": tc_tensor, "peak": tf32_peak, "unit": "TFLOP/s",
                         "frac": tc_tensor / tf32_peak, "peak_source": tf32_src, "traffic": None,
                         "kernel": "k_tc_gemm_tf32x3 (executed MMA flops / the kernel's CUDA-event time)",
                         "launch_avg_ms": kern_ms / max(kern_n, 1), "launches_per_step": kern_n / args.steps,
                         "phase_ms": gemm_ms / args.steps,
                         "phase_tflops": gemm_fl / (gemm_ms / 1000.0) / 1e12},
            "simt_gemm": {
                "value": nf / (ms_simt / 1000.0), "unit": UNIT, "ms_per_step": ms_simt,
                "beta2_rel_err_vs_fp64": float(np.max(errs_simt)),
                "beta2_rel_err_vs_fp64_median": float(np.median(errs_simt)),
                "note": "BF_PREC_MIXED_SIMT: the same solve with the class GEMMs on the FP32 SIMT pipes",
                "roofline": {"bound": "fp32-simt", "achieved": simt_fl / (simt_ms / 1000.0) / 1e12,
                             "peak": peak_fp32, "peak_source": fp32_src, "unit": "TFLOP/s",
                             "frac": simt_fl / (simt_ms / 1000.0) / 1e12 / peak_fp32,
                             "kernel": "k_rcgemm_c64 (whole propagation-matrix phase)",
                             "phase_ms": simt_ms / args.steps}}}
    print(json.dumps(line), flush=True)
    st.close()
    modes.close()
    h.close()


# --------------------------------------------------------------------------
# uneven batch and serving (the request loop of bf_server)
# --------------------------------------------------------------------------
def _build_request_stack(B, W, h, req, mode_cache=None):
    """A request's resident stack and, for the transformer, its mode basis.
    With mode_cache (a dict), requests on the same grid with the same mode
    set share one basis, as optimisers of one booster design do; shared
    bases are closed by the caller through the cache."""
    c = B.SeedCoordinateSystem(X=req["X"], Y=req["X"])
    sb = B.SeedSetupBoundaries(c, diskno=req["ndisk"], distance=req["distance"], epsilon=req["eps"],
                               relative_tilt_x=req["relative_tilt_x"], relative_tilt_y=req["relative_tilt_y"])
    sb.eps[np.isnan(sb.eps)] = 1e30
    st = B.Stack(sb, c, req["diskR"], handle=h)
    modes = None
    if req["solver"] == "transformer":
        key = (len(req["X"]), req["M"], req["waist"], req["diskR"])
        modes = None if mode_cache is None else mode_cache.get(key)
        if modes is None:
            pats, kt = W.lg_modes(c.X, c.Y, req["M"], req["waist"], req["diskR"])
            modes = B.SeedModes(c, ThreeDim=True, Mmax=req["M"], Lmax=0, diskR=req["diskR"], pattern_input=pats,
                                kT_arr=kt, handle=h)
            if mode_cache is not None:
                mode_cache[key] = modes
    return st, modes


def _close_all(stacks, mode_cache=None):
    for st, m in stacks:
        if m is not None and mode_cache is None:
            m.close()
        st.close()
    for m in (mode_cache or {}).values():
        m.close()


def _solve_plain(B, h, st, modes, req, precision="mixed"):
    """One request through the direct C ABI on handle h: beta^2 per frequency."""
    from bfgb300 import _lib
    fr = np.ascontiguousarray(req["freqs"], dtype=np.float64)
    if req["solver"] == "transformer":
        b2 = np.empty(len(fr))
        h.check(_lib.lib().bf_transformer(h.ptr, st._s, modes._m, len(fr), _lib.ptr(fr), _lib.BF_PROP_3D,
                                          B._prec(precision), None, None, None, 0, None, None, _lib.ptr(b2)))
        return b2
    return st.dancer(fr, nmax=req["nmax"], precision=precision)[1]


def _server_line(metric, value, n_done, wall, extra):
    line = {"metric": metric, "value": value, "unit": UNIT, "n_gpus": 1, "steps": int(n_done), "warmup": 0,
            "ms_per_step": 1000.0 * wall / max(n_done, 1), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c64 fields / overlap GEMM operands, f64 phases and solves",
            "data": "synthetic (seeded stacks, no dataset)"}
    line.update(extra)
    print(json.dumps(line), flush=True)


def run_uneven(args):
    """Uneven batch: a seeded sample of the 4096-stack distribution (disk count
    U{5..80}, grid {64,128,256}, U{64..1024} frequencies, half dancer / half
    transformer) solved through the serving engine (all requests submitted at
    once, 4 worker streams) and one after another on one handle ("plain");
    each request's beta^2 must be the same both ways.  An untimed pass first
    runs every bounce-loop request for a few bounces, so that the autotuner's
    first-solve trials are paid by neither arm."""
    import torch
    torch.cuda.set_device(0)
    import build as _b
    _b.build()
    import bfgb300 as B
    from bfgb300 import workloads as W
    reqs = W.config4_uneven()[:args.requests]
    h = B.Handle(0)
    mode_cache = {}   # requests on one grid with one mode set share a basis
    # untimed: the autotuner's first-solve trials for every stage shape of the
    # batch (a few bounces of each bounce-loop request), so that neither arm
    # below pays them and neither reuses the other's
    for r in reqs:
        if r["solver"] != "transformer":
            st, m = _build_request_stack(B, W, h, r, mode_cache)
            _solve_plain(B, h, st, m, dict(r, nmax=min(r["nmax"], 3)))
            st.close()
    # plain: one request after another on one handle; each stack is created
    # before and closed after its own (timed) solve, so that the workspaces of
    # hundreds of large stacks do not pile up on the device
    t_plain, plain = 0.0, []
    for r in reqs:
        st, m = _build_request_stack(B, W, h, r, mode_cache)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        plain.append(_solve_plain(B, h, st, m, r))
        t_plain += time.perf_counter() - t0
        st.close()
    batch_set = [_build_request_stack(B, W, h, r, mode_cache) for r in reqs]
    torch.cuda.synchronize()
    srv = B.Server(0, hbm_budget_bytes=int(180e9), n_workers=args.workers)
    try:
        clock = ClockSampler(0)
        clock.start()
        t0 = time.perf_counter()
        ids = [srv.submit(st, r["freqs"], r["solver"], modes=m, nmax=r["nmax"], precision="mixed")
               for (st, m), r in zip(batch_set, reqs)]
        res = [srv.wait(i) for i in ids]
        t_batch = time.perf_counter() - t0
        clocks = clock.stop()
        st_all, st_d, st_t = srv.stats(), srv.stats("dancer"), srv.stats("transformer")
    finally:
        srv.close()   # before the stacks it serves
    worst = max(float(np.max(np.abs(r["beta2"] - p) / np.abs(p))) for r, p in zip(res, plain))
    fpts = sum(len(r["freqs"]) for r in reqs)
    _close_all(batch_set, mode_cache)
    h.close()
    _server_line(
        "beta2 freq-points/s (uneven batch of disk stacks: 5-80 disks, 64/128/256 grids, 64-1024 freqs, "
        "dancer + transformer)", fpts / t_batch, len(reqs), t_batch,
        {"config": {"workload": f"uneven-batch-{len(reqs)}-of-4096-stacks", "requests": len(reqs),
                    "dancers": sum(r["solver"] == "dancer" for r in reqs), "workers": args.workers,
                    "dancer_bounces": reqs[0]["nmax"] + 1, "transformer_modes": reqs[0]["M"],
                    "hbm_budget_gb": 180, "l2": "no flush: per-request working sets > L2"},
         "plain_freqpts_per_s": fpts / t_plain, "batched_over_plain": t_plain / t_batch,
         "beta2_max_rel_diff_batched_vs_plain": worst,
         "latency_ms": {"p50": st_all["p50_ms"], "p99": st_all["p99_ms"], "max": st_all["max_ms"]},
         "per_solver": {"dancer": st_d, "transformer": st_t}, "evictions": st_all["evictions"],
         "clocks": clocks})


def _size_class(r):
    """Latency class of a request: solver, disk count band, grid, frequency band."""
    nd = r["ndisk"]
    band = "5-20" if nd <= 20 else ("21-40" if nd <= 40 else "41-80")
    nfb = "64-256" if len(r["freqs"]) <= 256 else "257-1024"
    return f"{r['solver']} {band} disks {r['n']}^2 {nfb} f"


def _open_loop(srv, nclients, rate, seconds, submit_one, seed=77, drain_s=20.0, weights=None):
    """Open-loop arrivals: a Poisson process of `rate` requests/s for
    `seconds`, each arrival assigned to a uniformly drawn client; the
    dispatcher submits at the scheduled time whatever the state of earlier
    requests (a client's requests queue behind each other on its stack).  A
    request's latency runs from its scheduled arrival to its completion: the
    server's submit-to-completion time plus the dispatcher's lag.  Completions
    are collected after the window (no polling thread competes with the
    dispatcher); requests still pending `drain_s` after the window are
    counted as unfinished.  weights: the clients' shares of the arrivals
    (default uniform).  Returns (records, wall seconds from the first
    arrival to the last completion, arrivals, unfinished, failed)."""
    import gc
    rng = np.random.default_rng(seed)
    n = int(rng.poisson(rate * seconds))
    t_arr = np.sort(rng.uniform(0.0, seconds, n))
    who = rng.integers(0, nclients, n) if weights is None else rng.choice(nclients, n, p=weights)
    sent = []
    gc.disable()   # no collector pause inside the dispatch loop
    try:
        t0 = time.perf_counter()
        for i in range(n):
            dt = t0 + t_arr[i] - time.perf_counter()
            if dt > 0:
                time.sleep(dt)
            t_s = time.perf_counter()
            lag = t_s - (t0 + t_arr[i])
            rid, cls = submit_one(int(who[i]))
            sent.append((rid, {"client": int(who[i]), "cls": cls, "lag_s": lag,
                               "submit_s": time.perf_counter() - t_s}))
    finally:
        gc.enable()
    deadline = time.perf_counter() + drain_s
    recs, unfinished, failed = [], 0, 0
    first, last = None, None
    for rid, meta in sent:
        try:
            res = srv.wait(rid, timeout_ms=int(max(0.0, deadline - time.perf_counter()) * 1000))
        except TimeoutError:
            unfinished += 1
            continue
        except Exception:
            failed += 1
            continue
        t_first = res["t_submit"] - meta["lag_s"]
        first = t_first if first is None else min(first, t_first)
        last = res["t_done"] if last is None else max(last, res["t_done"])
        recs.append(dict(meta, latency_ms=1e3 * (res["t_done"] - res["t_submit"] + meta["lag_s"])))
    wall = (last - first) if recs else seconds
    return recs, wall, n, unfinished, failed


def _optimiser_requests(nclients):
    """The optimiser class: 20-disk, 256-frequency transformer requests (8
    Laguerre-Gauss modes, 128x128 over 1 m), one seeded booster per client."""
    from bfgb300 import workloads as W
    reqs = []
    for k in range(nclients):
        rng = np.random.default_rng(500 + k)
        distance, eps, tx, ty = W.booster(20, rng.uniform(7.5e-3, 8.5e-3, 20))
        reqs.append(dict(solver="transformer", ndisk=20, n=128, nf=256, distance=distance, eps=eps,
                         relative_tilt_x=tx, relative_tilt_y=ty, X=W.symmetric_grid(128), diskR=0.15,
                         freqs=np.linspace(19.5e9, 20.5e9, 256), nmax=0, M=8, waist=0.03))
    return reqs


def run_serve(args, optimiser_class=False):
    """Serving loop, open loop: boost-factor solves arrive as a Poisson
    process of mean rate --rate (2000 requests/s) for --serve-seconds; each
    arrival is a step of one client, which moves that client's gaps by
    N(0, 10 um) and submits a solve of its resident stack
    (bf_request.distance).
    - optimiser_class (serve-opt): 32 optimiser clients (20-disk,
      256-frequency transformer requests), drawn uniformly.
    - otherwise (serve, the configuration-4 mix): the same 32 optimiser
      clients as interactive requests in the server's latency lane
      (--lane-workers reserved workers on high-priority streams) plus 16
      background clients whose stacks follow the uneven-batch distribution
      (5-80 disks, 64/128/256 grids, 64-1024 frequencies, dancers and
      transformers), at --bg-rate of the arrivals' rate.
    Latency percentiles are reported per request class."""
    import torch
    torch.cuda.set_device(0)
    import build as _b
    _b.build()
    import bfgb300 as B
    from bfgb300 import workloads as W
    n_int = 32
    reqs = _optimiser_requests(n_int)
    lanes = [0] * n_int
    classes = ["interactive: " + _size_class(r) for r in reqs] if not optimiser_class else \
        [_size_class(r) for r in reqs]
    n_bg = 0
    if not optimiser_class:
        bg = W.config4_uneven(seed=5, count=16)
        n_bg = len(bg)
        reqs = reqs + bg
        lanes = [1] * n_int + [0] * n_bg
        classes = classes + ["background: " + _size_class(r) for r in bg]
    nclients = len(reqs)
    h = B.Handle(0)
    mode_cache = {}
    stacks = [_build_request_stack(B, W, h, r, mode_cache) for r in reqs]
    n_lane = 0 if optimiser_class else args.lane_workers
    srv = B.Server(0, hbm_budget_bytes=int(180e9), n_workers=args.workers + n_lane,
                   reserve_hbm=not optimiser_class)
    try:
        if n_lane:
            srv.set_latency_lane(n_lane)

        # untimed warm-up on the serving server itself: one step per client
        # (builds the resident overlaps / plans), then two bursts of one step
        # from every interactive client at once (the group solves a burst
        # forms and their one-time tuning); the statistics window starts after it
        def warm(k):
            st, m = stacks[k]
            r = reqs[k]
            return srv.submit(st, r["freqs"], r["solver"], modes=m, distance=r["distance"], nmax=r["nmax"],
                              precision=args.serve_precision, lane=lanes[k])
        for k in range(nclients):
            srv.wait(warm(k))
        for _ in range(2):
            for i in [warm(k) for k in range(n_int)]:
                srv.wait(i)
        srv.reset_stats()
    except BaseException:
        srv.close()
        raise
    rngs = [np.random.default_rng(1000 + k) for k in range(nclients)]
    dist = [np.array(r["distance"]) for r in reqs]
    weights = None
    if n_bg:
        # background arrivals at bg_rate / rate of all arrivals
        pb = min(max(args.bg_rate / args.rate, 0.0), 1.0)
        weights = np.array([(1.0 - pb) / n_int] * n_int + [pb / n_bg] * n_bg)

    def submit_one(k):
        dist[k] = W.optimiser_step(dist[k], rngs[k])
        st, m = stacks[k]
        r = reqs[k]
        return srv.submit(st, r["freqs"], r["solver"], modes=m, distance=dist[k], nmax=r["nmax"],
                          precision=args.serve_precision, lane=lanes[k]), classes[k]

    try:
        clock = ClockSampler(0)
        clock.start()
        recs, wall, n_arr, unfinished, failed = _open_loop(srv, nclients, args.rate, args.serve_seconds,
                                                           submit_one, weights=weights,
                                                           drain_s=20.0 if optimiser_class else 120.0)
        clocks = clock.stop()
        st_all, st_d, st_t = srv.stats(), srv.stats("dancer"), srv.stats("transformer")
    finally:
        srv.close()   # cancels what is still queued, waits for what runs
    _close_all(stacks, mode_cache)
    h.close()
    lat = np.array([r["latency_ms"] for r in recs]) if recs else np.zeros(1)
    per_class = {}
    for cl in sorted(set(r["cls"] for r in recs)):
        v = np.array([r["latency_ms"] for r in recs if r["cls"] == cl])
        per_class[cl] = {"requests": int(len(v)), "p50_ms": float(np.percentile(v, 50)),
                         "p99_ms": float(np.percentile(v, 99)), "max_ms": float(v.max())}
    fpts = float(sum(len(reqs[r["client"]]["freqs"]) for r in recs))
    if optimiser_class:
        metric = (f"beta2 freq-points/s and p50/p99 latency, Poisson arrivals at {args.rate:g}/s from 32 "
                  f"optimiser clients, 20-disk 256-frequency transformer requests (8 LG modes, 128x128)")
        workload = "serve-optimiser-class"
    else:
        metric = (f"beta2 freq-points/s and per-class p50/p99 latency, Poisson arrivals at {args.rate:g}/s: 32 "
                  f"optimiser clients (20-disk 256-frequency transformer, latency lane) and 16 clients of the "
                  f"uneven-batch distribution ({args.bg_rate:g}/s)")
        workload = "serve-configuration-4-mix"
    _server_line(
        metric, fpts / wall, len(recs), wall,
        {"config": {"workload": workload, "arrivals": "poisson", "rate_per_s": args.rate,
                    "clients": nclients, "background_clients": n_bg,
                    "background_rate_per_s": args.bg_rate if n_bg else 0.0,
                    "seconds": args.serve_seconds, "workers": args.workers, "lane_workers": n_lane,
                    "hbm_budget_gb": 180, "gap_step_um": 10, "precision": args.serve_precision},
         "offered": n_arr, "completed": len(recs), "unfinished_after_drain": unfinished, "failed": failed,
         "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                        "mean": float(lat.mean()), "max": float(lat.max())},
         "latency_by_class": per_class,
         "requests_per_s": len(recs) / wall, "per_solver": {"dancer": st_d, "transformer": st_t},
         "dispatch_lag_ms_p99": float(np.percentile([1e3 * r["lag_s"] for r in recs], 99)) if recs else None,
         "dispatch_lag_ms_max": float(max(1e3 * r["lag_s"] for r in recs)) if recs else None,
         "submit_call_ms_p99": float(np.percentile([1e3 * r["submit_s"] for r in recs], 99)) if recs else None,
         "submit_call_ms_max": float(max(1e3 * r["submit_s"] for r in recs)) if recs else None,
         "evictions": st_all["evictions"], "batched": st_all.get("batched"), "clocks": clocks})


def run_serve_pgrid(args):
    """Serving loop on propagation-matrix grids: 32 optimiser clients, each
    with its own resident grid (20 disks, 256 frequencies, 8 Laguerre-Gauss
    modes, 128x128 over 1 m, 9 spacings from -200 um to +200 um, built at
    mixed precision).  Every step random-walks the per-disk shifts by
    N(0, 10 um) inside the grid and submits a "pgrid" request; the steps
    arrive open loop, a Poisson process of mean rate --rate (2000/s) with
    each arrival assigned to a uniformly drawn client.  This is the
    interpolated-matrix optimiser loop: a step solves the stack at the
    interpolated matrices instead of recomputing them."""
    import torch
    torch.cuda.set_device(0)
    import build as _b
    _b.build()
    import bfgb300 as B
    from bfgb300 import workloads as W
    nclients, n, nf, ndisk, M = 32, 128, 256, 20, 8
    sgrid = np.linspace(-2e-4, 2e-4, 9)
    freqs = np.linspace(19.5e9, 20.5e9, nf)
    h = B.Handle(0)
    X = W.symmetric_grid(n)
    c = B.SeedCoordinateSystem(X=X, Y=X)
    pats, kt = W.lg_modes(c.X, c.Y, M, 0.03, 0.15)
    modes = B.SeedModes(c, ThreeDim=True, Mmax=M, Lmax=0, diskR=0.15, pattern_input=pats, kT_arr=kt, handle=h)
    grids = []
    t0 = time.perf_counter()
    for k in range(nclients):
        rng = np.random.default_rng(500 + k)
        distance, eps, tx, ty = W.booster(ndisk, rng.uniform(7.5e-3, 8.5e-3, ndisk))
        sb = B.SeedSetupBoundaries(c, diskno=ndisk, distance=distance, epsilon=eps, relative_tilt_x=tx,
                                   relative_tilt_y=ty)
        grids.append(B.PGrid(sb, c, modes, freqs, sgrid, precision="mixed"))
    t_create = (time.perf_counter() - t0) / nclients
    srv = B.Server(0, hbm_budget_bytes=int(180e9), n_workers=args.workers)
    try:
        for g in grids:   # one warm-up step per client, untimed; the statistics window starts after it
            srv.wait(srv.submit(None, freqs, "pgrid", distance=np.zeros(ndisk), pgrid=g))
        srv.reset_stats()
    except BaseException:
        srv.close()
        raise
    lo, hi = sgrid[0], sgrid[-1]
    rngs = [np.random.default_rng(1000 + k) for k in range(nclients)]
    shifts = [np.zeros(ndisk) for _ in range(nclients)]

    def submit_one(k):
        shifts[k] = np.clip(shifts[k] + rngs[k].normal(0.0, 10e-6, ndisk), lo, hi)
        return srv.submit(None, freqs, "pgrid", distance=shifts[k], pgrid=grids[k]), "pgrid"

    try:
        clock = ClockSampler(0)
        clock.start()
        recs, wall, n_arr, unfinished, failed = _open_loop(srv, nclients, args.rate, args.serve_seconds,
                                                           submit_one)
        clocks = clock.stop()
        st_all = srv.stats()
    finally:
        srv.close()
    for g in grids:
        g.close()
    modes.close()
    h.close()
    lat = np.array([r["latency_ms"] for r in recs]) if recs else np.zeros(1)
    errors = [] if not failed else [f"{failed} failed requests"]
    _server_line(
        f"beta2 freq-points/s and p50/p99 latency, Poisson arrivals at {args.rate:g}/s from 32 optimiser clients, "
        "interpolated propagation-matrix grids (20 disks, 256 freqs, 8 LG modes, 128x128)",
        nf * len(recs) / wall, len(recs), wall,
        {"config": {"workload": "serve-pgrid-optimiser-class", "arrivals": "poisson", "rate_per_s": args.rate,
                    "clients": nclients, "disks": ndisk, "freqs": nf,
                    "modes": M, "grid": n, "spacings": len(sgrid), "spacing_range_um": [-200, 200],
                    "seconds": args.serve_seconds, "workers": args.workers, "gap_step_um": 10, "precision": "mixed"},
         "offered": n_arr, "completed": len(recs), "unfinished_after_drain": unfinished, "failed": failed,
         "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                        "mean": float(lat.mean()), "max": float(lat.max())},
         "requests_per_s": len(recs) / wall, "grid_create_s_per_client": t_create,
         "evictions": st_all["evictions"], "client_errors": errors[:3], "clocks": clocks})


def run_pgrid(args):
    """One optimiser on an interpolated propagation-matrix grid: 20 disks, 256
    frequencies, 8 Laguerre-Gauss modes, 128x128, 9 spacings, mixed precision;
    a step is bf_pgrid_transformer at new per-disk shifts (random walk N(0, 10
    um) inside the grid).  Device time with CUDA events on the library's
    stream; e2e is the host wall clock of the same calls (shifts in, beta^2
    out)."""
    import torch
    torch.cuda.set_device(0)
    import build as _b
    _b.build()
    import bfgb300 as B
    from bfgb300 import workloads as W
    n, nf, ndisk, M = 128, 256, 20, 8
    sgrid = np.linspace(-2e-4, 2e-4, 9)
    freqs = np.linspace(19.5e9, 20.5e9, nf)
    h = B.Handle(0)
    stream = torch.cuda.current_stream()
    h.set_stream(stream.cuda_stream)
    X = W.symmetric_grid(n)
    c = B.SeedCoordinateSystem(X=X, Y=X)
    pats, kt = W.lg_modes(c.X, c.Y, M, 0.03, 0.15)
    modes = B.SeedModes(c, ThreeDim=True, Mmax=M, Lmax=0, diskR=0.15, pattern_input=pats, kT_arr=kt, handle=h)
    rng = np.random.default_rng(500)
    distance, eps, tx, ty = W.booster(ndisk, rng.uniform(7.5e-3, 8.5e-3, ndisk))
    sb = B.SeedSetupBoundaries(c, diskno=ndisk, distance=distance, epsilon=eps, relative_tilt_x=tx,
                               relative_tilt_y=ty)
    t0 = time.perf_counter()
    g = B.PGrid(sb, c, modes, freqs, sgrid, precision="mixed")
    t_create = time.perf_counter() - t0
    shifts = [np.zeros(ndisk)]
    for _ in range(args.warmup + args.steps):
        shifts.append(np.clip(shifts[-1] + rng.normal(0.0, 10e-6, ndisk), sgrid[0], sgrid[-1]))
    for k in range(args.warmup):
        g.transformer(shifts[k])
    torch.cuda.synchronize()
    clock = ClockSampler(0)
    clock.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    e0.record(stream)
    for k in range(args.steps):
        g.transformer(shifts[args.warmup + k])
    e1.record(stream)
    torch.cuda.synchronize()
    wall = (time.perf_counter() - t0) / args.steps
    clocks = clock.stop()
    dev_ms = e0.elapsed_time(e1) / args.steps
    g.close()
    modes.close()
    h.close()
    print(json.dumps({"metric": "beta2 freq-points/s of one optimiser on an interpolated propagation-matrix grid "
                                "(20 disks, 256 freqs, 8 LG modes, 128x128)",
                      "value": nf / (dev_ms / 1000.0), "unit": UNIT, "n_gpus": 1, "steps": args.steps,
                      "warmup": args.warmup, "ms_per_step": dev_ms, "higher_is_better": True, "scaling": "weak",
                      "vs_baseline": None, "dtype": "c64 matrices, double-float chain, f64 spline and solve",
                      "data": "synthetic (seeded geometry)",
                      "config": {"workload": "pgrid-step-20disk-256f-8LG-128", "spacings": len(sgrid),
                                 "l2": "no flush: a step reads the grid's 2.8 MB of coefficients per frequency"},
                      "grid_create_s": t_create,
                      "e2e": {"value": nf / wall, "unit": UNIT, "ms_per_step": 1000.0 * wall,
                              "h2d_bytes_per_step": 8 * ndisk, "d2h_bytes_per_step": 8 * nf + 16 * nf * M},
                      "clocks": clocks}), flush=True)


def run_c1(args):
    """The reference's own CPU-runnable case: the plain dancer, complex128,
    mirror + 1 disk, 64x64 over 1 m, 20 GHz, 201 bounces, the default emission.
    GPU: the FP64 dancer through the C ABI (host buffers) per call; CPU: the FP64
    oracle's dancer on one core; the exit fields compared."""
    import torch
    torch.cuda.set_device(0)
    import build as _b
    _b.build()
    import bfgb300 as B
    from bfgb300 import workloads as W
    sys.path.insert(0, REPO)
    from oracle import bf_oracle as O
    w = W.config1_dancer()
    cb = B.SeedCoordinateSystem(X=w["X"], Y=w["Y"])
    co = O.seed_coordinate_system(X=w["X"], Y=w["Y"])
    kw = dict(diskno=1, distance=w["distance"], epsilon=w["eps"])
    sbb = B.SeedSetupBoundaries(cb, **kw)
    sbo = O.seed_setup_boundaries(co, **kw)
    for _ in range(args.warmup):
        B.dancer(0, w["nmax"], sbb, cb, f=20e9, diskR=w["diskR"])
    torch.cuda.synchronize()
    clock = ClockSampler(0)
    clock.start()
    ts = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        got = B.dancer(0, w["nmax"], sbb, cb, f=20e9, diskR=w["diskR"])
        ts.append(time.perf_counter() - t0)
    clocks = clock.stop()
    t_gpu = float(np.median(ts))
    t0 = time.perf_counter()
    ref = O.dancer(0, w["nmax"], sbo, co, f=20e9, diskR=w["diskR"])
    t_cpu = time.perf_counter() - t0
    err = float(np.linalg.norm(got - ref) / np.linalg.norm(ref))
    print(json.dumps({"metric": "beta2 freq-points/s (plain dancer, complex128, 1 disk, 64x64, 201 bounces)",
                      "value": 1.0 / t_gpu, "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
                      "ms_per_step": 1000.0 * t_gpu, "higher_is_better": True, "scaling": "weak",
                      "vs_baseline": None, "dtype": "f64", "data": "synthetic (the reference's own 1-disk setup)",
                      "config": {"workload": "dancer-1disk-64-201bounces", "timing": "host wall clock per C ABI call"},
                      "exit_field_rel_err_vs_oracle": err,
                      "cpu_baseline": {"value": 1.0 / t_cpu, "unit": UNIT, "cores": 1, "kind": "port",
                                       "sample": "the FP64 oracle's dancer, the whole case, one core"},
                      "clocks": clocks}), flush=True)


def run_peaks(args):
    """The measured arithmetic peaks that are the denominators of the SIMT and
    TF32 rooflines (FP32 FFMA, packed FP32x2 FFMA, FP64 DFMA and a cuBLAS
    8192^3 TF32 GEMM on this machine's GB300), as recorded in
    profiles/simt_peaks.json with the method that measured them."""
    sp = simt_peaks()
    if not sp:
        print(json.dumps({"metric": "measured arithmetic peaks", "unavailable": "profiles/simt_peaks.json missing"}),
              flush=True)
        return
    print(json.dumps({"metric": "measured arithmetic peaks", "value": sp["fp32_ffma_tflops"], "unit": "TFLOP/s",
                      "source": "profiles/simt_peaks.json (recorded measurement)", "peaks": sp}), flush=True)


def run_1d(args):
    """Batched 1D model: 4096 spacing configurations of the 20-disk booster
    (each gap moved by N(0, 10 um) from the seeded geometry) x 256 frequencies
    19.5-20.5 GHz per step, one FP64 launch (bf_transformer_1d_batch).  The
    plain path solves one configuration per 1D transformer call."""
    import torch
    torch.cuda.set_device(0)
    import build as _b
    _b.build()
    import bfgb300 as B
    from bfgb300 import workloads as W
    from bfgb300 import _lib
    w = W.config2_cheerleader()
    rng = np.random.default_rng(77)
    nconf, nf = 4096, 256
    confs = np.ascontiguousarray([W.optimiser_step(w["distance"], rng) for _ in range(nconf)])
    eps = np.ascontiguousarray(w["eps"], dtype=np.complex128)
    freqs = np.ascontiguousarray(np.linspace(19.5e9, 20.5e9, nf))
    h = B.Handle(0)
    stream = torch.cuda.current_stream()
    h.set_stream(stream.cuda_stream)
    b2 = np.empty((nconf, nf))
    L = _lib.lib()

    def step():
        h.check(L.bf_transformer_1d_batch(h.ptr, nconf, len(eps), _lib.ptr(confs), _lib.ptr(eps.view(np.float64)), nf,
                                          _lib.ptr(freqs), None, None, _lib.ptr(b2)))

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    clock = ClockSampler(0)
    clock.start()
    kern_ms = []
    prof = np.zeros(8)
    L.bf_set_profiling(h.ptr, 1)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
        h.check(L.bf_last_profile(h.ptr, _lib.ptr(prof)))
        kern_ms.append(prof[1])
    torch.cuda.synchronize()
    wall = (time.perf_counter() - t0) / args.steps
    L.bf_set_profiling(h.ptr, 0)
    clocks = clock.stop()
    kms = float(np.mean(kern_ms))
    # plain: the 1D transformer per configuration (frequencies batched), 32 configurations
    c1 = B.SeedCoordinateSystem(X=np.array([1e-7]), Y=np.array([1e-7]))
    m1 = B.SeedModes(c1, ThreeDim=False, handle=h)
    t0 = time.perf_counter()
    for c in range(32):
        sb = B.SeedSetupBoundaries(c1, diskno=20, distance=confs[c], epsilon=w["eps"].copy())
        B.transformer(sb, c1, m1, f=freqs, prop=B.propagator1D)
    plain = 32 * nf / (time.perf_counter() - t0)
    # accuracy: the oracle's 1D transformer on a sample of points
    sys.path.insert(0, REPO)
    from oracle import bf_oracle as O
    co = O.seed_coordinate_system(X=np.array([1e-7]), Y=np.array([1e-7]))
    mo = O.seed_modes(co, ThreeDim=False)
    errs = []
    for c, k in ((0, 0), (1000, 100), (4095, 255), (2048, 128)):
        sb = O.seed_setup_boundaries(co, diskno=20, distance=confs[c], epsilon=w["eps"].copy())
        ref = abs(O.transformer(sb, co, mo, f=freqs[k], prop=O.propagator1d)[0]) ** 2
        errs.append(abs(b2[c, k] - ref) / ref)
    m1.close()
    h.close()
    # FP64 roofline of k_tf1d: the explicit arithmetic of one region (complex
    # products 6 flops, sums 2: axion term 10, boundary factors 28, propagation
    # 12, phase argument 2 = 52 flops), not counting sincospi, over the FP64
    # DFMA rate measured by `bench.py --workload peaks` (nominal 1.25 TFLOP/s
    # without it)
    nregions = len(eps) - 1
    flops = 52.0 * nregions * nconf * nf
    sp = simt_peaks()
    fp64_peak, fp64_src = ((float(sp["fp64_dfma_tflops"]), "measured (DFMA probe, profiles/simt_peaks.json)")
                           if sp and sp.get("fp64_dfma_tflops") else (1.25, "nominal"))
    line = {"metric": "beta2 freq-points/s (batched 1D model, 20-disk booster, spacing configurations x frequencies)",
            "value": nconf * nf / (kms / 1000.0), "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": kms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded geometry, gap steps N(0, 10 um))",
            "config": {"workload": f"1d-20disk-{nconf}configs-{nf}f", "configs": nconf, "freqs": nf,
                       "timing": "value: k_tf1d device time (CUDA events, inputs resident); e2e: host wall clock "
                                 "around the C ABI call (host buffers in and out)",
                       "l2": "no flush: 9 MB working set, compute-bound"},
            "plain_freqpts_per_s": plain, "beta2_rel_err_vs_oracle_max": float(max(errs)),
            "roofline": {"bound": "fp64", "achieved": flops / (kms / 1000.0) / 1e12,
                         "peak": fp64_peak, "peak_source": fp64_src, "unit": "TFLOP/s",
                         "frac": flops / (kms / 1000.0) / 1e12 / fp64_peak,
                         "kernel": "k_tf1d", "flops_per_region": 52, "note": "sincospi/exp not counted"},
            "gpu_launches": args.steps, "clocks": clocks,
            "e2e": {"value": nconf * nf / wall, "unit": UNIT, "h2d_bytes_per_step": int(confs.nbytes + freqs.nbytes),
                    "d2h_bytes_per_step": int(b2.nbytes)}}
    print(json.dumps(line), flush=True)


def c2_config(w):
    """The `config` of the cheerleader workload, the same on both arms."""
    nf, nmax = len(w["freqs"]), w["nmax"]
    return {"workload": w["name"] + f"-{nf}f-{nmax + 1}bounces", "grid": len(w["X"]),
            "disks": (len(w["distance"]) - 2) // 2, "freqs": nf, "bounces": nmax + 1,
            "precision": "mixed", "per_gpu_request": f"one {nf}-frequency request per GPU",
            "l2": "no flush: per-step working set (phasor tables + fields) > L2"}


def run_reference(args):
    """The reference's algorithm on the host cores.  The reference is Julia
    (FFTW/LAPACK), which this machine does not have, so its FP64 numpy
    restatement (the oracle, pinned to the reference's golden vectors) runs
    instead, on every host core.  A step is a bounded sample of the request:
    as many of its frequencies as there are cores, each solved at the full
    bounce count by one process; freq-points/s = sample size / step wall.
    The warm-up steps start the process pool and run a one-bounce solve per
    process (imports, FFT set-up); a CPU solve has no other state to warm."""
    ws, rank, local = dist_env()
    if rank != 0:
        return
    over = {}
    if args.nf:
        over["nf"] = args.nf
    if args.nmax is not None:
        over["nmax"] = args.nmax
    w = workload(0, **over)
    P = os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    walls, per_proc = [], []
    with ctx.Pool(P) as pool:
        for k in range(max(args.warmup, 0)):
            cpu_sample(pool, w, sample_freqs(w, P, k), 0)
        t0 = time.perf_counter()
        for k in range(args.steps):
            wall, per = cpu_sample(pool, w, sample_freqs(w, P, k), w["nmax"])
            walls.append(wall)
            per_proc.append(max(per))
        timed = time.perf_counter() - t0
    ms_step = 1000.0 * timed / max(args.steps, 1)
    value = P / (ms_step / 1000.0)
    cb = dict(value=value, unit=UNIT, cores=P, kind="port",
              sample=f"per step {P} of the {len(w['freqs'])} frequencies (shifted by one index per step), "
                     f"each at the full {w['nmax'] + 1} bounces in one of {P} spawned processes; "
                     f"FP64 numpy oracle cheerleader")
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128 (FP64 oracle)",
            "data": "synthetic (seeded geometry, no dataset)",
            "config": c2_config(w),
            "impl": "reference", "cpu_baseline": cb,
            "reference_note": "the reference is Julia (not installed here or on the GPU box); its algorithm runs "
                              "as the FP64 numpy restatement pinned to the reference's golden vectors",
            "step_wall_s": {"median": statistics.median(walls), "max": max(walls)} if walls else None,
            "slowest_process_s_median": statistics.median(per_proc) if per_proc else None,
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--nf", type=int, default=0, help="override frequency count (testing only)")
    ap.add_argument("--nmax", type=int, default=None, help="override nmax (testing only)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--fused-variant", type=int, default=None,
                    help="force one fused-stage kernel variant (0-8, bit-identical results; profiling only)")
    ap.add_argument("--workload", default="cheerleader",
                    choices=["cheerleader", "transformer", "uneven", "serve", "serve-opt", "serve-pgrid", "1d", "peaks",
                             "c1", "pgrid"])
    ap.add_argument("--requests", type=int, default=24, help="uneven batch: requests of the seeded 4096")
    ap.add_argument("--workers", type=int, default=4, help="serving engine worker streams")
    ap.add_argument("--lane-workers", type=int, default=3,
                    help="serve: workers reserved, on high-priority streams, for the interactive clients")
    ap.add_argument("--bg-rate", type=float, default=0.5,
                    help="serve: arrivals per second of the uneven-batch background clients")
    ap.add_argument("--serve-seconds", type=float, default=10.0)
    ap.add_argument("--rate", type=float, default=2000.0, help="serving: mean Poisson arrival rate, requests/s")
    ap.add_argument("--serve-precision", default="mixed", help="serving: precision of the transformer requests")
    args = ap.parse_args()
    if args.workload == "transformer" and args.impl == "ours":
        run_transformer(args)
    elif args.workload == "uneven" and args.impl == "ours":
        run_uneven(args)
    elif args.workload == "1d" and args.impl == "ours":
        run_1d(args)
    elif args.workload == "pgrid" and args.impl == "ours":
        run_pgrid(args)
    elif args.workload == "c1" and args.impl == "ours":
        run_c1(args)
    elif args.workload == "peaks" and args.impl == "ours":
        run_peaks(args)
    elif args.workload == "serve-pgrid" and args.impl == "ours":
        run_serve_pgrid(args)
    elif args.workload in ("serve", "serve-opt") and args.impl == "ours":
        run_serve(args, optimiser_class=args.workload == "serve-opt")
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
