"""Generate tests/golden/c2_cheerleader_oracle.npz: the oracle's cheerleader
exit field and beta^2 at the full 20-disk cheerleader workload (128x128 grid
over 1 m, per-disk tilts, nmax = 400, i.e. 401 bounces) for a few of its 256
frequencies, one of them the spectrum's maximum.

The oracle needs about half a minute per frequency at this size, so the GPU
parity test and the benchmark's accuracy check read these values instead of
re-running it.  Run from the repository root:

    python tests/golden/make_c2_fixture.py [peak_index]

`peak_index` is the frequency index of the largest beta^2 of the 256-point
spectrum (from a solve of the same workload); the other indices are fixed.
The frequencies run in spawned processes, one per frequency.
"""
import multiprocessing as mp
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
for _p in (REPO, os.path.join(REPO, "boostfractor.jl_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

FIXED_INDEX = [0, 101, 255]
OUT = os.path.join(HERE, "c2_cheerleader_oracle.npz")


def _solve(fi):
    for _p in (REPO, os.path.join(REPO, "boostfractor.jl_gb300")):
        if _p not in sys.path:
            sys.path.insert(0, _p)
    from oracle import bf_oracle as O
    from bfgb300 import workloads as W
    w = W.config2_cheerleader()
    co = O.seed_coordinate_system(X=w["X"], Y=w["Y"])
    sb = O.seed_setup_boundaries(co, diskno=(len(w["distance"]) - 2) // 2, distance=w["distance"],
                                 epsilon=w["eps"].copy(), relative_tilt_x=w["relative_tilt_x"],
                                 relative_tilt_y=w["relative_tilt_y"])
    E = O.cheerleader(0, w["nmax"], sb, co, f=float(w["freqs"][fi]), diskR=w["diskR"])
    return E, O.boost_factor_rfp(E, co, w["diskR"])


def main(argv):
    from bfgb300 import workloads as W
    idx = sorted(set(FIXED_INDEX + [int(a) for a in argv]))
    w = W.config2_cheerleader()
    with mp.get_context("spawn").Pool(len(idx)) as pool:
        res = pool.map(_solve, idx)
    for fi, (_, b2) in zip(idx, res):
        print(f"index {fi:3d}  {w['freqs'][fi]:.6e} Hz  beta2 = {b2:.12g}", flush=True)
    np.savez_compressed(OUT, freq_index=np.array(idx), freqs=w["freqs"][idx],
                        exit_field=np.array([r[0] for r in res]), beta2=np.array([r[1] for r in res]),
                        peak_index=np.array([int(a) for a in argv][:1] or [-1]))


if __name__ == "__main__":
    main(sys.argv[1:])
