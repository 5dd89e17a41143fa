"""Generate tests/golden/c3_lg_oracle.npz: the oracle's transformer boost at
the full transformer workload (20 disks with surface maps, 64 Laguerre-Gauss
modes, 256x256 grid) for three of its 1024 frequencies.

The oracle needs about a minute per frequency at this size, so the GPU parity
test reads these values instead of re-running it.  Run from the repository
root:  python tests/golden/make_c3_fixture.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "boostfractor.jl_gb300"))

from oracle import bf_oracle as O          # noqa: E402
from bfgb300 import workloads as W         # noqa: E402

FREQ_INDEX = np.array([0, 341, 700])


def main():
    w = W.config3_transformer()
    c = O.seed_coordinate_system(X=w["X"], Y=w["Y"])
    m = O.seed_modes(c, ThreeDim=True, Mmax=w["M"], Lmax=w["L"], diskR=w["diskR"],
                     pattern_input=w["pattern_input"], kT_arr=w["kT_arr"])
    boosts = []
    for f in w["freqs"][FREQ_INDEX]:
        sb = O.seed_setup_boundaries(c, diskno=(len(w["distance"]) - 2) // 2, distance=w["distance"],
                                     epsilon=w["eps"].copy(), relative_tilt_x=w["relative_tilt_x"],
                                     relative_tilt_y=w["relative_tilt_y"],
                                     relative_surfaces=w["relative_surfaces"])
        boosts.append(O.transformer(sb, c, m, f=f, diskR=w["diskR"]))
        print(f"{f:.6e} Hz  beta2 = {np.sum(np.abs(boosts[-1]) ** 2):.12g}", flush=True)
    np.savez(os.path.join(HERE, "c3_lg_oracle.npz"), freq_index=FREQ_INDEX, freqs=w["freqs"][FREQ_INDEX],
             boost=np.array(boosts), beta2=np.sum(np.abs(np.array(boosts)) ** 2, axis=1))


if __name__ == "__main__":
    main()
