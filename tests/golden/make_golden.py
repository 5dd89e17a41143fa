"""Regenerate tests/golden/analytical1d.npz from the reference's own 1D model.

Run in a container that has the reference checkout (its src/Analytical1D.py
is plain numpy and runs as-is):

    python tests/golden/make_golden.py /path/to/BoostFractor.jl

Writes analytical1d.npz: |ax|^2 of the reference's 1D model
(src/Analytical1D.py:79-131, ``disk_system``) for seeded lossless stacks, the
independent cross-check of the transformer/cheerleader 1D limit.  The
full-size oracle fixtures are written by make_c2_fixture.py (cheerleader) and
make_c3_fixture.py (transformer).
"""
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from oracle import bf_oracle as O  # noqa: E402  (fixture generation is test infrastructure)


def analytical1d(ref_root):
    sys.path.insert(0, os.path.join(ref_root, "src"))
    import Analytical1D as A  # the reference's own 1D model
    rng = np.random.default_rng(1234)
    cases = []
    for nd, eps_d in ((1, 9.0), (5, 24.0), (20, 24.0)):
        spac = np.concatenate([rng.uniform(7.5e-3, 8.5e-3, nd), [0.0]])
        freqs = np.linspace(19.5e9, 20.5e9, 33)
        _, ax = A.disk_system(freqs.copy(), num_disk=nd, disk_epsilon=eps_d, spacings=spac.copy())
        cases.append((nd, eps_d, spac, freqs, np.abs(ax) ** 2))
    out = {}
    for k, (nd, eps_d, spac, freqs, b2) in enumerate(cases):
        out[f"nd_{k}"] = nd
        out[f"eps_{k}"] = eps_d
        out[f"spacings_{k}"] = spac
        out[f"freqs_{k}"] = freqs
        out[f"beta2_{k}"] = b2
    out["ncases"] = len(cases)
    np.savez(os.path.join(HERE, "analytical1d.npz"), **out)


def main():
    ref_root = sys.argv[1] if len(sys.argv) > 1 else None
    if not ref_root:
        sys.exit("usage: python tests/golden/make_golden.py /path/to/BoostFractor.jl")
    analytical1d(ref_root)


if __name__ == "__main__":
    main()
