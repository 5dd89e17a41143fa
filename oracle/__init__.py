"""CPU oracle for the boost-factor solvers.

TEST INFRASTRUCTURE ONLY.  This package is a plain FP64 numpy/scipy
restatement of the reference BoostFractor.jl algorithms (geometry,
propagators, recursive Fourier propagation, transformer mode matching).
It exists to check the CUDA product path and to time a CPU baseline.
Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import it.  The product (``boostfractor.jl_gb300``) never
imports, links or executes anything in this directory.

Parity pinning: every golden vector of the reference test suite
(test/runtests.jl:47, 52, 168, 171, 211, 214, 217, 221) is reproduced by
``tests/test_oracle_goldens.py`` at the reference's own tolerance
(isapprox default rtol = sqrt(eps(Float64))).
"""
