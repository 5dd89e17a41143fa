"""Golden vectors of the reference test suite (test/runtests.jl), as numbers.

These values are the reference's own known answers, read from
test/runtests.jl (line numbers given per entry).  They pin the CPU oracle;
the CUDA path is in turn checked against the oracle.
"""

# test/runtests.jl:47 -- gauss_profile(coords; z=1e-9, omega0=0.097, f=22e9)[4000]
GAUSS_4000 = 0.0954822450586725 - 4.408488908455253e-8j

# test/runtests.jl:52 -- unnormalized_match(g, 3g; dx, dy)
MATCH = 0.04433886791643955 - 5.80356296618764e-26j

# test/runtests.jl:168 -- modes2field(field2modes(nothing, ...))[5000]
MODES_FIELD_5000 = 0.03647557026951998 + 0.0j

# test/runtests.jl:171 -- calc_propagation_matrices(sbdry, coords, modes)[1][4,6]
PROPMAT_1_4_6 = 0.00021462613718063045 + 0.0j

# test/runtests.jl:211 -- cheerleader beta^2, Deps = 0:1:3pi
CHEERLEADER_BETA2 = [0.9541048836881387, 4.182537182036321, 18.70293960502623,
                     7.465918522414759, 10.764938064402624, 15.415614620919474,
                     1.2667394643264536, 1.9715312870420645, 27.119751483329694,
                     8.413847982210477]

# test/runtests.jl:214 -- dancer beta^2 (propagator1D on the 101x101 grid)
DANCER_BETA2 = [1.003029819130254, 5.497534861256151, 19.03228878235599,
                7.817723902385752, 12.610984927623164, 14.178962970482115,
                1.1434594478152733, 2.4841683203606983, 31.00826150988098,
                8.548916138820806]

# test/runtests.jl:217 -- transformer beta^2 = sum|boost|^2 (3D, Mmax=10, Lmax=0)
TRANSFORMER_BETA2 = [0.9219455134201273, 4.04056703852798, 18.28704972375292,
                     7.259610230310012, 10.454105269234187, 15.156155900849086,
                     1.2340396895028822, 1.8976994867509556, 26.47829858914631,
                     8.193191222497973]

# test/runtests.jl:221 -- transformer_trace_back full fields (regions x (R, L))
TRACE_BACK = [[1.4252452348787488 - 0.8148175624088544j, 1.42524523487875 - 0.8148175624088595j],
              [-0.7032500773811425 - 1.7882104943840833j, -2.135917787152056 + 3.420965357690683j],
              [1.0999399554091236 - 0.43257371611752315j, 2.199879910818247 - 0.8651474322350463j],
              [0.0 + 0.0j, 3.299819866227371 - 1.2977211483525695j]]

# test/runtests.jl:49-50 -- Julia isapprox default tolerance for Float64
RTOL = 1.4901161193847656e-08
