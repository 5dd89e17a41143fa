# BoostFractorGB300: the GB300 solvers behind BoostFractor.jl's public API.
#
# Thin ccall wrappers over libbfgb300.so (include/boostfractor_gb300.h).  The
# methods take the reference's own types (SetupBoundaries, CoordinateSystem,
# Modes) and keyword arguments, so a caller switches by replacing
# `BoostFractor.cheerleader(...)` with `BoostFractorGB300.cheerleader(...)`.
# Arrays are passed as they are: Julia's column-major ComplexF64 layout is the
# ABI's layout.
module BoostFractorGB300

using BoostFractor: SetupBoundaries, CoordinateSystem, Modes,
                    propagator, propagatorNoTilts, propagatorMomentumSpace, propagator1D
using LinearAlgebra: SingularException

const lib = get(ENV, "BFGB300_LIB", joinpath(@__DIR__, "..", "lib", "libbfgb300.so"))

const BF_PROP = Dict(propagator => 0, propagatorNoTilts => 1, propagatorMomentumSpace => 2,
                     propagator1D => 3)
const BF_PREC = Dict(:fp64 => 0, :mixed => 1, :tf32 => 2, :mixed_simt => 3)

mutable struct Handle
    ptr::Ptr{Cvoid}
end

function check(h::Handle, rc::Cint)
    rc == 0 && return nothing
    msg = unsafe_string(ccall((:bf_last_error, lib), Cstring, (Ptr{Cvoid},), h.ptr))
    rc == 1 && throw(ArgumentError(msg))
    rc == 6 && throw(SingularException(0))   # inv / \ of an exactly singular matrix (transformer.jl:247,346,356)
    error("libbfgb300 error $rc: $msg")
end

function Handle(device::Integer = 0; hbm_budget::Integer = 0)
    ref = Ref{Ptr{Cvoid}}(C_NULL)
    rc = ccall((:bf_create, lib), Cint, (Cint, Culonglong, Ptr{Ptr{Cvoid}}), device, hbm_budget, ref)
    rc == 0 || error("bf_create failed ($rc)")
    h = Handle(ref[])
    finalizer(x -> ccall((:bf_destroy, lib), Cint, (Ptr{Cvoid},), x.ptr), h)
    return h
end

const DEFAULT = Ref{Union{Nothing, Handle}}(nothing)
default_handle() = something(DEFAULT[], (DEFAULT[] = Handle(0)))

# resident stack (bf_stack_create)
function stack(h::Handle, bdry::SetupBoundaries, coords::CoordinateSystem, diskR)
    nd = length(bdry.distance)
    ref = Ref{Ptr{Cvoid}}(C_NULL)
    surf = any(!iszero, bdry.relative_surfaces) ? ComplexF64.(bdry.relative_surfaces) : C_NULL
    check(h, ccall((:bf_stack_create, lib), Cint,
        (Ptr{Cvoid}, Cint, Ptr{Float64}, Ptr{ComplexF64}, Ptr{ComplexF64}, Ptr{Float64}, Ptr{Float64},
         Ptr{ComplexF64}, Cint, Cint, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Float64,
         Ptr{Ptr{Cvoid}}),
        h.ptr, nd, Float64.(bdry.distance), ComplexF64.(bdry.r), ComplexF64.(bdry.eps),
        Float64.(bdry.relative_tilt_x), Float64.(bdry.relative_tilt_y), surf,
        length(coords.X), length(coords.Y), collect(Float64, coords.X), collect(Float64, coords.Y),
        collect(Float64, coords.kX), collect(Float64, coords.kY), diskR, ref))
    return ref[]
end
stack_destroy(h::Handle, s) = ccall((:bf_stack_destroy, lib), Cint, (Ptr{Cvoid}, Ptr{Cvoid}), h.ptr, s)

"""
    cheerleader(amin, nmax, bdry, coords; f=10.0e9, prop=propagator, emit=nothing,
                reflect=nothing, diskR=0.1, returnboth=false, precision=:fp64)

src/boost_fractor_recurprop.jl:226 on the GPU.  `f` may be a vector: the
frequencies are solved as one batch and the result gains a trailing frequency
dimension.
"""
function cheerleader(amin, nmax, bdry::SetupBoundaries, coords::CoordinateSystem; f=10.0e9,
                     prop=propagator, emit=nothing, reflect=nothing, diskR=0.1, returnboth=false,
                     precision=:fp64, handle=default_handle())
    freqs = Float64.(collect(f))
    nx, ny, nf = length(coords.X), length(coords.Y), length(freqs)
    right = Array{ComplexF64}(undef, nx, ny, nf)
    left = returnboth ? Array{ComplexF64}(undef, nx, ny, nf) : C_NULL
    s = stack(handle, bdry, coords, diskR)
    try
        check(handle, ccall((:bf_stack_cheerleader, lib), Cint,
            (Ptr{Cvoid}, Ptr{Cvoid}, Cint, Ptr{Float64}, Float64, Cint, Cint, Cint, Ptr{ComplexF64},
             Ptr{ComplexF64}, Cint, Float64, Cint, Ptr{ComplexF64}, Ptr{ComplexF64}, Ptr{Float64}),
            handle.ptr, s, nf, freqs, amin, nmax, BF_PROP[prop], BF_PREC[precision],
            emit === nothing ? C_NULL : ComplexF64.(emit), reflect === nothing ? C_NULL : ComplexF64.(reflect),
            returnboth, 0.0, 0, right, left, C_NULL))
    finally
        stack_destroy(handle, s)
    end
    r = f isa Number ? right[:, :, 1] : right
    returnboth || return r
    return (f isa Number ? left[:, :, 1] : left), r
end

"""
    dancer(amin, nmax, sbdry, coords; f=10.0e9, prop=propagator, emit=nothing,
           reflect=nothing, diskR=0.1, returnsum=true, immediatesum=true, precision=:fp64)

src/boost_fractor_recurprop.jl:25 on the GPU.
"""
function dancer(amin, nmax, sbdry::SetupBoundaries, coords::CoordinateSystem; f=10.0e9,
                prop=propagator, emit=nothing, reflect=nothing, diskR=0.1, returnsum=true,
                immediatesum=true, precision=:fp64, handle=default_handle())
    freqs = Float64.(collect(f))
    nx, ny, nf = length(coords.X), length(coords.Y), length(freqs)
    nslots = (returnsum || immediatesum) ? 1 : nmax + 1
    out = Array{ComplexF64}(undef, nx, ny, nslots, nf)
    s = stack(handle, sbdry, coords, diskR)
    try
        check(handle, ccall((:bf_stack_dancer, lib), Cint,
            (Ptr{Cvoid}, Ptr{Cvoid}, Cint, Ptr{Float64}, Float64, Cint, Cint, Cint, Ptr{ComplexF64},
             Ptr{ComplexF64}, Cint, Cint, Float64, Cint, Ptr{ComplexF64}, Ptr{Float64}),
            handle.ptr, s, nf, freqs, amin, nmax, BF_PROP[prop], BF_PREC[precision],
            emit === nothing ? C_NULL : ComplexF64.(emit), reflect === nothing ? C_NULL : ComplexF64.(reflect),
            returnsum, immediatesum, 0.0, 0, out, C_NULL))
    finally
        stack_destroy(handle, s)
    end
    r = nslots == 1 ? out[:, :, 1, :] : out
    return f isa Number ? selectdim(r, ndims(r), 1) |> collect : r
end

"""
    propagate!(E0, dz, diskR, eps, tilt_x, tilt_y, surface, lambda, coords; prop=propagator)

The `prop=` plug-in as one GPU call (src/boost_fractor.jl:137-227).
"""
function propagate!(E0::Matrix{ComplexF64}, dz, diskR, eps, tilt_x, tilt_y, surface, lambda,
                    coords::CoordinateSystem; prop=propagator, precision=:fp64, handle=default_handle())
    surf = surface isa AbstractArray && any(!iszero, surface) ? ComplexF64.(surface) : C_NULL
    check(handle, ccall((:bf_propagate, lib), Cint,
        (Ptr{Cvoid}, Cint, Cint, Ptr{ComplexF64}, Cint, Cint, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
         Ptr{Float64}, Float64, Float64, Float64, Float64, Float64, Float64, Ptr{ComplexF64}, Float64),
        handle.ptr, BF_PROP[prop], BF_PREC[precision], E0, size(E0, 1), size(E0, 2),
        collect(Float64, coords.X), collect(Float64, coords.Y), collect(Float64, coords.kX),
        collect(Float64, coords.kY), dz, diskR, real(eps), imag(eps), tilt_x, tilt_y, surf, lambda))
    return E0
end

"""
    transformer(bdry, coords, modes; f=10.0e9, prop=propagator, propagation_matrices=[],
                diskR=0.15, emit=nothing, reflect=nothing, precision=:fp64)

src/boost_fractor_transformer.jl:285 on the GPU (NaN permittivities of `bdry`
become 1e30 in place, like the reference).  `modes` is the reference's Modes;
its patterns are uploaded as `pattern_input`.
"""
function transformer(bdry::SetupBoundaries, coords::CoordinateSystem, modes::Modes; f=10.0e9,
                     prop=propagator, propagation_matrices=Matrix{ComplexF64}[], diskR=0.15,
                     emit=nothing, reflect=nothing, precision=:fp64, handle=default_handle())
    bdry.eps[isnan.(bdry.eps)] .= 1e30
    freqs = Float64.(collect(f))
    nf, nm = length(freqs), modes.M * (2modes.L + 1)
    mref = Ref{Ptr{Cvoid}}(C_NULL)
    check(handle, ccall((:bf_modes_create, lib), Cint,
        (Ptr{Cvoid}, Cint, Cint, Ptr{Float64}, Ptr{Float64}, Cint, Cint, Cint, Float64,
         Ptr{ComplexF64}, Ptr{ComplexF64}, Ptr{Ptr{Cvoid}}),
        handle.ptr, length(coords.X), length(coords.Y), collect(Float64, coords.X),
        collect(Float64, coords.Y), 1, modes.M, modes.L, diskR, modes.mode_patterns, modes.mode_kt, mref))
    s = stack(handle, bdry, coords, diskR)
    boost = Array{ComplexF64}(undef, nm, nf)
    refl = reflect === nothing ? C_NULL : Array{ComplexF64}(undef, nm, nf)
    pm = isempty(propagation_matrices) ? C_NULL : reduce(hcat, vec.(propagation_matrices))
    try
        check(handle, ccall((:bf_transformer, lib), Cint,
            (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Cint, Ptr{Float64}, Cint, Cint, Ptr{ComplexF64},
             Ptr{ComplexF64}, Ptr{ComplexF64}, Cint, Ptr{ComplexF64}, Ptr{ComplexF64}, Ptr{Float64}),
            handle.ptr, s, mref[], nf, freqs, BF_PROP[prop], BF_PREC[precision],
            emit === nothing ? C_NULL : ComplexF64.(emit), reflect === nothing ? C_NULL : ComplexF64.(reflect),
            pm, 0, boost, refl, C_NULL))
    finally
        stack_destroy(handle, s)
        ccall((:bf_modes_destroy, lib), Cint, (Ptr{Cvoid}, Ptr{Cvoid}), handle.ptr, mref[])
    end
    b = f isa Number ? boost[:, 1] : boost
    reflect === nothing && return b
    return b, (f isa Number ? refl[:, 1] : refl)
end

"""
    transformer_trace_back(reflected_beam, input_beam, bdry, coords, modes; inlcudes_axion=false,
                           f=10.0e9, prop=propagator, propagation_matrices=nothing, diskR=0.15,
                           emit=nothing, precision=:fp64)

src/boost_fractor_transformer.jl:372 on the GPU: the (Nregions, 2, nm) array
of per-region mode amplitudes.
"""
function transformer_trace_back(reflected_beam, input_beam, bdry::SetupBoundaries, coords::CoordinateSystem,
                                modes::Modes; inlcudes_axion=false, f=10.0e9, velocity_x=0, prop=propagator,
                                propagation_matrices=nothing, diskR=0.15, emit=nothing, precision=:fp64,
                                handle=default_handle())
    nm = modes.M * (2modes.L + 1)
    inp = ComplexF64.(collect(input_beam))
    ref = ComplexF64.(collect(reflected_beam))
    length(inp) + length(ref) == 2nm || throw(DimensionMismatch("vcat(input_beam, reflected_beam) needs 2nm elements"))
    mref = Ref{Ptr{Cvoid}}(C_NULL)
    check(handle, ccall((:bf_modes_create, lib), Cint,
        (Ptr{Cvoid}, Cint, Cint, Ptr{Float64}, Ptr{Float64}, Cint, Cint, Cint, Float64,
         Ptr{ComplexF64}, Ptr{ComplexF64}, Ptr{Ptr{Cvoid}}),
        handle.ptr, length(coords.X), length(coords.Y), collect(Float64, coords.X),
        collect(Float64, coords.Y), 1, modes.M, modes.L, diskR, modes.mode_patterns, modes.mode_kt, mref))
    s = stack(handle, bdry, coords, diskR)
    out = Array{ComplexF64}(undef, length(bdry.eps), 2, nm)
    pm = (propagation_matrices === nothing || isempty(propagation_matrices)) ? C_NULL :
         reduce(hcat, vec.(propagation_matrices))
    try
        check(handle, ccall((:bf_transformer_trace_back, lib), Cint,
            (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Cint, Ptr{Float64}, Cint, Cint, Ptr{ComplexF64},
             Ptr{ComplexF64}, Cint, Cint, Ptr{ComplexF64}, Ptr{ComplexF64}, Cint, Ptr{ComplexF64}),
            handle.ptr, s, mref[], 1, [Float64(f)], BF_PROP[prop], BF_PREC[precision], ref, inp, 0,
            inlcudes_axion, emit === nothing ? C_NULL : ComplexF64.(emit), pm, 0, out))
    finally
        stack_destroy(handle, s)
        ccall((:bf_modes_destroy, lib), Cint, (Ptr{Cvoid}, Ptr{Cvoid}), handle.ptr, mref[])
    end
    return out
end

# ---- optimiser utilities (examples/transformer_optim_utilities.jl) ----------

function modes_create(handle::Handle, coords::CoordinateSystem, modes::Modes, diskR)
    mref = Ref{Ptr{Cvoid}}(C_NULL)
    check(handle, ccall((:bf_modes_create, lib), Cint,
        (Ptr{Cvoid}, Cint, Cint, Ptr{Float64}, Ptr{Float64}, Cint, Cint, Cint, Float64,
         Ptr{ComplexF64}, Ptr{ComplexF64}, Ptr{Ptr{Cvoid}}),
        handle.ptr, length(coords.X), length(coords.Y), collect(Float64, coords.X),
        collect(Float64, coords.Y), 1, modes.M, modes.L, diskR, modes.mode_patterns, modes.mode_kt, mref))
    return mref[]
end

"""Propagation matrices over gap spacings x frequencies, resident on the GPU and
prefiltered for the spacing spline of Interpolations' BSpline(Cubic(Natural(OnCell())))."""
mutable struct PGrid
    handle::Handle
    stack::Ptr{Cvoid}
    modes::Ptr{Cvoid}
    grid::Ptr{Cvoid}
    freqs::Vector{Float64}
    nd::Int
    nm::Int
end

function release(g::PGrid)
    g.grid == C_NULL && return nothing
    ccall((:bf_pgrid_destroy, lib), Cint, (Ptr{Cvoid}, Ptr{Cvoid}), g.handle.ptr, g.grid)
    stack_destroy(g.handle, g.stack)
    ccall((:bf_modes_destroy, lib), Cint, (Ptr{Cvoid}, Ptr{Cvoid}), g.handle.ptr, g.modes)
    g.grid = C_NULL
    return nothing
end

# a copy of sbdry whose air gaps (regions 2:2:n_region) are tilted by (tx, ty) more
function tilt_gaps(sbdry::SetupBoundaries, tx, ty)
    gx = Float64.(collect(sbdry.relative_tilt_x))
    gy = Float64.(collect(sbdry.relative_tilt_y))
    gx[2:2:end] .+= tx
    gy[2:2:end] .+= ty
    return SetupBoundaries(copy(sbdry.distance), copy(sbdry.r), copy(sbdry.eps), gx, gy,
                           copy(sbdry.relative_surfaces))
end

"""
    calc_propagation_matrices_grid(sbdry, coords, modes, spacing_grid, frequencies;
                                   tilt_x_grid=0, tilt_y_grid=0, prop=propagator, diskR=0.15,
                                   precision=:fp64)

examples/transformer_optim_utilities.jl:10 on the GPU.  Returns a PGrid, which
is also the interpolation object.  With tilt grids the grid is built with the
gaps at their first tilt points, the only ones the reference's
interpolate_prop_matrix reads (itp(r, f, shift, 1, 1, ...)); the Python mirror's
PGrid.array() gives the whole 7-D array.
"""
function calc_propagation_matrices_grid(sbdry::SetupBoundaries, coords::CoordinateSystem, modes::Modes,
                                        spacing_grid::AbstractRange, frequencies; tilt_x_grid=0, tilt_y_grid=0,
                                        prop=propagator, diskR=0.15, precision=:fp64, handle=default_handle())
    freqs = Float64.(collect(frequencies))
    tx, ty = first(tilt_x_grid), first(tilt_y_grid)
    bd = (tx == 0 && ty == 0) ? sbdry : tilt_gaps(sbdry, tx, ty)
    m = modes_create(handle, coords, modes, diskR)
    s = stack(handle, bd, coords, diskR)
    ref = Ref{Ptr{Cvoid}}(C_NULL)
    rc = ccall((:bf_pgrid_create, lib), Cint,
        (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Cint, Ptr{Float64}, Cint, Float64, Float64, Cint, Cint,
         Ptr{Ptr{Cvoid}}),
        handle.ptr, s, m, length(freqs), freqs, length(spacing_grid), Float64(first(spacing_grid)),
        Float64(step(spacing_grid)), BF_PROP[prop], BF_PREC[precision], ref)
    if rc != 0
        stack_destroy(handle, s)
        ccall((:bf_modes_destroy, lib), Cint, (Ptr{Cvoid}, Ptr{Cvoid}), handle.ptr, m)
        check(handle, rc)
    end
    g = PGrid(handle, s, m, ref[], freqs, length(sbdry.distance), modes.M * (2modes.L + 1))
    finalizer(release, g)
    return g
end

"""utilities :56: the PGrid is its own interpolation object."""
construct_prop_matrix_interpolation(g::PGrid, spacing_grid=nothing) = g

"""utilities :78: Array{Matrix{ComplexF64}}(n_region, n_freq) at the shifts."""
function interpolate_prop_matrix(g::PGrid, dist_shift::AbstractVector)
    nf = length(g.freqs)
    out = Array{ComplexF64}(undef, g.nm, g.nm, g.nd, nf)
    check(g.handle, ccall((:bf_pgrid_matrices, lib), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Float64}, Ptr{ComplexF64}),
                          g.handle.ptr, g.grid, Float64.(dist_shift), out))
    return [out[:, :, r, f] for r in 1:g.nd, f in 1:nf]
end

"""
    calc_boostfactor_cost(dist_shift, itp::PGrid, frequencies, sbdry, coords, modes, m_reflect;
                          prop=propagator, diskR=0.15)

utilities :130 on the GPU: -p_norm(coupled power, -20) x soft_box_penalty, or
1000.0 outside the interpolation bounds.
"""
function calc_boostfactor_cost(dist_shift::AbstractVector, g::PGrid, frequencies, sbdry, coords, modes, m_reflect;
                               prop=propagator, diskR=0.15)
    Float64.(collect(frequencies)) == g.freqs || throw(ArgumentError("frequencies must be the grid's"))
    cost = Ref{Float64}(0.0)
    check(g.handle, ccall((:bf_pgrid_cost, lib), Cint,
        (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Float64}, Ptr{ComplexF64}, Float64, Ptr{Float64}, Ptr{Float64}),
        g.handle.ptr, g.grid, Float64.(dist_shift), ComplexF64.(collect(m_reflect)), -20.0, cost, C_NULL))
    return cost[]
end

end # module
