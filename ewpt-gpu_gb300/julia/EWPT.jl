# EWPT.jl -- Julia ccall binding of libewpt (include/ewpt.h).
#
# Keeps the reference driver's surface: `Params(ARGS)` reads the same 12
# positional arguments as gpu-kernels-rk4/parameters.jl:14-55, the 36 state
# arrays are CuArray{Float64,3} in the reference's order, and `rk4_step!`
# below is a drop-in for the reference kernel launch
#     @cuda threads=thrds blocks=blks rk4_step!(fields..., k..., momenta..., kt..., gw,...,γ)
# (gpu-kernels-rk4/main_rk4.jl:52-661, launched at :6155/:6226/:6298/:6370).
#
# Julia is not installed where this library is built and tested, so this
# file is exercised only through the same C ABI from Python (tests/).
module EWPT

const libewpt = joinpath(@__DIR__, "..", "build", "libewpt.so")

struct Params
    nx::Int32; ny::Int32; nz::Int32; precision::Int32
    dx::Float64; dt::Float64
    gw::Float64; gy::Float64; gp2::Float64
    lambda::Float64; vev::Float64; theta_w::Float64
    beta_w::Float64; beta_y::Float64; gamma_inp::Float64
    mH::Float64; t_sat::Float64
    thermal_init::Int32; device::Int32
    stencil_order::Int32   # 6, or 2/8/10/12: the diff_scheme.jl module `using`d by main_rk4.jl:33-35
end

const FP64 = Int32(0)
const FP32 = Int32(1)
const DF64 = Int32(2)

"""Params from the reference's 12 positional ARGS (parameters.jl:14-55)."""
function Params(args::Vector{String}; precision=FP64, thermal_init=false, device=0, stencil_order=6)
    N = parse(Int32, args[6])
    dx = parse(Float64, args[4])
    dt = dx / parse(Float64, args[5])
    gw = 0.65
    θ = asin(sqrt(0.22))
    lambda = 0.129
    vev = 1.0
    Params(N, N, N, precision, dx, dt, gw, gw * tan(θ), parse(Float64, args[7]), lambda, vev, θ,
           parse(Float64, args[11]), parse(Float64, args[10]), parse(Float64, args[1]),
           2.0 * sqrt(lambda) * vev, 2.0, Int32(thermal_init), Int32(device), Int32(stencil_order))
end

check(rc, ctx=C_NULL) = rc == 0 ? nothing :
    error("libewpt error $rc: " * unsafe_string(ccall((:ewpt_last_error, libewpt), Cstring, (Ptr{Cvoid},), ctx)))

mutable struct Lattice
    h::Ptr{Cvoid}
    p::Params
end

function Lattice(p::Params)
    r = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:ewpt_create, libewpt), Cint, (Ref{Params}, Ref{Ptr{Cvoid}}), p, r))
    L = Lattice(r[], p)
    finalizer(L) do x
        ccall((:ewpt_destroy, libewpt), Cint, (Ptr{Cvoid},), x.h)
    end
    L
end

"""Upload the 36 arrays (Julia Arrays on the host, or device pointers with on_device=1)."""
function set_state!(L::Lattice, arrays::Vector{<:AbstractArray{Float64,3}})
    ptrs = [pointer(a) for a in arrays]
    GC.@preserve arrays check(ccall((:ewpt_set_state, libewpt), Cint, (Ptr{Cvoid}, Ptr{Ptr{Float64}}, Int32),
                                    L.h, ptrs, 0), L.h)
end

function get_state!(arrays::Vector{<:AbstractArray{Float64,3}}, L::Lattice)
    ptrs = [pointer(a) for a in arrays]
    GC.@preserve arrays check(ccall((:ewpt_get_state, libewpt), Cint, (Ptr{Cvoid}, Ptr{Ptr{Float64}}, Int32),
                                    L.h, ptrs, 0), L.h)
end

"""nsteps RK4 steps with the J_ext/damp schedule of main_rk4.jl:5154-5172."""
step!(L::Lattice, nsteps::Integer=1) = check(ccall((:ewpt_step, libewpt), Cint, (Ptr{Cvoid}, Int32), L.h, nsteps), L.h)

"""Host state in, nsteps RK4 steps, host state out (ewpt_step_host): `y_in` and
`y_out` are nx x ny x nz x 36 Float64 arrays (may be the same array).  With
page-locked arrays (registered with cudaHostRegister, e.g. through
`CUDA.Mem.register`) an FP64 lattice overlaps the copies with the stencil
work; the result is that of set_state! + step! + get_state! in any case."""
function step_host!(y_out::Array{Float64,4}, L::Lattice, y_in::Array{Float64,4}, nsteps::Integer=1)
    n = 36 * Int(L.p.nx) * Int(L.p.ny) * Int(L.p.nz)
    length(y_in) == n && length(y_out) == n || error("y_in and y_out must hold 36 nx ny nz values")
    GC.@preserve y_in y_out check(ccall((:ewpt_step_host, libewpt), Cint,
                                        (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Int32), L.h, y_in, y_out, nsteps), L.h)
    y_out
end

"""The 20-column snapshot row (13 reference columns + total + Gauss columns)."""
function diagnostics(L::Lattice)
    out = zeros(Float64, 20)
    check(ccall((:ewpt_diagnostics, libewpt), Cint, (Ptr{Cvoid}, Ptr{Float64}), L.h, out), L.h)
    out
end

"""B (field=0), B_2 (1) or Higgs (2) spectrum in nbins log shells (mode=0) or
convolve_1d's unique-|n| bins (mode=1)."""
function spectrum(L::Lattice; field=0, mode=0, nbins=40)
    k = zeros(nbins); s = zeros(nbins); c = zeros(nbins); m = zeros(nbins); n = Ref{Int32}(0)
    check(ccall((:ewpt_spectrum, libewpt), Cint,
                (Ptr{Cvoid}, Int32, Int32, Int32, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ref{Int32}),
                L.h, field, mode, nbins, k, s, c, m, n), L.h)
    (k=k[1:n[]], sum=s[1:n[]], count=c[1:n[]], mean=m[1:n[]])
end

"""Thermal initial condition on the device (ewpt_init_thermal): Bose-Einstein
modes at temperature T with Higgs mass mH and W mass mW (defaults sqrt(2 lambda) vev
and g vev / 2), Gamma/Sigma the divergence of W/Y, momenta zero; `seed` fixes the state."""
function init_thermal!(L::Lattice, T; seed::Integer=0, mH=sqrt(2 * L.p.lambda) * L.p.vev, mW=L.p.gw * L.p.vev / 2)
    check(ccall((:ewpt_init_thermal, libewpt), Cint, (Ptr{Cvoid}, Float64, Float64, Float64, UInt64),
                L.h, T, mH, mW, UInt64(seed)), L.h)
end

"""Per-site fields as Julia arrays (nx, ny, nz, ncomp): field 0 = B_x,B_y,B_z
(the E_t of compute_Bx/By/Bz!), 1 = B_2, 2 = phi_1..phi_4, 3 = the energy
densities PE, KE, GE, EEW, MEW, EEY, MEY (compute_PE! .. compute_MEY!).
`fields(L; field=0)[:, :, :, 1]` is the reference's B_x E_t, so
`fft(fields(L)[:, :, :, 1])` is its B_x_fft (main_rk4.jl:6579-6580)."""
function fields(L::Lattice; field=0)
    n = ccall((:ewpt_field_components, libewpt), Int32, (Int32,), field)
    n > 0 || error("unknown field $field")
    out = zeros(Float64, L.p.nx, L.p.ny, L.p.nz, n)
    check(ccall((:ewpt_fields, libewpt), Cint, (Ptr{Cvoid}, Int32, Ptr{Float64}, Int32), L.h, field, out, 0), L.h)
    out
end

"""Drop-in for `@cuda rk4_step!(...)`: `inputs` = 20 fields then 16 momenta,
`outputs` = 20 k then 16 kt, all CuArray{Float64,3} device pointers (pass
`pointer.(arrays)` of CuArrays as UInt64 / Ptr{Float64})."""
function rk4_step!(p::Params, inputs::Vector{Ptr{Float64}}, outputs::Vector{Ptr{Float64}}, Jex, γ;
                   stream::Ptr{Cvoid}=C_NULL)
    @assert length(inputs) == 36 && length(outputs) == 36
    check(ccall((:ewpt_rk4_rates, libewpt), Cint,
                (Ref{Params}, Ptr{Ptr{Float64}}, Ptr{Ptr{Float64}}, Float64, Float64, Ptr{Cvoid}),
                p, inputs, outputs, Jex, γ, stream))
end

"""Launch shape of the stage kernels (ewpt_set_tiling): bx x by threads,
register variant `reg`, `pair` = 1 two sites per thread (FP32 form), 2 TMA tiles."""
set_tiling!(L::Lattice, bx, by; reg=0, pair=0) =
    check(ccall((:ewpt_set_tiling, libewpt), Cint, (Ptr{Cvoid}, Int32, Int32, Int32, Int32), L.h, bx, by, reg, pair), L.h)

"""FP32 form, compensated mode (ewpt_set_fp32_compensated): the gauge
Laplacians and Gauss-auxiliary gradients as float pairs; needs a tiling with
pair = 1, e.g. `set_tiling!(L, 64, 2; reg=2, pair=1)`."""
set_fp32_compensated!(L::Lattice, on::Bool=true) =
    check(ccall((:ewpt_set_fp32_compensated, libewpt), Cint, (Ptr{Cvoid}, Int32), L.h, on ? 1 : 0), L.h)

"""Bubble IC on the device (ewpt_init_bubbles; replaces the per-bubble
`initializer!` launches, main_rk4.jl:4930-4946, :5691-5697).  `bubbles` is
7 x nb: centre (1-based site indices for profile 0, physical units for
profile 1), then the direction d1..d4; profile 0 = the reference's rmag
profile, 1 = tanh with radius p0 and wall width p1."""
function init_bubbles!(L::Lattice, bubbles::Matrix{Float64}; profile=0, p0=0.0, p1=0.0)
    size(bubbles, 1) == 7 || error("bubbles must be 7 x nb")
    check(ccall((:ewpt_init_bubbles, libewpt), Cint, (Ptr{Cvoid}, Int32, Ptr{Float64}, Int32, Float64, Float64),
                L.h, size(bubbles, 2), bubbles, profile, p0, p1), L.h)
end

"""The 44 deviate arrays of run()'s thermal branch (main_rk4.jl:5348-5636),
drawn exactly as run() draws them: `Random.seed!(seed_value * iter);
rand(Normal(0.0, sqrt(2.0)), (Nx, Ny, Nz))` with iter = 5, 6, ... for W^1,
W^2, W^3 and Y (r_1, r_2, r_3, r_1_i, r_2_i, r_3_i, x_1 .. x_4 each), then
phi_1_k .. phi_4_k with seeds seed_value * 1 .. 4.  `normal` is the
sampler, e.g. `(dims) -> rand(Normal(0.0, sqrt(2.0)), dims)` from
Distributions (the reference's own dependency).  Returns an
(Nx, Ny, Nz, 44) array, the layout init_thermal_deviates! takes."""
function reference_deviates(p::Params, seed_value::Integer, normal, seed!)
    Nx, Ny, Nz = Int(p.nx), Int(p.ny), Int(p.nz)
    d = Array{Float64}(undef, Nx, Ny, Nz, 44)
    iter = 5
    for q in 1:40
        seed!(seed_value * iter)
        d[:, :, :, q] = normal((Nx, Ny, Nz))
        iter += 1
    end
    for a in 1:4
        seed!(seed_value * a)
        d[:, :, :, 40 + a] = normal((Nx, Ny, Nz))
    end
    d
end

"""The reference's thermal IC from given deviates (ewpt_init_thermal_deviates):
thermal_initializer_gauge!/phi! + bfft (main_rk4.jl:5029-5152) on the device.
The reference's own conventions are the defaults: mH^2 = meff_sq
(parameters.jl:37), massless gauge modes, 1-based mode indices."""
function init_thermal_deviates!(L::Lattice, T, deviates::Array{Float64,4}; mH=sqrt(8119.43 / 174.0^2), mW=0.0,
                                one_based=true)
    size(deviates) == (L.p.nx, L.p.ny, L.p.nz, 44) || error("deviates must be (nx, ny, nz, 44)")
    check(ccall((:ewpt_init_thermal_deviates, libewpt), Cint,
                (Ptr{Cvoid}, Float64, Float64, Float64, Ptr{Float64}, Int32, Int32),
                L.h, T, mH, mW, deviates, 0, one_based ? 1 : 0), L.h)
end

"""Thermal IC with Gauss-projected thermal momenta (ewpt_init_thermal_gauss)."""
function init_thermal_gauss!(L::Lattice, T; seed::Integer=0, gauss_iters=20, mH=sqrt(2 * L.p.lambda) * L.p.vev,
                             mW=L.p.gw * L.p.vev / 2)
    check(ccall((:ewpt_init_thermal_gauss, libewpt), Cint, (Ptr{Cvoid}, Float64, Float64, Float64, UInt64, Int32),
                L.h, T, mH, mW, UInt64(seed), gauss_iters), L.h)
end

"""Project the state's electric fields onto the Gauss law (ewpt_gauss_project)."""
gauss_project!(L::Lattice; iters=20) =
    check(ccall((:ewpt_gauss_project, libewpt), Cint, (Ptr{Cvoid}, Int32), L.h, iters), L.h)

"""A lattice cut into z-slabs (ewpt_slabs_create): the decomposition of
main_rk4_multiple.jl (update_halo!, boundary_x/y/z, :69-212) in one process,
slab m on devices[m]; `nz_local` planes per slab (default an even split)."""
mutable struct Slabs
    h::Ptr{Cvoid}
    p::Params
end
function Slabs(p::Params, n::Integer; nz_local=nothing, devices=nothing)
    r = Ref{Ptr{Cvoid}}(C_NULL)
    nzl = nz_local === nothing ? C_NULL : Int32.(nz_local)
    dev = devices === nothing ? C_NULL : Int32.(devices)
    rc = ccall((:ewpt_slabs_create, libewpt), Cint, (Ref{Params}, Int32, Ptr{Int32}, Ptr{Int32}, Ref{Ptr{Cvoid}}),
               p, n, nzl, dev, r)
    check(rc)
    s = Slabs(r[], p)
    finalizer(x -> ccall((:ewpt_slabs_destroy, libewpt), Cint, (Ptr{Cvoid},), x.h), s)
    s
end
slabs_check(rc, s::Slabs) = rc == 0 ? nothing :
    error("libewpt error $rc: " * unsafe_string(ccall((:ewpt_slabs_last_error, libewpt), Cstring, (Ptr{Cvoid},), s.h)))
"""Whole-lattice state, packed (nx, ny, nz, 36) on the host."""
set_state!(s::Slabs, y::Array{Float64,4}) =
    slabs_check(ccall((:ewpt_slabs_set_state, libewpt), Cint, (Ptr{Cvoid}, Ptr{Float64}, Int32), s.h, y, 0), s)
function get_state(s::Slabs)
    y = Array{Float64}(undef, s.p.nx, s.p.ny, s.p.nz, 36)
    slabs_check(ccall((:ewpt_slabs_get_state, libewpt), Cint, (Ptr{Cvoid}, Ptr{Float64}, Int32), s.h, y, 0), s)
    y
end
step!(s::Slabs, nsteps::Integer=1) =
    slabs_check(ccall((:ewpt_slabs_step, libewpt), Cint, (Ptr{Cvoid}, Int32), s.h, nsteps), s)

"""A batched ensemble of FP32-form members (ewpt_ensemble_create): `members`
is a vector of Params, one per realization."""
mutable struct Ensemble
    h::Ptr{Cvoid}
    members::Vector{Params}
end
function Ensemble(members::Vector{Params})
    r = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:ewpt_ensemble_create, libewpt), Cint, (Int32, Ptr{Params}, Ref{Ptr{Cvoid}}),
                length(members), members, r))
    e = Ensemble(r[], members)
    finalizer(x -> ccall((:ewpt_ensemble_destroy, libewpt), Cint, (Ptr{Cvoid},), x.h), e)
    e
end
ens_check(rc, e::Ensemble) = rc == 0 ? nothing :
    error("libewpt error $rc: " * unsafe_string(ccall((:ewpt_ensemble_last_error, libewpt), Cstring,
                                                      (Ptr{Cvoid},), e.h)))
"""Member m (0-based) from a packed (nx, ny, nz, 36) host state."""
set_state!(e::Ensemble, m::Integer, y::Array{Float64,4}) =
    ens_check(ccall((:ewpt_ensemble_set_state, libewpt), Cint, (Ptr{Cvoid}, Int32, Ptr{Float64}, Int32),
                    e.h, m, y, 0), e)
step!(e::Ensemble, nsteps::Integer=1) =
    ens_check(ccall((:ewpt_ensemble_step, libewpt), Cint, (Ptr{Cvoid}, Int32), e.h, nsteps), e)
"""Launch shape of ensemble member m (0-based; ewpt_ensemble_set_member_tiling)."""
set_member_tiling!(e::Ensemble, m::Integer, bx, by; reg=2, pair=1) =
    ens_check(ccall((:ewpt_ensemble_set_member_tiling, libewpt), Cint,
                    (Ptr{Cvoid}, Int32, Int32, Int32, Int32, Int32), e.h, m, bx, by, reg, pair), e)
function diagnostics(e::Ensemble, m::Integer)
    out = zeros(Float64, 20)
    ens_check(ccall((:ewpt_ensemble_diagnostics, libewpt), Cint, (Ptr{Cvoid}, Int32, Ptr{Float64}), e.h, m, out), e)
    out
end

end # module
