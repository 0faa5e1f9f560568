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

end # module
