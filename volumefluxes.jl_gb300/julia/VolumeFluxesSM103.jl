# VolumeFluxesSM103 -- the Julia glue that lets a VolumeFluxes.jl scenario run its
# 2D shallow-water step on GB300 through libvfsm103.so (include/volumefluxes_sm103.h).
#
# A maintainer adds this module beside the reference: it imports the module
# `VolumeFluxes` (src/SinFVM.jl:21; the package is named SinFVM in Project.toml),
# defines SM103Backend <: VolumeFluxes.Backend (src/backends/kernel_abstractions.jl:24),
# and overrides perform_step!, set_current_state!, current_interior_state and
# simulate_to_time (src/simulator.jl:114-212) for simulators on that backend, each
# with one ccall into the library. Unsupported configurations throw ArgumentError,
# as the reference's constructors do; there is no CPU fallback.
#
# Every ccall below is checked against the C header by tests/test_julia_glue.py
# (symbol, argument count, argument and return types). No Julia toolchain exists
# where this repository is built and tested, so the module itself is not run
# here; the Python package volumefluxes_sm103 drives the same entry points.

module VolumeFluxesSM103

import VolumeFluxes
using VolumeFluxes: Simulator, ConservedSystem, CartesianGrid, WallBC, ShallowWaterEquations,
    LinearReconstruction, CentralUpwind, RungeKutta2, ForwardEulerStepper, SourceTermBottom,
    ConstantRain, ConstantInfiltration, ImplicitFriction, ConstantBottomTopography,
    BottomTopography2D, friction_bsa2012, friction_fcg2016, friction_bh2021, InteriorVolume,
    PeriodicBC, NeumannBC, NoReconstruction, TimeDependentRain, HortonInfiltration, FunctionalRain, cell_center

const LIB = get(ENV, "VF_SM103_LIB", joinpath(@__DIR__, "..", "volumefluxes_sm103", "lib", "libvfsm103.so"))

# arithmetic (Float64 only): :reference rounds every operation as the reference
# does (bitwise equal to its CPU path); :faithful uses faithful quotients and
# fused multiply-adds (vf_set_arithmetic), held to a tolerance instead.
struct SM103Backend{RealType} <: VolumeFluxes.Backend
    realtype::Type{RealType}
    device::Int32
    arithmetic::Symbol
end
function SM103Backend(T::Type=Float64; device=0, arithmetic::Symbol=:reference)
    arithmetic in (:reference, :faithful) || throw(ArgumentError("arithmetic must be :reference or :faithful"))
    arithmetic === :faithful && T !== Float64 && throw(ArgumentError("faithful arithmetic is a Float64 mode"))
    SM103Backend{T}(T, Int32(device), arithmetic)
end
VolumeFluxes.name(::SM103Backend) = "SM103"

# Host-side volumes keep the reference's layout; the device copy lives in the library.
VolumeFluxes.create_buffer(b::SM103Backend, nvars::Int64, dims) = zeros(b.realtype, dims..., nvars)
VolumeFluxes.convert_to_backend(::SM103Backend, a::AbstractArray) = a

# Mirror of vf_config (include/volumefluxes_sm103.h); field order and types must match.
struct VfConfig
    abi_version::Int32; nx::Int32; ny::Int32; gc::Int32
    extent::NTuple{4,Float64}
    real_bytes::Int32
    g::Float64; rho::Float64; depth_cutoff::Float64; desingularizing_kappa::Float64
    reconstruction::Int32; theta::Float64
    n_sources::Int32; source_kind::NTuple{8,Int32}; source_rate::NTuple{8,Float64}
    source_aux::NTuple{16,Float64}   # double source_aux[8][2]: (f0, k) of a HortonInfiltration entry
    friction::Int32; friction_Cz::Float64
    stepper::Int32; bc::Int32; cfl::Float64
    bottom_is_constant::Int32; bottom_constant::Float64
    device::Int32
end

mutable struct Handle
    ptr::Ptr{Cvoid}
    function Handle(ptr)
        h = new(ptr)
        finalizer(x -> ccall((:vf_destroy, LIB), Cvoid, (Ptr{Cvoid},), x.ptr), h)
    end
end

check(h, rc) = rc == 0 ? nothing :
    let msg = unsafe_string(ccall((:vf_last_error, LIB), Cstring, (Ptr{Cvoid},), h))
        rc == -1 ? throw(ArgumentError(msg)) : error("libvfsm103 [$rc]: $msg")
    end

law(f) = f === friction_bsa2012 ? 1 : f === friction_fcg2016 ? 2 : f === friction_bh2021 ? 3 :
    throw(ArgumentError("unsupported friction law"))

function config(sim::Simulator{<:SM103Backend})
    sys, g, eq = sim.system, sim.grid, sim.system.equation
    sys isa ConservedSystem || throw(ArgumentError("SM103Backend runs ConservedSystem only"))
    eq isa ShallowWaterEquations || throw(ArgumentError("SM103Backend runs ShallowWaterEquations only"))
    rec = sys.reconstruction isa LinearReconstruction ? 1 : sys.reconstruction isa NoReconstruction ? 2 :
        throw(ArgumentError("unsupported reconstruction"))
    sys.numericalflux isa CentralUpwind || throw(ArgumentError("CentralUpwind only"))
    bc = g.boundary isa WallBC ? 1 : g.boundary isa PeriodicBC ? 2 : g.boundary isa NeumannBC ? 3 :
        throw(ArgumentError("WallBC, PeriodicBC or NeumannBC only"))
    g isa CartesianGrid{2} && g.ghostcells[1] == 2 || throw(ArgumentError("needs CartesianGrid(nx, ny; gc=2)"))
    kinds = zeros(Int32, 8); rates = zeros(8); aux = zeros(16)
    for (i, s) in enumerate(sys.source_terms)
        kinds[i], rates[i] = s isa SourceTermBottom ? (1, 0.0) :
                             s isa ConstantRain ? (2, s.rain_rate) :
                             s isa ConstantInfiltration ? (3, s.infiltration_rate) :
                             s isa TimeDependentRain ? (4, 0.0) :
                             s isa HortonInfiltration ? (5, s.fc) :
                             s isa FunctionalRain ? (6, 0.0) :
                             throw(ArgumentError("unsupported source term $(typeof(s))"))
        s isa HortonInfiltration && (aux[2i-1] = s.f0; aux[2i] = s.k)
    end
    fr = sys.implicit_source_term
    fcode, cz = fr === nothing ? (0, 0.0) : fr isa ImplicitFriction ? (law(fr.friction_function), fr.Cz) :
        throw(ArgumentError("unsupported implicit source term"))
    stepper = sim.timestepper isa RungeKutta2 ? 2 : sim.timestepper isa ForwardEulerStepper ? 1 :
        throw(ArgumentError("unsupported time stepper"))
    B = eq.B
    VfConfig(2, g.totalcells[1] - 4, g.totalcells[2] - 4, 2, Tuple(g.extent), sizeof(sim.backend.realtype),
             eq.g, eq.ρ, eq.depth_cutoff, eq.desingularizing_kappa, rec,
             rec == 1 ? sys.reconstruction.theta : 0.0,
             length(sys.source_terms), Tuple(kinds), Tuple(rates), Tuple(aux), fcode, cz, stepper, bc, sim.cfl,
             B isa ConstantBottomTopography ? 1 : 0, B isa ConstantBottomTopography ? B.B : 0.0,
             sim.backend.device)
end

# One device simulation per Simulator (the reference's Simulator is immutable).
const HANDLES = IdDict{Any,Handle}()
function handle(sim::Simulator{<:SM103Backend})
    get!(HANDLES, sim) do
        cfg = Ref(config(sim)); out = Ref{Ptr{Cvoid}}(C_NULL)
        check(C_NULL, ccall((:vf_create, LIB), Cint, (Ref{VfConfig}, Ref{Ptr{Cvoid}}), cfg, out))
        h = Handle(out[])
        if sim.backend.arithmetic === :faithful
            check(h.ptr, ccall((:vf_set_arithmetic, LIB), Cint, (Ptr{Cvoid}, Int32), h.ptr, 1))
        end
        B = sim.system.equation.B
        if B isa BottomTopography2D
            Bh = convert(Array{sim.backend.realtype}, collect(B.B))
            check(h.ptr, ccall((:vf_upload_bottom, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}), h.ptr, Bh))
        end
        for (i, s) in enumerate(sim.system.source_terms)
            if s isa TimeDependentRain
                check(h.ptr, ccall((:vf_set_source_table, LIB), Cint,
                    (Ptr{Cvoid}, Int32, Ptr{Float64}, Ptr{Float64}, Int32), h.ptr, i - 1,
                    collect(Float64, s.time), collect(Float64, s.rain_rates), length(s.time)))
            elseif s isa HortonInfiltration
                f = convert(Array{sim.backend.realtype}, collect(s.factor))
                check(h.ptr, ccall((:vf_set_source_field, LIB), Cint, (Ptr{Cvoid}, Int32, Ptr{Cvoid}),
                    h.ptr, i - 1, f))
            end
        end
        h
    end
end

function VolumeFluxes.set_current_state!(sim::Simulator{<:SM103Backend}, new_state)
    T = sim.backend.realtype
    planes = [T[x[k] for x in new_state] for k in 1:3]          # (nx, ny) column-major planes
    h = handle(sim)
    check(h.ptr, ccall((:vf_set_interior_state, LIB), Cint, (Ptr{Cvoid}, Ptr{T}, Ptr{T}, Ptr{T}),
                       h.ptr, planes[1], planes[2], planes[3]))
end

function VolumeFluxes.perform_step!(sim::Simulator{<:SM103Backend}, max_dt)
    dt = Ref{Float64}(0)
    h = handle(sim)
    T = sim.backend.realtype
    for (i, s) in enumerate(sim.system.source_terms)   # FunctionalRain, re-evaluated at the step's t
        s isa FunctionalRain || continue
        f = T[s.rain_function(sim.t[1], cell_center(sim.grid, I)...) for I in CartesianIndices(size(sim.grid))]
        check(h.ptr, ccall((:vf_set_source_field, LIB), Cint, (Ptr{Cvoid}, Int32, Ptr{Cvoid}), h.ptr, i - 1, f))
    end
    check(h.ptr, ccall((:vf_step, LIB), Cint, (Ptr{Cvoid}, Float64, Float64, Ref{Float64}),
                       h.ptr, max_dt, sim.t[1], dt))
    sim.current_timestep[1] = dt[]
end

# Reads the device state into the host volume, so collect(current_interior_state(sim).h) works unchanged.
function VolumeFluxes.current_interior_state(sim::Simulator{<:SM103Backend})
    vol = VolumeFluxes.current_state(sim)
    h = handle(sim)
    check(h.ptr, ccall((:vf_download_state, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}), h.ptr, vol._data))
    InteriorVolume(vol)
end

# Gauge values without a state download, e.g. inside an IntervalWriter callback:
# gauges are 1-based interior (i, j) pairs; returns a (3, n) array of (w, hu, hv).
function sample_cells(sim::Simulator{<:SM103Backend}, gauges::AbstractVector{<:Tuple{Int,Int}})
    T = sim.backend.realtype; h = handle(sim); n = length(gauges)
    i = Int32[g[1] - 1 for g in gauges]; j = Int32[g[2] - 1 for g in gauges]
    w = Vector{T}(undef, n); hu = Vector{T}(undef, n); hv = Vector{T}(undef, n)
    check(h.ptr, ccall((:vf_sample_cells, LIB), Cint,
        (Ptr{Cvoid}, Ptr{Int32}, Ptr{Int32}, Int32, Ptr{T}, Ptr{T}, Ptr{T}), h.ptr, i, j, n, w, hu, hv))
    permutedims(hcat(w, hu, hv))
end

# Device-resident time loop when no callback needs the host every step.
function VolumeFluxes.simulate_to_time(sim::Simulator{<:SM103Backend}, endtime; match_endtime=true,
                                       callback=nothing, show_progress=true, maximum_timestep=nothing)
    functional = any(s -> s isa FunctionalRain, sim.system.source_terms)
    (callback === nothing && !functional) || return invoke(VolumeFluxes.simulate_to_time, Tuple{Simulator,Any},
        sim, endtime; match_endtime, callback, show_progress, maximum_timestep)
    h = handle(sim); t = Ref{Float64}(0); n = Ref{Int64}(0); dt = Ref{Float64}(0)
    check(h.ptr, ccall((:vf_simulate, LIB), Cint,
        (Ptr{Cvoid}, Float64, Float64, Int32, Float64, Float64, Int64, Ref{Float64}, Ref{Int64}, Ref{Float64}),
        h.ptr, sim.t[1], endtime, match_endtime, maximum_timestep === nothing ? -1.0 : maximum_timestep,
        Inf, 0, t, n, dt))
    sim.t[1] = t[]; n[] > 0 && (sim.current_timestep[1] = dt[])
    nothing
end

# Many independent simulators at once: `simulate_to_time` for each, on the device.
function simulate_batch!(sims::AbstractVector{<:Simulator{<:SM103Backend}}, endtimes::AbstractVector{Float64})
    hs = [handle(s).ptr for s in sims]
    t0 = [s.t[1] for s in sims]
    n = length(sims); t = zeros(n); steps = zeros(Int64, n); dt = zeros(n); status = zeros(Int32, n)
    rc = ccall((:vf_batch_simulate, LIB), Cint,
        (Ptr{Ptr{Cvoid}}, Int32, Ptr{Float64}, Ptr{Float64}, Int32, Float64, Int64, Ptr{Cvoid},
         Ptr{Float64}, Ptr{Int64}, Ptr{Float64}, Ptr{Int32}),
        hs, n, t0, endtimes, 1, -1.0, 0, C_NULL, t, steps, dt, status)
    rc == 0 || error(unsafe_string(ccall((:vf_batch_last_error, LIB), Cstring, (Ptr{Cvoid},), C_NULL)))
    for (k, s) in enumerate(sims)
        s.t[1] = t[k]; steps[k] > 0 && (s.current_timestep[1] = dt[k])
    end
    status
end

# Reverse-mode gradient of the gauge loss w.r.t. the bottom corners and Manning's n,
# behind ChainRulesCore so Zygote-based optimisation loops pick it up.
using ChainRulesCore
function gauge_loss(sim_factory, B::Matrix{Float64}, n::Float64, gauges, target, dts)
    sim = sim_factory(B, n)                       # builds the SM103Backend simulator
    h = handle(sim)
    a = Ref{Ptr{Cvoid}}(C_NULL)
    check(h.ptr, ccall((:vf_adjoint_create, LIB), Cint, (Ptr{Cvoid}, Int32, Int32, Ref{Ptr{Cvoid}}),
                       h.ptr, length(dts), 0, a))
    adjoint_check(rc) = rc == 0 ? nothing :
        let msg = unsafe_string(ccall((:vf_adjoint_last_error, LIB), Cstring, (Ptr{Cvoid},), a[]))
            ccall((:vf_adjoint_destroy, LIB), Cvoid, (Ptr{Cvoid},), a[])
            rc == -1 ? throw(ArgumentError(msg)) : error("libvfsm103 adjoint [$rc]: $msg")
        end
    adjoint_check(ccall((:vf_adjoint_forward, LIB), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}),
                        a[], collect(Float64, dts), C_NULL))
    gi = Int32[g[1] - 1 for g in gauges]; gj = Int32[g[2] - 1 for g in gauges]
    loss = Ref{Float64}(0); gB = similar(B); gCz = Ref{Float64}(0)
    adjoint_check(ccall((:vf_adjoint_backward, LIB), Cint,
                        (Ptr{Cvoid}, Ptr{Int32}, Ptr{Int32}, Ptr{Float64}, Int32, Ref{Float64}, Ptr{Float64},
                         Ref{Float64}),
                        a[], gi, gj, collect(Float64, target), length(gi), loss, gB, gCz))
    ccall((:vf_adjoint_destroy, LIB), Cvoid, (Ptr{Cvoid},), a[])
    loss[], gB, 2n * gCz[]
end
function ChainRulesCore.rrule(::typeof(gauge_loss), f, B, n, gauges, target, dts)
    L, gB, gn = gauge_loss(f, B, n, gauges, target, dts)
    pullback(dL) = (NoTangent(), NoTangent(), dL .* gB, dL * gn, NoTangent(), NoTangent(), NoTangent())
    L, pullback
end

# Serving: a request loop over whole simulations (vf_server_*). The engine
# thread admits requests within an HBM budget and batches them; the caller
# submits and polls. Arrays keep the reference's layout (interior planes
# (nx, ny), corners (nx+2gc+1, ny+2gc+1)) and must stay alive until the
# request is reported done.
mutable struct Server
    ptr::Ptr{Cvoid}
end
server_check(s, rc) = rc == 0 ? nothing :
    let msg = unsafe_string(ccall((:vf_server_last_error, LIB), Cstring, (Ptr{Cvoid},), s))
        rc == -1 ? throw(ArgumentError(msg)) : error("libvfsm103 server [$rc]: $msg")
    end
function Server(; device=0, hbm_budget_bytes::Int64=Int64(120) * 2^30, max_steps::Int64=Int64(0))
    out = Ref{Ptr{Cvoid}}(C_NULL)
    server_check(C_NULL, ccall((:vf_server_create, LIB), Cint, (Int32, Int64, Ptr{Cvoid}, Int64, Ref{Ptr{Cvoid}}),
                               device, hbm_budget_bytes, C_NULL, max_steps, out))
    srv = Server(out[])
    finalizer(x -> ccall((:vf_server_destroy, LIB), Cint, (Ptr{Cvoid},), x.ptr), srv)
end
function submit!(srv::Server, sim::Simulator{<:SM103Backend}, w, hu, hv, endtime, out_w, out_hu, out_hv)
    cfg = Ref(config(sim)); ticket = Ref{Int64}(0)
    B = sim.system.equation.B
    Bh = B isa BottomTopography2D ? convert(Array{sim.backend.realtype}, collect(B.B)) : C_NULL
    server_check(srv.ptr, ccall((:vf_server_submit, LIB), Cint,
        (Ptr{Cvoid}, Ref{VfConfig}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Float64, Float64,
         Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ref{Int64}),
        srv.ptr, cfg, Bh, w, hu, hv, sim.t[1], endtime, out_w, out_hu, out_hv, ticket))
    ticket[]
end
function poll(srv::Server; capacity::Int=64)
    done = zeros(Int64, capacity); nd = Ref{Int32}(0)
    server_check(srv.ptr, ccall((:vf_server_poll, LIB), Cint, (Ptr{Cvoid}, Ptr{Int64}, Int32, Ref{Int32}),
                                srv.ptr, done, capacity, nd))
    done[1:nd[]]
end
function result(srv::Server, ticket::Int64)
    t = Ref{Float64}(0); steps = Ref{Int64}(0); dt = Ref{Float64}(0); status = Ref{Int32}(0)
    server_check(srv.ptr, ccall((:vf_server_result, LIB), Cint,
        (Ptr{Cvoid}, Int64, Ref{Float64}, Ref{Int64}, Ref{Float64}, Ref{Int32}), srv.ptr, ticket, t, steps, dt, status))
    server_check(srv.ptr, ccall((:vf_server_release, LIB), Cint, (Ptr{Cvoid}, Int64), srv.ptr, ticket))
    (t = t[], steps = steps[], last_dt = dt[], status = status[])
end

export SM103Backend, simulate_batch!, gauge_loss, Server, submit!, poll, result
end # module
