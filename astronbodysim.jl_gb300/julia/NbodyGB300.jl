"""
    NbodyGB300

Drop-in for AstroNbodySim.jl's DirectSum solver on the GPU device: the
`(DirectSum, GPU)` and `(Gravity, GPU)` methods of `src/directsumgpu/` are
re-defined to call libnbody_gb300.so through `ccall`.  The Julia host strips
units into structure-of-arrays buffers; the library keeps the particle state
resident on the GB300 and returns it on `get_all_data`.

Load after AstroNbodySim:

    using AstroNbodySim, NbodyGB300
    sim = Simulation(data; device = GPU(), GPU_Algorithm = Tiled(), ...)
    run(sim)

Only simulations whose `GPU_Algorithm` is `Tiled()` (declared but unimplemented
in the reference, `src/base/Traits.jl:32`) are routed here; `AllPairs()` keeps
the reference's CUDA.jl kernels.
"""
module NbodyGB300

using AstroNbodySim
using AstroNbodySim: Simulation, DirectSum, Gravity, GPU, Tiled, AdaptiveTimestep, ConstantTimestep
using StructArrays
using Unitful

const libnb = get(ENV, "NBODY_GB300_LIB",
                  joinpath(@__DIR__, "..", "csrc", "libnbody_gb300.so"))

# Mirrors `nb_params` of include/nbody_gb300.h (field order and types).
struct NbParams
    G::Float64
    softening::NTuple{6,Float64}
    law::Int32
    precision::Int32
    adaptive::Int32
    criterion::Int32
    dt::Float64
    eta::Float64
    min_step::Float64
    max_step::Float64
    time_base::Int64
    time_begin::Float64
    time_end::Float64
    device::Int32
    tile_j::Int32
    i_per_thread::Int32
    block::Int32
    j_split::Int32
    reserved::Int32
    bg_kind::Int32
    mond::Int32
    bg_gm::Float64
    bg_center::NTuple{3,Float64}
    bg_rg::Float64
    mond_acc0::Float64
    mond_nu_index::Float64
end

struct NbDiag
    kinetic::Float64
    potential::Float64
    momentum::NTuple{3,Float64}
    angular_momentum::NTuple{3,Float64}
end

mutable struct Handle
    ptr::Ptr{Cvoid}
    n::Int
end

const HANDLES = IdDict{Any,Handle}()

function check(h::Handle, rc::Integer)
    rc == 0 && return nothing
    msg = unsafe_string(ccall((:nb_last_error, libnb), Cstring, (Ptr{Cvoid},), h.ptr))
    error("libnbody_gb300 error $rc: $msg")
end

routed(sim) = sim.config.device.GPU_Algorithm isa Tiled

# unit stripping, in the simulation's unit system
lenunit(sim) = isnothing(sim.config.units) ? nothing : sim.config.units[1]
timeunit(sim) = isnothing(sim.config.units) ? nothing : sim.config.units[2]
strip(u, x) = isnothing(u) ? Float64(x) : Float64(ustrip(u, x))
stripG(sim) = Float64(ustrip(sim.config.constants.G))

accunit(sim) = isnothing(sim.config.units) ? nothing : sim.config.units[1] / sim.config.units[2]^2
mond_of(sim) = Int32(sim.config.grav.model isa AstroNbodySim.MOND1983Milgrom ? 1 : 0)

# Background-force closures (sim.bgforce) cannot cross the C ABI: analytic fields
# are selected through bg_kind / bg_gm / bg_center / bg_rg of NbParams instead.
function params(sim; precision = Int32(1), law = Int32(0))
    tc = sim.config.time
    step = tc.step
    soft = ntuple(k -> strip(lenunit(sim), sim.config.grav.ForceSofteningTable[k]), 6)
    tu = timeunit(sim)
    adaptive = step isa AdaptiveTimestep
    NbParams(stripG(sim), soft, law, precision, Int32(adaptive), Int32(0),
             adaptive ? 0.0 : strip(tu, step.dt),
             adaptive ? Float64(step.ErrTolTimestep) : 0.025,
             adaptive ? strip(tu, step.MinStep) : 1.0e-8,
             adaptive ? strip(tu, step.MaxStep) : Inf,
             adaptive ? Int64(step.TimeBase) : Int64(1) << 30,
             strip(tu, tc.Begin), strip(tu, tc.End), Int32(0), Int32(0), Int32(0), Int32(0),
             Int32(0), Int32(0),
             Int32(0), mond_of(sim), 0.0, (0.0, 0.0, 0.0), 0.0,
             mond_of(sim) == 0 ? 0.0 : strip(accunit(sim), sim.config.constants.ACC0),
             Float64(sim.config.grav.MOND_nuIndex))
end

"""Create the library handle for `sim` and upload its particles (replaces the
`cu(StructArray(d))` placement of src/base/Config.jl:1072-1088)."""
function attach!(sim::Simulation)
    haskey(HANDLES, sim) && return HANDLES[sim]
    p = Ref(params(sim))
    out = Ref{Ptr{Cvoid}}(C_NULL)
    rc = ccall((:nb_create, libnb), Cint, (Ref{NbParams}, Ref{Ptr{Cvoid}}), p, out)
    rc == 0 || error("nb_create failed: $rc")
    h = Handle(out[], 0)
    finalizer(x -> ccall((:nb_destroy, libnb), Cint, (Ptr{Cvoid},), x.ptr), h)
    d = StructArray(Array(sim.simdata))
    lu, tu = lenunit(sim), timeunit(sim)
    vu = isnothing(lu) ? nothing : lu / tu
    mu = isnothing(sim.config.units) ? nothing : sim.config.units[3]
    x = [strip(lu, p.x) for p in d.Pos]; y = [strip(lu, p.y) for p in d.Pos]; z = [strip(lu, p.z) for p in d.Pos]
    vx = [strip(vu, v.x) for v in d.Vel]; vy = [strip(vu, v.y) for v in d.Vel]; vz = [strip(vu, v.z) for v in d.Vel]
    m = [strip(mu, q) for q in d.Mass]
    t = Int32[Int(c) for c in d.Collection]
    n = length(d)
    GC.@preserve x y z vx vy vz m t begin
        check(h, ccall((:nb_upload, libnb), Cint,
                       (Ptr{Cvoid}, Int64, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
                        Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Int32}),
                       h.ptr, n, x, y, z, vx, vy, vz, m, t))
    end
    h.n = n
    HANDLES[sim] = h
    return h
end

handle(sim) = attach!(sim)

# -- (DirectSum, GPU) methods -------------------------------------------------

# src/directsumgpu/gravity.jl:36-45 (the GPU_Algorithm extension point)
function AstroNbodySim.compute_force(sim::Simulation, ::Tiled)
    h = handle(sim)
    check(h, ccall((:nb_compute_force, libnb), Cint, (Ptr{Cvoid}, Cint), h.ptr, 0))
end

# src/directsumgpu/timestep.jl:40-47
function AstroNbodySim.init_timesteps(sim::Simulation, g::Gravity, d::GPU)
    routed(sim) || return invoke(AstroNbodySim.init_timesteps, Tuple{Simulation,Gravity,GPU}, sim, g, d)
    h = handle(sim)
    check(h, ccall((:nb_init_timesteps, libnb), Cint, (Ptr{Cvoid},), h.ptr))
end

# src/directsumgpu/timestep.jl:210-212
function AstroNbodySim.leapfrog_half_kick(sim::Simulation, forward::Int, ::Gravity, ::GPU)
    h = handle(sim)
    check(h, ccall((:nb_half_kick, libnb), Cint, (Ptr{Cvoid}, Cint), h.ptr, forward))
end

# src/directsumgpu/timestep.jl:172-174
function AstroNbodySim.advance_and_find_timestep(sim::Simulation, ::Gravity, ::GPU)
    h = handle(sim)
    check(h, ccall((:nb_kick, libnb), Cint, (Ptr{Cvoid},), h.ptr))
end

# src/directsumgpu/timestep.jl:103-114
function AstroNbodySim.find_min_endstep(sim::Simulation, ::Gravity, ::GPU)
    h = handle(sim)
    v = Ref{Int64}(0)
    check(h, ccall((:nb_find_min_endstep, libnb), Cint, (Ptr{Cvoid}, Ref{Int64}), h.ptr, v))
    sim.timeinfo.min_endstep = v[]
    return v[]
end

# src/directsumgpu/timestep.jl:116-118 (check_sync_point_local on the device data)
function AstroNbodySim.check_sync_point(sim::Simulation, ::Gravity, ::GPU)
    h = handle(sim)
    v = Ref{Int32}(0)
    check(h, ccall((:nb_check_sync_point, libnb), Cint, (Ptr{Cvoid}, Ref{Int32}), h.ptr, v))
    return sim.outputinfo.syncflag = v[] != 0
end

# src/directsumgpu/timestep.jl:76-91: the host keeps TimeInfo, the device follows
function AstroNbodySim.drift_particles_kernel(sim::Simulation, ::AdaptiveTimestep, ::Gravity, ::GPU)
    h = handle(sim)
    check(h, ccall((:nb_drift_to_int, libnb), Cint, (Ptr{Cvoid}, Int64), h.ptr, sim.timeinfo.system_time_int))
end
function AstroNbodySim.drift_particles_kernel(sim::Simulation, ::ConstantTimestep, ::Gravity, ::GPU)
    h = handle(sim)
    t = strip(timeunit(sim), sim.timeinfo.system_time_float)
    check(h, ccall((:nb_drift_to_float, libnb), Cint, (Ptr{Cvoid}, Float64), h.ptr, t))
end

# New GPU method: src/directsum/potential.jl:142-148 has only a CPU version
function AstroNbodySim.compute_potential(sim::Simulation, ::DirectSum, ::GPU)
    h = handle(sim)
    check(h, ccall((:nb_compute_potential, libnb), Cint, (Ptr{Cvoid},), h.ptr))
end

function diag(sim, with_pot)
    h = handle(sim)
    r = Ref{NbDiag}()
    check(h, ccall((:nb_diagnostics, libnb), Cint, (Ptr{Cvoid}, Cint, Ref{NbDiag}), h.ptr, with_pot, r))
    return r[]
end

# src/directsum/potential.jl:150-153 and src/base/Energy.jl (GPU versions)
AstroNbodySim.total_potential(sim::Simulation, ::DirectSum, ::GPU) = diag(sim, 1).potential

# src/restart.jl:14-19: the (DirectSum, GPU) restart file holds the device image
function AstroNbodySim.saverestart(sim::Simulation, ::DirectSum, ::GPU)
    routed(sim) || return invoke(AstroNbodySim.saverestart, Tuple{Simulation,DirectSum,GPU}, sim, DirectSum(), GPU())
    h = handle(sim)
    nbytes = Ref{Int64}(0)
    check(h, ccall((:nb_checkpoint_size, libnb), Cint, (Ptr{Cvoid}, Ref{Int64}), h.ptr, nbytes))
    buf = Vector{UInt8}(undef, nbytes[])
    GC.@preserve buf check(h, ccall((:nb_checkpoint_save, libnb), Cint, (Ptr{Cvoid}, Ptr{UInt8}, Int64),
                                    h.ptr, buf, nbytes[]))
    write(joinpath(sim.config.output.dir, "restart.$(AstroNbodySim.Distributed.myid()).nbgb300"), buf)
    return nothing
end

"""Load a device image written by `saverestart` into the handle of `sim`
(a Simulation built with the same configuration), replacing its state."""
function loadrestart!(sim::Simulation, filename::AbstractString)
    h = handle(sim)
    buf = read(filename)
    GC.@preserve buf check(h, ccall((:nb_checkpoint_load, libnb), Cint, (Ptr{Cvoid}, Ptr{UInt8}, Int64),
                                    h.ptr, buf, length(buf)))
    return sim
end

"""Copy the resident state back into `sim.simdata` (units re-attached by the
caller's StructArray element types); replaces get_all_data for GPU
(src/base/Config.jl:1228-1230)."""
function download(sim::Simulation)
    h = handle(sim)
    n = h.n
    b = [Vector{Float64}(undef, n) for _ in 1:10]
    tb = Vector{Int64}(undef, n); te = Vector{Int64}(undef, n)
    GC.@preserve b tb te begin
        check(h, ccall((:nb_download, libnb), Cint,
                       (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
                        Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
                        Ptr{Int64}, Ptr{Int64}),
                       h.ptr, b..., tb, te))
    end
    return (x = b[1], y = b[2], z = b[3], vx = b[4], vy = b[5], vz = b[6],
            ax = b[7], ay = b[8], az = b[9], pot = b[10], ti_begstep = tb, ti_endstep = te)
end

end # module
