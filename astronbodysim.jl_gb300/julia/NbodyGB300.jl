"""
    NbodyGB300

Drop-in for AstroNbodySim.jl's DirectSum solver on the GPU device.  A
simulation built by the reference's constructor with `device = GPU()` is
handed to `NbodyGB300.route(sim)`, which uploads its particles to
libnbody_gb300.so and returns the same `Simulation` with a different data
field: `Simulation{NbDeviceData}`.  Every method below is defined for that type
only, so it is more specific than the reference's `(DirectSum, GPU)` /
`(Gravity, GPU)` methods for `Simulation`; no reference method is redefined,
and simulations that were not routed keep the reference's CUDA.jl path
untouched.

    using AstroNbodySim, NbodyGB300
    sim = NbodyGB300.route(Simulation(data; device = GPU(), ...))
    run(sim)                      # src/run.jl, unchanged

The library keeps the particle state and the time line resident on the GB300;
`get_all_data` downloads it.  Background-force closures (`sim.bgforce`) cannot
cross the C ABI: pass the analytic field they stand for as
`route(sim; bgfield = PointMassField(GM, center))` (or
`PseudoNewtonianField`); a simulation with closures and no `bgfield` is
refused instead of silently losing its field.
"""
module NbodyGB300

using AstroNbodySim
using AstroNbodySim: Simulation, DirectSum, Gravity, GPU, AdaptiveTimestep, ConstantTimestep
using PhysicalParticles: PVector
using StructArrays
using Unitful

const libnb = get(ENV, "NBODY_GB300_LIB",
                  joinpath(@__DIR__, "..", "csrc", "libnbody_gb300.so"))

# Mirrors `nb_params` of include/nbody_gb300.h (field order and types; the
# CPU test tests/test_julia_shim.py compares them with the header).
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
    algorithm::Int32
    bg_kind::Int32
    mond::Int32
    bg_gm::Float64
    bg_center::NTuple{3,Float64}
    bg_rg::Float64
    mond_acc0::Float64
    mond_nu_index::Float64
    stages::Int32
    resort_every::Int32
end

# Mirrors `nb_diag` of include/nbody_gb300.h.
struct NbDiag
    kinetic::Float64
    potential::Float64
    momentum::NTuple{3,Float64}
    angular_momentum::NTuple{3,Float64}
end

"""Analytic background fields the library applies after the direct sum
(postprocessing_force, src/directsumgpu/gravity.jl:64-79): a point mass
(the attractor of test/Local-Timestep.jl:746) or the pseudo-Newtonian field of
src/tools/BlackHole.jl:41-60.  GM, rg and center in the simulation's units."""
struct PointMassField
    GM
    center
end
struct PseudoNewtonianField
    GM
    rg
    center
end

"""Data field of a routed simulation: the library handle, the particle count
and the host copy of the particles as built by the reference's constructor
(kept for their types, IDs, collections and masses)."""
mutable struct NbDeviceData
    ptr::Ptr{Cvoid}
    n::Int
    host
end
Base.length(d::NbDeviceData) = d.n

const Routed = Simulation{<:NbDeviceData}

function check(ptr::Ptr{Cvoid}, rc::Integer)
    rc == 0 && return nothing
    msg = unsafe_string(ccall((:nb_last_error, libnb), Cstring, (Ptr{Cvoid},), ptr))
    error("libnbody_gb300 error $rc: $msg")
end
check(sim::Routed, rc::Integer) = check(sim.simdata.ptr, rc)
hptr(sim::Routed) = sim.simdata.ptr

# unit stripping, in the simulation's unit system
units(sim) = sim.config.units
lenunit(sim) = isnothing(units(sim)) ? nothing : units(sim)[1]
timeunit(sim) = isnothing(units(sim)) ? nothing : units(sim)[2]
massunit(sim) = isnothing(units(sim)) ? nothing : units(sim)[3]
velunit(sim) = isnothing(units(sim)) ? nothing : lenunit(sim) / timeunit(sim)
accunit(sim) = isnothing(units(sim)) ? nothing : lenunit(sim) / timeunit(sim)^2
strip(u, x) = isnothing(u) ? Float64(x) : Float64(ustrip(u, x))
unstrip(u, x) = isnothing(u) ? x : x * u
stripG(sim) = Float64(ustrip(sim.config.constants.G))

mond_of(sim) = Int32(sim.config.grav.model isa AstroNbodySim.MOND1983Milgrom ? 1 : 0)

function field_params(sim, bgfield)
    lu = lenunit(sim)
    if bgfield === nothing
        return Int32(0), 0.0, (0.0, 0.0, 0.0), 0.0
    end
    gm = isnothing(units(sim)) ? Float64(bgfield.GM) :
         Float64(ustrip(lu^3 / timeunit(sim)^2, bgfield.GM))
    c = ntuple(k -> strip(lu, bgfield.center[k]), 3)
    if bgfield isa PointMassField
        return Int32(1), gm, c, 0.0
    elseif bgfield isa PseudoNewtonianField
        return Int32(2), gm, c, strip(lu, bgfield.rg)
    end
    error("bgfield must be a PointMassField or a PseudoNewtonianField")
end

function params(sim; precision = Int32(1), law = Int32(0), bgfield = nothing, resort_every = 0)
    tc = sim.config.time
    step = tc.step
    soft = ntuple(k -> strip(lenunit(sim), sim.config.grav.ForceSofteningTable[k]), 6)
    tu = timeunit(sim)
    adaptive = step isa AdaptiveTimestep
    euler = tc.algorithm isa AstroNbodySim.Euler
    bg_kind, bg_gm, bg_center, bg_rg = field_params(sim, bgfield)
    mond = mond_of(sim)
    NbParams(stripG(sim), soft, law, precision, Int32(adaptive), Int32(0),
             adaptive ? 0.0 : strip(tu, step.dt),
             adaptive ? Float64(step.ErrTolTimestep) : 0.025,
             adaptive ? strip(tu, step.MinStep) : 1.0e-8,
             adaptive ? strip(tu, step.MaxStep) : Inf,
             adaptive ? Int64(step.TimeBase) : Int64(1) << 30,
             strip(tu, tc.Begin), strip(tu, tc.End),
             Int32(0),                 # device
             Int32(0), Int32(0), Int32(0), Int32(0),  # tile_j, i_per_thread, block, j_split: built-in rule
             Int32(euler ? 1 : 0),     # algorithm
             bg_kind, mond, bg_gm, bg_center, bg_rg,
             mond == 0 ? 0.0 : strip(accunit(sim), sim.config.constants.ACC0),
             Float64(sim.config.grav.MOND_nuIndex),
             Int32(0), Int32(resort_every))  # stages (built-in), resort_every (0 = 16)
end

"""
    route(sim; precision = :mixed, law = :spline, bgfield = nothing, resort_every = 0)

Uploads the particles of a `(DirectSum, GPU)` simulation built by the
reference's constructor (replacing its `cu(StructArray(d))` placement,
src/base/Config.jl:1072-1088) and returns the routed simulation.  The
snapshot schedule (`TimeBetweenSnapshots`, src/base/Config.jl:436-439,
749-750) goes to the device so that `step` splits its drifts at output times.
`law = :plummer` selects the r^2 + h^2 softening instead of the reference's
Gadget-2 spline; `precision = :fp64` the plain FP64 form.  `resort_every`
sets the steps between Morton re-orders of the sources in `step` (0 = 16,
1 = every step; the forces differ only by FP32 round-off).
"""
function route(sim::Simulation; precision = :mixed, law = :spline, bgfield = nothing, resort_every = 0)
    sim.config.solver.grav isa DirectSum || error("NbodyGB300 routes DirectSum simulations only")
    sim.config.device.type isa GPU || error("NbodyGB300 routes GPU simulations only")
    if !isempty(sim.bgforce) && bgfield === nothing
        error("sim.bgforce holds Julia closures, which cannot cross the C ABI: pass the field " *
              "as bgfield = PointMassField(GM, center) or PseudoNewtonianField(GM, rg, center)")
    end
    p = Ref(params(sim; precision = Int32(precision === :fp64 ? 0 : 1),
                   law = Int32(law === :plummer ? 1 : 0), bgfield, resort_every))
    out = Ref{Ptr{Cvoid}}(C_NULL)
    rc = ccall((:nb_create, libnb), Cint, (Ref{NbParams}, Ref{Ptr{Cvoid}}), p, out)
    check(C_NULL, rc)  # with a null handle nb_last_error gives the reason nb_create failed
    d = StructArray(Array(sim.simdata))
    dev = NbDeviceData(out[], length(d), d)
    finalizer(x -> ccall((:nb_destroy, libnb), Cint, (Ptr{Cvoid},), x.ptr), dev)
    lu, vu, mu = lenunit(sim), velunit(sim), massunit(sim)
    x = [strip(lu, q.x) for q in d.Pos]; y = [strip(lu, q.y) for q in d.Pos]; z = [strip(lu, q.z) for q in d.Pos]
    vx = [strip(vu, v.x) for v in d.Vel]; vy = [strip(vu, v.y) for v in d.Vel]; vz = [strip(vu, v.z) for v in d.Vel]
    m = [strip(mu, q) for q in d.Mass]
    t = Int32[Int(c) for c in d.Collection]
    GC.@preserve x y z vx vy vz m t begin
        check(dev.ptr, ccall((:nb_upload, libnb), Cint,
                             (Ptr{Cvoid}, Int64, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
                              Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Int32}),
                             dev.ptr, length(d), x, y, z, vx, vy, vz, m, t))
    end
    between = strip(timeunit(sim), sim.config.time.BetweenSnapshots)
    check(dev.ptr, ccall((:nb_set_snapshot_interval, libnb), Cint, (Ptr{Cvoid}, Float64),
                         dev.ptr, between))
    routed = Simulation(sim.config, sim.id, sim.pids, dev, sim.timeinfo, sim.outputinfo,
                        sim.loginfo, sim.physics, sim.stream, sim.visinfo, sim.buffer,
                        sim.bgforce, sim.bgpotential, sim.poststep)
    AstroNbodySim.registry[sim.id] = routed
    return routed
end

# -- forces -------------------------------------------------------------------

# compute_force(sim, DirectSum, GPU) (src/directsumgpu/gravity.jl:81-85): the
# direct sum of the active particles and postprocessing_force (:64-79) run on
# the device in one call; inactive particles keep their Acc as on the CPU path.
function AstroNbodySim.compute_force(sim::Routed, ::DirectSum, ::GPU)
    t_FORCE = time_ns()
    check(sim, ccall((:nb_compute_force, libnb), Cint, (Ptr{Cvoid}, Cint), hptr(sim), 0))
    AstroNbodySim.add_timer(sim, "FORCE", t_FORCE, time_ns())
end

# compute_potential(sim) (src/base/Potential.jl:20-24): the direct-sum
# potential, then the self-potential term (src/base/Potential.jl:5-16); the
# reference has a CPU version only (src/directsum/potential.jl:142-148).
function AstroNbodySim.compute_potential(sim::Routed)
    check(sim, ccall((:nb_compute_potential, libnb), Cint, (Ptr{Cvoid},), hptr(sim)))
    check(sim, ccall((:nb_remove_self_potential, libnb), Cint, (Ptr{Cvoid},), hptr(sim)))
end
AstroNbodySim.compute_potential(sim::Routed, ::DirectSum, ::GPU) =
    check(sim, ccall((:nb_compute_potential, libnb), Cint, (Ptr{Cvoid},), hptr(sim)))

# -- integrator (src/directsumgpu/timestep.jl) ---------------------------------

# :40-47
AstroNbodySim.init_timesteps(sim::Routed, ::Gravity, ::GPU) =
    check(sim, ccall((:nb_init_timesteps, libnb), Cint, (Ptr{Cvoid},), hptr(sim)))

# :210-212
AstroNbodySim.leapfrog_half_kick(sim::Routed, forward::Int, ::Gravity, ::GPU) =
    check(sim, ccall((:nb_half_kick, libnb), Cint, (Ptr{Cvoid}, Cint), hptr(sim), forward))

# :172-174
AstroNbodySim.advance_and_find_timestep(sim::Routed, ::Gravity, ::GPU) =
    check(sim, ccall((:nb_kick, libnb), Cint, (Ptr{Cvoid},), hptr(sim)))

# :103-114
function AstroNbodySim.find_min_endstep(sim::Routed, ::Gravity, ::GPU)
    v = Ref{Int64}(0)
    check(sim, ccall((:nb_find_min_endstep, libnb), Cint, (Ptr{Cvoid}, Ref{Int64}), hptr(sim), v))
    sim.timeinfo.min_endstep = v[]
    return v[]
end

# :116-118 (check_sync_point_local, src/base/Timestep.jl:146-157, on the device data)
function AstroNbodySim.check_sync_point(sim::Routed, ::Gravity, ::GPU)
    v = Ref{Int32}(0)
    check(sim, ccall((:nb_check_sync_point, libnb), Cint, (Ptr{Cvoid}, Ref{Int32}), hptr(sim), v))
    return sim.outputinfo.syncflag = v[] != 0
end

# :57-74: the host's TimeInfo was advanced by drift_particles_*_timestep; the
# device clock follows (constant steps drift by the float time difference, as
# the CPU path does, src/base/Timestep.jl:181-191)
AstroNbodySim.drift_particles_kernel(sim::Routed, ::AdaptiveTimestep, ::Gravity, ::GPU) =
    check(sim, ccall((:nb_drift_to_int, libnb), Cint, (Ptr{Cvoid}, Int64), hptr(sim),
                     sim.timeinfo.system_time_int))
AstroNbodySim.drift_particles_kernel(sim::Routed, ::ConstantTimestep, ::Gravity, ::GPU) =
    check(sim, ccall((:nb_drift_to_float, libnb), Cint, (Ptr{Cvoid}, Float64), hptr(sim),
                     strip(timeunit(sim), sim.timeinfo.system_time_float)))

function device_time(sim::Routed)
    ti = Ref{Int64}(0); tf = Ref{Float64}(0.0)
    check(sim, ccall((:nb_get_time, libnb), Cint, (Ptr{Cvoid}, Ref{Int64}, Ref{Float64}),
                     hptr(sim), ti, tf))
    ni = Ref{Int64}(0); nf = Ref{Float64}(0.0); at = Ref{Int32}(0); k = Ref{Int64}(0)
    check(sim, ccall((:nb_get_output_time, libnb), Cint,
                     (Ptr{Cvoid}, Ref{Int64}, Ref{Float64}, Ref{Int32}, Ref{Int64}),
                     hptr(sim), ni, nf, at, k))
    return ti[], tf[], ni[], nf[]
end

# step(sim, DirectSum, GPU) (:216-224): find_next_sync_point_and_drift with
# the snapshot schedule (src/base/Timestep.jl:197-245), force, kick -- one
# replay of the library's step graph, which stops the time line at every
# output time inside the step; the output function then runs on the state at
# that time (src/base/Timestep.jl:204-206, 234-236) and the next replay
# finishes the step.  TimeInfo follows the device clock.
function AstroNbodySim.step(sim::Routed, ::DirectSum, ::GPU)
    ti = sim.timeinfo
    tu = timeunit(sim)
    k = Ref{Int64}(0); at = Ref{Int32}(0)
    while true
        last_int, last_float = ti.system_time_int, ti.system_time_float
        check(sim, ccall((:nb_step_until_output, libnb), Cint,
                         (Ptr{Cvoid}, Int64, Ref{Int64}, Ref{Int32}), hptr(sim), 1, k, at))
        t_int, t_float, next_int, next_float = device_time(sim)
        ti.last_system_time_int = last_int
        ti.last_system_time_float = last_float
        ti.system_time_int = t_int
        ti.system_time_float = unstrip(tu, t_float)
        ti.dt = unstrip(tu, t_float - strip(tu, last_float))
        at[] == 0 && break
        # the reference moves next_output_time on after the output function
        sim.config.output.func(sim, sim.config.output.type)
        ti.next_output_time_int = next_int
        ti.next_output_time_float = unstrip(tu, next_float)
    end
    return nothing
end

# -- data and diagnostics --------------------------------------------------------

"""The resident state as the reference's particle StructArray on the host
(get_all_data for GPU, src/base/Config.jl:1228-1230): positions, velocities,
accelerations, potentials and time bins from the device, everything else from
the particles that were uploaded."""
function AstroNbodySim.get_all_data(sim::Routed, ::DirectSum, ::GPU)
    n = sim.simdata.n
    b = [Vector{Float64}(undef, n) for _ in 1:10]
    tb = Vector{Int64}(undef, n); te = Vector{Int64}(undef, n)
    GC.@preserve b tb te begin
        check(sim, ccall((:nb_download, libnb), Cint,
                         (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
                          Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
                          Ptr{Float64}, Ptr{Int64}, Ptr{Int64}),
                         hptr(sim), b..., tb, te))
    end
    d = deepcopy(sim.simdata.host)
    lu, vu, au = lenunit(sim), velunit(sim), accunit(sim)
    pu = isnothing(units(sim)) ? nothing : vu^2
    P = eltype(d.Pos)
    for i in 1:n
        d.Pos[i] = P(unstrip(lu, b[1][i]), unstrip(lu, b[2][i]), unstrip(lu, b[3][i]))
        d.Vel[i] = typeof(d.Vel[i])(unstrip(vu, b[4][i]), unstrip(vu, b[5][i]), unstrip(vu, b[6][i]))
        d.Acc[i] = typeof(d.Acc[i])(unstrip(au, b[7][i]), unstrip(au, b[8][i]), unstrip(au, b[9][i]))
        d.Potential[i] = unstrip(pu, b[10][i])
        d.Ti_begstep[i] = tb[i]
        d.Ti_endstep[i] = te[i]
    end
    return d
end
AstroNbodySim.get_local_data(sim::Routed, g::DirectSum, d::GPU) = AstroNbodySim.get_all_data(sim, g, d)

function diag(sim::Routed, with_pot)
    r = Ref{NbDiag}()
    check(sim, ccall((:nb_diagnostics, libnb), Cint, (Ptr{Cvoid}, Cint, Ref{NbDiag}), hptr(sim),
                     with_pot, r))
    return r[]
end

eunit(sim) = isnothing(units(sim)) ? nothing : massunit(sim) * velunit(sim)^2
punit(sim) = isnothing(units(sim)) ? nothing : massunit(sim) * velunit(sim)
lunit(sim) = isnothing(units(sim)) ? nothing : massunit(sim) * lenunit(sim) * velunit(sim)
vec3(sim, u, t) = PVector(unstrip(u, t[1]), unstrip(u, t[2]), unstrip(u, t[3]))

# src/base/Energy.jl:43-47, 61, 87-101 for the resident data (FP64 reductions
# on the device; the reference's GPU versions index device arrays, which
# CUDA.jl forbids)
AstroNbodySim.total_kinetic(sim::Routed) = unstrip(eunit(sim), diag(sim, 0).kinetic)
AstroNbodySim.total_potential(sim::Routed, ::DirectSum, ::GPU) = unstrip(eunit(sim), diag(sim, 1).potential)
AstroNbodySim.total_momentum(sim::Routed) = vec3(sim, punit(sim), diag(sim, 0).momentum)
AstroNbodySim.total_angular_momentum(sim::Routed) = vec3(sim, lunit(sim), diag(sim, 0).angular_momentum)

# set_softlen! for GPU (src/tools/SofteningLength.jl:87-89): the table in the
# configuration, then the device copy
function AstroNbodySim.set_softlen!(sim::Routed, h, ::DirectSum, ::GPU)
    AstroNbodySim.set_softlen_local!(sim, h)
    soft = [strip(lenunit(sim), s) for s in sim.config.grav.ForceSofteningTable]
    GC.@preserve soft check(sim, ccall((:nb_set_softening, libnb), Cint, (Ptr{Cvoid}, Ptr{Float64}),
                                       hptr(sim), soft))
end

# -- restart files ------------------------------------------------------------------

# saverestart(sim, DirectSum, GPU) (src/restart.jl:14-19): the device image
# (parameters incl. the time-integration algorithm, particles, time line and
# snapshot schedule) next to the reference's file name
function AstroNbodySim.saverestart(sim::Routed, ::DirectSum, ::GPU)
    nbytes = Ref{Int64}(0)
    check(sim, ccall((:nb_checkpoint_size, libnb), Cint, (Ptr{Cvoid}, Ref{Int64}), hptr(sim), nbytes))
    buf = Vector{UInt8}(undef, nbytes[])
    GC.@preserve buf check(sim, ccall((:nb_checkpoint_save, libnb), Cint,
                                      (Ptr{Cvoid}, Ptr{UInt8}, Int64), hptr(sim), buf, nbytes[]))
    write(joinpath(sim.config.output.dir, "restart.$(AstroNbodySim.Distributed.myid()).nbgb300"), buf)
    return nothing
end

"""Load a device image written by `saverestart` into a routed simulation
(loadrestart, src/restart.jl:129-139, for the device part), replacing its
state and time line."""
function loadrestart!(sim::Routed, filename::AbstractString)
    buf = read(filename)
    GC.@preserve buf check(sim, ccall((:nb_checkpoint_load, libnb), Cint,
                                      (Ptr{Cvoid}, Ptr{UInt8}, Int64), hptr(sim), buf, length(buf)))
    t_int, t_float, next_int, next_float = device_time(sim)
    tu = timeunit(sim)
    sim.timeinfo.system_time_int = t_int
    sim.timeinfo.system_time_float = unstrip(tu, t_float)
    sim.timeinfo.next_output_time_int = next_int
    sim.timeinfo.next_output_time_float = unstrip(tu, next_float)
    return sim
end

end # module
