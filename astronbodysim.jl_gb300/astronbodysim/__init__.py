"""astronbodysim -- GB300-native DirectSum gravity for AstroNbodySim.jl users.

The compute path is libnbody_gb300.so (hand-written CUDA for sm_103a) behind
the C ABI in include/nbody_gb300.h; this package is the host-side mirror of the
reference's Simulation/run API plus seeded initial conditions.
"""
from ._lib import NbodyError, load
from .engine import Engine
from .serve import RequestStream, ensemble_systems, serve
from .ics import collision, hernquist, plummer
from .gadget2 import internal_G, read_gadget2, write_gadget2, write_snapshot
from .sim import (DirectSum, Euler, GPU, Leapfrog, MOND1983Milgrom, Newton, PointMassField, PseudoNewtonianField,
                  Simulation, active_count, advance_and_find_timestep,
                  compute_force, compute_potential, const_step_count, counters, diagnostics,
                  drift_particles_adaptive_timestep, drift_particles_const_timestep,
                  find_min_endstep, force_and_potential_at_points, get_all_data,
                  check_sync_point, init_timesteps, leapfrog_half_kick, loadrestart, run, saverestart, set_softlen, step,
                  step_until_output,
                  total_angular_momentum, total_energy, total_kinetic, total_momentum,
                  total_potential)

__all__ = [
    "Euler", "Leapfrog", "MOND1983Milgrom", "Newton", "PointMassField", "PseudoNewtonianField",
    "read_gadget2", "write_gadget2", "write_snapshot", "internal_G",
    "Engine", "RequestStream", "ensemble_systems", "serve", "NbodyError", "load", "plummer", "hernquist", "collision", "DirectSum", "GPU", "Simulation",
    "active_count", "counters", "advance_and_find_timestep", "compute_force", "compute_potential",
    "const_step_count", "diagnostics", "drift_particles_adaptive_timestep",
    "drift_particles_const_timestep", "find_min_endstep", "force_and_potential_at_points",
    "get_all_data", "check_sync_point", "saverestart", "loadrestart", "init_timesteps", "leapfrog_half_kick", "run", "set_softlen", "step", "step_until_output",
    "total_angular_momentum", "total_energy", "total_kinetic", "total_momentum", "total_potential",
]
