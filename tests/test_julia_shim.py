"""CPU checks of the Julia ccall shim (astronbodysim.jl_gb300/julia/NbodyGB300.jl),
which cannot run here (no Julia toolchain):
* its NbParams / NbDiag structs have the fields of include/nbody_gb300.h and of
  the ctypes structures, in the same order and with the same types;
* every method it adds to AstroNbodySim is defined for routed simulations
  (Simulation{<:NbDeviceData}) only, so no reference method is redefined;
* every library symbol it calls is declared in the header."""
import ctypes
import os
import re

from conftest import REPO

SHIM = os.path.join(REPO, "astronbodysim.jl_gb300", "julia", "NbodyGB300.jl")
HEADER = os.path.join(REPO, "include", "nbody_gb300.h")

C_TO_JL = {"double": "Float64", "int32_t": "Int32", "int64_t": "Int64"}
CT_TO_JL = {ctypes.c_double: "Float64", ctypes.c_int32: "Int32", ctypes.c_int64: "Int64"}


def jl_struct(name):
    src = open(SHIM).read()
    m = re.search(r"^struct %s\n(.*?)^end" % name, src, flags=re.S | re.M)
    assert m, name
    fields = []
    for line in m.group(1).splitlines():
        line = line.split("#")[0].strip()
        if line:
            f, t = line.split("::")
            fields.append((f.strip(), t.strip()))
    return fields


def c_struct(name):
    src = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    m = re.search(r"typedef struct %s \{(.*?)\} %s;" % (name, name), src, flags=re.S)
    assert m, name
    fields = []
    for decl in m.group(1).split(";"):
        decl = decl.strip()
        if not decl:
            continue
        t, f = decl.split()
        a = re.match(r"(\w+)\[(\d+)\]", f)
        if a:
            fields.append((a.group(1), "NTuple{%s,%s}" % (a.group(2), C_TO_JL[t])))
        else:
            fields.append((f, C_TO_JL[t]))
    return fields


def ctypes_struct(cls):
    out = []
    for f, t in cls._fields_:
        if hasattr(t, "_length_"):
            out.append((f, "NTuple{%d,%s}" % (t._length_, CT_TO_JL[t._type_])))
        else:
            out.append((f, CT_TO_JL[t]))
    return out


def test_params_struct_matches_header_and_ctypes():
    from astronbodysim import _lib

    jl = jl_struct("NbParams")
    assert jl == c_struct("nb_params")
    assert jl == ctypes_struct(_lib.nb_params)


def test_diag_struct_matches_header_and_ctypes():
    from astronbodysim import _lib

    jl = jl_struct("NbDiag")
    assert jl == c_struct("nb_diag")
    assert jl == ctypes_struct(_lib.nb_diag)


def test_methods_extend_only_routed_simulations():
    src = open(SHIM).read()
    defs = re.findall(r"^(?:function )?AstroNbodySim\.([\w!]+)\((\w+)::([\w{}<:]+)", src, flags=re.M)
    assert len(defs) >= 15
    for fn, arg, typ in defs:
        assert typ == "Routed", (fn, arg, typ)
    # the integrator, force, data and diagnostics methods of the drop-in
    names = {fn for fn, _, _ in defs}
    for fn in ("compute_force", "compute_potential", "init_timesteps", "leapfrog_half_kick",
               "advance_and_find_timestep", "find_min_endstep", "check_sync_point",
               "drift_particles_kernel", "step", "get_all_data", "get_local_data",
               "total_kinetic", "total_potential", "total_momentum", "total_angular_momentum",
               "set_softlen!", "saverestart"):
        assert fn in names, fn
    assert "Routed = Simulation{<:NbDeviceData}" in src
    # no self-recursive fallbacks into overwritten methods
    assert "invoke(" not in src


def test_called_symbols_are_declared():
    src = open(SHIM).read()
    called = set(re.findall(r"ccall\(\(:(nb_\w+), libnb\)", src))
    hdr = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    declared = set(re.findall(r"\b(nb_[a-z0-9_]+)\s*\(", hdr))
    assert called and called <= declared, called - declared
