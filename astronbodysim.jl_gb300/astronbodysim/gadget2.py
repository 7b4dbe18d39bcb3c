"""Gadget-2 snapshot files (SnapFormat 1), the format the reference reads its
collision initial conditions from (examples/04-collisions/04-collisions.jl:21,
through AstroIO's read_gadget2) and writes its snapshots in
(src/base/Output.jl:36-51, through AstroIO's write_gadget2).

Layout, after the public Gadget-2 user guide (Springel 2005): a sequence of
Fortran records, each framed by a 4-byte length before and after it,

    HEAD  256 bytes: int32 Npart[6], float64 Massarr[6], float64 Time,
          float64 Redshift, int32 FlagSfr, int32 FlagFeedback, uint32 Nall[6],
          int32 FlagCooling, int32 NumFiles, float64 BoxSize, float64 Omega0,
          float64 OmegaLambda, float64 HubbleParam, int32 FlagAge,
          int32 FlagMetals, uint32 NallHW[6], int32 flag_entr_ics, 60 fill bytes
    POS   float[N][3]   particles ordered by type 0..5
    VEL   float[N][3]
    ID    uint32[N] (uint64 when the record says so)
    MASS  float[M]      only the particles of types whose Massarr is 0
    ...   gas blocks (U, RHO, ...) for type 0, not needed for gravity

Floats are single precision, or double when the record lengths say so.  The
byte order is found from the first record length (256).  Gadget type t maps to
the reference's Collection t + 1 (GAS = 1, HALO = 2, DISK = 3, BULGE = 4,
STAR = 5, BLACKHOLE = 6), which indexes the softening table.

Quantities stay in the file's internal units (by default kpc, km/s and
1e10 solar masses); internal_G() gives G in those units for Simulation(G=...).
"""
import struct

import numpy as np

_HEAD = "6i6d2d2i6I2i4d2i6Ii"
_HEAD_BYTES = struct.calcsize("<" + _HEAD)  # 196; padded to 256
_HEAD_FIELDS = ("Npart", "Massarr", "Time", "Redshift", "FlagSfr", "FlagFeedback", "Nall",
                "FlagCooling", "NumFiles", "BoxSize", "Omega0", "OmegaLambda", "HubbleParam",
                "FlagAge", "FlagMetals", "NallHW", "flag_entr_ics")
_HEAD_COUNTS = (6, 6, 1, 1, 1, 1, 6, 1, 1, 1, 1, 1, 1, 1, 1, 6, 1)


class Gadget2FormatError(ValueError):
    pass


def internal_G(G_cgs=6.6743e-8, length_cm=3.085678e21, mass_g=1.989e43, velocity_cm_s=1e5):
    """G in Gadget-2 internal units (length, mass, velocity; time = length /
    velocity).  The defaults are Gadget-2's kpc, 1e10 solar masses and km/s."""
    return G_cgs * mass_g / (length_cm * velocity_cm_s ** 2)


def _records(buf):
    if len(buf) < 4:
        raise Gadget2FormatError("file too short")
    first = buf[:4]
    if struct.unpack("<i", first)[0] == 256:
        end = "<"
    elif struct.unpack(">i", first)[0] == 256:
        end = ">"
    else:
        raise Gadget2FormatError("first record is not a 256-byte header (not SnapFormat 1)")
    recs = []
    off = 0
    while off < len(buf):
        if off + 4 > len(buf):
            raise Gadget2FormatError("truncated record marker at byte %d" % off)
        n = struct.unpack_from(end + "i", buf, off)[0]
        if n < 0 or off + 8 + n > len(buf):
            raise Gadget2FormatError("record at byte %d overruns the file" % off)
        m = struct.unpack_from(end + "i", buf, off + 4 + n)[0]
        if m != n:
            raise Gadget2FormatError("record markers differ at byte %d (%d vs %d)" % (off, n, m))
        recs.append(buf[off + 4:off + 4 + n])
        off += 8 + n
    return end, recs


def _parse_header(end, rec):
    vals = struct.unpack_from(end + _HEAD, rec, 0)
    h, k = {}, 0
    for name, c in zip(_HEAD_FIELDS, _HEAD_COUNTS):
        h[name] = list(vals[k:k + c]) if c > 1 else vals[k]
        k += c
    return h


def read_gadget2(path):
    """Reads one SnapFormat-1 file.  Returns (header, data) where data has
    pos (N,3), vel (N,3), mass (N,), collection (N,) int32 in 1..6, id (N,)
    as float64 / int arrays in file order (by type)."""
    with open(path, "rb") as f:
        buf = f.read()
    end, recs = _records(buf)
    header = _parse_header(end, recs[0])
    npart = np.array(header["Npart"], dtype=np.int64)
    n = int(npart.sum())
    if len(recs) < 4:
        raise Gadget2FormatError("need HEAD, POS, VEL and ID records, found %d" % len(recs))
    pos_rec, vel_rec, id_rec = recs[1], recs[2], recs[3]
    if len(pos_rec) == 12 * n:
        ft = np.dtype(end + "f4")
    elif len(pos_rec) == 24 * n:
        ft = np.dtype(end + "f8")
    else:
        raise Gadget2FormatError("POS record of %d bytes does not fit %d particles" % (len(pos_rec), n))
    if len(vel_rec) != len(pos_rec):
        raise Gadget2FormatError("VEL record size differs from POS")
    if len(id_rec) == 4 * n:
        it = np.dtype(end + "u4")
    elif len(id_rec) == 8 * n:
        it = np.dtype(end + "u8")
    else:
        raise Gadget2FormatError("ID record of %d bytes does not fit %d particles" % (len(id_rec), n))
    pos = np.frombuffer(pos_rec, dtype=ft).reshape(n, 3).astype(np.float64)
    vel = np.frombuffer(vel_rec, dtype=ft).reshape(n, 3).astype(np.float64)
    ids = np.frombuffer(id_rec, dtype=it).astype(np.int64)
    massarr = np.array(header["Massarr"], dtype=np.float64)
    coll = np.repeat(np.arange(1, 7, dtype=np.int32), npart)
    mass = massarr[coll - 1].copy()
    need = (massarr == 0.0) & (npart > 0)
    nvar = int(npart[need].sum())
    if nvar:
        if len(recs) < 5 or len(recs[4]) != nvar * ft.itemsize:
            raise Gadget2FormatError("MASS record missing or of the wrong size (%d masses)" % nvar)
        mv = np.frombuffer(recs[4], dtype=ft).astype(np.float64)
        mass[need[coll - 1]] = mv
    return header, {"pos": pos, "vel": vel, "mass": mass, "collection": coll, "id": ids}


def make_header(npart, massarr=None, time=0.0, redshift=0.0, boxsize=0.0, omega0=0.0,
                omega_lambda=0.0, hubble=0.0):
    npart = [int(v) for v in npart]
    return {"Npart": npart, "Massarr": list(massarr) if massarr is not None else [0.0] * 6,
            "Time": float(time), "Redshift": float(redshift), "FlagSfr": 0, "FlagFeedback": 0,
            "Nall": list(npart), "FlagCooling": 0, "NumFiles": 1, "BoxSize": float(boxsize),
            "Omega0": float(omega0), "OmegaLambda": float(omega_lambda), "HubbleParam": float(hubble),
            "FlagAge": 0, "FlagMetals": 0, "NallHW": [0] * 6, "flag_entr_ics": 0}


def write_gadget2(path, header, data, double=False, byteorder="<"):
    """Writes one SnapFormat-1 file.  data as returned by read_gadget2
    (pos, vel, mass, collection in 1..6, optional id); particles are written
    grouped by type, so header Npart is recomputed from the collections.
    Masses go to Massarr when a type's masses are all equal (and Massarr is not
    set to 0 for it in the header), otherwise to the MASS record."""
    end = byteorder
    coll = np.asarray(data["collection"], dtype=np.int32)
    order = np.argsort(coll, kind="stable")
    coll = coll[order]
    pos = np.asarray(data["pos"], dtype=np.float64).reshape(-1, 3)[order]
    vel = np.asarray(data["vel"], dtype=np.float64).reshape(-1, 3)[order]
    mass = np.asarray(data["mass"], dtype=np.float64)[order]
    ids = (np.asarray(data["id"], dtype=np.int64)[order] if "id" in data
           else np.arange(1, coll.size + 1, dtype=np.int64))
    npart = np.bincount(coll - 1, minlength=6)[:6]
    h = dict(header)
    h["Npart"] = [int(v) for v in npart]
    h["Nall"] = [int(v) for v in npart]
    massarr = [0.0] * 6
    hm = header.get("Massarr", [0.0] * 6)
    for t in range(6):
        mt = mass[coll == t + 1]
        if mt.size and np.all(mt == mt[0]) and hm[t] != 0.0:
            massarr[t] = float(mt[0])
    h["Massarr"] = massarr
    ft = np.dtype(end + ("f8" if double else "f4"))
    it = np.dtype(end + ("u8" if ids.max(initial=0) >= 2 ** 32 else "u4"))
    vals = []
    for name, c in zip(_HEAD_FIELDS, _HEAD_COUNTS):
        vals.extend(h[name] if c > 1 else [h[name]])
    head = struct.pack(end + _HEAD, *vals) + b"\0" * (256 - _HEAD_BYTES)
    var = np.array([massarr[t - 1] == 0.0 for t in coll], dtype=bool)
    recs = [head, pos.astype(ft).tobytes(), vel.astype(ft).tobytes(), ids.astype(it).tobytes()]
    if var.any():
        recs.append(mass[var].astype(ft).tobytes())
    with open(path, "wb") as f:
        for r in recs:
            f.write(struct.pack(end + "i", len(r)))
            f.write(r)
            f.write(struct.pack(end + "i", len(r)))


def write_snapshot(sim, path, time=None, double=False):
    """Snapshot of a Simulation's resident state (positions, velocities,
    masses, collections) as a Gadget-2 file; Time is the simulation time."""
    d = sim.download()
    if time is None:
        time = sim.time()[1]
    coll = sim.collection
    out = {"pos": d["pos"], "vel": d["vel"], "mass": d["mass"], "collection": coll}
    hdr = make_header(np.bincount(np.asarray(coll) - 1, minlength=6)[:6], massarr=[1.0] * 6,
                      time=time)
    write_gadget2(path, hdr, out, double=double)
