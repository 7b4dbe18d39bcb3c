"""Writes galaxy_subsample.npz: every 15th particle of the reference's
Gadget-2 collision fixture (examples/04-collisions/galaxy_littleendian.dat,
40000 halo + 20000 disk particles in kpc, km/s, 1e10 Msun), with masses
scaled by 15 so the total mass is kept, and the header fields the tests check.

Run in a checkout that has the reference project next to it:
    python tests/golden/make_galaxy_subsample.py /path/to/AstroNbodySim.jl
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "astronbodysim.jl_gb300"))

from astronbodysim.gadget2 import read_gadget2  # noqa: E402


def main(ref_root):
    path = os.path.join(ref_root, "examples", "04-collisions", "galaxy_littleendian.dat")
    header, d = read_gadget2(path)
    sel = np.arange(0, d["pos"].shape[0], 15)
    np.savez_compressed(os.path.join(HERE, "galaxy_subsample.npz"),
                        pos=d["pos"][sel], vel=d["vel"][sel], mass=d["mass"][sel] * 15.0,
                        collection=d["collection"][sel], id=d["id"][sel],
                        npart=np.array(header["Npart"]), massarr=np.array(header["Massarr"]),
                        n_total=d["pos"].shape[0], total_mass=d["mass"].sum())


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("ASTRONBODYSIM_REF", "."))
