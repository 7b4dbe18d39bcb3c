"""Gadget-2 SnapFormat-1 reader/writer (host side, no GPU)."""
import os
import struct

import numpy as np
import pytest

from astronbodysim import gadget2 as g2

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "galaxy_subsample.npz")


def _system(n, rng, types=(2, 3)):
    coll = np.sort(rng.choice(np.array(types, dtype=np.int32), n))
    return {"pos": rng.normal(size=(n, 3)) * 10.0, "vel": rng.normal(size=(n, 3)) * 100.0,
            "mass": rng.uniform(1e-4, 2e-4, n), "collection": coll,
            "id": np.arange(1, n + 1, dtype=np.int64)}


@pytest.mark.parametrize("double", [False, True])
@pytest.mark.parametrize("order", ["<", ">"])
def test_round_trip_with_mass_record(tmp_path, double, order):
    rng = np.random.default_rng(3)
    d = _system(1000, rng)
    hdr = g2.make_header([0] * 6, time=0.25)
    p = tmp_path / "snap.dat"
    g2.write_gadget2(str(p), hdr, d, double=double, byteorder=order)
    h, r = g2.read_gadget2(str(p))
    ft = np.float64 if double else np.float32
    assert h["Npart"][1] + h["Npart"][2] == 1000 and h["Time"] == 0.25
    np.testing.assert_array_equal(r["collection"], d["collection"])
    np.testing.assert_array_equal(r["pos"], d["pos"].astype(ft).astype(np.float64))
    np.testing.assert_array_equal(r["vel"], d["vel"].astype(ft).astype(np.float64))
    np.testing.assert_array_equal(r["mass"], d["mass"].astype(ft).astype(np.float64))
    np.testing.assert_array_equal(r["id"], d["id"])


def test_equal_masses_go_to_massarr(tmp_path):
    rng = np.random.default_rng(4)
    d = _system(600, rng)
    d["mass"] = np.where(d["collection"] == 2, 1e-3, 2e-4)
    hdr = g2.make_header([0] * 6, massarr=[1.0] * 6)
    p = tmp_path / "snap.dat"
    g2.write_gadget2(str(p), hdr, d)
    buf = p.read_bytes()
    n = 600
    # HEAD, POS, VEL, ID only: no MASS record
    assert len(buf) == (256 + 8) + 2 * (12 * n + 8) + (4 * n + 8)
    h, r = g2.read_gadget2(str(p))
    assert h["Massarr"][1] == 1e-3 and h["Massarr"][2] == 2e-4
    np.testing.assert_array_equal(r["mass"], d["mass"])


def test_galaxy_fixture_subsample(tmp_path):
    """The committed subsample of the reference's collision fixture: 40000 halo
    (type 1, Collection 2) and 20000 disk (type 2, Collection 3) particles with
    per-type masses in the header; written and read back unchanged."""
    z = np.load(GOLDEN)
    assert int(z["n_total"]) == 60000
    assert list(z["npart"]) == [0, 40000, 20000, 0, 0, 0]
    assert z["massarr"][0] == 0.0 and z["massarr"][1] > 0.0 and z["massarr"][2] > 0.0
    assert set(np.unique(z["collection"])) == {2, 3}
    d = {k: z[k] for k in ("pos", "vel", "mass", "collection", "id")}
    p = tmp_path / "sub.dat"
    g2.write_gadget2(str(p), g2.make_header([0] * 6, massarr=[1.0] * 6), d)
    _, r = g2.read_gadget2(str(p))
    np.testing.assert_array_equal(r["pos"], d["pos"])  # the fixture's values are float32
    np.testing.assert_array_equal(r["mass"], d["mass"])  # per-type masses travel in Massarr


@pytest.mark.skipif(not os.environ.get("ASTRONBODYSIM_REF"),
                    reason="set ASTRONBODYSIM_REF to a checkout of the reference project")
def test_reference_fixture_byte_identical_rewrite(tmp_path):
    path = os.path.join(os.environ["ASTRONBODYSIM_REF"], "examples", "04-collisions",
                        "galaxy_littleendian.dat")
    h, d = g2.read_gadget2(path)
    p = tmp_path / "re.dat"
    g2.write_gadget2(str(p), h, d)
    assert p.read_bytes() == open(path, "rb").read()


def test_format_errors(tmp_path):
    rng = np.random.default_rng(5)
    d = _system(10, rng)
    p = tmp_path / "s.dat"
    g2.write_gadget2(str(p), g2.make_header([0] * 6), d)
    buf = bytearray(p.read_bytes())
    bad = tmp_path / "bad.dat"
    b1 = bytearray(buf)
    struct.pack_into("<i", b1, 260, 255)  # trailing HEAD marker
    bad.write_bytes(bytes(b1))
    with pytest.raises(g2.Gadget2FormatError):
        g2.read_gadget2(str(bad))
    bad.write_bytes(bytes(buf[:-3]))
    with pytest.raises(g2.Gadget2FormatError):
        g2.read_gadget2(str(bad))
    bad.write_bytes(b"\x01\x01\x00\x00" + bytes(buf[4:]))  # first record of 257 bytes
    with pytest.raises(g2.Gadget2FormatError):
        g2.read_gadget2(str(bad))


def test_internal_G():
    # Gadget-2 internal units: kpc, km/s, 1e10 Msun -> G of about 43 000
    assert abs(g2.internal_G() - 43022.0) < 5.0
