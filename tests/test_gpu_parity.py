"""GPU parity: libnbody_gb300.so through its C ABI against the oracle and the
golden known answers.  Tolerances:
  FP64 form   : |a_gpu - a_oracle| <= 1e-12 |a_oracle| per force (and potential)
  mixed form  : median relative force error <= 1e-6, p99 <= 1e-5, max <= 1e-4
                (sources in Morton order, FP32 pairs relative to FP64 tile origins)
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def make_sim(nb, data, **kw):
    return nb.Simulation(data, **kw)


def rel_err(a, b):
    return np.linalg.norm(a - b, axis=-1) / np.linalg.norm(b, axis=-1)


@pytest.fixture(scope="module")
def plummer4096(nb):
    return nb.plummer(4096, seed=1)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_binary_static(nb, golden, precision):
    """test/StaticTest.jl:161-207 through the GPU path."""
    g = golden("binary_static.json")
    data = {"pos": np.array(g["pos"]), "vel": np.array(g["vel"]), "mass": np.full(2, g["mass"])}
    sim = make_sim(nb, data, G=g["G"], ForceSofteningTable=[g["softening"]] * 6,
                   ErrTolTimestep=g["eta"], precision=precision)
    nb.compute_force(sim)
    d = nb.get_all_data(sim)
    a = d["acc"]
    rtol = g["rtol"] if precision == "fp64" else 1e-6
    assert abs(a[0, 0] + a[1, 0]) <= rtol * abs(a[0, 0])
    np.testing.assert_allclose(abs(a[:, 0]), g["acc_abs"], rtol=rtol)
    np.testing.assert_allclose(nb.total_potential(sim), g["potential"], rtol=rtol)
    np.testing.assert_allclose(nb.total_kinetic(sim), g["kinetic"], rtol=g["rtol"])
    np.testing.assert_allclose(nb.total_energy(sim), g["energy"], rtol=rtol)
    nb.init_timesteps(sim)
    d = nb.get_all_data(sim)
    dt_sim = (d["ti_endstep"][0] - d["ti_begstep"][0]) * sim.TimeInterval
    assert dt_sim < g["dt_bound"]
    P = nb.total_momentum(sim)
    assert np.all(np.abs(P) <= g["rtol"] * g["mass"] * abs(g["vel"][0][1]))
    np.testing.assert_allclose(nb.total_angular_momentum(sim), g["angular_momentum"],
                               rtol=g["rtol"], atol=1e-30)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_box_probe(nb, golden, precision):
    """test/StaticTest.jl:299-350: force and potential at a probe point."""
    g = golden("box_probe.json")
    pos = np.array(g["pos"])
    data = {"pos": pos, "vel": np.zeros_like(pos), "mass": np.full(len(pos), g["mass"])}
    sim = make_sim(nb, data, G=g["G"], ForceSofteningTable=[g["softening"]] * 6, precision=precision)
    acc, pot = nb.force_and_potential_at_points(sim, np.array([g["probe"]]), g["softening"])
    rtol = 1e-14 if precision == "fp64" else 2e-6
    np.testing.assert_allclose(acc[0], g["acc"], rtol=rtol)
    np.testing.assert_allclose(pot[0], g["pot"], rtol=rtol)


@pytest.mark.parametrize("law", ["spline", "plummer"])
def test_fp64_force_matches_oracle_1e12(nb, oracle, plummer4096, law):
    """Plain FP64 GPU form vs the CPU Float64 direct sum: <= 1e-12 relative per force."""
    d = plummer4096
    h = 0.01
    sim = make_sim(nb, d, ForceSofteningTable=[h] * 6, precision="fp64", law=law)
    nb.compute_force(sim, want_potential=True)
    g = nb.get_all_data(sim)
    olaw = oracle.LAW_SPLINE_G2 if law == "spline" else oracle.LAW_PLUMMER
    a_ref, p_ref = oracle.force(d["pos"], d["mass"], d["pos"], h, law=olaw)
    e = rel_err(g["acc"], a_ref)
    assert e.max() <= 1e-12, e.max()
    ep = np.abs(g["pot"] - p_ref) / np.abs(p_ref)
    assert ep.max() <= 1e-12, ep.max()


@pytest.mark.parametrize("law", ["spline", "plummer"])
def test_mixed_force_error_quantiles(nb, oracle, plummer4096, law):
    d = plummer4096
    h = 0.01
    sim = make_sim(nb, d, ForceSofteningTable=[h] * 6, precision="mixed", law=law)
    nb.compute_force(sim, want_potential=True)
    g = nb.get_all_data(sim)
    olaw = oracle.LAW_SPLINE_G2 if law == "spline" else oracle.LAW_PLUMMER
    a_ref, p_ref = oracle.force(d["pos"], d["mass"], d["pos"], h, law=olaw)
    e = rel_err(g["acc"], a_ref)
    ep = np.abs(g["pot"] - p_ref) / np.abs(p_ref)
    assert np.median(e) <= 1e-6, np.median(e)
    assert np.quantile(e, 0.99) <= 1e-5, np.quantile(e, 0.99)
    assert e.max() <= 1e-4, e.max()
    assert np.median(ep) <= 1e-6 and np.quantile(ep, 0.99) <= 1e-5


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("n", [1, 2, 3, 255, 256, 257, 1000])
def test_ragged_sizes(nb, oracle, precision, n):
    """Ragged tiles, single particle (zero force), tiny systems."""
    d = nb.plummer(n, seed=n) if n > 1 else {"pos": np.zeros((1, 3)) + 0.25, "vel": np.zeros((1, 3)),
                                              "mass": np.ones(1)}
    h = 0.05
    sim = make_sim(nb, d, ForceSofteningTable=[h] * 6, precision=precision)
    nb.compute_force(sim, want_potential=True)
    g = nb.get_all_data(sim)
    a_ref, p_ref = oracle.force(d["pos"], d["mass"], d["pos"], h)
    if n == 1:
        assert np.all(g["acc"] == 0.0) and g["pot"][0] == 0.0
        return
    e = rel_err(g["acc"], a_ref)
    if precision == "fp64":
        assert e.max() <= 1e-12, e.max()
    else:
        assert np.median(e) <= 1e-6 and e.max() <= 1e-4, (np.median(e), e.max())


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_close_pairs_spline_branch(nb, oracle, precision):
    """Particles inside each other's softening length exercise r < h, both
    spline segments, and exactly coincident particles (r == 0)."""
    rng = np.random.default_rng(7)
    n = 600
    pos = rng.normal(scale=0.02, size=(n, 3))
    pos[10] = pos[11]  # coincident pair
    d = {"pos": pos, "vel": np.zeros_like(pos), "mass": rng.uniform(0.5, 1.5, n) / n}
    h = 0.02
    sim = make_sim(nb, d, ForceSofteningTable=[h] * 6, precision=precision)
    nb.compute_force(sim, want_potential=True)
    g = nb.get_all_data(sim)
    a_ref, p_ref = oracle.force(pos, d["mass"], pos, h)
    e = rel_err(g["acc"], a_ref)
    ep = np.abs(g["pot"] - p_ref) / np.abs(p_ref)
    if precision == "fp64":
        assert e.max() <= 1e-12 and ep.max() <= 1e-12
    else:
        assert np.median(e) <= 1e-5 and np.median(ep) <= 1e-6


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_far_offset_system(nb, oracle, precision):
    """A system far from the coordinate origin: the FP64 tile origins keep the
    mixed form's relative coordinates small."""
    d = nb.plummer(2048, seed=5)
    pos = d["pos"] + np.array([1.0e5, -3.0e4, 2.0e4])
    dd = {"pos": pos, "vel": d["vel"], "mass": d["mass"]}
    h = 0.01
    sim = make_sim(nb, dd, ForceSofteningTable=[h] * 6, precision=precision)
    nb.compute_force(sim)
    g = nb.get_all_data(sim)
    a_ref, _ = oracle.force(pos, d["mass"], pos, h)
    e = rel_err(g["acc"], a_ref)
    if precision == "fp64":
        assert e.max() <= 1e-10
    else:
        # positions ~1e5: FP32 relative coordinates within a tile keep ~1e-7 of the tile size
        assert np.median(e) <= 1e-4


def test_softening_table_by_type(nb, oracle):
    """Per-type softening (ForceSofteningTable indexed by Collection)."""
    d = nb.plummer(1024, seed=9)
    types = (np.arange(1024) % 6 + 1).astype(np.int32)
    table = [0.01, 0.02, 0.05, 0.1, 0.2, 0.3]
    dd = dict(d, collection=types)
    sim = make_sim(nb, dd, ForceSofteningTable=table, precision="fp64")
    nb.compute_force(sim, want_potential=True)
    g = nb.get_all_data(sim)
    th = np.array(table)[types - 1]
    a_ref, p_ref = oracle.force(d["pos"], d["mass"], d["pos"], th)
    assert rel_err(g["acc"], a_ref).max() <= 1e-12
    assert (np.abs(g["pot"] - p_ref) / np.abs(p_ref)).max() <= 1e-12


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_probe_points_match_oracle(nb, oracle, plummer4096, precision):
    d = plummer4096
    rng = np.random.default_rng(11)
    probes = rng.normal(size=(300, 3))
    sim = make_sim(nb, d, ForceSofteningTable=[0.01] * 6, precision=precision)
    acc, pot = nb.force_and_potential_at_points(sim, probes, 0.02)
    a_ref, p_ref = oracle.force(d["pos"], d["mass"], probes, 0.02)
    e = rel_err(acc, a_ref)
    ep = np.abs(pot - p_ref) / np.abs(p_ref)
    if precision == "fp64":
        assert e.max() <= 1e-12 and ep.max() <= 1e-12
    else:
        assert np.median(e) <= 1e-6 and e.max() <= 1e-4 and ep.max() <= 1e-5


def test_compute_potential_self_term(nb, oracle):
    """compute_potential(sim) adds +G m / (h / 2.8) as src/base/Potential.jl:5-24 does."""
    d = nb.plummer(512, seed=2)
    h = 0.01
    sim = make_sim(nb, d, ForceSofteningTable=[h] * 6, precision="fp64", G=2.0)
    nb.compute_potential(sim)
    g = nb.get_all_data(sim)
    _, p_ref = oracle.force(d["pos"], d["mass"], d["pos"], h, G=2.0)
    corr = 2.0 * d["mass"] / (h / 2.8)
    # the +2.8 G m / h term nearly cancels phi for some particles: bound the
    # error by the magnitude of the direct sum itself
    np.testing.assert_allclose(g["pot"], p_ref + corr, rtol=0, atol=1e-12 * np.abs(p_ref).max())


def test_invalid_arguments(nb):
    d = nb.plummer(64, seed=1)
    with pytest.raises(nb.NbodyError):
        nb.Simulation(d, ForceSofteningTable=[0.0] * 6)
    sim = nb.Simulation(d, ForceSofteningTable=[0.01] * 6)
    with pytest.raises(nb.NbodyError):
        nb.leapfrog_half_kick(sim, 2)
    with pytest.raises(nb.NbodyError):
        sim.upload(dict(d, collection=np.full(64, 9, dtype=np.int32)))
    with pytest.raises(nb.NbodyError):
        nb.set_softlen(sim, [0.01, 0.01, -1.0, 0.01, 0.01, 0.01])


@pytest.mark.parametrize("law", ["spline", "plummer"])
@pytest.mark.parametrize("n", [300, 5000, 70000])
def test_worklist_matches_direct_grid_and_is_deterministic(nb, oracle, law, n):
    """The persistent work-list force (block=-1) and the direct-grid force (block and
    i_per_thread given) agree; repeated evaluations are bit-identical."""
    d = nb.plummer(n, seed=31)
    h = 0.01
    a = nb.Simulation(d, ForceSofteningTable=[h] * 6, precision="mixed", law=law, block=-1)
    b = nb.Simulation(d, ForceSofteningTable=[h] * 6, precision="mixed", law=law, block=128,
                      i_per_thread=2)
    nb.compute_force(a, want_potential=True)
    ga = nb.get_all_data(a)
    nb.compute_force(a, want_potential=True)
    ga2 = nb.get_all_data(a)
    np.testing.assert_array_equal(ga["acc"], ga2["acc"])
    np.testing.assert_array_equal(ga["pot"], ga2["pot"])
    nb.compute_force(b, want_potential=True)
    gb = nb.get_all_data(b)
    assert rel_err(ga["acc"], gb["acc"]).max() <= 1e-6
    assert (np.abs(ga["pot"] - gb["pot"]) / np.abs(gb["pot"])).max() <= 1e-6
    if n <= 5000:
        olaw = oracle.LAW_SPLINE_G2 if law == "spline" else oracle.LAW_PLUMMER
        a_ref, _ = oracle.force(d["pos"], d["mass"], d["pos"], h, law=olaw)
        e = rel_err(ga["acc"], a_ref)
        assert np.median(e) <= 1e-6 and e.max() <= 1e-4


@pytest.mark.parametrize("law", ["spline", "plummer"])
@pytest.mark.parametrize("shape", [(128, 1, 2), (128, 2, 3), (256, 4, 4)])
@pytest.mark.parametrize("n", [300, 5000, 70000])
def test_j_split_matches_direct_grid_and_is_deterministic(nb, oracle, law, shape, n):
    """The direct grid with each i-block's source tiles split over j_split CTAs
    (partials joined in part order) agrees with the unsplit grid, is
    bit-identical between evaluations, and matches the oracle."""
    block, ipt, js = shape
    d = nb.plummer(n, seed=37)
    h = 0.01
    a = nb.Simulation(d, ForceSofteningTable=[h] * 6, precision="mixed", law=law, block=block,
                      i_per_thread=ipt, j_split=js)
    b = nb.Simulation(d, ForceSofteningTable=[h] * 6, precision="mixed", law=law, block=block,
                      i_per_thread=ipt)
    nb.compute_force(a, want_potential=True)
    ga = nb.get_all_data(a)
    nb.compute_force(a, want_potential=True)
    ga2 = nb.get_all_data(a)
    np.testing.assert_array_equal(ga["acc"], ga2["acc"])
    np.testing.assert_array_equal(ga["pot"], ga2["pot"])
    nb.compute_force(b, want_potential=True)
    gb = nb.get_all_data(b)
    assert rel_err(ga["acc"], gb["acc"]).max() <= 1e-6
    assert (np.abs(ga["pot"] - gb["pot"]) / np.abs(gb["pot"])).max() <= 1e-6
    if n <= 5000:
        olaw = oracle.LAW_SPLINE_G2 if law == "spline" else oracle.LAW_PLUMMER
        a_ref, p_ref = oracle.force(d["pos"], d["mass"], d["pos"], h, law=olaw)
        e = rel_err(ga["acc"], a_ref)
        assert np.median(e) <= 1e-6 and np.quantile(e, 0.99) <= 1e-5
        assert np.median(np.abs(ga["pot"] - p_ref) / np.abs(p_ref)) <= 1e-6


def test_j_split_adaptive_steps_match_unsplit(nb):
    """Adaptive block steps (active-subset forces through the device count) with
    j_split = 2 follow the unsplit run to FP32 round-off."""
    d = nb.plummer(3000, seed=41)
    kw = dict(ForceSofteningTable=[0.02] * 6, precision="mixed", ErrTolTimestep=0.025,
              MaxStep=1e-2, MinStep=1e-7, TimeEnd=0.05)
    a = nb.Simulation(d, block=128, i_per_thread=1, j_split=2, **kw)
    b = nb.Simulation(d, block=128, i_per_thread=1, **kw)
    nb.run(a)
    nb.run(b)
    ga, gb = nb.get_all_data(a), nb.get_all_data(b)
    # a timestep bin may flip where |a| sits on a power-of-two boundary
    assert np.mean(ga["ti_endstep"] == gb["ti_endstep"]) >= 0.99
    dp = np.abs(ga["pos"] - gb["pos"])
    assert np.median(dp) <= 1e-9 and dp.max() <= 1e-4


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_reupload_smaller_system_into_same_handle(nb, precision):
    """A handle that held 5000 particles and is re-uploaded with 3000 gives the
    forces of a fresh handle (no source tiles of the earlier upload remain)."""
    big = nb.plummer(5000, seed=43)
    small = nb.plummer(3000, seed=44)
    a = nb.Simulation(big, ForceSofteningTable=[0.01] * 6, precision=precision)
    nb.compute_force(a)
    a.upload(small)
    nb.compute_force(a, want_potential=True)
    b = nb.Simulation(small, ForceSofteningTable=[0.01] * 6, precision=precision)
    nb.compute_force(b, want_potential=True)
    ga, gb = nb.get_all_data(a), nb.get_all_data(b)
    np.testing.assert_array_equal(ga["acc"], gb["acc"])
    np.testing.assert_array_equal(ga["pot"], gb["pot"])


@pytest.mark.parametrize("law", ["spline", "plummer"])
def test_uniform_and_mixed_mass_tiles(nb, oracle, law):
    """Tiles whose sources share one mass take the far-tile loop with the mass
    applied once per tile; tiles with unequal masses the per-pair loop.  Both
    match the oracle, and a 1-ulp mass change on one particle (which moves its
    tile to the per-pair loop) changes no force beyond FP32 round-off."""
    n, h = 6000, 0.01
    d = nb.plummer(n, seed=97)
    d["mass"] = d["mass"].copy()
    d["mass"][n // 2:] *= np.random.default_rng(5).uniform(0.5, 1.5, n - n // 2)
    olaw = oracle.LAW_SPLINE_G2 if law == "spline" else oracle.LAW_PLUMMER
    sim = nb.Simulation(d, ForceSofteningTable=[h] * 6, precision="mixed", law=law)
    nb.compute_force(sim, want_potential=True)
    g = nb.get_all_data(sim)
    a_ref, p_ref = oracle.force(d["pos"], d["mass"], d["pos"], h, law=olaw)
    e = rel_err(g["acc"], a_ref)
    assert np.median(e) <= 1e-6 and np.quantile(e, 0.99) <= 1e-5
    assert np.median(np.abs(g["pot"] - p_ref) / np.abs(p_ref)) <= 1e-6

    u = nb.plummer(n, seed=98)
    v = dict(u, mass=u["mass"].copy())
    v["mass"][123] = np.nextafter(v["mass"][123], 1.0)
    ga, gb = [], []
    for dd, out in ((u, ga), (v, gb)):
        s = nb.Simulation(dd, ForceSofteningTable=[h] * 6, precision="mixed", law=law)
        nb.compute_force(s)
        out.append(nb.get_all_data(s)["acc"])
    assert rel_err(ga[0], gb[0]).max() <= 1e-6


def test_builtin_rule_at_large_n_matches_explicit_shape_and_oracle(nb, oracle):
    """Without a tuning table the library uses the direct grid with the
    j-split.  It agrees with an explicit unsplit shape and the oracle, repeats
    bit for bit, and survives re-uploads of smaller and larger systems into the
    same handle."""
    n, h = (1 << 17) + 5, 0.01
    d = nb.plummer(n, seed=101)
    a = nb.Simulation(d, ForceSofteningTable=[h] * 6, precision="mixed")
    b = nb.Simulation(d, ForceSofteningTable=[h] * 6, precision="mixed", block=128, i_per_thread=1)
    nb.compute_force(a)
    ga = nb.get_all_data(a)["acc"]
    nb.compute_force(a)
    np.testing.assert_array_equal(ga, nb.get_all_data(a)["acc"])
    nb.compute_force(b)
    # two mixed forms (tiles of 512, two targets per thread and the j-split
    # against tiles of 256, one target per thread unsplit) differ by their own
    # FP32 round-off: the mixed-form bars
    er = rel_err(ga, nb.get_all_data(b)["acc"])
    assert np.median(er) <= 1e-6 and np.quantile(er, 0.99) <= 1e-5 and er.max() <= 1e-4
    sub = np.arange(0, n, 512)
    a_ref, _ = oracle.force(d["pos"], d["mass"], d["pos"][sub], h)
    e = rel_err(ga[sub], a_ref)
    assert np.median(e) <= 1e-6 and np.quantile(e, 0.99) <= 1e-5
    small = nb.plummer(5000, seed=102)
    a.upload(small)
    nb.compute_force(a)
    c = nb.Simulation(small, ForceSofteningTable=[h] * 6, precision="mixed")
    nb.compute_force(c)
    np.testing.assert_array_equal(nb.get_all_data(a)["acc"], nb.get_all_data(c)["acc"])
    a.upload(d)
    nb.compute_force(a)
    np.testing.assert_array_equal(nb.get_all_data(a)["acc"], ga)
