"""GPU tests of the many-system engine (batching / continuous-batching serving)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def systems(nb, sizes, seed=0):
    out = []
    for k, n in enumerate(sizes):
        d = nb.plummer(n, seed=seed + k) if k % 2 == 0 else nb.hernquist(n, seed=seed + k)
        out.append(d)
    return out


def test_engine_matches_single_system_path(nb):
    """Each system of a batch follows the single-system run(sim) trajectory.
    Both are mixed precision but group sources into different tiles (14- vs
    21-bit Morton keys), so forces differ at the FP32 level (~1e-7 relative);
    over 20 steps positions agree to 1e-8 and velocities to 1e-6."""
    sizes = [300, 1000, 3000, 257]
    softs = [0.01, 0.005, 0.002, 0.02]
    dt, nsteps = 1e-3, 20
    ds = systems(nb, sizes, seed=3)
    eng = nb.Engine(max_particles=1 << 16, max_systems=64)
    ids = [eng.submit(d, s, dt, nsteps) for d, s in zip(ds, softs)]
    eng.run_until_idle()
    for d, s, rid, n in zip(ds, softs, ids, sizes):
        assert eng.poll(rid)[0] == nb._lib.NB_REQ_DONE
        got = eng.fetch(rid, n)
        sim = nb.Simulation(d, ForceSofteningTable=[s] * 6, TimeStep=dt, TimeEnd=1.0, precision="mixed")
        nb.run(sim, nsteps=nsteps)
        ref = nb.get_all_data(sim)
        np.testing.assert_allclose(got["pos"], ref["pos"], rtol=0, atol=1e-8)
        np.testing.assert_allclose(got["vel"], ref["vel"], rtol=0, atol=1e-6)
    st = eng.stats()
    assert st["done"] == len(sizes) and st["running"] == 0 and st["queued"] == 0
    assert st["interactions"] == pytest.approx(nsteps * sum(n * n for n in sizes))


def test_engine_vs_oracle(nb, oracle):
    d = nb.plummer(1500, seed=41)
    h, dt, nsteps = 0.01, 1e-3, 25
    eng = nb.Engine(max_particles=1 << 14, max_systems=8)
    rid = eng.submit(d, h, dt, nsteps)
    eng.run_until_idle()
    got = eng.fetch(rid, 1500)
    o = oracle.OracleSim(d["pos"], d["vel"], d["mass"], soft=[h] * 6, dt=dt, time_end=1.0)
    o.run_begin()
    o.step(nsteps)
    o.run_end()
    np.testing.assert_allclose(got["pos"], o.pos, rtol=0, atol=1e-7)
    np.testing.assert_allclose(got["vel"], o.vel, rtol=0, atol=1e-5)


def test_same_alone_and_in_the_mix(nb):
    """A system's result does not depend on the other systems (bit-identical):
    whole i-blocks per work item, per-system Morton keys."""
    target = nb.plummer(2000, seed=7)
    others = systems(nb, [512, 4096, 1000, 3333], seed=11)
    dt, h = 1e-3, 0.004
    alone = nb.Engine(max_particles=1 << 15, max_systems=16)
    ra = alone.submit(target, h, dt, 40)
    alone.run_until_idle()
    a = alone.fetch(ra, 2000)
    mix = nb.Engine(max_particles=1 << 15, max_systems=16, max_steps_per_call=7)
    r0 = mix.submit(others[0], 0.01, dt, 13)       # retires during the target's run
    r1 = mix.submit(others[1], 0.002, dt, 60)
    mix.run(5)                                      # others already running
    rt = mix.submit(target, h, dt, 40)
    mix.run(9)
    r2 = mix.submit(others[2], 0.006, dt, 25)       # admitted mid-run
    r3 = mix.submit(others[3], 0.003, dt, 3)
    mix.run_until_idle()
    b = mix.fetch(rt, 2000)
    np.testing.assert_array_equal(a["pos"], b["pos"])
    np.testing.assert_array_equal(a["vel"], b["vel"])
    for rid in (r0, r1, r2, r3):
        assert mix.poll(rid)[0] == nb._lib.NB_REQ_DONE


def test_admission_by_footprint(nb):
    """Only systems that fit the arena are resident; the rest queue (FIFO)."""
    ds = systems(nb, [3000, 3000, 3000], seed=21)
    eng = nb.Engine(max_particles=5000, max_systems=8, max_steps_per_call=4)
    ids = [eng.submit(d, 0.01, 1e-3, 8) for d in ds]
    eng.run(1)
    st = eng.stats()
    assert st["running"] == 1 and st["queued"] == 2 and st["resident_particles"] == 3000
    states = [eng.poll(r)[0] for r in ids]
    assert states == [nb._lib.NB_REQ_RUNNING, nb._lib.NB_REQ_QUEUED, nb._lib.NB_REQ_QUEUED]
    eng.run_until_idle()
    assert all(eng.poll(r)[0] == nb._lib.NB_REQ_DONE for r in ids)


def test_engine_errors_and_cancel(nb):
    eng = nb.Engine(max_particles=4096, max_systems=4)
    big = nb.plummer(5000, seed=1)
    with pytest.raises(nb.NbodyError) as ei:
        eng.submit(big, 0.01, 1e-3, 10)
    assert ei.value.code == nb._lib.NB_ERR_ADMISSION
    d = nb.plummer(1000, seed=2)
    r1 = eng.submit(d, 0.01, 1e-3, 10)
    r2 = eng.submit(d, 0.01, 1e-3, 10)
    eng.cancel(r2)
    assert eng.poll(r2)[0] == nb._lib.NB_REQ_CANCELLED
    with pytest.raises(nb.NbodyError):
        eng.fetch(r1, 1000)  # not finished
    eng.run_until_idle()
    assert eng.poll(r1)[0] == nb._lib.NB_REQ_DONE
    with pytest.raises(nb.NbodyError):
        eng.poll(999999)


@pytest.mark.parametrize("n", [2000, 20000])
@pytest.mark.parametrize("at", [21, 32])
def test_suspend_resume_is_bit_identical(nb, n, at):
    """A system evicted to the host after `at` steps (mid re-ordering period,
    and on a re-ordering step), kept out while others run, then resumed,
    ends bit-identical to the uninterrupted run.  n = 20000 is ordered by the
    global radix sort, n = 2000 in shared memory."""
    target = nb.plummer(n, seed=61)
    others = systems(nb, [700, 3000], seed=62)
    dt, nsteps = 1e-3, 60

    ref_eng = nb.Engine(max_particles=1 << 16, max_systems=8, max_steps_per_call=8)
    rid = ref_eng.submit(target, 0.01, dt, nsteps)
    ref_eng.run_until_idle()
    ref = ref_eng.fetch(rid, n)

    eng = nb.Engine(max_particles=1 << 16, max_systems=8, max_steps_per_call=at)
    tid = eng.submit(target, 0.01, dt, nsteps)
    oids = [eng.submit(d, 0.005, dt, 100) for d in others]
    eng.run()  # admits all, advances `at` steps
    assert eng.poll(tid) == (nb._lib.NB_REQ_RUNNING, at)
    eng.suspend(tid)
    assert eng.poll(tid)[0] == nb._lib.NB_REQ_SUSPENDED
    assert eng.stats()["running"] == 2
    eng.run(5)  # the others move on
    eng.resume(tid)
    eng.run_until_idle()
    got = eng.fetch(tid, n)
    np.testing.assert_array_equal(got["pos"], ref["pos"])
    np.testing.assert_array_equal(got["vel"], ref["vel"])
    for rid_, d in zip(oids, others):
        assert eng.poll(rid_)[0] == nb._lib.NB_REQ_DONE


def test_suspend_errors(nb):
    eng = nb.Engine(max_particles=1 << 14, max_systems=4)
    rid = eng.submit(nb.plummer(500, seed=63), 0.01, 1e-3, 10)
    with pytest.raises(nb.NbodyError):
        eng.suspend(rid)  # queued, not running
    with pytest.raises(nb.NbodyError):
        eng.resume(rid)  # not suspended
    eng.run(3)
    eng.suspend(rid)
    with pytest.raises(nb.NbodyError):
        eng.fetch(rid, 500)  # not finished
    eng.cancel(rid)
    assert eng.poll(rid)[0] == nb._lib.NB_REQ_CANCELLED


@pytest.mark.parametrize("shape", [(128, 1), (256, 1), (256, 2)])
def test_engine_launch_shapes_agree(nb, shape):
    """Every batch-force shape gives the default shape's trajectories to FP32
    round-off, and stays mix-independent (bit-identical alone and in a mix)."""
    ds = systems(nb, [300, 2000, 5000], seed=81)
    dt, nsteps = 1e-3, 10
    runs = {}
    for sh in [(128, 2), shape]:
        eng = nb.Engine(max_particles=1 << 15, max_systems=8, block=sh[0], i_per_thread=sh[1])
        ids = [eng.submit(d, 0.01, dt, nsteps) for d in ds]
        eng.run_until_idle()
        runs[sh] = [eng.fetch(i, d["pos"].shape[0]) for i, d in zip(ids, ds)]
    for a, b in zip(runs[(128, 2)], runs[shape]):
        np.testing.assert_allclose(a["pos"], b["pos"], rtol=0, atol=1e-9)
        np.testing.assert_allclose(a["vel"], b["vel"], rtol=0, atol=1e-7)
    eng = nb.Engine(max_particles=1 << 15, max_systems=8, block=shape[0], i_per_thread=shape[1])
    rid = eng.submit(ds[1], 0.01, dt, nsteps)
    eng.run_until_idle()
    alone = eng.fetch(rid, 2000)
    np.testing.assert_array_equal(alone["pos"], runs[shape][1]["pos"])
    np.testing.assert_array_equal(alone["vel"], runs[shape][1]["vel"])


def test_engine_rejects_unknown_shape(nb):
    with pytest.raises(nb.NbodyError):
        nb.Engine(max_particles=1 << 12, max_systems=4, block=512, i_per_thread=1)


def test_run_async_matches_blocking_run(nb):
    """Chunks launched with run_async (completed by the next call) and systems
    submitted while a chunk runs give results bit-identical to the same
    systems run with the blocking run()."""
    sizes = [400, 1500, 260, 3000, 900]
    softs = [0.01, 0.004, 0.02, 0.003, 0.008]
    steps = [30, 17, 45, 22, 9]
    ds = systems(nb, sizes, seed=21)
    out = {}
    for mode in ("blocking", "async"):
        eng = nb.Engine(max_particles=1 << 15, max_systems=16, max_steps_per_call=8)
        ids = {}
        if mode == "blocking":
            for k in range(5):
                ids[k] = eng.submit(ds[k], softs[k], 1e-3, steps[k])
            eng.run_until_idle()
        else:
            for k in range(2):
                ids[k] = eng.submit(ds[k], softs[k], 1e-3, steps[k])
            launched = eng.run_async(8)
            assert launched == 8
            # submitted while the first chunk runs; admitted at the next boundary
            for k in range(2, 5):
                ids[k] = eng.submit(ds[k], softs[k], 1e-3, steps[k])
            while True:
                st = eng.stats()
                if eng.run_async(8) == 0 and st["queued"] == 0:
                    break
            eng.sync()
        for k in range(5):
            assert eng.poll(ids[k])[0] == nb._lib.NB_REQ_DONE, (mode, k)
            out[(mode, k)] = eng.fetch(ids[k], sizes[k])
        eng.close()
    for k in range(5):
        np.testing.assert_array_equal(out[("async", k)]["pos"], out[("blocking", k)]["pos"])
        np.testing.assert_array_equal(out[("async", k)]["vel"], out[("blocking", k)]["vel"])


def test_systems_finishing_inside_a_chunk_are_held(nb):
    """A chunk runs as long as the resident system with the most steps left
    needs (up to max_steps_per_call); a system that makes its last step
    inside it is held on the device (no drift, force, kick or count) until the
    chunk ends.  Its result is bit-identical to running it alone, including a
    system of 0 steps (only the two half kicks), and the interaction count
    covers the steps actually made."""
    ds = systems(nb, [700, 1500, 300], seed=81)
    steps = [5, 40, 0]
    dt = 1e-3
    alone = []
    for d, k in zip(ds, steps):
        e1 = nb.Engine(max_particles=1 << 13, max_systems=4, max_steps_per_call=16)
        r = e1.submit(d, 0.01, dt, k)
        e1.run_until_idle()
        alone.append(e1.fetch(r, d["pos"].shape[0]))
        e1.close()
    eng = nb.Engine(max_particles=1 << 13, max_systems=4, max_steps_per_call=16)
    ids = [eng.submit(d, 0.01, dt, k) for d, k in zip(ds, steps)]
    assert eng.run() == 16                       # set by the 40-step system, not the 5-step one
    assert eng.poll(ids[0]) == (nb._lib.NB_REQ_DONE, 5)
    assert eng.poll(ids[2]) == (nb._lib.NB_REQ_DONE, 0)
    assert eng.poll(ids[1]) == (nb._lib.NB_REQ_RUNNING, 16)
    eng.run_until_idle()
    for d, rid, ref in zip(ds, ids, alone):
        got = eng.fetch(rid, d["pos"].shape[0])
        np.testing.assert_array_equal(got["pos"], ref["pos"])
        np.testing.assert_array_equal(got["vel"], ref["vel"])
    st = eng.stats()
    assert st["interactions"] == pytest.approx(sum(d["pos"].shape[0] ** 2 * k for d, k in zip(ds, steps)))


def test_large_systems_alone_and_in_the_mix(nb):
    """Systems above the shared-memory sort limit (16384) are ordered by a radix
    sort over their own particles only, at compact offsets.  Two of them among
    small systems end bit-identical to each running alone, whatever their
    ranks and arena places."""
    big = systems(nb, [20000, 17000], seed=91)
    small = systems(nb, [900, 3000, 500], seed=95)
    dt, steps = 1e-3, 12
    alone = []
    for d in big:
        e1 = nb.Engine(max_particles=1 << 16, max_systems=4, max_steps_per_call=5)
        r = e1.submit(d, 0.005, dt, steps)
        e1.run_until_idle()
        alone.append(e1.fetch(r, d["pos"].shape[0]))
        e1.close()
    eng = nb.Engine(max_particles=1 << 17, max_systems=8, max_steps_per_call=5)
    s0 = eng.submit(small[0], 0.01, dt, 30)
    b0 = eng.submit(big[0], 0.005, dt, steps)
    s1 = eng.submit(small[1], 0.01, dt, 7)
    eng.run(3)
    b1 = eng.submit(big[1], 0.005, dt, steps)
    s2 = eng.submit(small[2], 0.01, dt, 9)
    eng.run_until_idle()
    for rid, d, ref in ((b0, big[0], alone[0]), (b1, big[1], alone[1])):
        got = eng.fetch(rid, d["pos"].shape[0])
        np.testing.assert_array_equal(got["pos"], ref["pos"])
        np.testing.assert_array_equal(got["vel"], ref["vel"])
    for rid in (s0, s1, s2):
        assert eng.poll(rid)[0] == nb._lib.NB_REQ_DONE
