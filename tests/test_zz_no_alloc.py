"""GPU test of nb_force_noalloc, the force entry point that allocates no device
memory, for callers that cannot let the library call cudaMalloc (a Julia host
whose device arrays all come from CUDA.jl's pooled allocator, or a serving
process that reserves its HBM budget up front).

The caller's device arrays come from torch here.  The entry point is compared
with the handle path (nb_compute_force, mixed precision) on two calls in a row;
the two calls share the library's fixed scratch array, so the second call also
checks that nothing left over from the first one leaks into its result.  The
handle path runs the same kernels with another launch shape, so the FP32 sums
differ in order: the tolerance is the mixed-precision bar of the other GPU
tests (relative force and potential error: median <= 1e-6, p99 <= 1e-5,
max <= 1e-4).  Sizes: one particle, a partial tile, a mid size and the
maximum; with and without the potential.  A warm call must leave the device's
free memory unchanged.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_PARTICLES = 65536


def _dev(torch, a):
    return torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda:0")


def _call(lib, torch, n, cols, law, G, h, outs, want_pot=True):
    buf = ctypes.create_string_buffer(512)
    stream = torch.cuda.current_stream().cuda_stream
    ptr = lambda t: ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p()
    rc = lib.nb_force_noalloc(n, *[ptr(c) for c in cols], law, G, h,
                              *[ptr(o) for o in outs[:3]], ptr(outs[3] if want_pot else None),
                              ctypes.c_void_p(stream), buf, len(buf))
    return rc, buf.value.decode()


def _within_bar(got, ref):
    e = np.abs(got - ref) / np.maximum(np.abs(ref), 1e-300)
    return np.median(e) <= 1e-6 and np.quantile(e, 0.99) <= 1e-5 and e.max() <= 1e-4


@pytest.mark.parametrize("law", ["spline", "plummer"])
@pytest.mark.parametrize("n", [1, 257, 20000, MAX_PARTICLES])
@pytest.mark.parametrize("want_pot", [True, False])
def test_noalloc_matches_handle_path_twice(nb, law, n, want_pot):
    torch = pytest.importorskip("torch")
    from astronbodysim import _lib as L

    lib = L.load()
    h, G = 0.01, 1.5
    d = nb.plummer(n, seed=21) if n > 1 else {"pos": np.array([[0.3, -0.2, 0.1]]),
                                              "vel": np.zeros((1, 3)), "mass": np.ones(1)}
    sim = nb.Simulation(d, G=G, ForceSofteningTable=[h] * 6, TimeStep=1e-3, precision="mixed",
                        law=law)
    nb.compute_force(sim, want_potential=True)
    ref = nb.get_all_data(sim)
    cols = [_dev(torch, d["pos"][:, k]) for k in range(3)] + [_dev(torch, d["mass"])]
    ilaw = L.NB_LAW_SPLINE_G2 if law == "spline" else L.NB_LAW_PLUMMER
    for call in range(2):
        outs = [torch.full((n,), float("nan"), dtype=torch.float64, device="cuda:0") for _ in range(4)]
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        rc, msg = _call(lib, torch, n, cols, ilaw, G, h, outs, want_pot)
        assert rc == L.NB_OK, msg
        torch.cuda.synchronize()
        if call == 1:
            # the warm call takes no device memory
            assert torch.cuda.mem_get_info()[0] == free0
        acc = torch.stack(outs[:3], 1).cpu().numpy()
        assert np.all(np.isfinite(acc)), call
        if n == 1:
            assert np.all(acc == 0.0) and np.all(ref["acc"] == 0.0)
        else:
            na = np.linalg.norm(acc - ref["acc"], axis=1)
            e = na / np.linalg.norm(ref["acc"], axis=1)
            assert np.median(e) <= 1e-6 and np.quantile(e, 0.99) <= 1e-5 and e.max() <= 1e-4, call
        pot = outs[3].cpu().numpy()
        if want_pot:
            assert np.all(np.isfinite(pot)), call
            if n == 1:
                assert pot[0] == ref["pot"][0]
            else:
                assert _within_bar(pot, ref["pot"]), call
        else:
            assert np.all(np.isnan(pot)), "pot must stay untouched without a potential"


def test_noalloc_rejects_sizes_beyond_maximum(nb):
    torch = pytest.importorskip("torch")
    from astronbodysim import _lib as L

    lib = L.load()
    n = MAX_PARTICLES + 1
    cols = [torch.zeros(n, dtype=torch.float64, device="cuda:0") for _ in range(4)]
    outs = [torch.zeros(n, dtype=torch.float64, device="cuda:0") for _ in range(4)]
    rc, msg = _call(lib, torch, n, cols, L.NB_LAW_SPLINE_G2, 1.0, 0.01, outs)
    assert rc == L.NB_ERR_INVALID_ARG
    assert "65537" in msg and "65536" in msg
