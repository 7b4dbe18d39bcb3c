"""GPU test of nb_force_noalloc, the force entry point that allocates no device
memory, for callers that cannot let the library call cudaMalloc (a Julia host
whose device arrays all come from CUDA.jl's pooled allocator, or a serving
process that reserves its HBM budget up front).

The caller's device arrays come from torch here.  The entry point is compared
with the handle path (nb_compute_force, mixed precision) on two calls in a row;
the two calls share the library's fixed scratch array, so the second call also
checks that nothing left over from the first one leaks into its result.  The
tolerance is the mixed-precision force tolerance of the other GPU tests
(relative 1e-5 per particle); the two paths run the same kernels, so the
results normally agree bit for bit.
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


@pytest.mark.parametrize("law", ["spline", "plummer"])
def test_noalloc_matches_handle_path_twice(nb, law):
    torch = pytest.importorskip("torch")
    from astronbodysim import _lib as L

    lib = L.load()
    n, h, G = 20000, 0.01, 1.5
    d = nb.plummer(n, seed=21)
    sim = nb.Simulation(d, G=G, ForceSofteningTable=[h] * 6, TimeStep=1e-3, precision="mixed",
                        law=law)
    nb.compute_force(sim, want_potential=True)
    ref = nb.get_all_data(sim)
    cols = [_dev(torch, d["pos"][:, k]) for k in range(3)] + [_dev(torch, d["mass"])]
    ilaw = L.NB_LAW_SPLINE_G2 if law == "spline" else L.NB_LAW_PLUMMER
    for call in range(2):
        outs = [torch.full((n,), float("nan"), dtype=torch.float64, device="cuda:0") for _ in range(4)]
        rc, msg = _call(lib, torch, n, cols, ilaw, G, h, outs)
        assert rc == L.NB_OK, msg
        torch.cuda.synchronize()
        acc = torch.stack(outs[:3], 1).cpu().numpy()
        pot = outs[3].cpu().numpy()
        e = np.linalg.norm(acc - ref["acc"], axis=1) / np.linalg.norm(ref["acc"], axis=1)
        ep = np.abs(pot - ref["pot"]) / np.abs(ref["pot"])
        assert np.all(np.isfinite(acc)) and np.all(np.isfinite(pot)), call
        assert e.max() <= 1e-5, (call, e.max())
        assert ep.max() <= 1e-5, (call, ep.max())


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
