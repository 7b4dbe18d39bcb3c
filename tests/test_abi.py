"""CPU tests of the C ABI boundary: the library builds, loads, and exports every
entry point declared in include/*.h; host-only entry points behave."""
import ctypes
import glob
import os
import re

from conftest import REPO, gpu_available


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(REPO, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"\b(nb_[a-z0-9_]+)\s*\(", src):
            names.add(m.group(1))
    return names


def test_header_declares_core_api():
    names = declared_symbols()
    for n in ("nb_create", "nb_destroy", "nb_upload", "nb_download", "nb_compute_force",
              "nb_step", "nb_diagnostics", "nb_last_error"):
        assert n in names


def test_library_exports_every_declared_symbol(nb):
    from astronbodysim import _lib

    lib = ctypes.CDLL(_lib.library_path())
    missing = [n for n in sorted(declared_symbols()) if not hasattr(lib, n)]
    assert not missing, missing
    # the ctypes table covers exactly the declared API
    assert set(_lib.SIGNATURES) == declared_symbols()


def test_default_params_host_only(nb):
    from astronbodysim import _lib

    p = _lib.nb_params()
    _lib.load().nb_default_params(ctypes.byref(p))
    assert p.G == 1.0 and p.eta == 0.025 and p.min_step == 1e-8
    assert p.time_base == 1 << 30 and p.adaptive == 1
    assert list(p.softening) == [1e-4] * 6
    assert _lib.load().nb_version().startswith(b"nbody_gb300")


def test_create_without_gpu_fails_cleanly(nb):
    """Without a GPU nb_create returns NB_ERR_CUDA instead of crashing."""
    if gpu_available():
        return
    from astronbodysim import _lib

    p = _lib.nb_params()
    _lib.load().nb_default_params(ctypes.byref(p))
    h = ctypes.c_void_p()
    rc = _lib.load().nb_create(ctypes.byref(p), ctypes.byref(h))
    assert rc == _lib.NB_ERR_CUDA and not h.value


def test_invalid_params_rejected(nb):
    """Parameter validation runs before any device call."""
    from astronbodysim import _lib

    L = _lib.load()
    p = _lib.nb_params()
    L.nb_default_params(ctypes.byref(p))
    p.softening[2] = 0.0
    h = ctypes.c_void_p()
    assert L.nb_create(ctypes.byref(p), ctypes.byref(h)) == _lib.NB_ERR_INVALID_ARG
    L.nb_default_params(ctypes.byref(p))
    p.law = 7
    assert L.nb_create(ctypes.byref(p), ctypes.byref(h)) == _lib.NB_ERR_INVALID_ARG
    L.nb_default_params(ctypes.byref(p))
    p.adaptive = 0
    p.dt = 0.0
    assert L.nb_create(ctypes.byref(p), ctypes.byref(h)) == _lib.NB_ERR_INVALID_ARG
