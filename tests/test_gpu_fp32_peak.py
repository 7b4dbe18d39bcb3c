"""GPU test of the FP32 throughput probe that sets the roofline's denominator
(nb_selftest_fp32_peak): a chain of independent fma.rn.f32x2 on every SM,
timed with CUDA events, 2 flop per FMA lane.  On a GB300 it reads about
80 TFLOP/s (152 SMs x 128 lanes x 2 x 2.07 GHz = 80.5 nominal); the bounds
here only catch a broken probe (a kernel that does no work, or a unit error)."""
import ctypes

import pytest

pytestmark = pytest.mark.gpu


def test_fp32_peak_probe_reads_a_plausible_rate(nb):
    from astronbodysim import _lib as L

    lib = L.load()
    tf, ms = ctypes.c_double(), ctypes.c_double()
    assert lib.nb_selftest_fp32_peak(0, 1, ctypes.byref(tf), ctypes.byref(ms)) == L.NB_OK
    assert 40.0 <= tf.value <= 100.0, tf.value
    assert ms.value > 0.0
