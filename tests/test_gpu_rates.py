"""The rate micro-benchmarks behind the roofline denominators beyond the HBM copy
and bf16 GEMM rates (hyp_measure_peaks: FMA throughput and host-link copies; hyp_measure_layouts:
the mixed step's traffic in the two state layouts): they run, return finite positive
rates in a plausible order, and reject bad arguments."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _call(hyp, fn, *args, n):
    out = np.zeros(n)
    rc = getattr(hyp._lib.load(), fn)(*args, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    return rc, out


def test_measure_peaks(hyp):
    rc, out = _call(hyp, "hyp_measure_peaks", 1, 64 << 20, n=6)
    assert rc == hyp._lib.HYP_OK
    assert np.all(np.isfinite(out)) and np.all(out > 0)
    fp64, fp32, fp32x2 = out[:3]
    assert fp64 < fp32 and fp32x2 > 0.5 * fp32  # GB300: FP64 at 1/64 of FP32
    assert _call(hyp, "hyp_measure_peaks", 0, 64 << 20, n=6)[0] == hyp._lib.HYP_ERR_INVALID
    assert _call(hyp, "hyp_measure_peaks", 1, 1024, n=6)[0] == hyp._lib.HYP_ERR_INVALID


def test_measure_layouts(hyp):
    rc, out = _call(hyp, "hyp_measure_layouts", 1, 1 << 20, n=2)
    assert rc == hyp._lib.HYP_OK
    assert np.all(np.isfinite(out)) and np.all(out > 100.0)  # GB/s
    assert _call(hyp, "hyp_measure_layouts", 1, 100, n=2)[0] == hyp._lib.HYP_ERR_INVALID
