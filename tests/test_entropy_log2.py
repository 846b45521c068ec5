"""The float-float log2 of the GPU entropy sums (host evaluation of the same code)
against the f64 log2: absolute error below 1e-12 over the count range a
(wavelength, bin) cell can hold."""
import ctypes as C
import math

import numpy as np


def test_entropy_log2_error_bound():
    from compound_prism_designer import _native as N

    rng = np.random.default_rng(3)
    bits = rng.integers(1, 54, 20000)
    vals = [int(rng.integers(0, 2 ** int(b), dtype=np.uint64)) | 1 for b in bits]
    vals += [1, 2, 3, 255, 256, 257, 2 ** 31, 2 ** 31 + 1, 2 ** 41 - 1, 2 ** 53 - 1]
    out = np.zeros(2)
    worst = 0.0
    for c in vals:
        assert N.lib.cpd_entropy_log2(C.c_uint64(c), out.ctypes.data_as(C.POINTER(C.c_double))) == 0
        err = abs((out[0] + out[1]) - math.log2(c))
        worst = max(worst, err)
    assert worst < 1e-12, worst
