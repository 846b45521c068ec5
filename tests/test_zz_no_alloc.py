"""The entry point that allocates no device memory.

cpd_fitness_gpu_points_static exists for callers that cannot call cudaMalloc: a host
application that owns the GPU memory budget and forbids plug-in libraries to allocate,
or a latency-critical loop that must not pay the synchronisation an allocation can
bring. It keeps all of its scratch in one fixed device array (W <= 1024, R <= 4096,
B <= 128) that every call reuses.

The tests call it through the C ABI twice in a row on the same design, in each trace
mode, and compare each result with the allocating entry point (cpd_fitness_gpu_points)
on the same points, with the tolerances of the other parity tests: p(d|lambda) within
1e-6 absolute and the mutual information within 1e-4 relative. The second call also
shows that what the first call left in the shared array does not leak into the next
result. One case compares with the oracle directly, one runs without the p(d|lambda)
output, and one runs a near-critical design at the largest sizes, where the fixed
re-trace queue may run out (the call must then say CPD_NO_CAPACITY, never return a
wrong result). This file is named so that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

import oracle as O
import compound_prism_designer as cpd
from compound_prism_designer import _native as N
from compound_prism_designer import precision as P
from compound_prism_designer import synth

pytestmark = pytest.mark.gpu


def _static_call(spec, lam_u, ray_u, mode=cpd.TRACE_HYBRID, want_p=True):
    lam_u = np.ascontiguousarray(lam_u, dtype=np.float64)
    ray_u = np.ascontiguousarray(ray_u, dtype=np.float64)
    B = spec.detector_array.bin_count
    f = N.Fitness()
    p = np.zeros((lam_u.size, B)) if want_p else None
    dp = C.POINTER(C.c_double)
    rc = N.lib.cpd_fitness_gpu_points_static(C.byref(spec.design), lam_u.ctypes.data_as(dp), lam_u.size,
                                             ray_u.ctypes.data_as(dp), ray_u.size, mode, C.byref(f),
                                             p.ctypes.data_as(dp) if want_p else None)
    return rc, f, p


def _cases(f1):
    rng = np.random.default_rng(77)
    cases = [synth.spectrometer_from_dict(f1)]
    s6, _, _ = synth.random_design(rng, 6, 64)
    s3, _, _ = synth.random_design(rng, 3, 128)
    return cases + [s6, s3]


@pytest.mark.parametrize("mode", [cpd.TRACE_HYBRID, cpd.TRACE_FP32, cpd.TRACE_FP64],
                         ids=["hybrid", "fp32", "fp64"])
def test_static_entry_matches_allocating_entry_on_two_calls(f1, mode):
    # CPD_TRACE_FP64 re-traces every ray through the fixed 32768-entry queue: W R <= 32768
    lam_u = O.qrng_points(0.5, 512 if mode != cpd.TRACE_FP64 else 24)
    ray_u = O.qrng_points(0.5, 1024)
    for spec in _cases(f1):
        ref, p_ref = spec.gpu_fitness_points(lam_u, ray_u, mode=mode, want_p=True)
        for call in range(2):
            rc, f, p = _static_call(spec, lam_u, ray_u, mode)
            assert rc == N.OK, (call, N.status_string(rc))
            assert np.abs(p - p_ref).max() <= 1e-6, call
            assert abs(f.info - ref.info) <= 1e-4 * abs(ref.info) + 1e-9, (call, f.info, ref.info)
            assert f.hits == ref.hits and f.wavelengths == ref.wavelengths
            assert f.retraced == ref.retraced


def test_static_entry_without_p_output(f1):
    spec = _cases(f1)[1]
    lam_u = O.qrng_points(0.5, 256)
    ray_u = O.qrng_points(0.5, 2048)
    ref, _ = spec.gpu_fitness_points(lam_u, ray_u)
    for _ in range(2):
        rc, f, _ = _static_call(spec, lam_u, ray_u, want_p=False)
        assert rc == N.OK, N.status_string(rc)
        assert abs(f.info - ref.info) <= 1e-4 * abs(ref.info) + 1e-9, (f.info, ref.info)
        assert f.hits == ref.hits


def test_static_entry_matches_the_oracle(f1):
    lam_u = O.qrng_points(0.5, 384)
    ray_u = O.qrng_points(0.5, 1536)
    d = f1
    po, st = O.fitness_points(d, lam_u, ray_u, nthreads=8)
    rc, f, p = _static_call(synth.spectrometer_from_dict(d), lam_u, ray_u)
    assert rc == N.OK, N.status_string(rc)
    assert np.abs(p - po).max() <= 1e-6
    assert abs(f.info - st["info"]) <= 1e-4 * abs(st["info"])
    assert f.hits == st["hits"]


def test_static_entry_near_critical_design_at_the_largest_sizes():
    spec = P.study_population(314, n=2, B=128)[0][0]  # exit face within 2 degrees of TIR
    lam_u = P.synth_points(0.5, 1024)
    ray_u = P.synth_points(0.5, 4096, first=1)
    ref, p_ref = spec.gpu_fitness_points(lam_u, ray_u, want_p=True)
    for _ in range(2):
        rc, f, p = _static_call(spec, lam_u, ray_u)
        if rc == N.NO_CAPACITY:
            # more guard-band rays than the fixed queue holds: refused, not truncated
            assert ref.retraced > 32768
            continue
        assert rc == N.OK, N.status_string(rc)
        assert np.abs(p - p_ref).max() <= 1e-6
        assert abs(f.info - ref.info) <= 1e-4 * abs(ref.info) + 1e-9
        assert f.hits == ref.hits


def test_static_entry_rejects_sizes_beyond_its_array(f1):
    spec = synth.spectrometer_from_dict(f1)
    rc, _, _ = _static_call(spec, O.qrng_points(0.5, 2048), O.qrng_points(0.5, 64))
    assert rc == N.NO_CAPACITY
    rc, _, _ = _static_call(spec, O.qrng_points(0.5, 16), O.qrng_points(0.5, 8192))
    assert rc == N.NO_CAPACITY
    # every ray of the FP64 mode goes through the re-trace queue
    rc, _, _ = _static_call(spec, O.qrng_points(0.5, 512), O.qrng_points(0.5, 1024), cpd.TRACE_FP64)
    assert rc == N.NO_CAPACITY
    # the array is still usable after a refused call
    rc, _, _ = _static_call(spec, O.qrng_points(0.5, 16), O.qrng_points(0.5, 256))
    assert rc == N.OK
