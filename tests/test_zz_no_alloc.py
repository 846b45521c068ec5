"""The entry point that allocates no device memory.

cpd_fitness_gpu_points_static exists for callers that cannot call cudaMalloc: a host
application that owns the GPU memory budget and forbids plug-in libraries to allocate,
or a latency-critical loop that must not pay the synchronisation an allocation can
bring. It keeps all of its scratch in one fixed device array (W <= 1024, R <= 4096,
B <= 128) that every call reuses.

The test calls it through the C ABI twice in a row on the same design and compares each
result with the allocating entry point (cpd_fitness_gpu_points) on the same points, with
the tolerances of the other parity tests: p(d|lambda) within 1e-6 absolute and the
mutual information within 1e-4 relative. The second call also shows that what the first
call left in the shared array does not leak into the next result. This file is named so
that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

import oracle as O
import compound_prism_designer as cpd
from compound_prism_designer import _native as N
from compound_prism_designer import synth

pytestmark = pytest.mark.gpu


def _static_call(spec, lam_u, ray_u):
    lam_u = np.ascontiguousarray(lam_u, dtype=np.float64)
    ray_u = np.ascontiguousarray(ray_u, dtype=np.float64)
    B = spec.detector_array.bin_count
    f = N.Fitness()
    p = np.zeros((lam_u.size, B))
    dp = C.POINTER(C.c_double)
    rc = N.lib.cpd_fitness_gpu_points_static(C.byref(spec.design), lam_u.ctypes.data_as(dp), lam_u.size,
                                             ray_u.ctypes.data_as(dp), ray_u.size, cpd.TRACE_HYBRID, C.byref(f),
                                             p.ctypes.data_as(dp))
    return rc, f, p


def test_static_entry_matches_allocating_entry_on_two_calls(f1):
    rng = np.random.default_rng(77)
    cases = [synth.spectrometer_from_dict(f1)]
    s6, _, _ = synth.random_design(rng, 6, 64)
    s3, _, _ = synth.random_design(rng, 3, 128)
    cases += [s6, s3]
    lam_u = O.qrng_points(0.5, 512)
    ray_u = O.qrng_points(0.5, 1024)
    for spec in cases:
        ref, p_ref = spec.gpu_fitness_points(lam_u, ray_u, want_p=True)
        for call in range(2):
            rc, f, p = _static_call(spec, lam_u, ray_u)
            assert rc == N.OK, (call, N.status_string(rc))
            assert np.abs(p - p_ref).max() <= 1e-6, call
            assert abs(f.info - ref.info) <= 1e-4 * abs(ref.info) + 1e-9, (call, f.info, ref.info)
            assert f.hits == ref.hits and f.wavelengths == ref.wavelengths


def test_static_entry_rejects_sizes_beyond_its_array(f1):
    spec = synth.spectrometer_from_dict(f1)
    rc, _, _ = _static_call(spec, O.qrng_points(0.5, 2048), O.qrng_points(0.5, 64))
    assert rc == N.NO_CAPACITY
    rc, _, _ = _static_call(spec, O.qrng_points(0.5, 16), O.qrng_points(0.5, 8192))
    assert rc == N.NO_CAPACITY
