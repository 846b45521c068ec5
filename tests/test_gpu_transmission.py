"""Spectrometer.transmission_probability on the GPU against the oracle's restatement of
the reference's estimator, p_dets_l_wavelength (src/fitness.rs:5-34,48-69; the call of
src/pylib.rs:1028-1058).

The reference stops a wavelength at the first hit after which that hit's bin has
SEM <= 5e-3, pads every bin's Welford state to the ray count, and the bin that fired the
stop keeps a count one ahead. The GPU traces every ray in exact f64 and replays the
Welford updates in the reference's operation order, so the bar here is exact: the same
rays consumed per wavelength and the same p(d|lambda) bits (within the 1e-6 absolute bound
of the other parity tests, it is checked to be equal). fixed_n=True keeps the fixed-N
estimator (all max_m rays), checked against the oracle's fixed-N mode within 1e-6.
"""
import numpy as np
import pytest

import oracle as O
from compound_prism_designer import synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def designs(f1):
    rng = np.random.default_rng(20261211)
    out = [("F1", synth.spectrometer_from_dict(f1), f1)]
    for G, B in [(2, 16), (3, 32), (4, 64), (5, 128), (6, 64), (6, 128), (1, 32)]:
        s, d, _ = synth.random_design(rng, G, B)
        out.append((f"G{G}B{B}", s, d))
    return out


def _oracle(d, w, max_m):
    rows, rays = zip(*(O.p_dets_l_wavelength_count(d, x, max_m) for x in w))
    return np.array(rows), np.array(rays)


def test_reference_estimator_equals_oracle(designs):
    # inside the design range, beyond both ends, and where the beam misses the detector
    w = np.concatenate([np.linspace(0.5, 0.82, 21), [0.3, 0.45, 0.9, 1.2]])
    total = 0
    for name, s, d in designs:
        p, rays = s.transmission_probability(w, return_rays=True)
        po, ro = _oracle(d, w, 16384)
        assert np.array_equal(rays, ro), (name, rays, ro)
        assert np.abs(p - po).max() <= 1e-6, name
        assert np.array_equal(p, po), (name, np.abs(p - po).max())
        total += int(rays.sum())
    assert total > 0


@pytest.mark.parametrize("max_m", [1, 31, 257, 1000])
def test_small_ray_budgets(designs, max_m):
    name, s, d = designs[4]
    w = np.linspace(0.5, 0.82, 9)
    p, rays = s.transmission_probability(w, max_m=max_m, return_rays=True)
    po, ro = _oracle(d, w, max_m)
    assert np.array_equal(rays, ro) and np.array_equal(p, po), name
    assert (rays <= max_m).all()


@pytest.mark.parametrize("B", [1, 1024])
def test_detector_size_extremes(B):
    rng = np.random.default_rng(777 + B)
    s, d, _ = synth.random_design(rng, 4, B)
    w = np.linspace(0.5, 0.82, 7)
    p, rays = s.transmission_probability(w, max_m=8192, return_rays=True)
    po, ro = _oracle(d, w, 8192)
    assert np.array_equal(rays, ro) and np.array_equal(p, po)


def test_fixed_n_flag_keeps_the_fixed_estimator(designs):
    name, s, d = designs[0]
    w = np.linspace(0.5, 0.82, 17)
    p, rays = s.transmission_probability(w, max_m=1024, fixed_n=True, return_rays=True)
    dd = dict(d)
    dd["wavelength_bounds"] = (0.0, 1.0)
    po, _ = O.fitness_points(dd, w, O.qrng_points(0.5, 1024))
    assert np.abs(p - po).max() <= 1e-6
    assert (rays == 1024).all()
