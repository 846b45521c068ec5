"""Pins the C oracle to the reference's own known-answer tests.

* src/fitness.rs:153-257 -- known 3-glass design: size, info and deviation
  within the reference's relative tolerances.
* src/spectrometer/erf.rs:142-161 -- Shaw inverse normal CDF accuracy points.
"""
import math

import numpy as np
import pytest

import oracle as O
from conftest import load_golden


def test_f1_known_design_fitness(f1):
    g = load_golden("f1_known_design.json")
    size, info, dev = O.fitness_adaptive(f1, g["max_n"], g["max_m"])
    got = {"size": size, "info": info, "deviation": dev}
    for name, exp in g["expected"].items():
        rel = abs(got[name] - exp["value"]) / max(abs(got[name]), abs(exp["value"]))
        assert rel <= exp["rmax"], (name, got[name], exp)


@pytest.mark.parametrize("pt", load_golden("norminv_points.json")["points"], ids=lambda p: str(p["u"]))
def test_norminv_accuracy_points(pt):
    got = O.norminv(pt["u"])
    rel = abs(got - pt["exact"]) / max(abs(got), abs(pt["exact"]), 1e-300)
    assert rel <= pt["rmax"] or (pt["exact"] == 0.0 and got == 0.0)


def test_qrng_is_incremental_golden_ratio_sequence():
    pts = O.qrng_points(0.5, 5)
    alpha = 1.0 / 1.61803398874989484820458683436563
    st = 0.5
    for p in pts:
        st = (st + alpha) % 1.0
        assert p == st


def test_detector_positioning_and_geometry_f1(f1):
    # positions the detector for the reference's own design without error, and the
    # size/deviation the dump reports equal the adaptive fitness' values.
    dump = O.design_dump(f1)
    size, _, dev = O.fitness_adaptive(f1, 64, 256)
    assert dump[-2] == size and dump[-1] == dev


def test_fixed_points_vs_reference_welford_skip(f1):
    # p_dets_l_wavelength (src/fitness.rs:5-34) pads a bin with `skip(count)` and
    # then adds the hit with `next_sample`, so after a hit the bin's Welford count
    # is one ahead of the ray count. The final skip(count) absorbs the offset for
    # every bin except the one the LAST ray hit, whose mean is sum(t)/(R+1).
    # The fixed-N estimator is sum(t)/R for every bin; with no early stop (R=64 is
    # far below the SEM stop), the two agree exactly up to that one bin.
    R = 64
    ray_u = O.qrng_points(0.5, R)
    checked = 0
    for w in np.linspace(0.51, 0.81, 7):
        p_ad = O.p_dets_l_wavelength(f1, w, R)
        lam_u = np.array([(w - 0.5) / (0.82 - 0.5)])
        if 0.5 + (0.82 - 0.5) * lam_u[0] != w:
            continue
        p_fx, _ = O.fitness_points(f1, lam_u, ray_u)
        e, last_bin, _ = O.propagate(f1, w, ray_u[-1])
        expect = p_fx[0].copy()
        if e == O.OK:
            expect[last_bin] = expect[last_bin] * R / (R + 1)
        np.testing.assert_allclose(p_ad, expect, rtol=1e-13, atol=1e-15)
        checked += 1
    assert checked >= 3


def test_propagation_path_reaches_detector(f1):
    rows = O.propagation_path(f1, 0.6, 0.95)
    G = len(f1["glasses"])
    assert rows.shape == (G + 3, 4)
    # the last row lies on the detector line through det_position
    assert np.isfinite(rows).all()
