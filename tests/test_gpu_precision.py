"""Precision study on a small population: FP32-only and hybrid traces against the
all-FP64 trace, and the FP64 trace against the CPU oracle, on near-critical designs
(exit-face incidence within 2 degrees of total internal reflection) and ordinary ones.

Bounds (the parity bar of this path): the hybrid trace must agree with FP64 exactly on hit
bins, within 1e-6 absolute on p(d|lambda) and within 1e-4 relative on MI. The
FP64 trace must agree with the oracle within the 2^-32 fixed-point quantum on p and
1e-8 relative on MI. FP32-only has no bound; its errors are the study's output and
are only checked to be finite.
"""
import os

import numpy as np
import pytest

import oracle as O
import compound_prism_designer as cpd
from compound_prism_designer import precision as P
from compound_prism_designer import synth

pytestmark = pytest.mark.gpu
NTHREADS = max(1, min(16, os.cpu_count() or 1))


@pytest.fixture(scope="module")
def population():
    return P.study_population(314, n=8, B=128)


def test_hybrid_meets_the_bounds_near_and_far_from_tir(population):
    rng = np.random.default_rng(1)
    lam_u = P.synth_points(0.5, 512)
    ray_u = P.synth_points(0.5, 1024, first=1)
    pl, pr = rng.uniform(size=16384), rng.uniform(1e-9, 1 - 1e-9, size=16384)
    for spec, near, margin in population:
        if near:
            assert 0.0 < margin <= 2.0
        r = P.evaluate(spec, lam_u, ray_u, pl, pr)
        h = r["hybrid"]
        assert h["hit_index_mismatches"] == 0, (near, margin, h)
        assert h["p_max_abs_err"] <= 1e-6, (near, margin, h)
        assert h["mi_rel_err"] <= 1e-4, (near, margin, h)
        f = r["fp32"]
        assert np.isfinite(f["mi_rel_err"]) and np.isfinite(f["p_max_abs_err"])


def test_fp64_trace_equals_oracle_on_near_critical_designs(population):
    lam_u = O.qrng_points(0.5, 256)
    ray_u = O.qrng_points(0.5, 1024)
    for spec, near, margin in population[:4]:
        assert near
        d = synth.spec_dict(spec)
        f, p = spec.gpu_fitness_points(lam_u, ray_u, mode=cpd.TRACE_FP64, want_p=True)
        po, st = O.fitness_points(d, lam_u, ray_u, nthreads=NTHREADS)
        assert np.abs(p - po).max() <= 2.0 ** -32, margin
        assert abs(f.info - st["info"]) <= 1e-8 * abs(st["info"]) + 1e-9, margin
        assert f.hits == st["hits"]


def test_single_design_trace_with_overflowing_flag_lists():
    """The largest single-design pass whose trace takes equal shares of the ray slots
    (16384 wavelengths x 8192 rays): each warp's share holds ~37 k rays, and at this
    design's flag rate (1.3e-3 of the core rays in the host check) many warps flag more rays
    than their 32-entry lists hold, so the rest go through the global queue and its kernel.
    The result must equal the multi-design trace's (work items, every flagged ray queued)
    bit for bit, and the oracle on the same points within the parity bounds."""
    spec = P.study_population(314, n=8, B=128)[7][0]
    W, R, seed = 16384, 8192, 0.3
    single = spec.gpu_fitness_full([seed], max_n=W, max_eval=R)
    for o in cpd.fitness_batch([spec, spec], seeds=seed, max_n=W, max_eval=R):
        assert o.info == single.info and o.hits == single.hits and o.retraced == single.retraced
    assert single.retraced > 0
    lam_u, ray_u = O.gpu_points(seed, W), O.gpu_points(seed, R, first=1)
    f, p = spec.gpu_fitness_points(lam_u, ray_u, want_p=True)
    assert f.info == single.info and f.hits == single.hits
    po, st = O.fitness_points(synth.spec_dict(spec), lam_u, ray_u, nthreads=NTHREADS)
    assert np.abs(p - po).max() <= 1e-6
    assert abs(f.info - st["info"]) <= 1e-4 * abs(st["info"]) + 1e-9
    assert f.hits == st["hits"]
    print(f"retraced {f.retraced} of {f.rays} rays, MI rel err {abs(f.info - st['info']) / abs(st['info']):.2e}")


def test_summary_counts_classes(population):
    rows = []
    lam_u = P.synth_points(0.5, 64)
    ray_u = P.synth_points(0.5, 256, first=1)
    for i, (spec, near, margin) in enumerate(population):
        r = P.evaluate(spec, lam_u, ray_u, lam_u[:16], ray_u[:16])
        r.update(design=i, near_critical=near, margin_deg=margin)
        rows.append(r)
    s = P.summarize(rows)
    assert s["near_critical"]["designs"] == 4 and s["ordinary"]["designs"] == 4
    assert s["near_critical"]["hybrid"]["designs_over_1e-4_mi"] == 0


def test_far_reference_ray_design_on_the_gpu():
    """The design whose reference rays land ~1.9 m from the detector: the hybrid trace
    equals the oracle on the rows that once went wrong and stays within the bounds of
    the FP64 trace over all 8192 x 2048 points."""
    import json

    from conftest import GOLDEN

    case = json.load(open(os.path.join(GOLDEN, "regression_designs.json")))["far_reference_detector"]
    d = case["design"]
    spec = synth.spectrometer_from_dict(d)
    pts = case["points"]
    lam_all = P.synth_points(pts["lam_seed"], pts["wavelengths"])
    ray_u = P.synth_points(pts["ray_seed"], pts["rays"], first=pts["ray_first"])
    lam_bad = lam_all[case["bad_rows"]]
    f, p = spec.gpu_fitness_points(lam_bad, ray_u, mode=cpd.TRACE_HYBRID, want_p=True)
    po, st = O.fitness_points(d, lam_bad, ray_u, nthreads=NTHREADS)
    assert np.abs(p - po).max() <= 1e-6
    assert f.hits == st["hits"]
    f64, p64 = spec.gpu_fitness_points(lam_all, ray_u, mode=cpd.TRACE_FP64, want_p=True)
    fh, ph = spec.gpu_fitness_points(lam_all, ray_u, mode=cpd.TRACE_HYBRID, want_p=True)
    assert np.abs(ph - p64).max() <= 1e-6
    assert abs(fh.info - f64.info) <= 1e-4 * abs(f64.info)
    assert fh.hits == f64.hits
