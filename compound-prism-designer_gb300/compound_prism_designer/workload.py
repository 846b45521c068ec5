"""Seeded synthetic design parameters with the shapes and value ranges of the benchmark
workloads (no public dataset is involved). numpy only: this module imports nothing from
the package, so it can be loaded by file path where the native library must not be
(the benchmark's reference arm builds these designs with the CPU restatement alone).

* Glasses: Sellmeier-1 (b1, c1, b2, c2, b3, c3) with B1 in [0.5, 1.8], B2 in [0, 0.5],
  B3 in [0.5, 1.5], C1 in [0.003, 0.015], C2 in [0.01, 0.07], C3 in [80, 200] um^2,
  fitted to the reference's 6-coefficient Horner polynomial over the wavelength
  range on 100 evenly spaced points (AbstractGlass.horner_polynomial_fit,
  compound_prism_designer/glasscat.py:114-127; a linear least-squares problem,
  solved here directly).
* Geometry: G+1 face angles of alternating sign, |theta| in [0.1, 1.2] rad, zero
  separation lengths, height 20 mm, width 7 mm, exit-face curvature 0.05,
  anti-reflection coated.
* Beam: Gaussian, width 2, centred (y_mean = height/2). Wavelengths U[0.50, 0.82] um.
* Detector: B bins over 32 mm (slope 32/B, bin size 0.8*slope, intercept
  0.1*slope; for B = 32 these are the reference's spring.toml values), 45 degree
  maximum incidence, angle 0, positioned by the caller (acceptance 1.0).
"""
from __future__ import annotations

import math

import numpy as np

WAVELENGTHS = (0.5, 0.82)


def sellmeier1(sell, w):
    b1, c1, b2, c2, b3, c3 = sell
    w2 = np.asarray(w, dtype=np.float64) ** 2
    return np.sqrt(1 + b1 * w2 / (w2 - c1) + b2 * w2 / (w2 - c2) + b3 * w2 / (w2 - c3))


def horner_fit(sell, limits=WAVELENGTHS, order: int = 5) -> np.ndarray:
    """Least-squares degree-`order` polynomial through 100 points, highest degree first."""
    x = np.linspace(limits[0], limits[1], 100)
    y = sellmeier1(sell, x)
    A = np.vander(x, order + 1)
    coef, *_ = np.linalg.lstsq(A, y, rcond=None)
    return coef


def random_sellmeier(rng) -> tuple:
    b1, b2, b3 = rng.uniform(0.5, 1.8), rng.uniform(0.0, 0.5), rng.uniform(0.5, 1.5)
    c1, c2, c3 = rng.uniform(0.003, 0.015), rng.uniform(0.01, 0.07), rng.uniform(80, 200)
    return (b1, c1, b2, c2, b3, c3)


def detector_for_bins(B: int):
    slope = 32.0 / B
    return dict(bin_count=B, bin_size=0.8 * slope, linear_slope=slope, linear_intercept=0.1 * slope,
                length=32.0, max_incident_angle=math.radians(45.0), angle=0.0)


def draw_params(rng, G: int, B: int, *, height=20.0, width=7.0, curvature=0.05, beam_width=2.0,
                ar_coated=True, angle_range=(0.1, 1.2)) -> dict:
    """One draw of a design's parameters as the flat dict the builders take; the detector
    is not positioned yet (det_position (0, 0))."""
    sells = [random_sellmeier(rng) for _ in range(G)]
    mags = rng.uniform(angle_range[0], angle_range[1], G + 1)
    sign = 1.0 if rng.uniform() < 0.5 else -1.0
    det = detector_for_bins(B)
    return dict(glasses=[horner_fit(s).tolist() for s in sells],
                angles=[float(sign * (-1) ** i * m) for i, m in enumerate(mags)], lengths=[0.0] * G,
                curvature=curvature, height=height, width=width, ar_coated=ar_coated,
                bin_count=det["bin_count"], bin_size=det["bin_size"], linear_slope=det["linear_slope"],
                linear_intercept=det["linear_intercept"], det_length=det["length"],
                max_incident_angle=det["max_incident_angle"], det_angle=det["angle"], det_position=(0.0, 0.0),
                det_flipped=False, wavelength_bounds=WAVELENGTHS, beam_width=beam_width,
                beam_y_mean=height / 2)


def random_params(rng, G: int, B: int, accept, *, max_tries: int = 1000, **kw):
    """Draws until `accept(params)` returns the positioned parameter dict (None rejects the
    draw: the design raises RayTraceError or is invalid). Returns (params, rejections)."""
    rejected = 0
    for _ in range(max_tries):
        d = accept(draw_params(rng, G, B, **kw))
        if d is not None:
            return d, rejected
        rejected += 1
    raise RuntimeError("no valid design found")
