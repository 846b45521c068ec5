"""Seeded synthetic designs with the shapes and value ranges of the benchmark
workloads (no public dataset is involved).

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
  maximum incidence, angle 0, auto-positioned with acceptance 1.0.
Designs that raise RayTraceError are redrawn; the rejection count is returned.
"""
from __future__ import annotations

import math

import numpy as np

from . import (CompoundPrism, DetectorArray, GaussianBeam, Glass, RayTraceError, Spectrometer,
               UniformWavelengthDistribution, position_detector_array)

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


def random_design(rng, G: int, B: int, *, height=20.0, width=7.0, curvature=0.05, beam_width=2.0,
                  ar_coated=True, max_tries: int = 1000, angle_range=(0.1, 1.2)):
    """Returns (Spectrometer, params dict, rejections)."""
    rejected = 0
    for _ in range(max_tries):
        sells = [random_sellmeier(rng) for _ in range(G)]
        glasses = [Glass(f"s{i}", horner_fit(s)) for i, s in enumerate(sells)]
        mags = rng.uniform(angle_range[0], angle_range[1], G + 1)
        sign = 1.0 if rng.uniform() < 0.5 else -1.0
        angles = [float(sign * (-1) ** i * m) for i, m in enumerate(mags)]
        lengths = [0.0] * G
        try:
            cp = CompoundPrism(glasses, angles, lengths, curvature, height, width, ar_coated)
            wl = UniformWavelengthDistribution(WAVELENGTHS)
            beam = GaussianBeam(beam_width, height / 2)
            det = detector_for_bins(B)
            pos, flipped = position_detector_array(det["length"], det["angle"], cp, wl, beam, 1.0)
            da = DetectorArray(det["bin_count"], det["bin_size"], det["linear_slope"], det["linear_intercept"],
                               det["length"], det["max_incident_angle"], det["angle"], pos, flipped)
            spec = Spectrometer(cp, da, wl, beam)
            _ = spec.design
        except (RayTraceError, ValueError):
            rejected += 1
            continue
        return spec, spec_dict(spec), rejected
    raise RuntimeError("no valid design found")


def spec_dict(spec: Spectrometer) -> dict:
    """The flat parameter dict the oracle's loader takes."""
    cp, da = spec.compound_prism, spec.detector_array
    return dict(glasses=[g.glass.tolist() for g in cp.glasses], angles=list(cp.angles), lengths=list(cp.lengths),
                curvature=cp.curvature, height=cp.height, width=cp.width, ar_coated=cp.ar_coated,
                bin_count=da.bin_count, bin_size=da.bin_size, linear_slope=da.linear_slope,
                linear_intercept=da.linear_intercept, det_length=da.length,
                max_incident_angle=da.max_incident_angle, det_angle=da.angle, det_position=da.position,
                det_flipped=da.flipped, wavelength_bounds=spec.wavelengths.bounds,
                beam_width=spec.beam.width, beam_y_mean=spec.beam.y_mean)


def spectrometer_from_dict(d: dict) -> Spectrometer:
    glasses = [Glass(f"g{i}", c) for i, c in enumerate(d["glasses"])]
    cp = CompoundPrism(glasses, d["angles"], d["lengths"], d["curvature"], d["height"], d["width"],
                       d["ar_coated"])
    da = DetectorArray(d["bin_count"], d["bin_size"], d["linear_slope"], d["linear_intercept"], d["det_length"],
                       d["max_incident_angle"], d["det_angle"], d.get("det_position", (0.0, 0.0)),
                       d.get("det_flipped", False))
    return Spectrometer(cp, da, UniformWavelengthDistribution(d["wavelength_bounds"]),
                        GaussianBeam(d["beam_width"], d["beam_y_mean"]))


def population(seed: int, n: int, G_choices=(2, 3, 4, 5, 6), B_choices=(16, 32, 64, 128)):
    """n designs with G and B drawn uniformly from the given choices."""
    rng = np.random.default_rng(seed)
    out, rej = [], 0
    for _ in range(n):
        G = int(rng.choice(G_choices))
        B = int(rng.choice(B_choices))
        s, d, r = random_design(rng, G, B)
        out.append((s, d))
        rej += r
    return out, rej
