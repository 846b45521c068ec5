"""Seeded synthetic designs with the shapes and value ranges of the benchmark
workloads, built into Spectrometers. The parameter draws (glasses, angles, detector,
beam) are in `workload` (numpy only); this module builds and positions them with the
library and redraws designs that raise RayTraceError. The rejection count is returned.
"""
from __future__ import annotations

import numpy as np

from . import (CompoundPrism, DetectorArray, GaussianBeam, Glass, RayTraceError, Spectrometer,
               UniformWavelengthDistribution, position_detector_array)
from .workload import (WAVELENGTHS, detector_for_bins, draw_params, horner_fit, random_params,  # noqa: F401
                       random_sellmeier, sellmeier1)


def _accept(d: dict):
    """The positioned parameters of a draw, or None when the design cannot be built."""
    try:
        glasses = [Glass(f"s{i}", c) for i, c in enumerate(d["glasses"])]
        cp = CompoundPrism(glasses, d["angles"], d["lengths"], d["curvature"], d["height"], d["width"],
                           d["ar_coated"])
        wl = UniformWavelengthDistribution(d["wavelength_bounds"])
        beam = GaussianBeam(d["beam_width"], d["beam_y_mean"])
        pos, flipped = position_detector_array(d["det_length"], d["det_angle"], cp, wl, beam, 1.0)
        da = DetectorArray(d["bin_count"], d["bin_size"], d["linear_slope"], d["linear_intercept"],
                           d["det_length"], d["max_incident_angle"], d["det_angle"], pos, flipped)
        spec = Spectrometer(cp, da, wl, beam)
        _ = spec.design
    except (RayTraceError, ValueError):
        return None
    return spec


def random_design(rng, G: int, B: int, *, height=20.0, width=7.0, curvature=0.05, beam_width=2.0,
                  ar_coated=True, max_tries: int = 1000, angle_range=(0.1, 1.2)):
    """Returns (Spectrometer, params dict, rejections)."""
    spec, rejected = random_params(rng, G, B, _accept, max_tries=max_tries, height=height, width=width,
                                   curvature=curvature, beam_width=beam_width, ar_coated=ar_coated,
                                   angle_range=angle_range)
    return spec, spec_dict(spec), rejected


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
