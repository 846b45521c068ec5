"""Writes regression_designs.json: designs that once exposed a wrong decision of the
FP32 fast path, or that reach a branch of the pass no drawn design reaches, with the points
and rows that show it.

* far_reference_detector: design 196 of the precision-study population
  (compound_prism_designer.precision.study_population(20261207, 256, 128)); 2 prisms,
  0.24% of the beam reaches the detector, and the per-wavelength reference ray lands
  about 1.9 m from the detector, so the FP32 detector position of the rays that hit
  was summed from terms of ~2000 mm. With a purely absolute 1e-4 mm guard 22 of its
  16.8 M rays (8192 wavelengths x 2048 rays) were binned differently from the exact
  trace; the position guard now grows with those magnitudes.
* flat_face_tir_mid, flat_face_tir_last: designs that lose part of the band to total
  internal reflection at a flat face (face 2 of 4 prisms; face 5, the last flat face, of 6).
  At a flat face every ray of a wavelength has the same direction, so the per-wavelength
  setup decides the loss for the whole row; with the setup's flat-face chain split over two
  warps (direction and position), the direction warp has to stop the position warp there.
  No design of the drawn populations loses a row at a flat face. Each is a drawn design
  (seed 7 of the draw sequence below) with one apex angle scaled up, and its detector
  re-positioned on the part of the band that passes (the positioning traces the band's
  edges, and one edge is now lost); the wavelength bounds stay the drawn ones.
  `tir_rows` lists the wavelength rows (indices into the points) whose trace the oracle
  stops at a flat face with total internal reflection.

Run from the repository root: python tests/golden/make_regression_designs.py
"""
import copy
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.join(HERE, "..", "..")
sys.path.insert(0, os.path.join(ROOT, "compound-prism-designer_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from compound_prism_designer import precision as P  # noqa: E402
from compound_prism_designer import synth  # noqa: E402
import oracle as O  # noqa: E402

TIR = 3  # the oracle's total-internal-reflection status


def flat_face_tir(drawn: dict, k: int, scale: float, lam_u) -> dict:
    d = copy.deepcopy(drawn)
    d["angles"] = list(d["angles"])
    d["angles"][k] *= scale
    lo, hi = d["wavelength_bounds"]
    errs = np.array([O.propagate(d, lo + (hi - lo) * u, 0.5)[0] for u in lam_u])
    lost = lam_u[errs == TIR]
    assert lost.size, "no row lost to total internal reflection"
    if lost.min() > 0.5:
        band = (lo, lo + (hi - lo) * lost.min() * 0.98)
    else:
        band = (lo + (hi - lo) * (lost.max() + (1.0 - lost.max()) * 0.02), hi)
    e, pos, flipped = O.position_detector(dict(d, wavelength_bounds=list(band)), 1.0)
    assert e == 0, e
    return dict(d, det_position=list(pos), det_flipped=flipped)


def main():
    pop = P.study_population(20261207, 256, 128)
    spec, near, margin = pop[196]
    out = {"far_reference_detector": {
        "design": synth.spec_dict(spec),
        "points": {"lam_seed": 0.5, "wavelengths": 8192, "ray_seed": 0.5, "rays": 2048, "ray_first": 1,
                   "policy": "compound_prism_designer.precision.synth_points"},
        # wavelength rows (indices into the 8192 points) where the absolute guard erred
        "bad_rows": [110, 800, 1309, 1422, 2003, 2089, 2448, 2923, 2980],
    }}

    rng = np.random.default_rng(7)
    drawn = []
    for _ in range(11):
        G = int(rng.choice([3, 4, 5, 6]))
        B = int(rng.choice([32, 64]))
        drawn.append(synth.random_design(rng, G, B)[1])
    scales = np.linspace(1.02, 1.6, 30)
    W, R, seed = 2048, 1024, 0.5
    lam_u = O.gpu_points(seed, W)
    for name, trial, k, i in (("flat_face_tir_mid", 8, 2, 20), ("flat_face_tir_last", 10, 5, 27)):
        d = flat_face_tir(drawn[trial], k, float(scales[i]), lam_u)
        lo, hi = d["wavelength_bounds"]
        G = len(d["glasses"])
        stops = [O.stop_face(d, lo + (hi - lo) * u, d["beam_y_mean"]) for u in lam_u]
        tir_rows = [r for r, (face, st) in enumerate(stops) if face < G and face >= 0 and st == TIR]
        out[name] = {
            "design": d,
            "points": {"seed": seed, "wavelengths": W, "rays": R, "ray_first": 1,
                       "policy": "oracle.gpu_points"},
            "tir_faces": sorted({stops[r][0] for r in tir_rows}),
            "tir_rows": tir_rows,
        }
    with open(os.path.join(HERE, "regression_designs.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
