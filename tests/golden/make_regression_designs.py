"""Writes regression_designs.json: designs that once exposed a wrong decision of the
FP32 fast path, with the points and rays that showed it.

* far_reference_detector: design 196 of the precision-study population
  (compound_prism_designer.precision.study_population(20261207, 256, 128)); 2 prisms,
  0.24% of the beam reaches the detector, and the per-wavelength reference ray lands
  about 1.9 m from the detector, so the FP32 detector position of the rays that hit
  was summed from terms of ~2000 mm. With a purely absolute 1e-4 mm guard 22 of its
  16.8 M rays (8192 wavelengths x 2048 rays) were binned differently from the exact
  trace; the position guard now grows with those magnitudes.

Run from the repository root: python tests/golden/make_regression_designs.py
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "compound-prism-designer_gb300"))

from compound_prism_designer import precision as P  # noqa: E402
from compound_prism_designer import synth  # noqa: E402


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
    with open(os.path.join(HERE, "regression_designs.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
