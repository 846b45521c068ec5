"""Regenerates the golden fixtures in this folder from the reference sources.

Run in a container where the reference project is checked out; its path is the
required first argument. Nothing here runs during the tests:
the tests read the JSON files this script writes.

* f1_known_design.json -- the known 3-glass design of the reference's
  `fitness::tests::test_with_known_prism` (src/fitness.rs:153-257), its
  expected fitness and tolerances, parsed out of the Rust source.
* norminv_points.json -- the accuracy points of `erf::test::test_shaw`
  (src/spectrometer/erf.rs:142-161); the exact quantiles, which the Rust test
  takes from statrs, come from scipy.special.ndtri.
* glass_fits.json -- synthetic Sellmeier-1 glasses fitted to the 6-coefficient
  Horner polynomial by the reference's own `AbstractGlass.horner_polynomial_fit`
  (compound_prism_designer/glasscat.py:114-127), imported from the reference
  with a stand-in for its compiled `Glass` class.
"""
from __future__ import annotations

import importlib.util
import json
import math
import os
import re
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _floats(text: str):
    return [float(x) for x in re.findall(r"-?\d+\.\d+(?:e-?\d+)?|-?\d+(?=\s*[,\]])", text)]


def f1(ref: str):
    src = open(os.path.join(ref, "src", "fitness.rs")).read()
    test = src[src.index("fn test_with_known_prism"):]
    glasses = [_floats(m) for m in re.findall(r"coefficents:\s*\[([^\]]*)\]", test)]
    angles = _floats(re.search(r"let angles = \[([^\]]*)\]", test).group(1))
    height = float(re.search(r"let height = ([\d.]+);", test).group(1))
    width = float(re.search(r"let width = ([\d.]+);", test).group(1))
    curv = float(re.search(r"signed_normalized_curvature: ([\d.]+)", test).group(1))
    bounds = _floats(re.search(r"bounds: \(([^)]*)\)", test).group(1))
    bw = float(re.search(r"width: ([\d.]+),\s*y_mean", test).group(1))
    ym = float(re.search(r"y_mean: ([\d.]+)", test).group(1))
    nbin = int(re.search(r"const NBIN: usize = (\d+);", test).group(1))
    pmt = float(re.search(r"let pmt_length = ([\d.]+);", test).group(1))
    maxang = float(re.search(r"let spec_max_accepted_angle = \(([\d.]+)_f64\)", test).group(1))
    det = re.search(r"LinearDetectorArray::new\(\s*NBIN as u32,\s*([\d.]+),\s*([\d.]+),\s*([\d.]+),", test)
    coat = re.search(r"width,\s*(true|false),\s*\);", test).group(1) == "true"
    checks = {}
    for name, val, tol in re.findall(r"assert_float_eq!\((\w+), ([\d.]+), rmax <= ([\d.e-]+)\)", test):
        checks[name] = {"value": float(val), "rmax": float(tol)}
    max_n, max_m = (int(x.replace("_", "")) for x in
                    re.search(r"fitness\(&spec, ([\d_]+), ([\d_]+)\)", test).groups())
    return {
        "source": "src/fitness.rs:153-257 (fitness::tests::test_with_known_prism)",
        "design": {
            "glasses": glasses,
            "angles_deg": angles,
            "lengths": [0.0] * len(glasses),
            "curvature": curv,
            "height": height,
            "width": width,
            "ar_coated": coat,
            "bin_count": nbin,
            "bin_size": float(det.group(1)),
            "linear_slope": float(det.group(2)),
            "linear_intercept": float(det.group(3)),
            "det_length": pmt,
            "max_incident_angle_deg": maxang,
            "det_angle": 0.0,
            "acceptance": 1.0,
            "wavelength_bounds": bounds,
            "beam_width": bw,
            "beam_y_mean": ym,
        },
        "max_n": max_n,
        "max_m": max_m,
        "expected": checks,
    }


def norminv_points(ref: str):
    from scipy.special import ndtri

    src = open(os.path.join(ref, "src", "spectrometer", "erf.rs")).read()
    test = src[src.index("fn test_shaw"):src.index("fn test_fast_shaw")]
    pts = []
    for u, tol in re.findall(r"norminv\(([\d.e-]+)\), n\.inverse_cdf\([\d.e-]+\), rmax <= ([\d.e-]+)\)", test):
        pts.append({"u": float(u), "exact": float(ndtri(float(u))), "rmax": float(tol)})
    return {"source": "src/spectrometer/erf.rs:142-161 (erf::test::test_shaw)", "points": pts}


def glass_fits(ref: str, n: int = 8, seed: int = 20261203):
    pkg = types.ModuleType("cpd_ref_pkg")
    pkg.__path__ = []
    sys.modules["cpd_ref_pkg"] = pkg
    stub = types.ModuleType("cpd_ref_pkg.compound_prism_designer")

    class Glass:  # stands in for the compiled pyo3 class (src/pylib.rs:37-95)
        ORDER = 5

        def __init__(self, name, coefficents):
            self.name = name
            self.glass = list(coefficents)

    stub.Glass = Glass
    sys.modules["cpd_ref_pkg.compound_prism_designer"] = stub
    spec = importlib.util.spec_from_file_location(
        "cpd_ref_pkg.glasscat", os.path.join(ref, "compound_prism_designer", "glasscat.py"))
    gc = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(gc)
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        b1, b2, b3 = rng.uniform(0.5, 1.8), rng.uniform(0.0, 0.5), rng.uniform(0.5, 1.5)
        c1, c2, c3 = rng.uniform(0.003, 0.015), rng.uniform(0.01, 0.07), rng.uniform(80, 200)
        sell = (b1, c1, b2, c2, b3, c3)  # Sellmeier1 order (glasscat.py:144-152)
        g = gc.Sellmeier1(f"synthetic{i}", sell, (0.3, 2.5))
        glass, chisq = g.into_glass((0.5, 0.82))
        out.append({"sellmeier1": list(sell), "limits": [0.5, 0.82],
                    "horner": [float(c) for c in glass.glass], "chisq": float(chisq)})
    return {"source": "compound_prism_designer/glasscat.py:114-127,144-152", "glasses": out}


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the reference project>")
    ref = sys.argv[1]
    for name, obj in (("f1_known_design.json", f1(ref)),
                      ("norminv_points.json", norminv_points(ref)),
                      ("glass_fits.json", glass_fits(ref))):
        with open(os.path.join(HERE, name), "w") as f:
            json.dump(obj, f, indent=1)
        print("wrote", name)


if __name__ == "__main__":
    main()
