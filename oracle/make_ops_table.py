"""Writes roofline/ops_per_ray.json: the frozen operation table of the fitness path.

The op-counting build of the oracle (ops_count.cpp over cpd_oracle_model.h, the
reference's f64 per-ray trace) traces the rays of a seeded synthetic population and
counts every operation. Per prism count G (1..6): the mean per ray over every traced ray
(rays lost at a face stop there, as in the reference), the mean per ray that reached a
detector bin, and, booked apart, the per-wavelength work the reference repeats per ray
(Glass::calc_n at each face) and the beam's inverse CDF per start height. FLOP = add +
mul + 2 fma + compare; div, sqrt and log are counted apart.

Population: 12 designs per G drawn like the benchmark workloads
(compound_prism_designer/workload.py, 64 bins, positioned by the oracle), each traced
over 64 wavelengths x 512 rays of the GPU seed policy (seed 0.5).

Run from the repository root: python oracle/make_ops_table.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(ROOT, "compound-prism-designer_gb300", "compound_prism_designer"))

import oracle as O  # noqa: E402
import workload  # noqa: E402  (numpy only; loaded without the library's package)

OUT = os.path.join(ROOT, "roofline", "ops_per_ray.json")
DESIGNS, W, R, B = 12, 64, 512, 64


def flop(c):
    return c["add"] + c["mul"] + 2 * c["fma"] + c["cmp"]


def per(c, n):
    out = {k: v / n for k, v in c.items()}
    out["flop"] = flop(c) / n
    return out


def main():
    lam = O.gpu_points(0.5, W)
    ray = O.gpu_points(0.5, R, first=1)
    table = {}
    for G in range(1, 7):
        rng = np.random.default_rng(20261212 + G)
        tot = {n: dict.fromkeys(O.OP_KINDS, 0) for n in ("ray", "lambda", "hit_ray", "beam")}
        hits = 0
        for _ in range(DESIGNS):
            d, _ = workload.random_params(rng, G, B, O.accept_params)
            c, h = O.ops_trace(d, lam, ray)
            _, st = O.fitness_points(d, lam, ray)
            assert h == st["hits"], "the counting build must trace what the oracle traces"
            hits += h
            for n in tot:
                for k in O.OP_KINDS:
                    tot[n][k] += c[n][k]
        rays = DESIGNS * W * R
        table[str(G)] = {
            "per_ray": per(tot["ray"], rays),
            "per_hit_ray": per(tot["hit_ray"], max(hits, 1)),
            "per_ray_calc_n": per(tot["lambda"], rays),
            "per_start_height": per(tot["beam"], DESIGNS * R),
            "hit_fraction": hits / rays,
            "rays": rays,
        }
        print(G, round(table[str(G)]["per_ray"]["flop"], 1), round(table[str(G)]["per_hit_ray"]["flop"], 1),
              round(table[str(G)]["hit_fraction"], 3))
    doc = {
        "description": "operations per traced ray of the reference's per-ray f64 formulation "
                       "(src/spectrometer/ray.rs:485-499, spectrometer.rs:265-303,421-427), counted by the "
                       "op-counting build of the oracle (oracle/ops_count.cpp over oracle/cpd_oracle_model.h)",
        "convention": "flop = add + mul + 2 fma + cmp; div, sqrt, log, trig counted apart; other = neg, abs, "
                      "copysign, sign bit, trunc; calc_n (per wavelength, repeated per ray by the reference) "
                      "and the beam inverse CDF (per start height) booked apart",
        "sample": f"{DESIGNS} designs per G from compound_prism_designer/workload.py ({B} bins, seeds "
                  f"20261212+G), each over {W} wavelengths x {R} rays (GPU seed policy, seed 0.5)",
        "generator": "python oracle/make_ops_table.py",
        "by_glasses": table,
    }
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    with open(OUT, "w") as f:
        json.dump(doc, f, indent=1, sort_keys=True)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
