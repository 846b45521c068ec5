"""Precision study: the FP32-only and the hybrid GPU traces against the all-FP64 GPU trace.

Population: n designs with B detector bins, prism counts 2..6, half of them
near-critical -- at the beam centre, for the shortest, middle and longest
wavelength, the incidence on the curved exit face is within `max_margin_deg`
(2 degrees) below the total-internal-reflection angle, so a large share of the beam
is lost there and many rays pass close to the TIR threshold. The other half are
ordinary designs of the same ranges (synth.random_design).

Per design, on identical QMC points (W wavelengths x R rays, seed 0.5):
  * CPD_TRACE_FP64 is the reference: every ray traced in exact f64, the same
    operation order as the reference's f64 CPU path (src/spectrometer/ray.rs), so its
    p(d|lambda) equals the CPU oracle's to within the 2^-32 fixed-point quantum;
  * CPD_TRACE_FP32 (FP32 trace, no guard bands, no re-trace) and CPD_TRACE_HYBRID
    (FP32 trace, guard-band rays re-traced in f64) are compared with it:
    relative MI error, max |delta p(d|lambda)|, and, on `pairs` random
    (wavelength, ray) pairs traced one by one, the number of rays whose hit bin
    differs and the max relative transmittance error of the rays that agree.

Run: python -m compound_prism_designer.precision --out study.json
"""
from __future__ import annotations

import argparse
import json
import math
import time

import numpy as np

from . import RayTraceError, TRACE_FP32, TRACE_FP64, TRACE_HYBRID, default_context
from . import synth


def exit_margin_deg(spec, y: float, w: float) -> float:
    """Degrees between the TIR angle and the incidence angle on the curved exit face
    for the ray entering at height y with wavelength w (-inf: the ray does not leave)."""
    cp = spec.compound_prism
    try:
        p, d = cp.exit_ray(y, w)
    except RayTraceError:
        return -math.inf
    D = cp._design
    nx = (p.x - D.exit_center[0]) / D.exit_radius
    ny = (p.y - D.exit_center[1]) / D.exit_radius
    cos_out = abs(d.x * nx + d.y * ny)
    sin_out = math.sqrt(max(0.0, 1.0 - cos_out * cos_out))
    n = cp.glasses[-1](w)
    return math.degrees(math.asin(1.0 / n) - math.asin(min(1.0, sin_out / n)))


def design_margin_deg(spec) -> float:
    wmin, wmax = spec.wavelengths.bounds
    y = spec.beam.y_mean
    return min(exit_margin_deg(spec, y, w) for w in (wmin, 0.5 * (wmin + wmax), wmax))


def near_critical_design(rng, G: int, B: int, max_margin_deg: float = 2.0, max_tries: int = 200_000):
    """A design whose exit-face incidence is within (0, max_margin_deg] of TIR."""
    for _ in range(max_tries):
        try:
            spec, _, _ = synth.random_design(rng, G, B, max_tries=1)
        except RuntimeError:
            continue
        m = design_margin_deg(spec)
        if 0.0 < m <= max_margin_deg:
            return spec, m
    raise RuntimeError("no near-critical design found")


def study_population(seed: int, n: int = 256, B: int = 128, near_fraction: float = 0.5,
                     max_margin_deg: float = 2.0):
    """[(spec, near_critical, margin_deg)] with G uniform in 2..6."""
    rng = np.random.default_rng(seed)
    out = []
    n_near = int(round(n * near_fraction))
    for i in range(n):
        G = int(rng.integers(2, 7))
        if i < n_near:
            spec, m = near_critical_design(rng, G, B, max_margin_deg)
            out.append((spec, True, m))
        else:
            spec, _, _ = synth.random_design(rng, G, B)
            out.append((spec, False, design_margin_deg(spec)))
    return out


def evaluate(spec, lam_u, ray_u, pair_lam, pair_ray, context=None) -> dict:
    """Errors of FP32-only and hybrid against the FP64 trace for one design."""
    ctx = context or default_context()
    f64, p64 = spec.gpu_fitness_points(lam_u, ray_u, mode=TRACE_FP64, want_p=True, context=ctx)
    b64, t64, _ = spec.trace_rays(pair_lam, pair_ray, mode=TRACE_FP64, context=ctx)
    res = {"mi_fp64": f64.info, "hit_fraction": f64.hits / f64.rays, "h_det": f64.h_det, "h_cond": f64.h_cond}
    for name, mode in (("fp32", TRACE_FP32), ("hybrid", TRACE_HYBRID)):
        f, p = spec.gpu_fitness_points(lam_u, ray_u, mode=mode, want_p=True, context=ctx)
        b, t, fl = spec.trace_rays(pair_lam, pair_ray, mode=mode, context=ctx)
        same = b == b64
        hit = same & (b64 < spec.detector_array.bin_count)
        t_rel = np.abs(t[hit] - t64[hit]) / np.maximum(np.abs(t64[hit]), 1e-300)
        res[name] = {
            "mi": f.info,
            "mi_rel_err": abs(f.info - f64.info) / abs(f64.info) if f64.info != 0 else abs(f.info),
            "p_max_abs_err": float(np.abs(p - p64).max()),
            "hit_index_mismatches": int((~same).sum()),
            "t_max_rel_err": float(t_rel.max()) if t_rel.size else 0.0,
            "retraced_rays": int(f.retraced),
            "retraced_pairs": int(fl.sum()),
        }
    return res


def run(seed: int = 20261207, n: int = 256, B: int = 128, W: int = 8192, R: int = 2048, pairs: int = 65536,
        context=None, log=None) -> dict:
    t0 = time.perf_counter()
    pop = study_population(seed, n, B)
    t_pop = time.perf_counter() - t0
    rng = np.random.default_rng(seed + 1)
    lam_u = synth_points(0.5, W)
    ray_u = synth_points(0.5, R, first=1)
    pair_lam = rng.uniform(size=pairs)
    pair_ray = rng.uniform(1e-9, 1 - 1e-9, size=pairs)
    rows = []
    t1 = time.perf_counter()
    for i, (spec, near, margin) in enumerate(pop):
        r = evaluate(spec, lam_u, ray_u, pair_lam, pair_ray, context)
        r.update(design=i, near_critical=near, margin_deg=margin, prisms=len(spec.compound_prism.glasses))
        rows.append(r)
        if log and (i + 1) % 32 == 0:
            log(f"{i + 1}/{n} designs")
    t_eval = time.perf_counter() - t1
    return {"config": {"designs": n, "bins": B, "wavelengths": W, "rays_per_wavelength": R, "pairs": pairs,
                       "seed": seed, "near_critical": sum(1 for _, nr, _ in pop if nr), "max_margin_deg": 2.0},
            "summary": summarize(rows), "designs": rows, "seconds": {"population": t_pop, "evaluate": t_eval}}


def synth_points(seed: float, n: int, first: int = 0) -> np.ndarray:
    """u_i = fract(seed + (first + i)/phi): the golden-ratio QMC points of the GPU
    policy (computed here without the fused multiply-add; every mode gets the same
    array, which is all the comparison needs)."""
    alpha = 0.6180339887498948482045868343656381177203091798057628621354486227
    i = np.arange(first, first + n, dtype=np.float64)
    v = i * alpha + seed
    return v - np.trunc(v)


def summarize(rows) -> dict:
    out = {}
    for cls, sel in (("near_critical", [r for r in rows if r["near_critical"]]),
                     ("ordinary", [r for r in rows if not r["near_critical"]])):
        if not sel:
            continue
        c = {"designs": len(sel), "median_hit_fraction": float(np.median([r["hit_fraction"] for r in sel]))}
        for mode in ("fp32", "hybrid"):
            mi = np.array([r[mode]["mi_rel_err"] for r in sel])
            pe = np.array([r[mode]["p_max_abs_err"] for r in sel])
            hm = np.array([r[mode]["hit_index_mismatches"] for r in sel])
            c[mode] = {"mi_rel_err_max": float(mi.max()), "mi_rel_err_median": float(np.median(mi)),
                       "designs_over_1e-4_mi": int((mi > 1e-4).sum()), "p_abs_err_max": float(pe.max()),
                       "designs_over_1e-6_p": int((pe > 1e-6).sum()), "hit_mismatches_total": int(hm.sum()),
                       "designs_with_hit_mismatch": int((hm > 0).sum())}
        out[cls] = c
    return out


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--designs", type=int, default=256)
    ap.add_argument("--bins", type=int, default=128)
    ap.add_argument("--wavelengths", type=int, default=8192)
    ap.add_argument("--rays", type=int, default=2048)
    ap.add_argument("--pairs", type=int, default=65536)
    ap.add_argument("--seed", type=int, default=20261207)
    ap.add_argument("--out", default=None)
    a = ap.parse_args(argv)
    res = run(a.seed, a.designs, a.bins, a.wavelengths, a.rays, a.pairs, log=print)
    print(json.dumps({"config": res["config"], "summary": res["summary"], "seconds": res["seconds"]}, indent=1))
    if a.out:
        with open(a.out, "w") as f:
            json.dump(res, f)


if __name__ == "__main__":
    main()
