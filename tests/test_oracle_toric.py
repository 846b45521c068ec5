"""The reference's 3-D spectrometer (fiber beam, toric lenses) restated in the oracle
(oracle/cpd_oracle_toric.c), and what it computes. No GPU calls.

* approx_cbrt (src/spectrometer/cbrt.rs:49-68) meets the reference's own accuracy test
  (test_cbrt_f32, cbrt.rs:95-108: relative error <= 3e-5 on [1e-5, 1024]).
* The closed-form quartic (sympy_soln, src/spectrometer/toric.rs:41-141) agrees with a
  polynomial root finder where the ray-torus quartic has two real roots, and yields NaN
  for every root where it has four (its general branch takes the square root of the
  resolvent cubic's negative discriminant).
* On the fiber configuration of the reference's optimizer (designer.py:203-265 with
  spring.toml's fiber-core-radius 0.050 and numerical-aperture 0.32, the curvature
  bounds of designer.py:127), the axial ray cannot pass the first toric lens of any
  design, so detector positioning raises RayTraceError for every design, although for
  most of them the ray does cross the lens inside its bounds.
"""
import math

import numpy as np

import oracle as O
from compound_prism_designer import workload


def _quartic(R2, r2, dms, dpv, dpn, nv):
    """Coefficients of the ray-torus quartic in the distance (toric.rs:163-172)."""
    return [1.0, 4 * dpv, -2 * (r2 + R2 - dms - 2 * dpv ** 2 - 2 * R2 * nv ** 2),
            -4 * (r2 + R2 - dms) * dpv + 8 * R2 * dpn * nv,
            (r2 - R2) ** 2 - 2 * (R2 + r2) * dms + dms ** 2 + 4 * R2 * dpn ** 2]


def _real_roots(c):
    return sorted(x.real for x in np.roots(c) if abs(x.imag) < 1e-7 * max(1.0, abs(x.real)))


def test_approx_cbrt_meets_the_reference_accuracy():
    v = np.exp(np.random.default_rng(1).uniform(math.log(1e-5), math.log(1024.0), 20000)).astype(np.float32)
    err = max(abs(O.approx_cbrt(float(x)) / math.pow(float(x), 1 / 3) - 1.0) for x in v)
    assert err <= 3e-5, err
    assert O.approx_cbrt(-8.0) == -O.approx_cbrt(8.0)


def test_closed_form_roots_two_real_and_four_real():
    rng = np.random.default_rng(3)
    two_err, four_nan, four = [], 0, 0
    for _ in range(6000):
        R = rng.uniform(0.5, 20.0)
        r = rng.uniform(0.05, 0.9) * R
        n = rng.normal(size=3)
        n /= np.linalg.norm(n)
        v = rng.normal(size=3)
        v /= np.linalg.norm(v)
        dp = rng.normal(size=3) * R * 2
        args = (r * r, R * R, dp @ dp, dp @ v, dp @ n, n @ v)
        real = _real_roots(_quartic(R * R, r * r, dp @ dp, dp @ v, dp @ n, n @ v))
        cf = O.toric_roots(*args)
        fin = np.sort(cf[np.isfinite(cf)])
        if len(real) == 4:
            four += 1
            four_nan += int(np.isnan(cf).all())
        elif len(real) == 2 and len(fin) == 2:
            two_err.append(max(abs(a - b) for a, b in zip(fin, real)) / R)
    assert four > 20 and four_nan == four  # every root NaN whenever all four are real
    assert len(two_err) > 500 and np.median(two_err) < 1e-3  # the algebra is the quartic's


def _designer_fiber_design(rng, G=4, H=25.0, width=7.0):
    """One design of the reference optimizer's fiber configuration (designer.py:108-265,
    spring.toml with the fiber beam): parameters uniform within the optimizer's bounds,
    synthetic glasses."""
    height = rng.uniform(0.0001 * H, H)
    return dict(glasses=[workload.horner_fit(workload.random_sellmeier(rng)).tolist() for _ in range(G)],
                angles=list(rng.uniform(-math.pi / 2, math.pi / 2, G + 1)),
                lengths=list(np.arctanh(rng.uniform(0, 1, G)) * H / 4),
                curv0=(-rng.uniform(1e-5, 1), rng.uniform(1e-5, 1)), curv1=(rng.uniform(1e-5, 1), rng.uniform(1e-5, 1)),
                height=height, width=width, ar_coated=True, bin_count=32, bin_size=0.8, linear_slope=1.0,
                linear_intercept=0.1, det_length=32.0, max_incident_angle=math.radians(45.0),
                det_angle=rng.uniform(-math.pi, math.pi), wavelength_bounds=(0.5, 0.82), fiber_radius=0.05,
                fiber_na=0.32, fiber_center_y=height * rng.uniform(0, 1))


def _first_lens_has_hit(d):
    """Whether the axial ray from the fiber centre meets the first toric lens inside its
    bounds, by a polynomial root finder (ToricLens::from_hyperplane, toric.rs:221-262)."""
    a0, h = d["angles"][0], d["height"]
    n = np.array([-math.cos(a0), -math.sin(a0), 0.0])
    p = np.array([abs(n[1] / n[0]) * h / 2, h / 2, 0.0])
    spc, ntc = d["curv0"]
    chord = abs(h / n[0])
    pr = chord * 0.5 / abs(spc)
    tr = d["width"] * 0.5 / ntc
    apothem = math.sqrt(pr * pr - chord * chord * 0.25)
    c = n * math.copysign(apothem + tr, spc) + p
    tn = np.array([-n[1], n[0], 0.0])
    bn = n if spc < 0 else -n
    o = np.array([0.0, d["fiber_center_y"], 0.0])
    v = np.array([1.0, 0.0, 0.0])
    dp = o - c
    for t in _real_roots(_quartic(tr * tr, pr * pr, dp @ dp, dp @ v, dp @ tn, tn @ v)):
        s = bn @ (o + v * t - p)
        if t >= 0 and 0 <= s <= pr - apothem:
            return True
    return False


def test_designer_fiber_configuration_cannot_be_positioned():
    rng = np.random.default_rng(1)
    n, failed, with_hit = 200, 0, 0
    for _ in range(n):
        d = _designer_fiber_design(rng)
        e, _, _ = O.position_detector3(d, 1.0)
        failed += e != O.OK
        with_hit += _first_lens_has_hit(d)
    assert failed == n               # every design raises RayTraceError
    assert with_hit > 0.6 * n        # although most axial rays do cross the first lens


def test_positioned_3d_design_loses_every_ray_at_the_first_lens():
    """With the detector placed by hand (designer.py's position branch), the fitness of a
    fiber design: every ray stops at the first toric lens, so p(d|lambda) is zero."""
    rng = np.random.default_rng(5)
    d = _designer_fiber_design(rng)
    d["det_position"], d["det_flipped"] = (60.0, d["height"] / 2), False
    q = O.qrng3_points(0.5, 512)
    lam = np.repeat(np.linspace(0.0, 1.0, 16), 512)
    bins, ts, status, nan, calls = O.trace_pairs3(d, lam, np.tile(q, (16, 1)))
    assert (bins == d["bin_count"]).all() and (calls == 1).all()
    assert (status == O.NO_SURFACE_INTERSECTION).all() and (nan > 0).mean() > 0.9
    p, st = O.fitness_points3(d, np.linspace(0.0, 1.0, 16), q)
    assert st["hits"] == 0 and st["info"] == 0.0 and not p.any()
