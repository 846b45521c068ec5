"""Host side of the product against the oracle (no GPU): design tables, detector
positioning, cpu_fitness, propagation path, exit ray, glass index and the
Python API's argument checks and errors (src/pylib.rs)."""
import math

import numpy as np
import pytest

import oracle as O
import compound_prism_designer as cpd
from compound_prism_designer import synth
from conftest import load_golden


def _tables(spec, G):
    D = spec.design
    out = []
    for i in range(G):
        out += [D.face_point[i][0], D.face_point[i][1], D.face_normal[i][0], D.face_normal[i][1]]
    out += [D.exit_center[0], D.exit_center[1], D.exit_radius, D.exit_bound_center[0], D.exit_bound_center[1],
            D.exit_bound_r2]
    out += [D.det_normal[0], D.det_normal[1], D.det_direction[0], D.det_direction[1], D.min_ci, D.size,
            D.deviation]
    return np.array(out)


@pytest.fixture(scope="module")
def designs(f1):
    rng = np.random.default_rng(5)
    out = [(synth.spectrometer_from_dict(f1), f1)]
    for G, B in [(1, 8), (2, 16), (3, 32), (4, 64), (5, 128), (6, 64)]:
        s, d, _ = synth.random_design(rng, G, B)
        out.append((s, d))
    return out


def test_design_tables_bit_identical_to_oracle(designs):
    for s, d in designs:
        G = len(d["glasses"])
        np.testing.assert_array_equal(_tables(s, G), O.design_dump(d))


def test_detector_positioning_bit_identical(designs):
    for s, d in designs:
        e, pos, fl = O.position_detector(d, 1.0)
        assert e == O.OK
        got = cpd.position_detector_array(d["det_length"], d["det_angle"], s.compound_prism, s.wavelengths,
                                          s.beam, 1.0)
        assert got == (pos, fl)


def test_cpu_fitness_bit_identical_to_oracle(designs):
    for s, d in designs[:4]:
        ref = O.fitness_adaptive(d, 2048, 2048)
        f = s.cpu_fitness(max_n=2048, max_m=2048)
        assert (f.size, f.info, f.deviation) == ref


def test_cpu_fitness_f1_golden(f1):
    g = load_golden("f1_known_design.json")
    f = synth.spectrometer_from_dict(f1).cpu_fitness()
    got = {"size": f.size, "info": f.info, "deviation": f.deviation}
    for name, exp in g["expected"].items():
        assert abs(got[name] - exp["value"]) / abs(exp["value"]) <= exp["rmax"]


def test_ray_trace_matches_propagation_path(designs):
    for s, d in designs:
        for w in (0.5, 0.63, 0.82):
            y = d["beam_y_mean"]
            np.testing.assert_array_equal(s.ray_trace(w, y), O.propagation_path(d, w, y))


def test_exit_ray_and_errors(f1):
    s = synth.spectrometer_from_dict(f1)
    rows = O.propagation_path(f1, 0.6, 0.95)
    o, u = s.compound_prism.exit_ray(0.95, 0.6)
    G = len(f1["glasses"])
    assert (o.x, o.y, u.x, u.y) == tuple(rows[G + 1])
    with pytest.raises(cpd.RayTraceError):
        s.compound_prism.exit_ray(1e6, 0.6)  # starts far above the prism: misses the entry face


def test_glass_index_and_norminv():
    c = [-0.19660238, 0.85166448, -1.49929414, 1.35438084, -0.64424681, 1.62434799]
    import ctypes

    g = cpd.Glass("N-PK52A", c)
    arr = (ctypes.c_double * 6)(*c)
    for w in (0.5, 0.6, 0.82):
        assert g(w) == O.lib().orc_calc_n(arr, w)
    from compound_prism_designer import _native as N

    for u in (1e-10, 0.1, 0.5, 0.7, 0.999):
        assert N.lib.cpd_norminv(u) == O.norminv(u)


def test_constructor_argument_checks():
    g = cpd.Glass("a", [0, 0, 0, 0, 0, 1.5])
    with pytest.raises(ValueError, match="len\\(glasses\\) \\+ 1 != len\\(angles\\)"):
        cpd.CompoundPrism([g, g], [0.1, -0.2], [0, 0], 0.05, 20, 7, True)
    with pytest.raises(ValueError, match="len\\(glasses\\) != len\\(lengths\\)"):
        cpd.CompoundPrism([g], [0.1, -0.2], [0, 0], 0.05, 20, 7, True)
    with pytest.raises(ValueError, match="Maximum of 6 prisms"):
        cpd.CompoundPrism([g] * 7, [0.1] * 8, [0] * 7, 0.05, 20, 7, True)
    with pytest.raises(ValueError, match="Incorrect coefficents length"):
        cpd.Glass("b", [1, 2, 3])
    with pytest.raises(ValueError):
        cpd.UniformWavelengthDistribution((0.8, 0.5))
    with pytest.raises(NotImplementedError):
        cpd.CompoundPrism([g], [0.1, -0.2], [0], ((0.1, 0.1), (0.1, 0.1)), 20, 7, True)


def test_positioning_raises_raytrace_error():
    # a single glass with n = 1 everywhere deviates nothing: both rays are parallel
    g = cpd.Glass("air", [0, 0, 0, 0, 0, 1.0])
    cp = cpd.CompoundPrism([g], [0.3, -0.3], [0.0], 0.05, 20, 7, True)
    with pytest.raises(cpd.RayTraceError):
        cpd.position_detector_array(32, 0.0, cp, cpd.UniformWavelengthDistribution((0.5, 0.82)),
                                    cpd.GaussianBeam(2, 10), 1.0)


def test_synthetic_glass_fit_matches_reference_fit():
    gf = load_golden("glass_fits.json")
    for g in gf["glasses"]:
        mine = synth.horner_fit(g["sellmeier1"], tuple(g["limits"]))
        x = np.linspace(0.5, 0.82, 50)
        # the same least-squares optimum: scipy's curve_fit stops at its default ftol, so the
        # fitted indices agree to ~1e-9, three orders below the fit's own RMS residual
        rms = np.sqrt(g["chisq"] / 100)
        np.testing.assert_allclose(np.polyval(mine, x), np.polyval(g["horner"], x), rtol=0, atol=1e-8)
        assert np.max(np.abs(np.polyval(mine, x) - np.polyval(g["horner"], x))) < 1e-2 * rms


def test_pickle_round_trip(f1):
    import pickle

    s = synth.spectrometer_from_dict(f1)
    s2 = pickle.loads(pickle.dumps(s))
    assert bytes(s2.design) == bytes(s.design)
