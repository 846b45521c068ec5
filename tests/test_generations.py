"""Host side of the serving workload: whole-generation design building and the
synthetic optimizer's genome operators. No GPU calls."""
import ctypes as C

import numpy as np

import compound_prism_designer as cpd
from compound_prism_designer import _native as N
from compound_prism_designer import generations as gen
from compound_prism_designer import synth


def _class_path_design(pop, cat, i):
    G = int(pop.G[i])
    glasses = [cpd.Glass("g", cat[k]) for k in pop.glass_idx[i, :G]]
    cp = cpd.CompoundPrism(glasses, pop.angles[i, :G + 1], [0.0] * G, pop.curvature[i], pop.height[i], 7.0, True)
    wl = cpd.UniformWavelengthDistribution(synth.WAVELENGTHS)
    beam = cpd.GaussianBeam(2.0, pop.height[i] * pop.y_frac[i])
    det = synth.detector_for_bins(int(pop.B[i]))
    pos, fl = cpd.position_detector_array(det["length"], pop.det_angle[i], cp, wl, beam, 1.0)
    da = cpd.DetectorArray(det["bin_count"], det["bin_size"], det["linear_slope"], det["linear_intercept"],
                           det["length"], det["max_incident_angle"], pop.det_angle[i], pos, fl)
    return cpd.Spectrometer(cp, da, wl, beam)


def test_batch_build_equals_the_class_path_bitwise():
    rng = np.random.default_rng(3)
    cat = gen.glass_catalog(rng, 8)
    pop = gen.random_population(rng, 64, len(cat))
    d, ok = gen.build(pop, cat)
    assert 0 < ok.sum() < 64 or ok.all()
    for i in range(64):
        if ok[i]:
            s = _class_path_design(pop, cat, i)
            assert bytes(s.design) == d[i].tobytes()
        else:
            assert not d[i].tobytes().strip(b"\0")


def test_batch_build_without_positioning_uses_the_given_detector():
    rng = np.random.default_rng(4)
    cat = gen.glass_catalog(rng, 8)
    pop = gen.initial_population(rng, 8, cat)
    p = gen.to_params(pop, cat)
    placed, st = cpd.build_designs(p, acceptance=1.0)
    assert (st == N.OK).all()
    for i in range(8):
        q = N.SpectrometerParams.from_buffer_copy(p[i].tobytes())
        pos = (C.c_double * 2)()
        fl = C.c_int32(0)
        assert N.lib.cpd_position_detector_array(C.byref(q), 1.0, pos, C.byref(fl)) == N.OK
        p[i]["det_position"] = tuple(pos)
        p[i]["det_flipped"] = fl.value
    again, st2 = cpd.build_designs(p, acceptance=0.0)
    assert (st2 == N.OK).all()
    assert again.tobytes() == placed.tobytes()


def test_perturbation_stays_in_range_and_keeps_prism_and_bin_counts():
    rng = np.random.default_rng(5)
    cat = gen.glass_catalog(rng, 16)
    parents = gen.random_population(rng, 32, len(cat))
    off = gen.perturb(rng, parents, 4096, len(cat))
    assert set(np.unique(off.G)) <= set(gen.G_CHOICES) and set(np.unique(off.B)) <= set(gen.B_CHOICES)
    mag = np.abs(off.angles)
    assert mag.min() >= gen.ANGLE_MAG[0] and mag.max() <= gen.ANGLE_MAG[1]
    for k, r in (("curvature", gen.CURVATURE), ("height", gen.HEIGHT), ("y_frac", gen.Y_MEAN),
                 ("det_angle", gen.DET_ANGLE)):
        v = getattr(off, k)
        assert v.min() >= r[0] and v.max() <= r[1]
    assert (off.glass_idx >= 0).all() and (off.glass_idx < len(cat)).all()


def test_survival_keeps_the_best():
    rng = np.random.default_rng(6)
    pop = gen.random_population(rng, 10, 4)
    info = np.arange(10, dtype=float)
    keep = gen.survive(pop, info, 3)
    assert np.array_equal(keep.height, pop.height[[9, 8, 7]])


def test_near_critical_designs_sit_within_two_degrees_of_tir():
    from compound_prism_designer import precision as P

    pop = P.study_population(99, n=4, B=128)
    for spec, near, margin in pop[:2]:
        assert near and 0.0 < margin <= 2.0
        # the margin is the smallest over three wavelengths: the middle one leaves too
        assert P.exit_margin_deg(spec, spec.beam.y_mean, 0.66) >= margin
    for spec, near, margin in pop[2:]:
        assert not near
