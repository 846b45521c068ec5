"""Designs built on the GPU from parameter records (cpd_design_build_device,
cpd_fitness_gpu_batch_params, cpd_server_submit_params) against the host build
(cpd_design_build_batch, the C++ restatement pinned to the reference's geometry by
tests/test_host_api.py and the oracle's design dump).

Tolerances: the device uses CUDA's f64 sin/cos where the host uses the C library's, so
a table may differ in its last bits (relative 1e-14); the build status (including the
ray-trace errors of detector positioning) must be equal. Fitness of a design built on the
device: within the parity bounds of the host-built design's (MI 1e-4 relative), and
bitwise equal where the two tables are bitwise equal.
"""
import numpy as np
import pytest

import compound_prism_designer as cpd
from compound_prism_designer import _native as N
from compound_prism_designer import generations as gen

pytestmark = pytest.mark.gpu

FLOAT_FIELDS = ("glass", "face_point", "face_normal", "height", "exit_center", "exit_radius", "exit_bound_center",
                "exit_bound_r2", "bin_size", "linear_slope", "linear_intercept", "min_ci", "det_length", "det_normal",
                "det_position", "det_direction", "wavelength_bounds", "beam_width", "beam_y_mean", "size",
                "deviation")


def _params(n=300, seed=5):
    rng = np.random.default_rng(seed)
    cat = gen.glass_catalog(rng, 32)
    return gen.to_params(gen.random_population(rng, n, len(cat)), cat)


@pytest.mark.parametrize("acceptance", [1.0, 0.0])
def test_device_records_match_host(acceptance):
    p = _params()
    dh, sh = cpd.build_designs(p, acceptance=acceptance)
    dd, sd = cpd.build_designs(p, acceptance=acceptance, device=True)
    assert np.array_equal(sh, sd), np.nonzero(sh != sd)[0][:10]
    ok = sh == 0
    assert ok.sum() > 50
    if acceptance > 0:
        assert (~ok).sum() > 0  # positioning failures exercised too
    for k in ("nglass", "bin_count", "ar_coated"):
        assert np.array_equal(dh[k][ok], dd[k][ok]), k
    for k in FLOAT_FIELDS:
        a, b = dh[k][ok], dd[k][ok]
        assert np.allclose(a, b, rtol=1e-14, atol=1e-14 * np.abs(a).max()), k


def test_batch_params_matches_host_built():
    p = _params(160, seed=9)
    dh, sh = cpd.build_designs(p, acceptance=1.0)
    ok = np.nonzero(sh == 0)[0]
    # host-built designs through the ordinary batch
    specs = []
    for i in ok:
        sp = cpd.Spectrometer.__new__(cpd.Spectrometer)
        sp._design = N.Design.from_buffer_copy(dh[i].tobytes())
        specs.append(sp)
    ref = cpd.fitness_batch(specs, seeds=0.5, max_n=64, max_eval=2048)
    out = cpd.fitness_batch_params(p, acceptance=1.0, seeds=0.5, max_n=64, max_eval=2048)
    assert np.array_equal(out["status"][sh != 0], sh[sh != 0])  # build errors reported per design
    assert (out["info"][sh != 0] == 0).all()
    dd, _ = cpd.build_designs(p, acceptance=1.0, device=True)
    same = 0
    for j, i in enumerate(ok):
        r, o = ref[j], out[i]
        assert o["status"] in (N.OK, N.NOT_CONVERGED)
        assert abs(o["info"] - r.info) <= 1e-4 * abs(r.info) + 1e-9, (i, o["info"], r.info)
        assert abs(o["size"] - r.size) <= 1e-12 * r.size and abs(o["deviation"] - r.deviation) <= 1e-12
        if dd[i].tobytes() == dh[i].tobytes():
            same += 1
            assert o["info"] == r.info and o["hits"] == r.hits, i
    assert same > 0


def test_server_params_alone_equals_mix():
    p = _params(96, seed=13)
    alone = cpd.fitness_batch_params(p[:8], acceptance=1.0, seeds=0.25, max_n=32, max_eval=1024)
    with cpd.Server(mem_budget_bytes=1 << 28, slots=2) as sv:
        r1 = sv.submit_params(p, acceptance=1.0, seeds=0.25, max_n=32, max_eval=1024)
        r2 = sv.submit_params(p[:8], acceptance=1.0, seeds=0.25, max_n=32, max_eval=1024)
        mix, _ = sv.wait(r1, timeout=120)
        few, _ = sv.wait(r2, timeout=120)
    for k in ("info", "h_cond", "h_det", "hits", "status", "size", "deviation"):
        assert np.array_equal(mix[k][:8], alone[k]), k
        assert np.array_equal(few[k], alone[k]), k


def test_generations_serve_with_device_build():
    with cpd.Server(mem_budget_bytes=1 << 30, slots=2) as sv:
        r = gen.serve(sv, generations=3, sizes=(64, 128), mu=64, device_build=True, seed=3)
    assert r["designs"] >= 3 * 64 and r["best_info"] is not None and r["best_info"] > 0
