"""The FP32 fast path's decisions and the float-float re-trace, checked on the host
against the exact f64 trace (tests/fastpath_check.cpp compiled here with g++ from the
product's model headers).

The host build uses IEEE single-precision sqrt and division where the device uses
its approximate MUFU instructions (the float-float reciprocal and square root refine
either to ~2^-46), so this checks the guard-band logic and the float-float algebra, not
the device rounding; the GPU parity tests check the device itself."""
import json
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, PKG_DIR, ROOT
from compound_prism_designer import precision as P
from compound_prism_designer import synth


@pytest.fixture(scope="module")
def fastpath_bin(tmp_path_factory):
    out = tmp_path_factory.mktemp("fastpath") / "fastpath_check"
    csrc = os.path.join(PKG_DIR, "csrc")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-I", csrc, "-I",
                    os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "fastpath_check.cpp"),
                    os.path.join(csrc, "cpd_host.cpp"), "-o", str(out)], check=True)
    return out


def _run(fastpath_bin, tmp_path, spec, lam_u, ray_u):
    dp, lp, rp = tmp_path / "d.bin", tmp_path / "l.bin", tmp_path / "r.bin"
    dp.write_bytes(bytes(spec.design))
    np.asarray(lam_u, dtype=np.float64).tofile(lp)
    np.asarray(ray_u, dtype=np.float64).tofile(rp)
    out = subprocess.run([str(fastpath_bin), str(dp), str(len(lam_u)), str(len(ray_u)), str(lp), str(rp)],
                         capture_output=True, text=True, check=True).stdout.split()
    return dict(zip(out[0::2], map(int, out[1::2])))


def test_far_reference_ray_design(fastpath_bin, tmp_path):
    case = json.load(open(os.path.join(GOLDEN, "regression_designs.json")))["far_reference_detector"]
    spec = synth.spectrometer_from_dict(case["design"])
    pts = case["points"]
    lam_u = P.synth_points(pts["lam_seed"], pts["wavelengths"])[case["bad_rows"]]
    ray_u = P.synth_points(pts["ray_seed"], pts["rays"], first=pts["ray_first"])
    r = _run(fastpath_bin, tmp_path, spec, lam_u, ray_u)
    assert r["rays"] == len(lam_u) * len(ray_u)
    assert r["mismatches"] == 0 and r["outside_band_hits"] == 0 and r["df_mismatches"] == 0, r


def test_random_designs(fastpath_bin, tmp_path):
    rng = np.random.default_rng(8)
    lam_u = P.synth_points(0.3, 256)
    ray_u = P.synth_points(0.3, 1024, first=1)
    for G, B in [(2, 16), (3, 32), (4, 64), (5, 128), (6, 64), (6, 128)]:
        spec, _, _ = synth.random_design(rng, G, B)
        r = _run(fastpath_bin, tmp_path, spec, lam_u, ray_u)
        assert r["mismatches"] == 0 and r["outside_band_hits"] == 0 and r["df_mismatches"] == 0, (G, B, r)
        assert r["flagged"] < 0.01 * r["rays"], (G, B, r)
        # adaptive sampling's decision guard (kTqDelta = 2 quanta of 2^-20) assumes the
        # fast path's transmittance error stays below 2^-19 ~ 1.9e-6; keep a margin
        assert r["fast_t_relerr_e9"] < 1000, (G, B, r)


@pytest.mark.parametrize("name", ["flat_face_tir_mid", "flat_face_tir_last"])
def test_rows_lost_at_a_flat_face(fastpath_bin, tmp_path, name):
    """Part of the band is lost to total internal reflection at a flat face: the per-row
    setup must drop exactly those rows, and decide the rest like the exact trace."""
    import oracle as O

    case = json.load(open(os.path.join(GOLDEN, "regression_designs.json")))[name]
    spec = synth.spectrometer_from_dict(case["design"])
    pts = case["points"]
    lam_all = O.gpu_points(pts["seed"], pts["wavelengths"])
    lost = np.zeros(lam_all.size, dtype=bool)
    lost[case["tir_rows"]] = True
    sel = np.arange(0, lam_all.size, 4)
    ray_u = O.gpu_points(pts["seed"], 256, first=pts["ray_first"])
    r = _run(fastpath_bin, tmp_path, spec, lam_all[sel], ray_u)
    assert lost[sel].any() and not lost[sel].all()
    assert r["mismatches"] == 0 and r["outside_band_hits"] == 0 and r["df_mismatches"] == 0, r
