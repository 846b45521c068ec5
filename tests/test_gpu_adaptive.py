"""GPU adaptive sampling (CPD_SAMPLING_ADAPTIVE) against the oracle's restatement of
the reference kernel's per-wavelength SEM stop (orc_fitness_adaptive_points; pinned to
the kernel's own Welford rule in tests/test_oracle_adaptive.py).

Tolerances:
* rays consumed: exactly equal (sum over wavelengths). The stop decisions are exact
  integer tests; a decision that the FP32 transmittances cannot settle is redone on the
  float-float path, so the GPU decides like the oracle;
* hits: exactly equal;
* p(d|lambda): within 1e-6 absolute; MI within 1e-4 relative.
"""
import os

import numpy as np
import pytest

import oracle as O
import compound_prism_designer as cpd
from compound_prism_designer import precision as P
from compound_prism_designer import synth

pytestmark = pytest.mark.gpu

NTHREADS = max(1, min(16, os.cpu_count() or 1))
ADAPTIVE = cpd.TRACE_HYBRID | cpd.SAMPLING_ADAPTIVE


@pytest.fixture(scope="module")
def designs(f1):
    rng = np.random.default_rng(20261205)
    out = [("F1", synth.spectrometer_from_dict(f1), f1)]
    for G, B in [(2, 16), (3, 32), (4, 64), (5, 128), (6, 64), (6, 128)]:
        s, d, _ = synth.random_design(rng, G, B)
        out.append((f"G{G}B{B}", s, d))
    return out


def _check(s, d, lam_u, ray_u, mode=ADAPTIVE):
    f, p = s.gpu_fitness_points(lam_u, ray_u, mode=mode, want_p=True)
    po, st, counts = O.fitness_adaptive_points(d, lam_u, ray_u, nthreads=NTHREADS)
    assert f.rays == int(counts.sum()), (f.rays, int(counts.sum()))
    assert f.hits == st["hits"], (f.hits, st["hits"])
    err_p = np.abs(p - po).max()
    assert err_p <= 1e-6, err_p
    assert abs(f.info - st["info"]) <= 1e-4 * abs(st["info"]) + 1e-9, (f.info, st["info"])
    return f, counts


@pytest.mark.parametrize("W,R", [(128, 8192), (64, 1000)])
def test_adaptive_points_equal_oracle(designs, W, R):
    lam_u = O.qrng_points(0.5, W)
    ray_u = O.qrng_points(0.25, R)
    stopped = 0
    for name, s, d in designs:
        f, counts = _check(s, d, lam_u, ray_u)
        stopped += int((counts < R).sum())
    if R >= 8192:
        assert stopped > 0  # the stop rule was exercised (1000 rays are too few to stop)


def test_adaptive_exact_path_decides_the_same(designs):
    """Every wavelength on the float-float path (SAMPLING_EXACT) stops after the same
    rounds as the default FP32-with-fallback path, and both match the oracle."""
    lam_u = O.qrng_points(0.5, 96)
    ray_u = O.qrng_points(0.25, 4096)
    for name, s, d in designs:
        fa, _ = _check(s, d, lam_u, ray_u)
        fe, _ = _check(s, d, lam_u, ray_u, mode=ADAPTIVE | cpd.SAMPLING_EXACT)
        assert fa.rays == fe.rays and fa.hits == fe.hits, name
        assert fe.retraced >= fe.hits  # every ray of the band went through the float-float path


def test_adaptive_gpu_seed_policy(designs):
    """gpu_fitness(adaptive=True): the GPU seed policy's points, the multi-seed loop, and
    the rays consumed reported in cpd_fitness.rays."""
    seed = 0.3
    for name, s, d in designs[:4]:
        f = s.gpu_fitness_full(seed, max_n=128, max_eval=8192, adaptive=True)
        lam_u = P.synth_points(seed, 128)
        ray_u = P.synth_points(seed, 8192, first=1)
        po, st, counts = O.fitness_adaptive_points(d, lam_u, ray_u, nthreads=NTHREADS)
        assert f.rays == int(counts.sum()), name
        assert f.hits == st["hits"], name
        assert abs(f.info - st["info"]) <= 1e-4 * abs(st["info"]) + 1e-9, name


def test_adaptive_f1_within_reference_gpu_bar(f1):
    """The known design through gpu_fitness with the reference's defaults and adaptive
    sampling: info within the reference's own CPU-vs-GPU bar (relative 1e-2,
    benches/benchmark.rs:153-157) of the golden value 0.7407 (src/fitness.rs:250-257)."""
    s = synth.spectrometer_from_dict(f1)
    f = s.gpu_fitness_full(0.5, max_n=256, max_eval=16384, adaptive=True)
    assert abs(f.info - 0.7407) <= 1e-2 * 0.7407, f.info
    assert f.rays < 256 * 16384  # some wavelengths stopped early


def test_adaptive_batch_bitwise_equal_alone(designs):
    """A design's adaptive result does not depend on what shares its pass."""
    ds = [s for _, s, _ in designs]
    seeds = [0.5, 0.25, 0.5, 0.75, 0.5, 0.1, 0.5]
    max_n = [64, 128, 32, 64, 64, 16, 64]
    max_eval = [4096, 2048, 8192, 4096, 1000, 4096, 4096]
    mix = cpd.fitness_batch(ds, seeds=seeds, max_n=max_n, max_eval=max_eval, mode=ADAPTIVE)
    for i, s in enumerate(ds):
        one = cpd.fitness_batch([s], seeds=seeds[i], max_n=max_n[i], max_eval=max_eval[i], mode=ADAPTIVE)[0]
        for k in ("info", "h_cond", "h_det", "max_sem", "rays", "hits", "status"):
            assert getattr(mix[i], k) == getattr(one, k), (i, k, getattr(mix[i], k), getattr(one, k))


def test_adaptive_server_matches_batch(designs):
    ds = [s for _, s, _ in designs]
    ref = cpd.fitness_batch(ds, seeds=0.5, max_n=64, max_eval=4096, mode=ADAPTIVE)
    with cpd.Server(mem_budget_bytes=1 << 30, slots=2) as sv:
        rid = sv.submit(ds, seeds=0.5, max_n=64, max_eval=4096, mode=ADAPTIVE)
        out, _ = sv.wait(rid, timeout=120)
    for i in range(len(ds)):
        for k in ("info", "rays", "hits"):
            assert out[i][k] == getattr(ref[i], k), (i, k)


def test_adaptive_rejects_other_trace_modes(designs):
    _, s, _ = designs[0]
    lam_u = O.qrng_points(0.5, 8)
    ray_u = O.qrng_points(0.5, 64)
    for mode in (cpd.TRACE_FP32 | cpd.SAMPLING_ADAPTIVE, cpd.TRACE_FP64 | cpd.SAMPLING_ADAPTIVE,
                 cpd.TRACE_HYBRID | cpd.SAMPLING_EXACT):
        with pytest.raises(ValueError):
            s.gpu_fitness_points(lam_u, ray_u, mode=mode)


@pytest.mark.parametrize("W", [1, 33, 500, 2000])
def test_adaptive_ragged_sizes(designs, W):
    """Rounds past the last ray, a single partial round, and every width of the round groups
    (16 warps per row for a few rows, 4 at 2-7 rows per SM, 2 when rows fill the GPU)."""
    for R in (1, 31, 33, 1000):
        lam_u = O.qrng_points(0.5, W)
        ray_u = O.qrng_points(0.25, R)
        for name, s, d in designs[:3]:
            _check(s, d, lam_u, ray_u)
