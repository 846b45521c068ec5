"""The adaptive-sampling oracle (orc_fitness_adaptive_points) pinned against the
reference GPU kernel's own stop rule.

`_kernel_row` below is a literal restatement of src/spectrometer/kernel.rs:127-189 in
f64: rounds of 32 rays; for each bin a round hit (in increasing bin order, the warp_min
loop of kernel.rs:147-170) a 32-sample Welford of the round (the hits' t, zeros
elsewhere) merged into the bin's state with Welford's `+` (welford.rs:86-91); stop when
the round hit some bin and every merged state passes sem_le_error_threshold
(welford.rs:80-84); p = the state's mean padded with zeros to every ray consumed
(Welford::skip, kernel.rs:181-189). It runs on the oracle's own per-ray (bin, t).

The oracle does the same merges in exact integer arithmetic on t quantized to 2^-20.
The two must stop every wavelength after the same round, except where the literal f64
test is within a hair of its threshold (quantization and rounding can flip only those).
"""
import numpy as np
import pytest

import oracle as O
from compound_prism_designer import synth

MAX_ERR_SQ = 5e-3 * 5e-3


def _kernel_row(bins, ts, nbin, R):
    """Returns (rays consumed, p[nbin], smallest relative margin of a deciding test)."""
    state = {}
    count = 0
    margin = np.inf
    for r0 in range(0, R, 32):
        b = bins[r0:r0 + 32]
        t = ts[r0:r0 + 32]
        count += 32
        hit = b < nbin
        finished = bool(hit.any())
        for bb in sorted(set(b[hit].tolist())):
            x = np.where(b == bb, t, 0.0)
            wm = x.sum() / 32.0
            wm2 = ((x - wm) ** 2).sum()
            c, m, m2 = state.get(bb, (0.0, 0.0, 0.0))
            cn = c + 32.0
            delta = wm - m
            mean = (c * m + 32.0 * wm) / cn
            m2n = m2 + wm2 + delta * delta * c * 32.0 / cn
            state[bb] = (cn, mean, m2n)
            thr = MAX_ERR_SQ * (cn * (cn - 1.0))
            margin = min(margin, abs(m2n - thr) / thr)
            finished = finished and m2n < thr
        if finished:
            break
    p = np.zeros(nbin)
    for bb, (c, m, _) in state.items():
        p[bb] = c * m / count
    return count, p, margin


def _designs(f1):
    rng = np.random.default_rng(77)
    out = [("F1", f1)]
    for G, B in [(2, 16), (3, 32), (4, 64), (6, 128)]:
        _, d, _ = synth.random_design(rng, G, B)
        out.append((f"G{G}B{B}", d))
    return out


@pytest.mark.parametrize("W,R", [(16, 8192)])
def test_oracle_adaptive_matches_kernel_rule(f1, W, R):
    lam_u = O.qrng_points(0.5, W)
    ray_u = O.qrng_points(0.25, R)
    flips = 0
    for name, d in _designs(f1):
        p, st, counts = O.fitness_adaptive_points(d, lam_u, ray_u, nthreads=4)
        bins, ts = O.trace_pairs(d, np.repeat(lam_u, R), np.tile(ray_u, W))
        bins = bins.reshape(W, R)
        ts = ts.reshape(W, R)
        nbin = int(d["bin_count"])
        hits = 0
        for k in range(W):
            c, pk, margin = _kernel_row(bins[k], ts[k], nbin, R)
            hits += int((bins[k][:counts[k]] < nbin).sum())
            if c != counts[k]:
                # only a test within rounding distance of its threshold may decide otherwise
                assert margin < 1e-5, (name, k, c, counts[k], margin)
                flips += 1
                continue
            assert np.abs(pk - p[k]).max() <= 1e-9, (name, k)
        assert st["hits"] == hits, name
    assert flips <= 1


def test_oracle_adaptive_single_bin_stops_after_one_round(f1):
    """A wavelength whose 32 rays all land in one bin with nearly equal t passes the
    SEM test at once: one round, p = that bin's mean t."""
    lam_u = O.qrng_points(0.5, 16)
    # a narrow ray band: every start height within a tiny range around the beam centre
    ray_u = 0.5 + 1e-7 * (O.qrng_points(0.5, 256) - 0.5)
    p, st, counts = O.fitness_adaptive_points(f1, lam_u, ray_u)
    bins, ts = O.trace_pairs(f1, np.repeat(lam_u, 32), np.tile(ray_u[:32], 16))
    bins = bins.reshape(16, 32)
    for k in range(16):
        if (bins[k] < f1["bin_count"]).all() and len(set(bins[k].tolist())) == 1:
            assert counts[k] == 32
            # t is accumulated as round(2^31 t): p within 2^-31 of the exact mean
            assert abs(p[k].sum() - ts.reshape(16, 32)[k].mean()) < 1e-9


def test_oracle_adaptive_partial_last_round(f1):
    """R not a multiple of 32: the last round is shorter and counts only its rays."""
    lam_u = O.qrng_points(0.5, 8)
    for R in (1, 31, 33, 100):
        ray_u = O.qrng_points(0.5, R)
        p, st, counts = O.fitness_adaptive_points(f1, lam_u, ray_u)
        assert (counts >= 1).all() and (counts <= R).all()
        # a wavelength that ran out of rays consumed exactly R
        full = counts[counts > R - ((R - 1) % 32 + 1)]
        assert (full == R).all(), (R, counts)
        assert np.isfinite(p).all() and (p >= 0).all() and (p.sum(axis=1) <= 1 + 1e-12).all()


def test_oracle_adaptive_equals_fixed_n_over_rays_consumed(f1):
    """Each adaptive row is the fixed-N estimate over the rays it consumed (up to the
    2^-31 quantization of t)."""
    lam_u = O.qrng_points(0.5, 12)
    ray_u = O.qrng_points(0.5, 512)
    p, st, counts = O.fitness_adaptive_points(f1, lam_u, ray_u)
    for k in range(12):
        pf, _ = O.fitness_points(f1, lam_u[k:k + 1], ray_u[:counts[k]])
        assert np.abs(pf[0] - p[k]).max() <= 1e-9
