"""The batched form at the population config's full per-design size, against the oracle:
16 designs of 6 prisms and 128 bins, 4096 wavelengths x 1024 rays each (the largest
designs of the 1024-design population), in one batched pass, each on its own seed.
Every design's MI must be within 1e-4 relative of the oracle's on the same points and its
hit count equal (one of them reaches its detector with no ray: MI 0 on both sides); a
sampled design's p(d|lambda) is compared through the single-design
call (the batch gives each design the same bits as its single call)."""
import os

import numpy as np
import pytest

import oracle as O
import compound_prism_designer as cpd
from compound_prism_designer import synth

pytestmark = pytest.mark.gpu
NTHREADS = max(1, min(16, os.cpu_count() or 1))
W, R, G, B, N_DESIGNS = 4096, 1024, 6, 128, 16


def test_full_size_batch_equals_oracle():
    rng = np.random.default_rng(20261213)
    pairs = [synth.random_design(rng, G, B)[:2] for _ in range(N_DESIGNS)]
    specs = [s for s, _ in pairs]
    seeds = 0.1 + 0.05 * np.arange(N_DESIGNS)
    outs = cpd.fitness_batch(specs, seeds=seeds, max_n=W, max_eval=R)
    worst = 0.0
    for (s, d), seed, f in zip(pairs, seeds, outs):
        lam, ray = O.gpu_points(seed, W), O.gpu_points(seed, R, first=1)
        _, st = O.fitness_points(d, lam, ray, nthreads=NTHREADS, want_p=False)
        # a design may reach its detector with no ray at all (MI 0): the bound has a floor
        assert abs(f.info - st["info"]) <= 1e-4 * abs(st["info"]) + 1e-12, (seed, f.info, st["info"])
        if st["info"] != 0.0:
            worst = max(worst, abs(f.info - st["info"]) / abs(st["info"]))
        assert f.hits == st["hits"], seed
        assert f.rays == W * R and f.wavelengths == W
    # p(d|lambda) of one design at full size through the single-design call
    s, d = pairs[3]
    lam, ray = O.gpu_points(seeds[3], W), O.gpu_points(seeds[3], R, first=1)
    f1, p = s.gpu_fitness_points(lam, ray, want_p=True)
    po, st = O.fitness_points(d, lam, ray, nthreads=NTHREADS)
    assert np.abs(p - po).max() <= 1e-6
    assert f1.info == outs[3].info and f1.hits == outs[3].hits
    print(f"max MI rel err over {N_DESIGNS} full-size designs: {worst:.2e}")
