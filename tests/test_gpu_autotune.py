"""The launch-shape autotuner: it picks a shape from its candidate set, remembers it
per batch class, and the results it produces are bitwise those of any fixed shape."""
import numpy as np
import pytest

import compound_prism_designer as cpd
from compound_prism_designer import synth

pytestmark = pytest.mark.gpu
FIELDS = ("info", "h_cond", "h_det", "max_sem", "hits", "retraced", "fast_rays", "status")


@pytest.fixture(scope="module")
def batch():
    pop, _ = synth.population(777, 24)
    rng = np.random.default_rng(3)
    return [s for s, _ in pop], rng.integers(64, 512, 24)


def test_autotuner_picks_a_candidate_and_keeps_results(batch):
    specs, W = batch
    ctx = cpd.Context(0)
    ctx.set_launch_shape(32, 8)
    ref = cpd.fitness_batch(specs, max_n=W, max_eval=1024, context=ctx)
    rt, w, ms = cpd.autotune_batch(specs, max_n=W, max_eval=1024, context=ctx)
    # the powers of two 4..256 or a tile that makes whole rounds of the resident warps
    assert 2 <= rt <= 4096 and w in (2, 4, 8) and ms > 0
    assert ctx.launch_shape() == (rt, w)
    got = cpd.fitness_batch(specs, max_n=W, max_eval=1024, context=ctx)
    for a, b in zip(ref, got):
        for f in FIELDS:
            assert getattr(a, f) == getattr(b, f), f
    ctx.close()


def test_autotune_mode_uses_the_remembered_shape_of_a_class(batch):
    specs, W = batch
    ctx = cpd.Context(0)
    rt, w, _ = cpd.autotune_batch(specs, max_n=W, max_eval=1024, context=ctx)
    other = (16, 2) if (rt, w) != (16, 2) else (256, 8)
    ctx.set_launch_shape(*other)
    ctx.set_autotune(True)
    cpd.fitness_batch(specs, max_n=W, max_eval=1024, context=ctx)
    assert ctx.launch_shape() == (rt, w)
    ctx.close()
