"""compound_prism_designer.multigpu with the real batched GPU evaluator: a population split
over two contexts (two device threads; this run has one GPU, so both contexts share it)
gives, record for record, the single batched call's results -- the partition, the threads
and the reassembly change nothing (integer accumulation)."""
import numpy as np
import pytest

import compound_prism_designer as cpd
from compound_prism_designer import multigpu, synth

pytestmark = pytest.mark.gpu


def test_population_over_two_contexts_equals_one_batch():
    pop, _ = synth.population(6161, 24)
    specs = [s for s, _ in pop]
    W = np.random.default_rng(1).integers(64, 513, len(specs))
    ref = cpd.fitness_batch(specs, seeds=0.4, max_n=W, max_eval=1024)
    outs = multigpu.fitness_population(specs, seeds=0.4, max_n=W, max_eval=1024, devices=[0, 0])
    for r, o in zip(ref, outs):
        assert r.info == o["info"] and r.hits == o["hits"] and r.status == o["status"]
        assert r.wavelengths == o["wavelengths"] and r.retraced == o["retraced"]
