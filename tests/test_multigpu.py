"""Population fitness over several GPUs (compound_prism_designer.multigpu) on the CPU: the
dispatch itself runs -- partition by ray counts, one evaluator per device or per rank,
results back in population order, and for one process per GPU the host-side all-gather
over a gloo group of two ranks -- with the oracle standing in for each device's batched
GPU evaluation (this container has no GPU). The gathered results must equal one
evaluator's over the whole population, record for record."""
import os
import socket

import numpy as np
import pytest

from conftest import ROOT

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from compound_prism_designer import _native as N  # noqa: E402
from compound_prism_designer import multigpu, synth  # noqa: E402


def _population():
    pop, _ = synth.population(5151, 9)
    specs = [s for s, _ in pop]
    dicts = [d for _, d in pop]
    rng = np.random.default_rng(3)
    W = rng.integers(8, 40, len(pop))
    return specs, dicts, W


def _stand_in(dicts):
    """evaluate(indices, items) with the oracle on each design's own points."""
    import oracle as O

    def evaluate(idx, items):
        out = np.zeros(len(idx), dtype=N.FITNESS_DTYPE)
        for k, (i, it) in enumerate(zip(idx, items)):
            lam = O.gpu_points(float(it["seed"]), int(it["max_n"]))
            ray = O.gpu_points(float(it["seed"]), int(it["max_eval"]), first=1)
            _, st = O.fitness_points(dicts[i], lam, ray, want_p=False)
            out[k]["info"], out[k]["hits"] = st["info"], st["hits"]
            out[k]["wavelengths"], out[k]["rays"] = int(it["max_n"]), int(it["max_n"]) * int(it["max_eval"])
            out[k]["size"] = st["size"]
        return out

    return evaluate


def test_partition_covers_the_population_once():
    items = np.zeros(7, dtype=N.BATCH_ITEM_DTYPE)
    items["max_n"] = [10, 40, 5, 5, 30, 8, 20]
    items["max_eval"] = 64
    parts = multigpu.partition(items, 3)
    assert sorted(int(i) for p in parts for i in p) == list(range(7))
    loads = [int((items["max_n"][p] * 64).sum()) for p in parts]
    assert max(loads) - min(loads) <= 40 * 64


def test_one_process_several_devices_equals_one_device():
    specs, dicts, W = _population()
    one = multigpu.fitness_population(specs, seeds=0.3, max_n=W, max_eval=64, evaluators=[_stand_in(dicts)])
    three = multigpu.fitness_population(specs, seeds=0.3, max_n=W, max_eval=64,
                                        evaluators=[_stand_in(dicts) for _ in range(3)])
    assert one.tobytes() == three.tobytes()
    assert (one["wavelengths"] == W).all() and (one["hits"] > 0).any()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_path):
    import sys

    for p in (ROOT, os.path.join(ROOT, "compound-prism-designer_gb300"), os.path.join(ROOT, "oracle")):
        if p not in sys.path:
            sys.path.insert(0, p)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from compound_prism_designer import multigpu as mg

    specs, dicts, W = _population()
    dp = mg.DistributedPopulation(evaluate_factory=lambda d, mode: _stand_in(dicts))
    outs = dp.evaluate(specs, seeds=0.3, max_n=W, max_eval=64)
    np.save(out_path + f".{rank}.npy", np.frombuffer(outs.tobytes(), dtype=np.uint8))
    dist.destroy_process_group()


def test_two_gloo_ranks_all_gather_the_single_process_results(tmp_path):
    specs, dicts, W = _population()
    ref = multigpu.fitness_population(specs, seeds=0.3, max_n=W, max_eval=64, evaluators=[_stand_in(dicts)])
    out = str(tmp_path / "pop")
    mp.start_processes(_rank_main, args=(2, _free_port(), out), nprocs=2, start_method="spawn")
    for r in range(2):
        got = np.load(out + f".{r}.npy").tobytes()
        assert got == ref.tobytes(), r
