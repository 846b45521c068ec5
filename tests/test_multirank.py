"""The multi-GPU path on the CPU: two gloo ranks shard a population by design, each
evaluates its own shard (with the oracle standing in for the GPU, which this container
does not have), and the gathered results equal the single-process evaluation. Also
checks the bench's host barrier and max/sum reductions."""
import os
import socket

import numpy as np
import pytest

from conftest import ROOT

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from compound_prism_designer import sharding  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _population():
    from compound_prism_designer import synth

    pop, _ = synth.population(4242, 6)
    rng = np.random.default_rng(7)
    W = rng.integers(8, 33, len(pop))
    return [d for _, d in pop], W


def _evaluate(d, W):
    import oracle as O

    lam = O.qrng_points(0.5, int(W))
    ray = O.qrng_points(0.5, 64)
    _, st = O.fitness_points(d, lam, ray, nthreads=1, want_p=False)
    return np.array([st["info"], st["h_cond"], st["h_det"]])


def _rank_main(rank, world, port, out_path):
    import sys

    for p in (ROOT, os.path.join(ROOT, "compound-prism-designer_gb300"), os.path.join(ROOT, "oracle")):
        if p not in sys.path:
            sys.path.insert(0, p)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    import bench

    D = bench.Dist()
    designs, W = _population()
    mine = sharding.shard_for_rank([int(w) * 64 for w in W], rank, world)
    res = torch.zeros(len(designs), 3, dtype=torch.float64)
    for i in mine:
        res[i] = torch.from_numpy(_evaluate(designs[i], W[i]))
    D.barrier()
    dist.all_reduce(res, op=dist.ReduceOp.SUM)  # shards are disjoint: the sum is a gather
    mx = D.max(float(rank + 1))
    sm = D.sum(float(len(mine)))
    if rank == 0:
        np.save(out_path, np.concatenate([res.numpy().ravel(), [mx, sm]]))
    dist.destroy_process_group()


def test_shard_by_work_is_balanced_and_complete():
    work = [5, 1, 9, 3, 3, 8, 2, 7]
    parts = sharding.shard_by_work(work, 3)
    assert sorted(i for p in parts for i in p) == list(range(len(work)))
    loads = [sum(work[i] for i in p) for p in parts]
    assert max(loads) - min(loads) <= max(work)
    assert sharding.shard_by_work(work, 1) == [list(range(len(work)))]


def test_two_gloo_ranks_gather_the_single_process_results(tmp_path):
    designs, W = _population()
    ref = np.stack([_evaluate(d, w) for d, w in zip(designs, W)])
    out = str(tmp_path / "r.npy")
    mp.start_processes(_rank_main, args=(2, _free_port(), out), nprocs=2, start_method="spawn")
    got = np.load(out)
    np.testing.assert_array_equal(got[:-2].reshape(ref.shape), ref)
    assert got[-2] == 2.0 and got[-1] == len(designs)
