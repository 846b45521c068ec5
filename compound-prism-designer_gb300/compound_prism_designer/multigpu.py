"""Population fitness over several GPUs.

Designs are independent, so a population is split by design and no collective touches
the data path. The partition is sharding.shard_by_work on each design's ray count
(wavelengths x rays); it depends only on the work list, so every participant computes the
same one without communicating. Two forms:

* fitness_population(designs, ..., devices=[0, 1, ...]): one process drives several GPUs,
  one Context per device and one host thread per device (ctypes releases the GIL while a
  batch runs); the results come back in population order.
* DistributedPopulation: one process per GPU (torchrun). Every rank evaluates its own
  shard on its own device, then one host-side all-gather of the shards' result records
  (a torch.distributed object collective over the group, gloo or nccl) gives every rank
  the whole population's results.

Both take an `evaluate(indices, items) -> records` hook that evaluates the designs at
`indices` (with their batch items) on one device; the default is the batched GPU form
(cpd_fitness_gpu_batch) on that device's context.
"""
from __future__ import annotations

import ctypes as C
import threading
from typing import Callable, Optional, Sequence

import numpy as np

from . import TRACE_HYBRID, Context, _check, _design_array, _items
from . import _native as N
from .sharding import shard_by_work

Evaluator = Callable[[np.ndarray, np.ndarray], np.ndarray]


def batch_evaluator(designs: np.ndarray, mode: int, context: Context) -> Evaluator:
    """evaluate(indices, items): the designs at `indices` in one cpd_fitness_gpu_batch call
    on `context`'s device; an N.FITNESS_DTYPE record per design."""
    def evaluate(indices: np.ndarray, items: np.ndarray) -> np.ndarray:
        n = int(indices.size)
        outs = np.zeros(n, dtype=N.FITNESS_DTYPE)
        if n == 0:
            return outs
        d = np.ascontiguousarray(designs[indices])
        it = np.ascontiguousarray(items)
        _check(N.lib.cpd_fitness_gpu_batch(context.handle, d.ctypes.data_as(C.POINTER(N.Design)),
                                           it.ctypes.data_as(C.POINTER(N.BatchItem)), n, int(mode),
                                           outs.ctypes.data_as(C.POINTER(N.Fitness))), "fitness_batch")
        return outs
    return evaluate


def partition(items: np.ndarray, world: int) -> list[np.ndarray]:
    """Design indices per participant, balanced on ray counts (max_n x max_eval)."""
    work = items["max_n"].astype(np.float64) * items["max_eval"].astype(np.float64)
    return [np.asarray(p, dtype=np.int64) for p in shard_by_work(list(work), world)]


def fitness_population(designs, *, seeds=0.5, max_n=256, max_eval=16_384, mode: int = TRACE_HYBRID,
                       devices: Optional[Sequence[int]] = None,
                       evaluators: Optional[Sequence[Evaluator]] = None) -> np.ndarray:
    """Fitness of a population on several GPUs of this process (one thread and one batched
    call per device). designs: Spectrometers or an N.DESIGN_DTYPE array; seeds, max_n and
    max_eval scalars or per-design sequences. Returns N.FITNESS_DTYPE records in order."""
    d = _design_array(designs)
    n = d.size
    items = _items(n, seeds, max_n, max_eval)
    if evaluators is None:
        devs = list(devices) if devices else [0]
        evaluators = [batch_evaluator(d, mode, Context(dev)) for dev in devs]
    parts = partition(items, len(evaluators))
    outs = np.zeros(n, dtype=N.FITNESS_DTYPE)
    errors: list[BaseException] = []

    def run(k: int):
        try:
            idx = parts[k]
            outs[idx] = evaluators[k](idx, items[idx])
        except BaseException as e:  # noqa: BLE001
            errors.append(e)

    threads = [threading.Thread(target=run, args=(k,)) for k in range(len(evaluators))]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    if errors:
        raise errors[0]
    return outs


class DistributedPopulation:
    """One rank per GPU: each rank evaluates its shard of a population on its own device and
    every rank receives the whole population's results (one all-gather of result records,
    host side). `group`: a torch.distributed process group (default: the world)."""

    def __init__(self, *, group=None, device: Optional[int] = None, evaluate_factory=None):
        import torch.distributed as dist

        self._dist = dist
        self._group = group
        self.rank = dist.get_rank(group)
        self.world = dist.get_world_size(group)
        self._device = device
        self._factory = evaluate_factory
        self._ctx: Optional[Context] = None

    def _evaluator(self, d: np.ndarray, mode: int) -> Evaluator:
        if self._factory is not None:
            return self._factory(d, mode)
        if self._ctx is None:
            self._ctx = Context(self.rank if self._device is None else self._device)
        return batch_evaluator(d, mode, self._ctx)

    def evaluate(self, designs, *, seeds=0.5, max_n=256, max_eval=16_384, mode: int = TRACE_HYBRID) -> np.ndarray:
        d = _design_array(designs)
        n = d.size
        items = _items(n, seeds, max_n, max_eval)
        mine = partition(items, self.world)[self.rank]
        recs = self._evaluator(d, mode)(mine, items[mine])
        gathered: list = [None] * self.world
        self._dist.all_gather_object(gathered, (mine.tolist(), recs.tobytes()), group=self._group)
        outs = np.zeros(n, dtype=N.FITNESS_DTYPE)
        for idx, blob in gathered:
            outs[np.asarray(idx, dtype=np.int64)] = np.frombuffer(blob, dtype=N.FITNESS_DTYPE)
        return outs
