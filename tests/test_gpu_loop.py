"""The device-resident serving loop (cpd_loop_*): one persistent kernel whose CTAs take
whole designs from a ring in mapped host memory.

* Every design's result is bitwise the one it gets alone (cpd_fitness_gpu_batch with one
  design), whatever else is in flight, from any submitting thread: the loop runs the
  pass's device code per design and every sum is an integer.
* A design whose W x B cells do not fit a slab is refused at submit (CPD_NO_CAPACITY):
  admission is by histogram memory.
* The kernel's one wait, for new work, is bounded: with nothing published the CTAs leave
  after the idle limit (the host reads their exit counts), and the next submission
  relaunches the kernel.
"""
import ctypes as C
import threading
import time

import numpy as np
import pytest

import compound_prism_designer as cpd
from compound_prism_designer import _native as N
from compound_prism_designer import generations as gen

pytestmark = pytest.mark.gpu

FIELDS = ("info", "h_cond", "h_det", "max_sem", "hits", "retraced", "fast_rays", "wavelengths", "status", "rays",
          "size", "deviation")


@pytest.fixture(scope="module")
def designs():
    rng = np.random.default_rng(2025)
    cat = gen.glass_catalog(rng, 16)
    pop = gen.initial_population(rng, 48, cat)
    d, ok = gen.build(pop, cat)
    assert ok.all()
    return d


def _alone(design_rec, seed, max_n, max_eval):
    items = (N.BatchItem * 1)()
    items[0].seed, items[0].max_n, items[0].max_eval = seed, max_n, max_eval
    outs = (N.Fitness * 1)()
    rc = N.lib.cpd_fitness_gpu_batch(cpd.default_context().handle, N.Design.from_buffer_copy(design_rec.tobytes()),
                                     items, 1, cpd.TRACE_HYBRID, outs)
    assert rc == N.OK, N.status_string(rc)
    return outs[0]


def _same(a, rec):
    for f in FIELDS:
        assert getattr(a, f) == rec[f], (f, getattr(a, f), rec[f])


def test_results_in_the_loop_equal_results_alone(designs):
    d = designs
    plan = [(0, 12, 0.25, 64, 1024), (12, 20, 0.5, 128, 2048), (20, 33, 0.75, 32, 4096), (33, 48, 0.125, 96, 512)]
    with cpd.LoopServer(1 << 30, max_cells=1 << 16, max_rows=1024) as lp:
        ids = [lp.submit(d[a:b], seeds=s, max_n=W, max_eval=R) for a, b, s, W, R in plan]
        results = [lp.wait(i, timeout=120) for i in ids]
        st = lp.stats()
    assert st["designs_done"] == 48 and st["device_designs"] == 48 and st["kernel_launches"] >= 1
    for (a, b, s, W, R), (outs, lat) in zip(plan, results):
        assert lat > 0
        for k in range(b - a):
            _same(_alone(d[a + k], s, W, R), outs[k])


def test_threads_submit_concurrently(designs):
    d = designs
    out = {}
    with cpd.LoopServer(1 << 30, max_cells=1 << 16, max_rows=1024) as lp:
        def client(tag, sl, seed):
            out[tag] = lp.wait(lp.submit(d[sl], seeds=seed, max_n=64, max_eval=2048), timeout=120)[0]

        th = [threading.Thread(target=client, args=(i, slice(8 * i, 8 * i + 8), 0.1 + 0.1 * i)) for i in range(6)]
        for t in th:
            t.start()
        for t in th:
            t.join()
    for i in range(6):
        for k in range(8):
            _same(_alone(d[8 * i + k], 0.1 + 0.1 * i, 64, 2048), out[i][k])


def test_loop_matches_the_plain_call(designs):
    d = designs
    ctx = cpd.default_context()
    with cpd.LoopServer(1 << 30) as lp:
        outs, _ = lp.wait(lp.submit(d[:4], seeds=0.625, max_n=128, max_eval=8192), timeout=120)
    for k in range(4):
        f = N.Fitness()
        seeds = np.array([0.625])
        rc = N.lib.cpd_fitness_gpu(ctx.handle, N.Design.from_buffer_copy(d[k].tobytes()), seeds.ctypes.data_as(N._dp),
                                   1, 128, 2, 8192, f)
        assert rc in (N.OK, N.NOT_CONVERGED)
        assert f.info == outs[k]["info"] and f.hits == outs[k]["hits"] and f.status == outs[k]["status"]


def test_admission_by_histogram_slab(designs):
    d = designs
    with cpd.LoopServer(64 << 20, max_cells=1 << 12, max_rows=256) as lp:
        # 128 rows x B bins fits 4096 cells only for B <= 32
        B = d["bin_count"]
        small, big = np.nonzero(B <= 32)[0][:2], np.nonzero(B > 32)[0][:1]
        assert small.size and big.size
        outs, _ = lp.wait(lp.submit(d[small], max_n=128, max_eval=1024), timeout=60)
        assert (outs["wavelengths"] == 128).all()
        items = np.zeros(1, dtype=N.BATCH_ITEM_DTYPE)
        items["seed"], items["max_n"], items["max_eval"] = 0.5, 128, 1024
        rid = C.c_uint64(0)
        big_rec = np.ascontiguousarray(d[big])
        rc = N.lib.cpd_loop_submit(lp._h, big_rec.ctypes.data, items.ctypes.data, 1, cpd.TRACE_HYBRID, C.byref(rid))
        assert rc == N.NO_CAPACITY
        rc = N.lib.cpd_loop_submit(lp._h, big_rec.ctypes.data, items.ctypes.data, 1, cpd.TRACE_FP64, C.byref(rid))
        assert rc == N.INVALID_ARGUMENT
        assert lp.stats()["ctas"] >= 1


def test_idle_wait_runs_out_and_the_loop_relaunches(designs):
    d = designs
    with cpd.LoopServer(1 << 30, max_cells=1 << 16, max_rows=1024, idle_ms=20) as lp:
        a, _ = lp.wait(lp.submit(d[:3], seeds=0.5, max_n=64, max_eval=1024), timeout=60)
        time.sleep(0.5)  # nothing is published: every CTA's wait for work runs out
        st = lp.stats()
        assert st["idle_exits"] == st["ctas"] and st["kernel_launches"] == 1 and st["stop_exits"] == 0
        b, _ = lp.wait(lp.submit(d[:3], seeds=0.5, max_n=64, max_eval=1024), timeout=60)
        st = lp.stats()
        assert st["kernel_launches"] == 2
    for k in range(3):
        assert a[k].tobytes() == b[k].tobytes()


def test_generational_driver_on_the_loop():
    with cpd.LoopServer(2 << 30) as lp:
        r = gen.serve(lp, generations=4, sizes=(64, 128), seed=7)
    assert r["designs"] > 0 and r["p99_ms"] >= r["p50_ms"] > 0
