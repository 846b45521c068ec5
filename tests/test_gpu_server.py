"""The continuous-batching server: every design's result is bitwise the one it gets
alone, whatever else shares its passes, however the memory budget splits the work,
and whichever thread submitted it.

"Alone" is cpd_fitness_gpu_batch with a single design (the same estimator, seed
policy and trace mode). The accumulation is integer fixed point, so equality is
exact; the tests compare the full result records except the wall-clock fields.
"""
import threading

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
    rng = np.random.default_rng(2024)
    cat = gen.glass_catalog(rng, 16)
    pop = gen.initial_population(rng, 48, cat)
    d, ok = gen.build(pop, cat)
    assert ok.all()
    return d, pop


def _alone(design_rec, seed, max_n, max_eval, mode):
    spec_design = N.Design.from_buffer_copy(design_rec.tobytes())
    items = (N.BatchItem * 1)()
    items[0].seed, items[0].max_n, items[0].max_eval = seed, max_n, max_eval
    outs = (N.Fitness * 1)()
    ctx = cpd.default_context()
    rc = N.lib.cpd_fitness_gpu_batch(ctx.handle, spec_design, items, 1, mode, outs)
    assert rc == N.OK, N.status_string(rc)
    return outs[0]


def _same(a, b_rec):
    for f in FIELDS:
        assert getattr(a, f) == b_rec[f], (f, getattr(a, f), b_rec[f])


def test_results_alone_equal_results_in_the_mix(designs):
    d, pop = designs
    rng = np.random.default_rng(5)
    # requests of different sizes, sample counts and seeds, in flight together
    plan = [(0, 12, 0.25, 64, 1024), (12, 20, 0.5, 128, 2048), (20, 33, 0.75, 32, 4096), (33, 48, 0.125, 96, 512)]
    with cpd.Server(mem_budget_bytes=1 << 30, slots=3, max_designs_per_pass=8) as sv:
        ids = [sv.submit(d[a:b], seeds=s, max_n=W, max_eval=R) for a, b, s, W, R in plan]
        results = [sv.wait(i, timeout=120) for i in ids]
        st = sv.stats()
    assert st["designs_done"] == 48 and st["passes"] >= 6
    for (a, b, s, W, R), (outs, lat) in zip(plan, results):
        assert lat > 0
        for k in range(b - a):
            _same(_alone(d[a + k], s, W, R, cpd.TRACE_HYBRID), outs[k])
    del rng


def test_tight_budget_runs_one_design_per_pass_with_identical_results(designs):
    d, _ = designs
    with cpd.Server(mem_budget_bytes=1, slots=2) as sv:
        i1 = sv.submit(d[:6], seeds=0.5, max_n=64, max_eval=1024)
        i2 = sv.submit(d[6:10], seeds=0.5, max_n=64, max_eval=1024)
        o1, _ = sv.wait(i1, timeout=120)
        o2, _ = sv.wait(i2, timeout=120)
        st = sv.stats()
    assert st["passes"] == 10
    for k in range(6):
        _same(_alone(d[k], 0.5, 64, 1024, cpd.TRACE_HYBRID), o1[k])
    for k in range(4):
        _same(_alone(d[6 + k], 0.5, 64, 1024, cpd.TRACE_HYBRID), o2[k])


def test_trace_modes_mix_and_threads_submit_concurrently(designs):
    d, _ = designs
    out = {}

    def client(tag, sl, mode):
        rid = sv.submit(d[sl], seeds=0.3, max_n=64, max_eval=2048, mode=mode)
        out[tag] = sv.wait(rid, timeout=120)[0]

    with cpd.Server(mem_budget_bytes=64 << 20, slots=2, max_designs_per_pass=16) as sv:
        th = [threading.Thread(target=client, args=(t, sl, m))
              for t, sl, m in (("h", slice(0, 16), cpd.TRACE_HYBRID), ("d", slice(16, 24), cpd.TRACE_FP64),
                               ("f", slice(24, 40), cpd.TRACE_FP32))]
        for t in th:
            t.start()
        for t in th:
            t.join()
    for tag, sl, m in (("h", range(0, 16), cpd.TRACE_HYBRID), ("d", range(16, 24), cpd.TRACE_FP64),
                       ("f", range(24, 40), cpd.TRACE_FP32)):
        for k, i in enumerate(sl):
            _same(_alone(d[i], 0.3, 64, 2048, m), out[tag][k])


def test_wait_times_out_then_completes(designs):
    d, _ = designs
    with cpd.Server(mem_budget_bytes=1, slots=1) as sv:
        rid = sv.submit(d[:40], seeds=0.5, max_n=512, max_eval=8192)
        with pytest.raises(TimeoutError):
            sv.wait(rid, timeout=0.0)
        outs, lat = sv.wait(rid, timeout=300)
    assert (outs["status"] == N.OK).sum() + (outs["status"] == N.NOT_CONVERGED).sum() == 40
    _same(_alone(d[7], 0.5, 512, 8192, cpd.TRACE_HYBRID), outs[7])


def test_server_matches_the_plain_call(designs):
    """Through the server, a design evaluated with the reference optimizer's sampling
    (max_n=128, max_eval=8192, one seed) gives the plain gpu_fitness result."""
    d, _ = designs
    ctx = cpd.default_context()
    with cpd.Server(slots=2) as sv:
        outs, _ = sv.wait(sv.submit(d[:4], seeds=0.625, max_n=128, max_eval=8192), timeout=120)
    for k in range(4):
        f = N.Fitness()
        seeds = np.array([0.625])
        rc = N.lib.cpd_fitness_gpu(ctx.handle, N.Design.from_buffer_copy(d[k].tobytes()),
                                   seeds.ctypes.data_as(N._dp), 1, 128, 2, 8192, f)
        assert rc in (N.OK, N.NOT_CONVERGED)
        assert f.info == outs[k]["info"] and f.hits == outs[k]["hits"]
