"""Benchmark of the compound-prism fitness path on GB300.

Default workload (N=1): the plain one-design GPU call -- 6 prisms, 64 detector
bins, 4096 QMC wavelengths x 1024 rays (4,194,304 rays per design), FP32 trace
with FP64/int64 accumulation and entropy. A step is one gpu_fitness call of one
design. Also measured on the same run, under "forms": the batched population form
(1024 designs of mixed G, B, W in one captured launch sequence), the serving form
(a continuous-batching server fed by a synthetic generational optimizer: designs/s,
p50/p99 request latency) and adaptive sampling (the reference kernel's per-wavelength
SEM stop) beside fixed N at the reference optimizer's sampling; each form's results
are checked against the oracle on sampled designs (mi_check).

  value   designs/s with inputs resident on the device: 1 / (device time of the pass)
  e2e     designs/s through the C ABI with host buffers (design + point tables H2D,
          result D2H, inside the timed call)
  roofline  FP32 roofline of the dominant kernel (the trace kernel): the algorithmic
          FLOP of the reference's per-ray formulation (the frozen table
          roofline/ops_per_ray.json, counted by the op-counting build of the oracle) x
          the design's rays / kernel time, against a live FP32 FMA throughput probe;
          beside it the executed fast-path count and the SFU bound (live probe)
  cpu_baseline  the C oracle (the reference CPU algorithm restated) on all host cores,
          whole designs, fixed N on the GPU call's own points and the reference's
          adaptive estimator

  --impl reference  times the reference's CPU path (the oracle port: the reference
          itself is Rust and cannot be built here) on the same design and points, built
          and positioned by the oracle alone (the library is not imported).

Multi-GPU: designs are independent; each rank evaluates its own designs on its own
GPU with no collective (weak scaling); rank 0 prints the aggregate.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "compound-prism-designer_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

METRIC = "MI fitness designs/sec, batched-serving vs plain at <=1e-4 rel MI err; p50/p99 ms"
G_PLAIN, B_PLAIN, W_PLAIN, R_PLAIN = 6, 64, 4096, 1024
PLAIN_SEED = 20261203 + 1
# The frozen per-ray operation table of the reference's formulation, keyed by prism count.
OPS_TABLE = os.path.join(ROOT, "roofline", "ops_per_ray.json")
# FP32 arithmetic of fast_ray on its full path for an anti-reflection-coated design (exit
# face, refraction, detector, binning and the guard-band thresholds): adds/muls count 1,
# FMAs 2, comparisons 0; the 5 hardware estimates (2 sqrt, 3 reciprocals) and the floor
# are not counted. Rays lost early execute fewer, so this is an upper bound per evaluated
# ray. (102 before the exit-face terms became polynomials in dz and the exit direction was
# taken along the detector from dp.)
FLOP_PER_FAST_RAY = 82
# Special-function-unit results of fast_ray's full path: 2 square-root and 3 reciprocal
# estimates.
SFU_PER_FAST_RAY = 5
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one trace_spans_kernel
# launch of this workload, from the ncu capture summarised in
# profiles/fitness_pass_plain_g6_b64_w4096_r1024.md (the figure is copied here when the
# kernel is re-profiled; bench.py reads no profile file).
TRACE_TRAFFIC_BYTES = 3045888


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rk = int(os.environ.get("RANK", "0"))
    lrk = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rk, lrk


class Dist:
    """Host-side barrier and max-reduction over ranks (gloo; no data-path collective)."""

    def __init__(self):
        self.ws, self.rank, self.local = dist_info()
        self.pg = None
        if self.ws > 1:
            import torch.distributed as dist

            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo", rank=self.rank, world_size=self.ws)
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, v: float) -> float:
        if not self.pg:
            return v
        import torch

        t = torch.tensor([v], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def sum(self, v: float) -> float:
        if not self.pg:
            return v
        import torch

        t = torch.tensor([v], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.SUM)
        return float(t.item())


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() in ("active", "1"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "samples": len(sm), "reasons": sorted(reasons)}


def l2_flusher():
    """Writes 512 MiB (> the 129 MB L2) between timed steps."""
    try:
        import torch

        buf = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device="cuda")

        def flush():
            buf.fill_(1)
            torch.cuda.synchronize()

        return flush, "flushed between steps (512 MiB device write)"
    except Exception as e:  # noqa: BLE001
        return (lambda: None), f"not flushed ({type(e).__name__})"


def plain_design():
    import numpy as np
    from compound_prism_designer import synth

    spec, d, rej = synth.random_design(np.random.default_rng(PLAIN_SEED), G_PLAIN, B_PLAIN)
    return spec, d


def batched_population(n=1024, seed=20261205, with_params=False):
    import numpy as np
    from compound_prism_designer import synth

    pop, rej = synth.population(seed, n)
    rng = np.random.default_rng(seed + 1)
    W = rng.integers(512, 4097, n)
    if with_params:
        return [s for s, _ in pop], [d for _, d in pop], W, rej
    return [s for s, _ in pop], W, rej


def record_to_dict(rec) -> dict:
    """A cpd_spectrometer_params record (numpy) as the flat parameter dict of the oracle."""
    G = int(rec["nglass"])
    f = float
    return dict(glasses=[[f(c) for c in rec["glass"][g]] for g in range(G)],
                angles=[f(a) for a in rec["angles"][:G + 1]], lengths=[f(v) for v in rec["lengths"][:G]],
                curvature=f(rec["curvature"]), height=f(rec["height"]), width=f(rec["width"]),
                ar_coated=bool(rec["ar_coated"]), bin_count=int(rec["bin_count"]), bin_size=f(rec["bin_size"]),
                linear_slope=f(rec["linear_slope"]), linear_intercept=f(rec["linear_intercept"]),
                det_length=f(rec["det_length"]), max_incident_angle=f(rec["max_incident_angle"]),
                det_angle=f(rec["det_angle"]), det_position=(f(rec["det_position"][0]), f(rec["det_position"][1])),
                det_flipped=bool(rec["det_flipped"]),
                wavelength_bounds=(f(rec["wavelength_bounds"][0]), f(rec["wavelength_bounds"][1])),
                beam_width=f(rec["beam_width"]), beam_y_mean=f(rec["beam_y_mean"]))


def oracle_check(cases, adaptive=False, nthreads=None):
    """The oracle on the GPU results of sampled designs, on their own points (GPU seed
    policy): cases = [(params dict, seed, W, R, gpu info, gpu hits, gpu rays)]. Returns the
    largest relative MI error, and whether hits (and, adaptive, rays consumed) are equal."""
    import oracle as O

    nthreads = nthreads or os.cpu_count() or 1
    worst, equal, rows = 0.0, True, []
    for d, seed, W, R, info, hits, rays in cases:
        lam, ray_u = O.gpu_points(seed, W), O.gpu_points(seed, R, first=1)
        if adaptive:
            _, st, counts = O.fitness_adaptive_points(d, lam, ray_u, nthreads=nthreads)
            same = hits == st["hits"] and rays == int(counts.sum())
        else:
            _, st = O.fitness_points(d, lam, ray_u, nthreads=nthreads, want_p=False)
            same = hits == st["hits"]
        # a design whose rays all miss the detector has MI 0 on both sides
        rel = abs(info - st["info"]) / abs(st["info"]) if st["info"] != 0.0 else (0.0 if info == 0.0 else 1.0)
        worst = max(worst, rel)
        equal = equal and same
        rows.append({"W": W, "R": R, "G": len(d["glasses"]), "B": d["bin_count"], "rel_err": rel})
    return {"designs": len(cases), "max_rel_err": worst, "tolerance": 1e-4,
            "hits_equal" if not adaptive else "hits_and_rays_equal": equal, "per_design": rows}


def cpu_oracle_rate(d, W, R, target_s=10.0, nthreads=None, gpu_info=None):
    """Oracle (reference CPU algorithm) on all host threads, whole designs for at least
    target_s, on the points of the plain GPU call (seed 0.5, the GPU policy): fixed N, the
    GPU's own estimator. The oracle's MI on those points is the check of the GPU's
    (gpu_info). Beside it the reference's adaptive estimator (reference_adaptive)."""
    import oracle as O

    nthreads = nthreads or os.cpu_count() or 1
    lam_all = O.gpu_points(0.5, W)
    ray_u = O.gpu_points(0.5, R, first=1)
    done, t0 = 0, time.perf_counter()
    while done == 0 or time.perf_counter() - t0 < target_s:
        _, st = O.fitness_points(d, lam_all, ray_u, nthreads=nthreads, want_p=False)
        done += 1
    dt = time.perf_counter() - t0
    out = {"value": done / dt, "unit": "designs/s", "cores": nthreads, "kind": "port",
           "sample": f"{done} whole designs of the benchmark workload ({W} wavelengths x {R} rays each, "
                     f"{done * W * R} rays, {dt:.1f} s, {nthreads} threads, fixed N on the GPU call's points)",
           "reference_adaptive": reference_adaptive_rate(d, W, R, nthreads),
           "config0": config0_rates(nthreads)}
    if gpu_info is not None:
        out["mi_check"] = {"gpu_mi": gpu_info, "oracle_mi": st["info"],
                           "rel_err": abs(gpu_info - st["info"]) / abs(st["info"]), "tolerance": 1e-4}
    return out


def config0_rates(nthreads, target_s=2.0):
    """The reference's CPU-runnable case (3 prisms, 32 bins, 64 wavelengths x 256 rays, the
    reference CPU point set from 0.5): the oracle's fixed-N rate, one design per thread, and
    the reference's adaptive fitness with max_n = 64, max_m = 256."""
    from concurrent.futures import ThreadPoolExecutor

    import numpy as np
    import oracle as O
    from compound_prism_designer import synth

    _, d, _ = synth.random_design(np.random.default_rng(20261203), 3, 32)
    lam, ray_u = O.qrng_points(0.5, 64), O.qrng_points(0.5, 256)
    _, st = O.fitness_points(d, lam, ray_u)
    done, t0 = 0, time.perf_counter()
    with ThreadPoolExecutor(nthreads) as ex:
        while done == 0 or time.perf_counter() - t0 < target_s:
            list(ex.map(lambda _: O.fitness_points(d, lam, ray_u, want_p=False), range(nthreads * 8)))
            done += nthreads * 8
    fixed = done / (time.perf_counter() - t0)
    ad = reference_adaptive_rate(d, 64, 256, nthreads, target_s=target_s)
    return {"workload": "3 prisms, 32 bins, 64 wavelengths x 256 rays (reference CPU points from 0.5)",
            "fixed_n_designs_per_s": fixed, "fixed_n_mi": st["info"], "reference_adaptive": ad, "cores": nthreads}


def reference_adaptive_rate(d, max_n, max_m, nthreads, target_s=3.0):
    """The reference CPU fitness as it runs (src/fitness.rs:79-147: SEM stops per
    wavelength and across wavelengths, its own point set), one design per thread as the
    reference is single-threaded per design, whole designs for at least target_s."""
    from concurrent.futures import ThreadPoolExecutor

    import oracle as O

    res = [O.fitness_adaptive(d, max_n, max_m)]
    done, t0 = 0, time.perf_counter()
    with ThreadPoolExecutor(nthreads) as ex:  # ctypes releases the GIL during each call
        while done == 0 or time.perf_counter() - t0 < target_s:
            res = list(ex.map(lambda _: O.fitness_adaptive(d, max_n, max_m), range(nthreads * 4)))
            done += len(res)
    dt = time.perf_counter() - t0
    _, _, _, n_w, n_r = O.fitness_adaptive_work(d, max_n, max_m)
    return {"value": done / dt, "unit": "designs/s", "cores": nthreads, "max_n": max_n, "max_m": max_m,
            "info": res[0][1], "wavelengths_used": n_w, "rays_traced": n_r,
            "sample": f"{done} whole designs, one per thread, {dt:.2f} s",
            "note": "a different estimator: stops each wavelength at the first hit whose bin's SEM <= 5e-3 "
                    "and stops the wavelengths once every bin's SEM across them is <= 5e-3"}


def adaptive_form(ctx, n=256):
    """Adaptive sampling (the reference kernel's per-wavelength SEM stop) at the reference
    optimizer's sampling, 128 wavelengths x up to 8192 rays: the plain call over n
    generation-0 designs and the same designs as one batched pass, each beside fixed N."""
    import numpy as np
    from compound_prism_designer import _native as N
    from compound_prism_designer import generations as gen

    W, R = 128, 8192
    rng = np.random.default_rng(11)
    cat = gen.glass_catalog(rng, 64)
    pop = gen.initial_population(rng, n, cat)
    designs, ok = gen.build(pop, cat)
    dd = [N.Design.from_buffer_copy(designs[i].tobytes()) for i in range(len(designs))]
    nb = len(dd)
    darr = (N.Design * nb)(*dd)
    items = (N.BatchItem * nb)()
    for i in range(nb):
        items[i].seed, items[i].max_n, items[i].max_eval = 0.5, W, R
    outs = (N.Fitness * nb)()
    seeds = np.array([0.5])
    f = N.Fitness()
    out = {"workload": f"{nb} designs (G in 2..6, B in 16..128), {W} wavelengths x up to {R} rays, seed 0.5"}
    for name, sampling in (("fixed", 0), ("adaptive", N.SAMPLING_ADAPTIVE)):
        for x in dd[:4]:
            N.lib.cpd_fitness_gpu_ex(ctx.handle, x, seeds.ctypes.data_as(N._dp), 1, W, 2, R, sampling, f)
        rays = 0
        t0 = time.perf_counter()
        for x in dd:
            N.lib.cpd_fitness_gpu_ex(ctx.handle, x, seeds.ctypes.data_as(N._dp), 1, W, 2, R, sampling, f)
            rays += f.rays
        out[f"plain_{name}_designs_per_s"] = nb / (time.perf_counter() - t0)
        out[f"plain_{name}_rays_fraction"] = rays / (nb * W * R)
        ms = []
        for _ in range(4):
            N.lib.cpd_fitness_gpu_batch(ctx.handle, darr, items, nb, N.TRACE_HYBRID | sampling, outs)
            ms.append(ctx.last_timing()[0])
        out[f"batch_{name}_ms_device"] = min(ms[1:])
        out[f"batch_{name}_designs_per_s_device"] = nb / (min(ms[1:]) / 1e3)
        if sampling:
            # the oracle on 8 designs of the batch (their rays consumed must be equal too)
            recs = gen.to_params(pop, cat)[ok]
            idx = np.linspace(0, nb - 1, 8).astype(int)
            import oracle as O

            cases = []
            for i in idx:
                dct = O.accept_params(record_to_dict(recs[i]))
                cases.append((dct, 0.5, W, R, outs[i].info, outs[i].hits, outs[i].rays))
            out["mi_check"] = oracle_check(cases, adaptive=True)
    return out


def serving_form(ctx, generations=200):
    """The serving loop fed by the synthetic generational optimizer: 200 generations,
    batch sizes 64..2048, 128 wavelengths x 8192 rays per design (the reference
    optimizer's gpu_fitness sampling), once with batches submitted back to back
    (capacity) and once as a Poisson process at 70% of that capacity (latency). Beside
    it, the plain one-design call on the same sampling."""
    import ctypes as C

    import numpy as np
    import compound_prism_designer as cpd
    from compound_prism_designer import _native as N
    from compound_prism_designer import generations as gen

    W, R = 128, 8192
    out = {"workload": f"{generations} generations, batch sizes uniform 64..2048, G in 2..6, B in 16..128, "
                       f"{W} wavelengths x {R} rays per design, one seed per generation"}
    # plain call, same sampling, one design per call (ray table cached: same seed)
    rng = np.random.default_rng(11)
    cat = gen.glass_catalog(rng, 64)
    pop = gen.initial_population(rng, 256, cat)
    designs, ok = gen.build(pop, cat)
    dd = [N.Design.from_buffer_copy(designs[i].tobytes()) for i in range(len(designs))]
    seeds = np.array([0.5])
    f = N.Fitness()
    for i in range(8):
        N.lib.cpd_fitness_gpu(ctx.handle, dd[i], seeds.ctypes.data_as(N._dp), 1, W, 2, R, f)
    t0 = time.perf_counter()
    for x in dd:
        N.lib.cpd_fitness_gpu(ctx.handle, x, seeds.ctypes.data_as(N._dp), 1, W, 2, R, f)
    plain = len(dd) / (time.perf_counter() - t0)
    out["plain_designs_per_s"] = plain
    # the server's passes hold up to 256 designs of this sampling: tune the launch shape on
    # such a pass (the server uses the context's shape) and time it alone
    n_b = min(256, len(dd))
    darr = (N.Design * n_b)(*dd[:n_b])
    items = (N.BatchItem * n_b)()
    for i in range(n_b):
        items[i].seed, items[i].max_n, items[i].max_eval = 0.5, W, R
    rt_, w_, ms_ = C.c_uint32(0), C.c_uint32(0), C.c_double(0.0)
    N.lib.cpd_autotune_batch(ctx.handle, darr, items, n_b, 0, C.byref(rt_), C.byref(w_), C.byref(ms_))
    out["pass_shape"] = {"ray_tile": rt_.value, "warps_per_cta": w_.value}
    out["gpu_pass_designs_per_s"] = n_b / (ms_.value * 1e-3)
    with cpd.Server(mem_budget_bytes=8 << 30, slots=2, max_designs_per_pass=256, context=ctx) as sv:
        gen.serve(sv, generations=5, seed=1)  # warm-up: buffers, caches
        # the server alone: 64 requests of 1024 pre-built designs submitted at once
        pre = gen.perturb(rng, pop, 1024, len(cat))
        pd, pok = gen.build(pre, cat)
        pd = pd[pok]
        t0 = time.perf_counter()
        rids = [sv.submit(pd, seeds=0.25 + 0.001 * i, max_n=W, max_eval=R) for i in range(64)]
        for r_ in rids:
            sv.wait(r_)
        cap_pre = 64 * len(pd) / (time.perf_counter() - t0)
        sat = gen.serve(sv, generations=generations, seed=2)
        cap = sat["designs_per_s"]
        mean_gap = sat["mean_batch"] / (0.7 * cap)
        poi = gen.serve(sv, generations=generations, seed=3, mean_interarrival_s=mean_gap)
        # the same back-to-back load with the designs built on the device (parameter
        # records submitted; no host build step)
        dev = gen.serve(sv, generations=generations, seed=2, device_build=True)
        st = sv.stats()
        # the oracle on a request of 8 designs served by the same server
        import oracle as O

        recs = gen.to_params(pre, cat)[pok]
        idx = np.linspace(0, len(pd) - 1, 8).astype(int)
        rid = sv.submit(pd[idx], seeds=0.375, max_n=W, max_eval=R)
        souts, _ = sv.wait(rid)
        cases = [(O.accept_params(record_to_dict(recs[i])), 0.375, W, R, float(souts["info"][k]),
                  int(souts["hits"][k]), W * R) for k, i in enumerate(idx)]
        out["mi_check"] = oracle_check(cases)
    # the device-resident loop: the same loads through one persistent kernel that takes the
    # designs from a ring in mapped memory (cpd_loop_*)
    with cpd.LoopServer(8 << 30, max_cells=1 << 16, max_rows=1024, ray_tile=256, context=ctx) as lp:
        gen.serve(lp, generations=5, seed=1)  # warm-up
        t0 = time.perf_counter()
        rids = [lp.submit(pd, seeds=0.25 + 0.001 * i, max_n=W, max_eval=R) for i in range(64)]
        for r_ in rids:
            lp.wait(r_)
        loop_pre = 64 * len(pd) / (time.perf_counter() - t0)
        lsat = gen.serve(lp, generations=generations, seed=2)
        lgap = lsat["mean_batch"] / (0.7 * lsat["designs_per_s"])
        lpoi = gen.serve(lp, generations=generations, seed=3, mean_interarrival_s=lgap)
        rid = lp.submit(pd[idx], seeds=0.375, max_n=W, max_eval=R)
        louts, _ = lp.wait(rid)
        lcases = [(O.accept_params(record_to_dict(recs[i])), 0.375, W, R, float(louts["info"][k]),
                   int(louts["hits"][k]), W * R) for k, i in enumerate(idx)]
        lstats = lp.stats()
    for r in (lsat, lpoi):
        r.pop("latency_ms")
    out["loop"] = {"back_to_back": lsat, "poisson_70pct": dict(lpoi, mean_interarrival_ms=1e3 * lgap),
                   "designs_per_s": lsat["designs_per_s"], "loop_only_designs_per_s": loop_pre,
                   "p50_ms": lpoi["p50_ms"], "p99_ms": lpoi["p99_ms"],
                   "speedup_vs_plain": lsat["designs_per_s"] / plain, "stats": lstats,
                   "mi_check": oracle_check(lcases)}
    for r in (sat, poi, dev):
        r.pop("latency_ms")
    out["back_to_back"] = sat
    out["back_to_back_device_build"] = dev
    out["poisson_70pct"] = dict(poi, mean_interarrival_ms=1e3 * mean_gap)
    out["designs_per_s"] = cap
    out["server_only_designs_per_s"] = cap_pre
    out["p50_ms"], out["p99_ms"] = poi["p50_ms"], poi["p99_ms"]
    out["speedup_vs_plain"] = cap / plain
    out["server_stats"] = st
    return out


def run_batch_only(args):
    """--batch-only N: the batched form on N designs (W 512..4096, R 1024), one pass per
    step, for profiler captures; prints one JSON line of device times."""
    import compound_prism_designer as cpd

    pop, Ws, _ = batched_population()
    pop, Ws = pop[:args.batch_only], Ws[:args.batch_only]
    ctx = cpd.Context(0)
    rt, wp = (int(v) for v in (args.shape or "64,8").split(","))
    ctx.set_launch_shape(rt, wp)
    for _ in range(args.warmup):
        cpd.fitness_batch(pop, seeds=0.5, max_n=Ws, max_eval=R_PLAIN, context=ctx)
    ms = []
    for _ in range(args.steps):
        cpd.fitness_batch(pop, seeds=0.5, max_n=Ws, max_eval=R_PLAIN, context=ctx)
        ms.append(ctx.last_timing()[0])
    print(json.dumps({"form": "batched", "designs": len(pop), "rays": int(sum(int(w) for w in Ws) * R_PLAIN),
                      "ms": ms, "shape": [rt, wp]}), flush=True)


def run_adaptive_only(args):
    """--adaptive-only N: the adaptive form's batched pass (adaptive sampling, 128
    wavelengths x up to 8192 rays) on N generation-0 designs, for profiler captures;
    prints one JSON line of device times."""
    import numpy as np
    import compound_prism_designer as cpd
    from compound_prism_designer import generations as gen

    rng = np.random.default_rng(11)
    cat = gen.glass_catalog(rng, 64)
    pop = gen.initial_population(rng, args.adaptive_only, cat)
    designs, ok = gen.build(pop, cat)
    specs = []
    for i in range(len(designs)):
        sp = cpd.Spectrometer.__new__(cpd.Spectrometer)
        sp._design = cpd._native.Design.from_buffer_copy(designs[i].tobytes())
        specs.append(sp)
    ctx = cpd.Context(0)
    mode = cpd.TRACE_HYBRID | cpd.SAMPLING_ADAPTIVE
    for _ in range(args.warmup):
        cpd.fitness_batch(specs, seeds=0.5, max_n=128, max_eval=8192, mode=mode, context=ctx)
    ms, rays = [], 0
    for _ in range(args.steps):
        outs = cpd.fitness_batch(specs, seeds=0.5, max_n=128, max_eval=8192, mode=mode, context=ctx)
        ms.append(ctx.last_timing()[0])
        rays = sum(o.rays for o in outs)
    print(json.dumps({"form": "adaptive batch", "designs": len(specs), "rays": int(rays), "ms": ms}), flush=True)


def _workload_module():
    """compound_prism_designer/workload.py loaded by file path: the numpy-only parameter
    draws, without importing the library's package (which would load libcpd.so)."""
    import importlib.util

    path = os.path.join(ROOT, "compound-prism-designer_gb300", "compound_prism_designer", "workload.py")
    spec = importlib.util.spec_from_file_location("cpd_workload", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def run_reference(args, dist):
    """--impl reference: the reference's CPU fitness path (the oracle port, f64, all host
    threads) on the plain workload's own design and points. The design is drawn by the same
    seeded numpy generator as the GPU arm's and built and positioned by the oracle alone;
    the library's package is never imported. A step is one whole design, fixed N on the GPU
    call's points (the same work as a GPU step); the reference's adaptive estimator (its
    cpu_fitness, with its early stops) is timed beside it."""
    if dist.rank != 0:
        return
    import numpy as np
    import oracle as O

    wl = _workload_module()
    d, rej = wl.random_params(np.random.default_rng(PLAIN_SEED), G_PLAIN, B_PLAIN, O.accept_params)
    nthreads = os.cpu_count() or 1
    lam = O.gpu_points(0.5, W_PLAIN)
    ray_u = O.gpu_points(0.5, R_PLAIN, first=1)
    for _ in range(args.warmup):
        O.fitness_points(d, lam, ray_u, nthreads=nthreads, want_p=False)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        _, st = O.fitness_points(d, lam, ray_u, nthreads=nthreads, want_p=False)
    dt = time.perf_counter() - t0
    rate = args.steps / dt
    adaptive = reference_adaptive_rate(d, W_PLAIN, R_PLAIN, nthreads)
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": "designs/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": plain_config("none (CPU)"), "same_config": True,
        "cpu_baseline": {"value": rate, "unit": "designs/s", "cores": nthreads, "kind": "port",
                         "sample": f"each step one whole design: {W_PLAIN} wavelengths x {R_PLAIN} rays, fixed N "
                                   f"on the GPU call's points; {args.steps} steps, {dt:.1f} s"},
        "e2e": {"value": rate, "unit": "designs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "mi": st["info"], "hits": st["hits"], "design_rejections": rej,
        "reference_adaptive": adaptive,
        "library_imported": "compound_prism_designer" in sys.modules,
        "note": "reference is Rust (nightly, un-vendored git deps): not buildable here; the oracle restates "
                "its CPU fitness path (src/fitness.rs, src/spectrometer/*.rs) in C, f64, on all host threads",
    }
    print(json.dumps(line), flush=True)


def plain_config(l2):
    return {"workload": f"plain gpu_fitness call, one design per call: {G_PLAIN} prisms, {B_PLAIN} bins, "
                        f"{W_PLAIN} wavelengths x {R_PLAIN} rays ({W_PLAIN * R_PLAIN} rays)",
            "prisms": G_PLAIN, "bins": B_PLAIN, "wavelengths": W_PLAIN, "rays_per_wavelength": R_PLAIN,
            "trace": "fp32 fast path; guard-band rays re-traced in float-float",
            "accumulation": "int64 fixed point; float-float entropy",
            "l2": l2}


def load_ops_table() -> dict:
    with open(OPS_TABLE) as fh:
        return json.load(fh)["by_glasses"]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-extras", action="store_true", help="main line only (for profiler runs)")
    ap.add_argument("--shape", default=None,
                    help="fixed launch shape RAY_TILE,WARPS instead of the autotuner (for profiler runs)")
    ap.add_argument("--batch-only", type=int, default=0, metavar="N",
                    help="profiler run: only the batched form, on the first N designs of its population")
    ap.add_argument("--adaptive-only", type=int, default=0, metavar="N",
                    help="profiler run: only the adaptive form's batched pass, on N designs")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    dist = Dist()
    if args.impl == "reference":
        run_reference(args, dist)
        return

    import numpy as np
    import compound_prism_designer as cpd

    if args.batch_only:
        run_batch_only(args)
        return
    if args.adaptive_only:
        run_adaptive_only(args)
        return
    ctx = cpd.Context(dist.local)
    if args.shape:
        rt, wp = (int(v) for v in args.shape.split(","))
        ctx.set_launch_shape(rt, wp)
    else:
        ctx.set_autotune(True)  # the first warm-up call tunes the launch shape of this class
    spec, d = plain_design()
    flush, l2_note = l2_flusher()
    seeds = [0.5]
    nwarp = ctx.launch_shape()[1] if args.shape else 8

    def step():
        t0 = time.perf_counter()
        f = spec.gpu_fitness_full(seeds, max_n=W_PLAIN, nwarp=nwarp, max_eval=R_PLAIN, context=ctx)
        wall = time.perf_counter() - t0
        ms, launches = ctx.last_timing()
        h2d, d2h = ctx.last_transfer_bytes()
        return f, wall, ms, launches, h2d, d2h

    for _ in range(args.warmup):
        step()
        flush()
    plain_shape = ctx.launch_shape()
    clocks = ClockSampler(dist.local)
    dist.barrier()
    clocks.start()
    dev_ms, walls, launches_total = [], [], 0
    t_start = time.perf_counter()
    for _ in range(args.steps):
        f, wall, ms, launches, h2d, d2h = step()
        dev_ms.append(ms)
        walls.append(wall)
        launches_total += launches
        flush()
    t_total = time.perf_counter() - t_start
    clk = clocks.stop()
    dist.barrier()
    dev_s = dist.max(sum(dev_ms) / 1e3)
    wall_s = dist.max(sum(walls))
    designs = dist.sum(float(args.steps))
    value = designs / dev_s
    e2e = designs / wall_s

    extras = {}
    peak = None
    if not args.no_extras and dist.rank == 0:
        try:
            # per-kernel CUDA events on the pass's stream (they stand between the kernels,
            # so these passes run without the programmatic overlap): the median of 10 passes,
            # L2 flushed before each like the timed steps
            ctx.set_profiling(True)
            kts = []
            for _ in range(10):
                flush()
                fp = spec.gpu_fitness_full(seeds, max_n=W_PLAIN, nwarp=nwarp, max_eval=R_PLAIN, context=ctx)
                kts.append(ctx.last_kernel_times())
            kt = {k: statistics.median(x[k] for x in kts) for k in kts[0]}
            ctx.set_profiling(False)
            peak = max(ctx.fp32_peak_tflops(2048) for _ in range(3))
            sfu_peak = max(ctx.sfu_peak_gops(2048) for _ in range(3))
            ops = load_ops_table()[str(G_PLAIN)]["per_ray"]
            rays = W_PLAIN * R_PLAIN
            t_trace = kt["trace"] * 1e-3
            t_pass = statistics.median(dev_ms) * 1e-3
            alg = rays * ops["flop"] / t_trace / 1e12
            alg_pass = rays * ops["flop"] / t_pass / 1e12
            executed = fp.fast_rays * FLOP_PER_FAST_RAY / t_trace / 1e12
            sfu_alg = rays * (ops["div"] + ops["sqrt"] + ops["log"]) / t_trace / 1e9
            sfu_exec = fp.fast_rays * SFU_PER_FAST_RAY / t_trace / 1e9
            extras["roofline"] = {
                "bound": "fp32", "achieved": alg, "peak": peak, "unit": "TFLOP/s", "frac": alg / peak,
                "traffic": TRACE_TRAFFIC_BYTES,
                "traffic_source": "ncu capture of trace_spans_kernel on this workload (dram__bytes_read.sum + "
                                  "dram__bytes_write.sum), profiles/fitness_pass_plain_g6_b64_w4096_r1024.md",
                "kernel": "trace_spans_kernel", "kernel_ms": kt,
                "frac_algorithmic": alg / peak,
                "frac_algorithmic_pass": alg_pass / peak,
                "frac_executed": executed / peak,
                "flop_per_ray_algorithmic": ops["flop"],
                "flop_basis": "the design's W x R rays x the frozen per-ray FLOP of the reference's formulation "
                              f"(roofline/ops_per_ray.json, G={G_PLAIN}), over the trace kernel's time "
                              "(frac_algorithmic) and over the whole pass (frac_algorithmic_pass); frac_executed: "
                              f"{FLOP_PER_FAST_RAY} FP32 FLOP per ray the fast path evaluated",
                "sfu": {"peak_gops": sfu_peak, "algorithmic_gops": sfu_alg, "frac_algorithmic": sfu_alg / sfu_peak,
                        "executed_gops": sfu_exec, "frac_executed": sfu_exec / sfu_peak,
                        "per_ray_algorithmic": ops["div"] + ops["sqrt"] + ops["log"],
                        "per_fast_ray_executed": SFU_PER_FAST_RAY,
                        "peak_source": "measured live: reciprocal-square-root chains on all SMs "
                                       "(cpd_measure_sfu_peak)"},
                "fast_rays": fp.fast_rays, "flop_per_fast_ray": FLOP_PER_FAST_RAY,
                "peak_source": "measured live: FP32 FMA probe on all SMs (cpd_measure_fp32_peak)",
                "retraced": fp.retraced, "hits": fp.hits}
        except Exception as e:  # noqa: BLE001
            extras["roofline"] = {"error": repr(e)}
        try:
            pop, pdicts, Ws, rej = batched_population(with_params=True)
            t_tune = time.perf_counter()
            tuned = cpd.autotune_batch(pop, seeds=0.5, max_n=Ws, max_eval=R_PLAIN, context=ctx)
            t_tune = time.perf_counter() - t_tune
            for _ in range(2):
                cpd.fitness_batch(pop, seeds=0.5, max_n=Ws, max_eval=R_PLAIN, context=ctx)
            bt = []
            bdev = []
            for _ in range(3):
                flush()
                t0 = time.perf_counter()
                outs = cpd.fitness_batch(pop, seeds=0.5, max_n=Ws, max_eval=R_PLAIN, context=ctx)
                bt.append(time.perf_counter() - t0)
                bdev.append(ctx.last_timing()[0])
            nb = len(pop)
            ctx.set_profiling(True)
            cpd.fitness_batch(pop, seeds=0.5, max_n=Ws, max_eval=R_PLAIN, context=ctx)
            bk = ctx.last_kernel_times()
            ctx.set_profiling(False)
            if peak is None:
                peak = max(ctx.fp32_peak_tflops(2048) for _ in range(3))
            table = load_ops_table()
            bflop = sum(int(w) * R_PLAIN * table[str(len(dd["glasses"]))]["per_ray"]["flop"]
                        for dd, w in zip(pdicts, Ws))
            idx = np.linspace(0, nb - 1, 8).astype(int)
            bcheck = oracle_check([(pdicts[i], 0.5, int(Ws[i]), R_PLAIN, outs[i].info, outs[i].hits, 0) for i in idx])
            extras["forms"] = {"batched": {
                "mi_check": bcheck,
                "roofline": {"achieved": bflop / (bk["trace"] * 1e-3) / 1e12, "unit": "TFLOP/s",
                             "frac_algorithmic": bflop / (bk["trace"] * 1e-3) / 1e12 / peak,
                             "frac_algorithmic_pass": bflop / (min(bdev) * 1e-3) / 1e12 / peak,
                             "basis": "sum over designs of W x R x the frozen per-ray FLOP of its prism count"},
                "kernel_ms": bk,
                "workload": f"{nb} designs, G in 2..6, B in 16..128, W in 512..4096, R={R_PLAIN}",
                "designs_per_s_device": nb / (min(bdev) / 1e3), "designs_per_s_e2e": nb / min(bt),
                "ms_device": min(bdev), "ms_e2e": 1e3 * min(bt), "rays": int(sum(int(w) for w in Ws) * R_PLAIN),
                "rays_per_s_device": sum(int(w) for w in Ws) * R_PLAIN / (min(bdev) / 1e3),
                "speedup_vs_plain_e2e": (nb / min(bt)) / e2e,
                "autotuned_shape": {"ray_tile": tuned[0], "warps_per_cta": tuned[1], "best_ms": tuned[2],
                                    "tuning_s": t_tune}}}
        except Exception as e:  # noqa: BLE001
            extras["forms"] = {"error": repr(e)}
        try:
            extras.setdefault("forms", {})["serving"] = serving_form(ctx)
        except Exception as e:  # noqa: BLE001
            extras.setdefault("forms", {})["serving"] = {"error": repr(e)}
        try:
            extras.setdefault("forms", {})["adaptive"] = adaptive_form(ctx)
        except Exception as e:  # noqa: BLE001
            extras.setdefault("forms", {})["adaptive"] = {"error": repr(e)}
        try:
            extras["cpu_baseline"] = cpu_oracle_rate(d, W_PLAIN, R_PLAIN, gpu_info=f.info)
        except Exception as e:  # noqa: BLE001
            extras["cpu_baseline"] = {"error": repr(e)}

    if dist.rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "designs/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * dev_s / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": dict(plain_config(l2_note), launch_shape={"ray_tile": plain_shape[0],
                                                                "warps_per_cta": plain_shape[1],
                                                                "picked_by": "--shape" if args.shape else
                                                                "autotuner (first warm-up call)"}),
            "e2e": {"value": e2e, "unit": "designs/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "ms_per_step": 1e3 * wall_s / args.steps},
            "gpu_launches": launches_total, "clocks": clk, "wall_s": t_total,
            "mi": f.info, "retraced_per_step": f.retraced,
            "rays_per_s": value * W_PLAIN * R_PLAIN, "rays_per_s_e2e": e2e * W_PLAIN * R_PLAIN,
        }
        line.update(extras)
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
