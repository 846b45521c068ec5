"""Synthetic generational optimizer traffic for the serving form.

The reference's optimizer (designer.py:116-300, an AGE-MOEA population driven by
pymoo) turns a parameter vector into a Spectrometer (create_spectrometer,
designer.py:203-265) and calls gpu_fitness(seeds=rand(1), max_n=128,
max_eval=8192) once per design (designer.py:276). This module produces the same
kind of load without pymoo: a population of parameter vectors with mixed prism
counts (2-6) and bin counts (16-128); each generation's offspring are Gaussian
perturbations (sigma = 5% of each parameter's range, clipped) of parents drawn from
the current population; after a generation is evaluated the population keeps the
best designs by mutual information (a (mu + lambda) survival, the simplest stand-in
for AGE-II's survival). Everything is vectorised over a generation: parameter
records are numpy arrays of the C ABI's cpd_spectrometer_params, built in one call
(build_designs, detectors auto-positioned with acceptance 1.0).

Glasses come from a fixed synthetic catalog (Sellmeier ranges of synth.py, fitted
to the Horner form), indexed per prism like the reference's glass_indices.
"""
from __future__ import annotations

import math

import numpy as np

from . import _native as N
from . import build_designs
from .synth import WAVELENGTHS, horner_fit, random_sellmeier

# parameter ranges (continuous part of the genome)
ANGLE_MAG = (0.1, 1.2)     # |apex angle|, rad
CURVATURE = (0.01, 0.1)
HEIGHT = (15.0, 25.0)      # mm
Y_MEAN = (0.3, 0.7)        # beam centre / height
DET_ANGLE = (-0.6, 0.6)    # rad
SIGMA_FRAC = 0.05
G_CHOICES = (2, 3, 4, 5, 6)
B_CHOICES = (16, 32, 64, 128)


def glass_catalog(rng, n: int = 64) -> np.ndarray:
    """n synthetic glasses, Horner coefficients (n, 6), highest degree first."""
    return np.array([horner_fit(random_sellmeier(rng)) for _ in range(n)])


class Population:
    """Genomes of a population: G, B, glass indices, signed angle magnitudes,
    curvature, height, beam y fraction, detector angle (all arrays over individuals)."""

    def __init__(self, G, B, glass_idx, angles, curvature, height, y_frac, det_angle):
        self.G = np.asarray(G, dtype=np.int32)
        self.B = np.asarray(B, dtype=np.int32)
        self.glass_idx = np.asarray(glass_idx, dtype=np.int32)     # (n, 6)
        self.angles = np.asarray(angles, dtype=np.float64)          # (n, 7), magnitude with sign
        self.curvature = np.asarray(curvature, dtype=np.float64)
        self.height = np.asarray(height, dtype=np.float64)
        self.y_frac = np.asarray(y_frac, dtype=np.float64)
        self.det_angle = np.asarray(det_angle, dtype=np.float64)

    def __len__(self):
        return self.G.size

    def take(self, idx) -> "Population":
        return Population(self.G[idx], self.B[idx], self.glass_idx[idx], self.angles[idx], self.curvature[idx],
                          self.height[idx], self.y_frac[idx], self.det_angle[idx])

    @staticmethod
    def concat(a: "Population", b: "Population") -> "Population":
        return Population(*[np.concatenate([getattr(a, k), getattr(b, k)])
                            for k in ("G", "B", "glass_idx", "angles", "curvature", "height", "y_frac",
                                      "det_angle")])


def random_population(rng, n: int, n_glasses: int) -> Population:
    G = rng.choice(G_CHOICES, n)
    B = rng.choice(B_CHOICES, n)
    gi = rng.integers(0, n_glasses, (n, N.MAX_GLASS))
    mags = rng.uniform(*ANGLE_MAG, (n, N.MAX_GLASS + 1))
    sign = np.where(rng.uniform(size=(n, 1)) < 0.5, 1.0, -1.0)
    alt = (-1.0) ** np.arange(N.MAX_GLASS + 1)
    return Population(G, B, gi, sign * alt * mags, rng.uniform(*CURVATURE, n), rng.uniform(*HEIGHT, n),
                      rng.uniform(*Y_MEAN, n), rng.uniform(*DET_ANGLE, n))


def perturb(rng, parents: Population, n: int, n_glasses: int) -> Population:
    """n offspring: Gaussian perturbation, sigma = 5% of each range, of random parents.
    Each glass index is redrawn with probability 1/(G+1)."""
    idx = rng.integers(0, len(parents), n)
    o = parents.take(idx)

    def step(x, lo_hi):
        lo, hi = lo_hi
        return np.clip(x + rng.normal(0.0, SIGMA_FRAC * (hi - lo), x.shape), lo, hi)

    mag = step(np.abs(o.angles), ANGLE_MAG)
    angles = np.sign(o.angles) * mag
    redraw = rng.uniform(size=o.glass_idx.shape) < 1.0 / (o.G[:, None] + 1.0)
    gi = np.where(redraw, rng.integers(0, n_glasses, o.glass_idx.shape), o.glass_idx)
    return Population(o.G, o.B, gi, angles, step(o.curvature, CURVATURE), step(o.height, HEIGHT),
                      step(o.y_frac, Y_MEAN), step(o.det_angle, DET_ANGLE))


def to_params(pop: Population, catalog: np.ndarray, *, width: float = 7.0, beam_width: float = 2.0) -> np.ndarray:
    """Parameter records (N.PARAMS_DTYPE) of a population; detectors as synth.detector_for_bins."""
    n = len(pop)
    p = np.zeros(n, dtype=N.PARAMS_DTYPE)
    G = pop.G
    p["nglass"] = G
    p["ar_coated"] = 1
    gl = catalog[pop.glass_idx]                                    # (n, 6, 6)
    gmask = np.arange(N.MAX_GLASS)[None, :] < G[:, None]
    p["glass"] = np.where(gmask[:, :, None], gl, 0.0)
    amask = np.arange(N.MAX_GLASS + 1)[None, :] <= G[:, None]
    p["angles"] = np.where(amask, pop.angles, 0.0)
    p["curvature"] = pop.curvature
    p["height"] = pop.height
    p["width"] = width
    slope = 32.0 / pop.B
    p["bin_count"] = pop.B
    p["bin_size"] = 0.8 * slope
    p["linear_slope"] = slope
    p["linear_intercept"] = 0.1 * slope
    p["det_length"] = 32.0
    p["max_incident_angle"] = math.radians(45.0)
    p["det_angle"] = pop.det_angle
    p["wavelength_bounds"] = np.array(WAVELENGTHS)
    p["beam_width"] = beam_width
    p["beam_y_mean"] = pop.height * pop.y_frac
    return p


def build(pop: Population, catalog: np.ndarray):
    """(designs, ok mask) of a population, detectors auto-positioned (acceptance 1.0)."""
    designs, status = build_designs(to_params(pop, catalog), acceptance=1.0)
    return designs, status == N.OK


def initial_population(rng, n: int, catalog: np.ndarray, max_rounds: int = 50) -> Population:
    """n individuals whose designs build (redraws the ones that raise a ray-trace error)."""
    keep = None
    for _ in range(max_rounds):
        cand = random_population(rng, 2 * n, len(catalog))
        _, ok = build(cand, catalog)
        cand = cand.take(np.nonzero(ok)[0])
        keep = cand if keep is None else Population.concat(keep, cand)
        if len(keep) >= n:
            return keep.take(np.arange(n))
    raise RuntimeError("could not draw a valid initial population")


def survive(pop: Population, info: np.ndarray, mu: int) -> Population:
    """(mu + lambda) survival on mutual information."""
    order = np.argsort(-info, kind="stable")[:mu]
    return pop.take(order)


def serve(server, *, generations: int = 200, sizes=(64, 2048), mean_interarrival_s: float = 0.0, mu: int = 512,
          max_n: int = 128, max_eval: int = 8192, seed: int = 0, mode: int = 0, catalog_size: int = 64,
          device_build: bool = False):
    """Drives `server` (a compound_prism_designer.Server) with `generations` batches.

    Batch sizes are uniform in [sizes[0], sizes[1]]; batches arrive as a Poisson process
    with the given mean inter-arrival time (0: each batch is submitted as soon as it is
    built). Each batch is one request: the offspring of the current population, all
    sampled with one seed drawn for that generation (common random numbers within a
    generation), max_n wavelengths x max_eval rays per design as the reference
    optimizer's gpu_fitness call (designer.py:276). A collector thread waits for the
    requests in order, records each request's latency (submit to completion, measured
    by the server) and updates the population by (mu + lambda) survival on mutual
    information (a design that did not reach the SEM stop or failed counts as -inf).
    device_build: submit the offspring's parameter records and let the server build the
    designs on the device (Server.submit_params) instead of building them here.

    Returns a dict: designs, generations, seconds (first submit to last completion),
    designs_per_s, latency_ms list, p50_ms, p99_ms, mean_batch, best_info."""
    import threading
    import time

    rng = np.random.default_rng(seed)
    catalog = glass_catalog(rng, catalog_size)
    state = {"pop": initial_population(rng, mu, catalog)}
    state["info"] = np.full(len(state["pop"]), -np.inf)
    lock = threading.Lock()
    submitted = []          # (request id, offspring population, n)
    cv = threading.Condition()
    lat, done_t, best = [], [], []
    n_designs = 0

    def collector():
        k = 0
        while k < generations:
            with cv:
                while len(submitted) <= k:
                    cv.wait()
                rid, off = submitted[k]
            outs, ms = server.wait(rid)
            done_t.append(time.perf_counter())
            lat.append(ms)
            info = np.where(outs["status"] == 0, outs["info"], -np.inf)
            with lock:
                merged = Population.concat(state["pop"], off)
                minfo = np.concatenate([state["info"], info])
                order = np.argsort(-minfo, kind="stable")[:mu]
                state["pop"] = merged.take(order)
                state["info"] = minfo[order]
                best.append(float(state["info"][0]))
            k += 1

    th = threading.Thread(target=collector, daemon=True)
    th.start()
    gaps = rng.exponential(mean_interarrival_s, generations) if mean_interarrival_s > 0 else np.zeros(generations)
    t0 = time.perf_counter()
    t_next = t0
    first_submit = None
    for g in range(generations):
        t_next += gaps[g]
        now = time.perf_counter()
        if t_next > now:
            time.sleep(t_next - now)
        n = int(rng.integers(sizes[0], sizes[1] + 1))
        with lock:
            parents = state["pop"]
        off = perturb(rng, parents, n, len(catalog))
        if device_build:
            # every offspring goes to the device; the ones that fail to build come back
            # with their ray-trace status and lose the survival
            keep = np.arange(len(off))
            rid = server.submit_params(to_params(off, catalog), acceptance=1.0, seeds=float(rng.uniform()),
                                       max_n=max_n, max_eval=max_eval, mode=mode)
        else:
            designs, ok = build(off, catalog)
            keep = np.nonzero(ok)[0]
            off = off.take(keep)
            rid = server.submit(designs[keep], seeds=float(rng.uniform()), max_n=max_n, max_eval=max_eval,
                                mode=mode)
        if first_submit is None:
            first_submit = time.perf_counter()
        n_designs += keep.size
        with cv:
            submitted.append((rid, off))
            cv.notify()
    th.join()
    secs = done_t[-1] - first_submit
    lat_a = np.asarray(lat)
    return {"designs": n_designs, "generations": generations, "seconds": secs, "designs_per_s": n_designs / secs,
            "latency_ms": lat, "p50_ms": float(np.percentile(lat_a, 50)), "p99_ms": float(np.percentile(lat_a, 99)),
            "mean_batch": n_designs / generations, "best_info": best[-1] if best else None,
            "best_info_first": best[0] if best else None}
