"""GB300 drop-in for the fitness path of jdtatz/compound-prism-designer.

Same module name, classes, methods, argument names and defaults as the
reference's pyo3 extension (src/pylib.rs; stub
compound_prism_designer/compound_prism_designer.pyi), so an optimizer written
against the reference (designer.py:203-300) runs unchanged. Every call goes
through the C ABI of libcpd.so (include/cpd.h); gpu_fitness runs the
sm_103a kernels and has no CPU fallback.

Out of scope (they raise NotImplementedError): the 3-D FiberBeam/toric-lens
variant and the matplotlib drawing helpers (polygons, surfaces). The reference's 3-D
ray-torus intersection (src/spectrometer/toric.rs:41-201) takes the square root of a
negative discriminant whenever a ray meets the torus four times, so in the reference
optimizer's fiber configuration no design can be positioned and every ray is lost at the
first toric lens; the 3-D path is not reproduced on the GPU.
"""
from __future__ import annotations

import ctypes as C
import math
import threading
from typing import Optional, Sequence

import numpy as np

from . import _native as N

__all__ = [
    "RayTraceError", "CudaError", "Glass", "DesignFitness", "Vector2D", "UnitVector2D",
    "UniformWavelengthDistribution", "GaussianBeam", "FiberBeam", "CompoundPrism",
    "position_detector_array", "DetectorArray", "Spectrometer", "Context", "default_context",
    "fitness_batch", "fitness_batch_params", "autotune_batch", "build_designs", "Server", "TRACE_HYBRID", "TRACE_FP32", "TRACE_FP64",
    "SAMPLING_ADAPTIVE", "SAMPLING_EXACT",
]

TRACE_HYBRID = N.TRACE_HYBRID
TRACE_FP32 = N.TRACE_FP32
TRACE_FP64 = N.TRACE_FP64
# OR into a trace mode (TRACE_HYBRID | SAMPLING_ADAPTIVE), or pass adaptive=True to
# gpu_fitness: the reference kernel's per-wavelength SEM stop (src/spectrometer/kernel.rs:127-178)
SAMPLING_ADAPTIVE = N.SAMPLING_ADAPTIVE
SAMPLING_EXACT = N.SAMPLING_EXACT


class RayTraceError(Exception):
    """A geometric failure (src/spectrometer/ray.rs:10-16)."""


class CudaError(Exception):
    """A CUDA failure (src/pylib.rs:26-35)."""


def _check(code: int, what: str = "") -> int:
    if code in (N.OK, N.NOT_CONVERGED):
        return code
    msg = N.status_string(code)
    if code in N.RAYTRACE_ERRORS:
        raise RayTraceError(msg)
    if code == N.CUDA_ERROR:
        raise CudaError(f"{what}: {msg}" if what else msg)
    if code == N.NOT_IMPLEMENTED:
        raise NotImplementedError(msg)
    raise ValueError(f"{what}: {msg}" if what else msg)


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _seed_array(seeds):
    """A few seeds as a ctypes double array (the per-call path: a numpy pointer costs
    several microseconds, a small ctypes array well under one)."""
    if type(seeds) is list and all(type(v) is float for v in seeds):
        vals = seeds  # the common per-call form, without a numpy round trip
    elif isinstance(seeds, np.ndarray):
        vals = seeds.ravel().tolist()
    elif isinstance(seeds, (float, int)):
        vals = [seeds]
    else:
        vals = np.asarray(seeds, dtype=np.float64).ravel().tolist()
    return (C.c_double * len(vals))(*vals), len(vals)


class Glass:
    """Glass(name, coefficents): the 6-coefficient Horner dispersion polynomial
    (src/pylib.rs:37-95, src/spectrometer/glasscat.rs:7-22)."""

    ORDER = 5

    def __init__(self, name: str, coefficents):
        c = np.ascontiguousarray(coefficents, dtype=np.float64).reshape(-1)
        if c.size != self.ORDER + 1:
            raise ValueError("Incorrect coefficents length")
        self.name = str(name)
        self._c = c

    @property
    def glass(self) -> np.ndarray:
        return self._c.copy()

    def __call__(self, w: float) -> float:
        return N.lib.cpd_glass_index(_dp(self._c), float(w))

    def __getnewargs__(self):
        return (self.name, self._c.copy())

    def __reduce__(self):
        return (Glass, (self.name, self._c.copy()))

    def __repr__(self):
        return f"Glass(name={self.name!r}, coefficents={self._c.tolist()})"


class DesignFitness:
    """DesignFitness(size, info, deviation) (src/pylib.rs:103-153)."""

    def __init__(self, size: float, info: float, deviation: float):
        self.size = float(size)
        self.info = float(info)
        self.deviation = float(deviation)

    def __getnewargs__(self):
        return (self.size, self.info, self.deviation)

    def __reduce__(self):
        return (DesignFitness, self.__getnewargs__())

    def __repr__(self):
        return f"DesignFitness(size={self.size}, info={self.info}, deviation={self.deviation})"


class Vector2D:
    def __init__(self, x: float, y: float):
        self.x = float(x)
        self.y = float(y)

    def __iter__(self):
        return iter((self.x, self.y))

    def __getnewargs__(self):
        return (self.x, self.y)

    def __repr__(self):
        return f"Vector2D(x={self.x}, y={self.y})"


class UnitVector2D(Vector2D):
    def __init__(self, x: float, y: float):
        # UnitVector::try_new: |v| within rmax 1e-3 of 1 (vector.rs:300-312, src/pylib.rs:215-220)
        n = math.hypot(x, y)
        if not abs(n - 1.0) <= 1e-3 * max(n, 1.0):
            raise ValueError("x^2 + y^2 != 1")
        super().__init__(x, y)

    def __repr__(self):
        return f"UnitVector2D(x={self.x}, y={self.y})"


class UniformWavelengthDistribution:
    """UniformWavelengthDistribution(bounds) (src/pylib.rs:290-331)."""

    def __init__(self, bounds):
        lo, hi = (float(b) for b in bounds)
        if hi < lo:
            raise ValueError("lower bound > upper bound")
        self.bounds = (lo, hi)

    def __getnewargs__(self):
        return (self.bounds,)


class GaussianBeam:
    """GaussianBeam(width, y_mean) (src/pylib.rs:357-385)."""

    def __init__(self, width: float, y_mean: float):
        self.width = float(width)
        self.y_mean = float(y_mean)

    def __getnewargs__(self):
        return (self.width, self.y_mean)

    def __repr__(self):
        return f"GaussianBeam(width={self.width}, y_mean={self.y_mean})"


class FiberBeam:
    """FiberBeam(core_radius, numerical_aperture, center_y) (src/pylib.rs:387-430).
    Constructible for API compatibility; the 3-D fiber-beam trace is not built."""

    def __init__(self, core_radius: float, numerical_aperture: float, center_y: float):
        self.core_radius = float(core_radius)
        self.numerical_aperture = float(numerical_aperture)
        self.center_y = float(center_y)

    @property
    def y_mean(self) -> float:
        return self.center_y

    @property
    def width(self) -> float:
        return self.core_radius

    def __getnewargs__(self):
        return (self.core_radius, self.numerical_aperture, self.center_y)


def _fill_prism(p: N.SpectrometerParams, glasses, angles, lengths, curvature, height, width, ar_coated):
    G = len(glasses)
    p.nglass = G
    p.ar_coated = int(bool(ar_coated))
    for g, glass in enumerate(glasses):
        for i, c in enumerate(glass._c):
            p.glass[g][i] = float(c)
    for i, a in enumerate(angles):
        p.angles[i] = float(a)
    for i, l in enumerate(lengths):
        p.lengths[i] = float(l)
    p.curvature = float(curvature)
    p.height = float(height)
    p.width = float(width)


class CompoundPrism:
    """CompoundPrism(glasses, angles, lengths, curvature, height, width, ar_coated)
    (src/pylib.rs:658-812)."""

    def __init__(self, glasses: Sequence[Glass], angles, lengths, curvature, height: float, width: float,
                 ar_coated: bool):
        glasses = list(glasses)
        angles = [float(a) for a in np.asarray(angles, dtype=np.float64).reshape(-1)]
        lengths = [float(l) for l in np.asarray(lengths, dtype=np.float64).reshape(-1)]
        # argument checks of SizedCompoundPrism::new (src/pylib.rs:524-540)
        if len(angles) < 2:
            raise ValueError("`angles` must have at least 2 elements")
        if len(glasses) > N.MAX_GLASS:
            raise ValueError(f"Maximum of {N.MAX_GLASS} prisms are allowed")
        if len(glasses) != len(angles) - 1:
            raise ValueError("len(glasses) + 1 != len(angles)")
        if len(glasses) != len(lengths):
            raise ValueError("len(glasses) != len(lengths)")
        if isinstance(curvature, (tuple, list)):
            raise NotImplementedError(
                "the 3-D toric-lens compound prism is not built: the reference's closed-form ray-torus "
                "intersection (toric.rs:41-141) yields NaN whenever a ray meets the torus four times, so no "
                "design of its fiber configuration can be positioned")
        self.glasses = glasses
        self.angles = angles
        self.lengths = lengths
        self.curvature = float(curvature)
        self.height = float(height)
        self.width = float(width)
        self.ar_coated = bool(ar_coated)
        # the prism tables alone (a placeholder detector makes the design complete)
        p = N.SpectrometerParams()
        self._fill(p)
        p.bin_count, p.bin_size, p.linear_slope, p.det_length = 1, 1.0, 1.0, 1.0
        p.wavelength_bounds[0], p.wavelength_bounds[1] = 0.5, 0.5
        d = N.Design()
        _check(N.lib.cpd_design_build(C.byref(p), C.byref(d)), "CompoundPrism")
        self._design = d

    def _fill(self, p: N.SpectrometerParams):
        _fill_prism(p, self.glasses, self.angles, self.lengths, self.curvature, self.height, self.width,
                    self.ar_coated)

    def __getnewargs__(self):
        return (self.glasses, self.angles, self.lengths, self.curvature, self.height, self.width, self.ar_coated)

    def __reduce__(self):
        return (CompoundPrism, self.__getnewargs__())

    def exit_ray(self, y: float, wavelength: float):
        out = np.zeros(4)
        _check(N.lib.cpd_exit_ray(C.byref(self._design), float(y), float(wavelength), _dp(out)))
        return Vector2D(out[0], out[1]), UnitVector2D(out[2], out[3])

    def final_midpt_and_normal(self):
        """(arc mid point, unit vector at the last angle) (src/pylib.rs:782-793)."""
        d = self._design
        a = self.angles[-1]
        return Vector2D(d.exit_bound_center[0], d.exit_bound_center[1]), UnitVector2D(math.cos(a), math.sin(a))

    def surfaces(self):
        raise NotImplementedError("drawing helpers are not part of the GPU fitness path")

    def polygons(self):
        raise NotImplementedError("drawing helpers are not part of the GPU fitness path")

    def __repr__(self):
        return (f"CompoundPrism(glasses={[g.name for g in self.glasses]}, angles={self.angles}, "
                f"lengths={self.lengths}, curvature={self.curvature}, height={self.height}, "
                f"width={self.width}, ar_coated={self.ar_coated})")


def _fill_source(p: N.SpectrometerParams, wavelengths, beam):
    if not isinstance(wavelengths, UniformWavelengthDistribution):
        raise TypeError("wavelengths must be a UniformWavelengthDistribution")
    p.wavelength_bounds[0], p.wavelength_bounds[1] = wavelengths.bounds
    if isinstance(beam, GaussianBeam):
        p.beam_width = beam.width
        p.beam_y_mean = beam.y_mean
    elif isinstance(beam, FiberBeam):
        raise NotImplementedError("No kernel compiled for this Spectrometer")
    else:
        raise TypeError("beam must be a GaussianBeam")


def position_detector_array(length: float, angle: float, compound_prism: CompoundPrism, wavelengths, beam,
                            acceptance: float):
    """position_detector_array (src/pylib.rs:815-838)."""
    p = N.SpectrometerParams()
    compound_prism._fill(p)
    _fill_source(p, wavelengths, beam)
    p.det_length = float(length)
    p.det_angle = float(angle)
    pos = np.zeros(2)
    fl = C.c_int32(0)
    _check(N.lib.cpd_position_detector_array(C.byref(p), float(acceptance), _dp(pos), C.byref(fl)))
    return (float(pos[0]), float(pos[1])), bool(fl.value)


class DetectorArray:
    """DetectorArray(bin_count, bin_size, linear_slope, linear_intercept, length,
    max_incident_angle, angle, position, flipped) (src/pylib.rs:840-955)."""

    def __init__(self, bin_count: int, bin_size: float, linear_slope: float, linear_intercept: float,
                 length: float, max_incident_angle: float, angle: float, position, flipped: bool):
        self.bin_count = int(bin_count)
        self.bin_size = float(bin_size)
        self.linear_slope = float(linear_slope)
        self.linear_intercept = float(linear_intercept)
        self.length = float(length)
        self.max_incident_angle = float(max_incident_angle)
        self.angle = float(angle)
        self.position = (float(position[0]), float(position[1]))
        self.flipped = bool(flipped)

    def __getnewargs__(self):
        return (self.bin_count, self.bin_size, self.linear_slope, self.linear_intercept, self.length,
                self.max_incident_angle, self.angle, self.position, self.flipped)

    def __reduce__(self):
        return (DetectorArray, self.__getnewargs__())


class Context:
    """A GPU context (one per device): stream, pooled device buffers, captured CUDA
    graphs. The reference keeps one cached context behind a mutex
    (src/cuda_fitness.rs:322-363); this one is thread-safe too."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        _check(N.lib.cpd_context_create(int(device), C.byref(h)), "cpd_context_create")
        self._h = h
        self.device = device

    @property
    def handle(self):
        return self._h

    def close(self):
        if self._h:
            N.lib.cpd_context_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_launch_shape(self, ray_tile: int = 0, warps_per_cta: int = 0):
        _check(N.lib.cpd_set_launch_shape(self._h, int(ray_tile), int(warps_per_cta)))

    def launch_shape(self):
        rt, w = C.c_uint32(0), C.c_uint32(0)
        _check(N.lib.cpd_get_launch_shape(self._h, C.byref(rt), C.byref(w)))
        return rt.value, w.value

    def last_timing(self):
        ms = C.c_double(0.0)
        n = C.c_uint32(0)
        _check(N.lib.cpd_last_timing(self._h, C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def set_autotune(self, on: bool = True):
        """Batched calls pick their launch shape with the autotuner (per batch class)."""
        _check(N.lib.cpd_set_autotune(self._h, int(bool(on))))

    def set_profiling(self, on: bool = True):
        _check(N.lib.cpd_set_profiling(self._h, int(bool(on))))

    def last_kernel_times(self) -> dict:
        ms = np.zeros(4)
        _check(N.lib.cpd_last_kernel_times(self._h, _dp(ms)))
        return dict(zip(("setup", "trace", "retrace", "entropy"), ms.tolist()))

    def last_transfer_bytes(self):
        h, d = C.c_uint64(0), C.c_uint64(0)
        _check(N.lib.cpd_last_transfer_bytes(self._h, C.byref(h), C.byref(d)))
        return h.value, d.value

    def fp32_peak_tflops(self, iters: int = 4096) -> float:
        t = C.c_double(0.0)
        _check(N.lib.cpd_measure_fp32_peak(self._h, int(iters), C.byref(t)))
        return t.value

    def sfu_peak_gops(self, iters: int = 2048) -> float:
        """Measured special-function-unit throughput (reciprocal-square-root estimates), G/s."""
        t = C.c_double(0.0)
        _check(N.lib.cpd_measure_sfu_peak(self._h, int(iters), C.byref(t)))
        return t.value


_contexts: dict[int, Context] = {}
_ctx_lock = threading.Lock()


def default_context(device: int = 0) -> Context:
    with _ctx_lock:
        ctx = _contexts.get(device)
        if ctx is None:
            ctx = Context(device)
            _contexts[device] = ctx
        return ctx


class Spectrometer:
    """Spectrometer(compound_prism, detector_array, wavelengths, beam) (src/pylib.rs:957-1170)."""

    def __init__(self, compound_prism: CompoundPrism, detector_array: DetectorArray, wavelengths, beam):
        self.compound_prism = compound_prism
        self.detector_array = detector_array
        self.wavelengths = wavelengths
        self.beam = beam
        self._design = None

    def __getnewargs__(self):
        return (self.compound_prism, self.detector_array, self.wavelengths, self.beam)

    def __reduce__(self):
        return (Spectrometer, self.__getnewargs__())

    def params(self) -> N.SpectrometerParams:
        p = N.SpectrometerParams()
        self.compound_prism._fill(p)
        _fill_source(p, self.wavelengths, self.beam)
        da = self.detector_array
        p.bin_count = da.bin_count
        p.bin_size = da.bin_size
        p.linear_slope = da.linear_slope
        p.linear_intercept = da.linear_intercept
        p.det_length = da.length
        p.max_incident_angle = da.max_incident_angle
        p.det_angle = da.angle
        p.det_position[0], p.det_position[1] = da.position
        p.det_flipped = int(da.flipped)
        return p

    @property
    def design(self) -> N.Design:
        """The built f64 design tables (cpd_design) this spectrometer evaluates."""
        if self._design is None:
            d = N.Design()
            _check(N.lib.cpd_design_build(C.byref(self.params()), C.byref(d)), "Spectrometer")
            self._design = d
        return self._design

    @property
    def position(self):
        d = self.design
        return (d.det_position[0], d.det_position[1])

    @property
    def direction(self):
        d = self.design
        return (d.det_direction[0], d.det_direction[1])

    def cpu_fitness(self, *, max_n: int = 16_384, max_m: int = 16_384) -> DesignFitness:
        """The reference's adaptive f64 host estimator (src/pylib.rs:1008-1026)."""
        f = N.Fitness()
        _check(N.lib.cpd_fitness_cpu(C.byref(self.design), int(max_n), int(max_m), C.byref(f)))
        return DesignFitness(f.size, f.info, f.deviation)

    def gpu_fitness(self, seeds, *, max_n: int = 256, nwarp: int = 2, max_eval: int = 16_384,
                    adaptive: bool = False, context: Optional[Context] = None) -> Optional[DesignFitness]:
        """GPU fitness (src/pylib.rs:1085-1135): None if the SEM stop was not met.
        adaptive: each wavelength stops at the reference kernel's per-wavelength SEM test
        (src/spectrometer/kernel.rs:127-178) instead of using all max_eval rays."""
        f = self.gpu_fitness_full(seeds, max_n=max_n, nwarp=nwarp, max_eval=max_eval, adaptive=adaptive,
                                  context=context)
        if f.status == N.NOT_CONVERGED:
            return None
        return DesignFitness(f.size, f.info, f.deviation)

    def gpu_fitness_full(self, seeds, *, max_n: int = 256, nwarp: int = 2, max_eval: int = 16_384,
                         adaptive: bool = False, context: Optional[Context] = None) -> N.Fitness:
        sarr, ns = _seed_array(seeds)
        ctx = context or default_context()
        f = N.Fitness()
        if adaptive:
            _check(N.lib.cpd_fitness_gpu_ex(ctx.handle, C.byref(self.design), sarr, ns, int(max_n),
                                            int(nwarp), int(max_eval), N.SAMPLING_ADAPTIVE, C.byref(f)),
                   "gpu_fitness")
        else:
            _check(N.lib.cpd_fitness_gpu(ctx.handle, C.byref(self.design), sarr, ns, int(max_n),
                                         int(nwarp), int(max_eval), C.byref(f)), "gpu_fitness")
        return f

    def gpu_fitness_points(self, lam_u, ray_u, *, mode: int = TRACE_HYBRID, want_p: bool = False,
                           context: Optional[Context] = None):
        """The estimator on explicit wavelength and ray u-points (parity entry): fixed N, or
        adaptive sampling with mode | SAMPLING_ADAPTIVE (rays taken in the given order)."""
        lam_u = np.ascontiguousarray(lam_u, dtype=np.float64)
        ray_u = np.ascontiguousarray(ray_u, dtype=np.float64)
        ctx = context or default_context()
        f = N.Fitness()
        p = np.zeros((lam_u.size, self.detector_array.bin_count)) if want_p else None
        _check(N.lib.cpd_fitness_gpu_points(ctx.handle, C.byref(self.design), _dp(lam_u), lam_u.size, _dp(ray_u),
                                            ray_u.size, int(mode), C.byref(f),
                                            _dp(p) if p is not None else None), "gpu_fitness_points")
        return f, p

    def trace_rays(self, lam_u, ray_u, *, mode: int = TRACE_HYBRID, context: Optional[Context] = None):
        """One ray per (lam_u[i], ray_u[i]): (bins, t, retraced) (propagation_test_kernel twin)."""
        lam_u = np.ascontiguousarray(lam_u, dtype=np.float64)
        ray_u = np.ascontiguousarray(ray_u, dtype=np.float64)
        n = lam_u.size
        bins = np.zeros(n, dtype=np.uint32)
        ts = np.zeros(n)
        fl = np.zeros(n, dtype=np.uint8)
        ctx = context or default_context()
        _check(N.lib.cpd_trace_rays(ctx.handle, C.byref(self.design), _dp(lam_u), _dp(ray_u), n, int(mode),
                                    bins.ctypes.data_as(C.POINTER(C.c_uint32)), _dp(ts),
                                    fl.ctypes.data_as(C.POINTER(C.c_uint8))), "trace_rays")
        return bins, ts, fl.astype(bool)

    def transmission_probability(self, wavelengths, *, max_m: int = 16_384, fixed_n: bool = False,
                                 return_rays: bool = False, context: Optional[Context] = None):
        """p(d|lambda) for each given wavelength, shape (len(wavelengths), bin_count)
        (src/pylib.rs:1028-1058): the reference's estimator, p_dets_l_wavelength
        (src/fitness.rs:5-69), which stops a wavelength at the first hit whose bin's SEM is
        <= 5e-3 (at most max_m rays). fixed_n=True traces all max_m rays instead.
        return_rays=True also returns the rays each wavelength consumed."""
        w = np.ascontiguousarray(wavelengths, dtype=np.float64).reshape(-1)
        ctx = context or default_context()
        out = np.zeros((w.size, self.detector_array.bin_count))
        rays = np.zeros(w.size, dtype=np.uint32)
        _check(N.lib.cpd_transmission_probability_ex(ctx.handle, C.byref(self.design), _dp(w), w.size, int(max_m),
                                                     N.TP_FIXED_N if fixed_n else 0, _dp(out),
                                                     rays.ctypes.data_as(C.POINTER(C.c_uint32))),
               "transmission_probability")
        return (out, rays) if return_rays else out

    def ray_trace(self, wavelength: float, inital_y: float) -> np.ndarray:
        """Propagation path rows (x, y, ux, uy) (src/pylib.rs:1060-1083)."""
        G = len(self.compound_prism.glasses)
        rows = np.zeros((G + 3, 4))
        n = C.c_uint32(0)
        _check(N.lib.cpd_ray_trace(C.byref(self.design), float(wavelength), float(inital_y), _dp(rows),
                                   C.byref(n)))
        return rows[: n.value].copy()

    def __repr__(self):
        return (f"Spectrometer({self.compound_prism!r}, detector_array={self.detector_array.__dict__}, "
                f"wavelengths={self.wavelengths.bounds}, beam={self.beam!r})")


def _pack_designs(designs):
    """The designs' records (Spectrometers or cpd_design structs) as one ctypes array:
    their buffers joined in one pass (a Python loop of struct copies costs ~2 us each)."""
    n = len(designs)
    blob = b"".join([memoryview(s.design if isinstance(s, Spectrometer) else s) for s in designs])
    return (N.Design * n).from_buffer_copy(blob)


def _batch_records(spectrometers, seeds, max_n, max_eval):
    n = len(spectrometers)
    designs = _pack_designs(spectrometers)
    items = (N.BatchItem * n).from_buffer(_items(n, 0.5 if seeds is None else seeds, max_n, max_eval))
    return n, designs, items


def fitness_batch(spectrometers: Sequence[Spectrometer], *, seeds=None, max_n=256, max_eval=16_384,
                  mode: int = TRACE_HYBRID, context: Optional[Context] = None):
    """Batched GPU fitness of many designs in one launch sequence (no reference
    counterpart). max_n, max_eval and seeds may be scalars or per-design sequences.
    Returns a list of cpd_fitness records (status OK or NOT_CONVERGED per design)."""
    n, designs, items = _batch_records(spectrometers, seeds, max_n, max_eval)
    outs = (N.Fitness * n)()
    ctx = context or default_context()
    _check(N.lib.cpd_fitness_gpu_batch(ctx.handle, designs, items, n, int(mode), outs), "fitness_batch")
    return list(outs)


def autotune_batch(spectrometers: Sequence[Spectrometer], *, seeds=None, max_n=256, max_eval=16_384,
                   mode: int = TRACE_HYBRID, context: Optional[Context] = None):
    """Runs the launch-shape autotuner on a batch (cpd_autotune_batch) and leaves the
    fastest shape set on the context. Returns (ray_tile, warps_per_cta, best_ms)."""
    n, designs, items = _batch_records(spectrometers, seeds, max_n, max_eval)
    ctx = context or default_context()
    rt, w, ms = C.c_uint32(0), C.c_uint32(0), C.c_double(0.0)
    _check(N.lib.cpd_autotune_batch(ctx.handle, designs, items, n, int(mode), C.byref(rt), C.byref(w),
                                    C.byref(ms)), "autotune_batch")
    return rt.value, w.value, ms.value


def build_designs(params: np.ndarray, acceptance: float = 0.0, *, device: bool = False,
                  context: Optional[Context] = None):
    """Builds a whole generation of designs from an array of N.PARAMS_DTYPE records (no
    reference counterpart; the reference builds one Spectrometer per call,
    designer.py:203-265). With acceptance in (0, 1] each detector is placed by
    position_detector_array first. device=True builds them on the GPU
    (cpd_design_build_device). Returns (designs, status): an N.DESIGN_DTYPE array and the
    per-design status codes (0 = built)."""
    params = np.ascontiguousarray(params, dtype=N.PARAMS_DTYPE)
    n = params.size
    designs = np.zeros(n, dtype=N.DESIGN_DTYPE)
    status = np.zeros(n, dtype=np.int32)
    if device:
        ctx = context or default_context()
        _check(N.lib.cpd_design_build_device(ctx.handle, params.ctypes.data, n, float(acceptance),
                                             designs.ctypes.data, status.ctypes.data_as(C.POINTER(C.c_int32))),
               "build_designs")
    else:
        _check(N.lib.cpd_design_build_batch(params.ctypes.data, n, float(acceptance), designs.ctypes.data,
                                            status.ctypes.data_as(C.POINTER(C.c_int32))), "build_designs")
    return designs, status


def _items(n, seeds, max_n, max_eval):
    items = np.zeros(n, dtype=N.BATCH_ITEM_DTYPE)
    items["seed"] = np.broadcast_to(np.asarray(seeds, dtype=np.float64), (n,))
    items["max_n"] = np.broadcast_to(np.asarray(max_n), (n,))
    items["max_eval"] = np.broadcast_to(np.asarray(max_eval), (n,))
    return items


def fitness_batch_params(params: np.ndarray, *, acceptance: float = 0.0, seeds=0.5, max_n=256, max_eval=16_384,
                         mode: int = TRACE_HYBRID, context: Optional[Context] = None) -> np.ndarray:
    """The batched fitness of designs built on the device from N.PARAMS_DTYPE records
    (cpd_fitness_gpu_batch_params). Returns an N.FITNESS_DTYPE array; status holds a
    design's build error (a RayTraceError code) where it could not be built."""
    params = np.ascontiguousarray(params, dtype=N.PARAMS_DTYPE)
    n = params.size
    items = _items(n, seeds, max_n, max_eval)
    outs = np.zeros(n, dtype=N.FITNESS_DTYPE)
    ctx = context or default_context()
    _check(N.lib.cpd_fitness_gpu_batch_params(ctx.handle, params.ctypes.data, items.ctypes.data, n,
                                              float(acceptance), int(mode), outs.ctypes.data),
           "fitness_batch_params")
    return outs


def _design_array(designs) -> np.ndarray:
    if isinstance(designs, np.ndarray):
        return np.ascontiguousarray(designs, dtype=N.DESIGN_DTYPE)
    return np.frombuffer(_pack_designs(designs), dtype=N.DESIGN_DTYPE)


class LoopServer:
    """The device-resident serving loop (cpd_loop_*, no reference counterpart).

    One persistent kernel; each CTA owns a histogram slab and evaluates whole designs
    taken from a ring in mapped host memory, with no host step between designs. A design
    is admitted when its W x B cells fit a slab (max_cells, max_rows); the GPU memory for
    histograms is hist_budget_bytes. Fixed N with the hybrid trace. The methods are
    those of Server; each design's result is bitwise the one it gets alone."""

    def __init__(self, hist_budget_bytes: int = 4 << 30, *, max_cells: int = 0, max_rows: int = 0,
                 ring_capacity: int = 0, ctas_per_sm: int = 0, idle_ms: int = 0, ray_tile: int = 0,
                 context: Optional[Context] = None):
        self._ctx = context or default_context()
        cfg = N.LoopConfig(int(hist_budget_bytes), int(max_cells), int(max_rows), int(ring_capacity),
                           int(ctas_per_sm), int(idle_ms), int(ray_tile))
        h = C.c_void_p()
        _check(N.lib.cpd_loop_create(self._ctx.handle, C.byref(cfg), C.byref(h)), "cpd_loop_create")
        self._h = h
        self._sizes: dict[int, int] = {}
        self._lock = threading.Lock()

    def submit(self, designs, *, seeds=0.5, max_n=128, max_eval=8192, mode: int = TRACE_HYBRID) -> int:
        """Queues designs (Spectrometers or an N.DESIGN_DTYPE array); returns the request id."""
        d = _design_array(designs)
        n = d.size
        items = _items(n, seeds, max_n, max_eval)
        rid = C.c_uint64(0)
        _check(N.lib.cpd_loop_submit(self._h, d.ctypes.data, items.ctypes.data, n, int(mode), C.byref(rid)),
               "cpd_loop_submit")
        with self._lock:
            self._sizes[rid.value] = n
        return rid.value

    def wait(self, request_id: int, timeout: Optional[float] = None):
        """(results, latency_ms) as Server.wait."""
        with self._lock:
            n = self._sizes[request_id]
        outs = np.zeros(n, dtype=N.FITNESS_DTYPE)
        lat = C.c_double(0.0)
        remaining = math.inf if timeout is None else float(timeout)
        while True:
            step = min(remaining, 1.0)
            rc = N.lib.cpd_loop_wait(self._h, request_id, outs.ctypes.data, step * 1e3, C.byref(lat))
            if rc != N.TIMEOUT:
                break
            remaining -= step
            if remaining <= 0:
                raise TimeoutError(f"request {request_id} not done")
        with self._lock:
            del self._sizes[request_id]
        _check(rc, "cpd_loop_wait")
        return outs, lat.value

    def stats(self) -> dict:
        r = N.LoopReport()
        _check(N.lib.cpd_loop_stats(self._h, C.byref(r)), "cpd_loop_stats")
        return r.as_dict()

    def close(self):
        if self._h:
            N.lib.cpd_loop_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass


class Server:
    """Continuous-batching fitness server on one GPU (no reference counterpart).

    Requests arrive from any thread with submit(); a native worker admits their designs
    in arrival order into passes while the device bytes of the designs in flight stay
    within mem_budget_bytes, and keeps up to `slots` passes in flight on separate
    streams. Each design's result is bitwise the one it gets alone."""

    def __init__(self, mem_budget_bytes: int = 8 << 30, slots: int = 2, max_designs_per_pass: int = 256,
                 context: Optional[Context] = None):
        self._ctx = context or default_context()
        h = C.c_void_p()
        _check(N.lib.cpd_server_create(self._ctx.handle, int(mem_budget_bytes), int(slots),
                                       int(max_designs_per_pass), C.byref(h)), "cpd_server_create")
        self._h = h
        self._sizes: dict[int, int] = {}
        self._lock = threading.Lock()

    def submit(self, designs, *, seeds=0.5, max_n=128, max_eval=8192, mode: int = TRACE_HYBRID) -> int:
        """Queues designs (Spectrometers or an N.DESIGN_DTYPE array); max_n, max_eval and
        seeds may be scalars or per-design sequences. Returns the request id at once."""
        d = _design_array(designs)
        n = d.size
        items = np.zeros(n, dtype=N.BATCH_ITEM_DTYPE)
        items["seed"] = np.broadcast_to(np.asarray(seeds, dtype=np.float64), (n,))
        items["max_n"] = np.broadcast_to(np.asarray(max_n), (n,))
        items["max_eval"] = np.broadcast_to(np.asarray(max_eval), (n,))
        rid = C.c_uint64(0)
        _check(N.lib.cpd_server_submit(self._h, d.ctypes.data, items.ctypes.data, n, int(mode), C.byref(rid)),
               "cpd_server_submit")
        with self._lock:
            self._sizes[rid.value] = n
        return rid.value

    def submit_params(self, params, *, acceptance: float = 0.0, seeds=0.5, max_n=128, max_eval=8192,
                      mode: int = TRACE_HYBRID) -> int:
        """Queues N.PARAMS_DTYPE records; the designs are built on the device inside their
        pass (cpd_server_submit_params). Returns the request id at once."""
        p = np.ascontiguousarray(params, dtype=N.PARAMS_DTYPE)
        n = p.size
        items = _items(n, seeds, max_n, max_eval)
        rid = C.c_uint64(0)
        _check(N.lib.cpd_server_submit_params(self._h, p.ctypes.data, items.ctypes.data, n, float(acceptance),
                                              int(mode), C.byref(rid)), "cpd_server_submit_params")
        with self._lock:
            self._sizes[rid.value] = n
        return rid.value

    def wait(self, request_id: int, timeout: Optional[float] = None):
        """Waits for a request (timeout in seconds, None = forever). Returns (results,
        latency_ms): an N.FITNESS_DTYPE array (status NOT_CONVERGED marks a design whose
        SEM stayed above 5e-3) and the time from submit to completion. Raises
        TimeoutError when the timeout passes first; the request stays queued."""
        with self._lock:
            n = self._sizes[request_id]
        outs = np.zeros(n, dtype=N.FITNESS_DTYPE)
        lat = C.c_double(0.0)
        remaining = math.inf if timeout is None else float(timeout)
        while True:
            step = min(remaining, 1.0)
            rc = N.lib.cpd_server_wait(self._h, request_id, outs.ctypes.data, step * 1e3, C.byref(lat))
            if rc != N.TIMEOUT:
                break
            remaining -= step
            if remaining <= 0:
                raise TimeoutError(f"request {request_id} not done")
        with self._lock:
            del self._sizes[request_id]
        _check(rc, "cpd_server_wait")
        return outs, lat.value

    def stats(self) -> dict:
        v = [C.c_uint64(0) for _ in range(4)]
        _check(N.lib.cpd_server_stats(self._h, *[C.byref(x) for x in v]))
        return dict(zip(("designs_done", "passes", "max_passes_in_flight", "pending_designs"),
                        (x.value for x in v)))

    def close(self):
        if self._h:
            N.lib.cpd_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
