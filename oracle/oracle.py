"""ctypes loader for the C oracle -- TEST INFRASTRUCTURE ONLY.

The oracle is a double-precision restatement of the reference's CPU fitness
path (src/fitness.rs and src/spectrometer/*.rs of jdtatz/compound-prism-designer).
Only tests, the smoke check and the benchmark's CPU-baseline/reference legs
import this module; the product package never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liborc.so")
OPS_LIB_PATH = os.path.join(HERE, "_build", "liborc_ops.so")

MAX_GLASS = 6
(OK, NO_SURFACE_INTERSECTION, OUT_OF_BOUNDS, TOTAL_INTERNAL_REFLECTION,
 ANGULAR_RESPONSE_TOO_WEAK) = range(5)
INVALID = 10


class OrcSpec(C.Structure):
    _fields_ = [
        ("nglass", C.c_int32),
        ("ar_coated", C.c_int32),
        ("glass", (C.c_double * 6) * MAX_GLASS),
        ("angles", C.c_double * (MAX_GLASS + 1)),
        ("lengths", C.c_double * MAX_GLASS),
        ("curvature", C.c_double),
        ("height", C.c_double),
        ("width", C.c_double),
        ("bin_count", C.c_uint32),
        ("det_flipped", C.c_int32),
        ("bin_size", C.c_double),
        ("linear_slope", C.c_double),
        ("linear_intercept", C.c_double),
        ("det_length", C.c_double),
        ("max_incident_angle", C.c_double),
        ("det_angle", C.c_double),
        ("det_position", C.c_double * 2),
        ("wmin", C.c_double),
        ("wmax", C.c_double),
        ("beam_width", C.c_double),
        ("beam_y_mean", C.c_double),
    ]


def _stale() -> bool:
    if not os.path.exists(LIB_PATH):
        return True
    t = os.path.getmtime(LIB_PATH)
    srcs = ("cpd_oracle.c", "cpd_oracle_toric.c", "cpd_oracle.h", "cpd_oracle_model.h", "ops_count.cpp", "build.sh")
    return any(os.path.getmtime(os.path.join(HERE, f)) > t for f in srcs)


def build(force: bool = False) -> str:
    if force or _stale():
        subprocess.check_call(["bash", os.path.join(HERE, "build.sh")])
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        dp = C.POINTER(C.c_double)
        up = C.POINTER(C.c_uint32)
        sp = C.POINTER(OrcSpec)
        L.orc_norminv.restype = C.c_double
        L.orc_norminv.argtypes = [C.c_double]
        L.orc_calc_n.restype = C.c_double
        L.orc_calc_n.argtypes = [dp, C.c_double]
        L.orc_qrng_points.argtypes = [C.c_double, C.c_size_t, dp]
        L.orc_gpu_points.argtypes = [C.c_double, C.c_uint64, C.c_size_t, dp]
        L.orc_position_detector.argtypes = [sp, C.c_double, dp, C.POINTER(C.c_int32)]
        L.orc_propagate.argtypes = [sp, C.c_double, C.c_double, up, dp]
        L.orc_design_dump.argtypes = [sp, dp]
        L.orc_propagation_path.argtypes = [sp, C.c_double, C.c_double, dp]
        L.orc_stop_face.argtypes = [sp, C.c_double, C.c_double, C.POINTER(C.c_int)]
        L.orc_fitness_adaptive.argtypes = [sp, C.c_size_t, C.c_size_t, dp]
        L.orc_fitness_adaptive_work.argtypes = [sp, C.c_size_t, C.c_size_t, dp, C.POINTER(C.c_uint64),
                                                C.POINTER(C.c_uint64)]
        L.orc_p_dets_l_wavelength.argtypes = [sp, C.c_double, C.c_size_t, dp]
        L.orc_p_dets_l_wavelength_count.argtypes = [sp, C.c_double, C.c_size_t, dp, C.POINTER(C.c_uint64)]
        L.orc_fitness_points.argtypes = [sp, dp, C.c_size_t, dp, C.c_size_t, C.c_int, dp, dp,
                                         C.POINTER(C.c_uint64)]
        L.orc_fitness_adaptive_points.argtypes = [sp, dp, C.c_size_t, dp, C.c_size_t, C.c_int, dp, dp,
                                                  C.POINTER(C.c_uint64), up]
        L.orc_trace_pairs.argtypes = [sp, dp, dp, C.c_size_t, up, dp]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def make_spec(d: dict) -> OrcSpec:
    """Fill an OrcSpec from the flat parameter dict used across the tests."""
    s = OrcSpec()
    G = len(d["glasses"])
    s.nglass = G
    s.ar_coated = int(bool(d["ar_coated"]))
    for g, coeffs in enumerate(d["glasses"]):
        for i, c in enumerate(coeffs):
            s.glass[g][i] = float(c)
    for i, a in enumerate(d["angles"]):
        s.angles[i] = float(a)
    for i, l in enumerate(d["lengths"]):
        s.lengths[i] = float(l)
    s.curvature = float(d["curvature"])
    s.height = float(d["height"])
    s.width = float(d["width"])
    s.bin_count = int(d["bin_count"])
    s.det_flipped = int(bool(d.get("det_flipped", False)))
    s.bin_size = float(d["bin_size"])
    s.linear_slope = float(d["linear_slope"])
    s.linear_intercept = float(d["linear_intercept"])
    s.det_length = float(d["det_length"])
    s.max_incident_angle = float(d["max_incident_angle"])
    s.det_angle = float(d["det_angle"])
    pos = d.get("det_position", (0.0, 0.0))
    s.det_position[0] = float(pos[0])
    s.det_position[1] = float(pos[1])
    s.wmin, s.wmax = (float(x) for x in d["wavelength_bounds"])
    s.beam_width = float(d["beam_width"])
    s.beam_y_mean = float(d["beam_y_mean"])
    return s


def norminv(x: float) -> float:
    return lib().orc_norminv(float(x))


def qrng_points(seed: float, n: int) -> np.ndarray:
    out = np.empty(n, dtype=np.float64)
    lib().orc_qrng_points(float(seed), n, _dp(out))
    return out


def gpu_points(seed: float, n: int, first: int = 0) -> np.ndarray:
    """The GPU seed policy's points u_i = fract(fma(first + i, 1/phi, seed))."""
    out = np.empty(n, dtype=np.float64)
    lib().orc_gpu_points(float(seed), int(first), n, _dp(out))
    return out


def accept_params(d: dict):
    """A drawn design positioned by the oracle (acceptance 1.0), or None when it raises
    RayTraceError or its tables are not finite: the same decision the library's builder
    takes, so a seeded draw sequence gives the same designs on both sides."""
    e, pos, fl = position_detector(d, 1.0)
    if e != OK:
        return None
    dd = dict(d, det_position=pos, det_flipped=fl)
    s = make_spec(dd)
    out = np.zeros(4 * len(dd["glasses"]) + 6 + 5 + 2)
    if lib().orc_design_dump(C.byref(s), _dp(out)) != OK or not np.isfinite(out).all():
        return None
    return dd


def position_detector(d: dict, acceptance: float = 1.0):
    s = make_spec(d)
    pos = np.zeros(2)
    fl = C.c_int32(0)
    e = lib().orc_position_detector(C.byref(s), float(acceptance), _dp(pos), C.byref(fl))
    return e, (float(pos[0]), float(pos[1])), bool(fl.value)


def design_dump(d: dict) -> np.ndarray:
    s = make_spec(d)
    G = len(d["glasses"])
    out = np.zeros(4 * G + 6 + 5 + 2)
    e = lib().orc_design_dump(C.byref(s), _dp(out))
    assert e == OK, e
    return out


def propagate(d: dict, wavelength: float, ray_u: float):
    s = make_spec(d)
    b = C.c_uint32(0)
    t = C.c_double(0.0)
    e = lib().orc_propagate(C.byref(s), float(wavelength), float(ray_u), C.byref(b), C.byref(t))
    return e, b.value, t.value


def propagation_path(d: dict, wavelength: float, initial_y: float) -> np.ndarray:
    s = make_spec(d)
    G = len(d["glasses"])
    rows = np.zeros((G + 3, 4))
    n = lib().orc_propagation_path(C.byref(s), float(wavelength), float(initial_y), _dp(rows))
    return rows[: max(n, 0)]


def stop_face(d: dict, wavelength: float, initial_y: float):
    """(face, status): where the prism trace of this wavelength and start height stops
    (0..G-1 the flat faces, G the curved exit face, -1 none) and the error it stops with."""
    s = make_spec(d)
    st = C.c_int(0)
    k = lib().orc_stop_face(C.byref(s), float(wavelength), float(initial_y), C.byref(st))
    assert k >= -1, k
    return k, st.value


def fitness_adaptive(d: dict, max_n: int = 16384, max_m: int = 16384):
    s = make_spec(d)
    out = np.zeros(3)
    e = lib().orc_fitness_adaptive(C.byref(s), max_n, max_m, _dp(out))
    assert e == OK, e
    return float(out[0]), float(out[1]), float(out[2])


def fitness_adaptive_work(d: dict, max_n: int = 16384, max_m: int = 16384):
    """(size, info, deviation, wavelengths used, rays traced) of the reference CPU fitness."""
    s = make_spec(d)
    out = np.zeros(3)
    nw, nr = C.c_uint64(0), C.c_uint64(0)
    e = lib().orc_fitness_adaptive_work(C.byref(s), max_n, max_m, _dp(out), C.byref(nw), C.byref(nr))
    assert e == OK, e
    return float(out[0]), float(out[1]), float(out[2]), int(nw.value), int(nr.value)


def p_dets_l_wavelength(d: dict, wavelength: float, max_m: int = 16384) -> np.ndarray:
    s = make_spec(d)
    out = np.zeros(int(d["bin_count"]))
    e = lib().orc_p_dets_l_wavelength(C.byref(s), float(wavelength), max_m, _dp(out))
    assert e == OK, e
    return out


def p_dets_l_wavelength_count(d: dict, wavelength: float, max_m: int = 16384):
    """(p(d|lambda)[B], rays consumed) of the reference's adaptive per-bin estimator."""
    s = make_spec(d)
    out = np.zeros(int(d["bin_count"]))
    n = C.c_uint64(0)
    e = lib().orc_p_dets_l_wavelength_count(C.byref(s), float(wavelength), max_m, _dp(out), C.byref(n))
    assert e == OK, e
    return out, int(n.value)


def fitness_points(d: dict, lam_u, ray_u, nthreads: int = 1, want_p: bool = True):
    """Fixed-N estimator on explicit points. Returns (p[W,B] or None, stats dict)."""
    s = make_spec(d)
    lam_u = np.ascontiguousarray(lam_u, dtype=np.float64)
    ray_u = np.ascontiguousarray(ray_u, dtype=np.float64)
    W, R, B = lam_u.size, ray_u.size, int(d["bin_count"])
    p = np.zeros((W, B)) if want_p else None
    st = np.zeros(4)
    hits = C.c_uint64(0)
    e = lib().orc_fitness_points(C.byref(s), _dp(lam_u), W, _dp(ray_u), R, int(nthreads),
                                 _dp(p) if p is not None else None, _dp(st), C.byref(hits))
    assert e == OK, e
    return p, {"info": float(st[0]), "h_cond": float(st[1]), "h_det": float(st[2]),
               "size": float(st[3]), "hits": int(hits.value)}


def fitness_adaptive_points(d: dict, lam_u, ray_u, nthreads: int = 1):
    """Adaptive sampling on explicit points (rays in the given order, 32 per round).
    Returns (p[W,B], stats dict, counts[W] = rays consumed per wavelength)."""
    s = make_spec(d)
    lam_u = np.ascontiguousarray(lam_u, dtype=np.float64)
    ray_u = np.ascontiguousarray(ray_u, dtype=np.float64)
    W, R, B = lam_u.size, ray_u.size, int(d["bin_count"])
    p = np.zeros((W, B))
    st = np.zeros(4)
    hits = C.c_uint64(0)
    counts = np.zeros(W, dtype=np.uint32)
    e = lib().orc_fitness_adaptive_points(C.byref(s), _dp(lam_u), W, _dp(ray_u), R, int(nthreads), _dp(p),
                                          _dp(st), C.byref(hits), counts.ctypes.data_as(C.POINTER(C.c_uint32)))
    assert e == OK, e
    return p, {"info": float(st[0]), "h_cond": float(st[1]), "h_det": float(st[2]),
               "size": float(st[3]), "hits": int(hits.value)}, counts


def trace_pairs(d: dict, lam_u, ray_u):
    s = make_spec(d)
    lam_u = np.ascontiguousarray(lam_u, dtype=np.float64)
    ray_u = np.ascontiguousarray(ray_u, dtype=np.float64)
    n = lam_u.size
    bins = np.zeros(n, dtype=np.uint32)
    ts = np.zeros(n)
    e = lib().orc_trace_pairs(C.byref(s), _dp(lam_u), _dp(ray_u), n,
                              bins.ctypes.data_as(C.POINTER(C.c_uint32)), _dp(ts))
    assert e == OK, e
    return bins, ts


OP_KINDS = ("add", "mul", "fma", "div", "sqrt", "cmp", "log", "trig", "other")


def ops_trace(d: dict, lam_u, ray_u):
    """The op-counting build of the model (ops_count.cpp) over W x R rays: totals per
    operation kind for the per-ray work, the per-wavelength work the reference repeats per
    ray (calc_n), the rays that reached a bin, and the R start heights; plus the hits."""
    build()
    L = C.CDLL(OPS_LIB_PATH)
    u64 = C.POINTER(C.c_uint64)
    L.orc_ops_trace.argtypes = [C.POINTER(OrcSpec), C.POINTER(C.c_double), C.c_size_t, C.POINTER(C.c_double),
                                C.c_size_t, u64, u64, u64, u64, u64]
    assert L.orc_ops_kinds() == len(OP_KINDS)
    s = make_spec(d)
    lam_u = np.ascontiguousarray(lam_u, dtype=np.float64)
    ray_u = np.ascontiguousarray(ray_u, dtype=np.float64)
    bufs = [np.zeros(len(OP_KINDS), dtype=np.uint64) for _ in range(4)]
    hits = C.c_uint64(0)
    e = L.orc_ops_trace(C.byref(s), _dp(lam_u), lam_u.size, _dp(ray_u), ray_u.size,
                        *[b.ctypes.data_as(u64) for b in bufs], C.byref(hits))
    assert e == OK, e
    names = ("ray", "lambda", "hit_ray", "beam")
    return {n: dict(zip(OP_KINDS, (int(v) for v in b))) for n, b in zip(names, bufs)}, int(hits.value)


class OrcSpec3(C.Structure):
    _fields_ = [("base", OrcSpec), ("curv0", C.c_double * 2), ("curv1", C.c_double * 2),
                ("fiber_radius", C.c_double), ("fiber_na", C.c_double), ("fiber_center_y", C.c_double)]


def make_spec3(d: dict) -> OrcSpec3:
    """The 3-D spectrometer: the flat dict of make_spec plus curv0 / curv1 (poloidal, toroidal)
    and fiber_radius / fiber_na / fiber_center_y."""
    s = OrcSpec3()
    base = dict(d)
    base.setdefault("curvature", 0.0)
    base.setdefault("beam_width", 0.0)
    base.setdefault("beam_y_mean", d["fiber_center_y"])
    s.base = make_spec(base)
    s.curv0[0], s.curv0[1] = (float(v) for v in d["curv0"])
    s.curv1[0], s.curv1[1] = (float(v) for v in d["curv1"])
    s.fiber_radius = float(d["fiber_radius"])
    s.fiber_na = float(d["fiber_na"])
    s.fiber_center_y = float(d["fiber_center_y"])
    return s


def _lib3():
    L = lib()
    if not getattr(L, "_orc3", False):
        sp3 = C.POINTER(OrcSpec3)
        dp = C.POINTER(C.c_double)
        up = C.POINTER(C.c_uint32)
        L.orc_approx_cbrt.restype = C.c_double
        L.orc_approx_cbrt.argtypes = [C.c_double]
        L.orc_toric_roots.argtypes = [C.c_double] * 6 + [dp]
        L.orc3_qrng_points.argtypes = [C.c_double, C.c_size_t, dp]
        L.orc3_position_detector.argtypes = [sp3, C.c_double, dp, C.POINTER(C.c_int32)]
        L.orc3_trace_pairs.argtypes = [sp3, dp, dp, C.c_size_t, up, dp, C.POINTER(C.c_int32), up, up]
        L.orc3_fitness_points.argtypes = [sp3, dp, C.c_size_t, dp, C.c_size_t, dp, dp, C.POINTER(C.c_uint64)]
        L._orc3 = True
    return L


def approx_cbrt(x: float) -> float:
    return _lib3().orc_approx_cbrt(float(x))


def toric_roots(r_2, R_2, dp_magn_sq, dp_v, dp_n, n_v) -> np.ndarray:
    out = np.zeros(4)
    _lib3().orc_toric_roots(r_2, R_2, dp_magn_sq, dp_v, dp_n, n_v, _dp(out))
    return out


def qrng3_points(seed: float, n: int) -> np.ndarray:
    out = np.zeros((n, 4))
    _lib3().orc3_qrng_points(float(seed), n, _dp(out))
    return out


def position_detector3(d: dict, acceptance: float = 1.0):
    s = make_spec3(d)
    pos = np.zeros(2)
    fl = C.c_int32(0)
    e = _lib3().orc3_position_detector(C.byref(s), float(acceptance), _dp(pos), C.byref(fl))
    return e, (float(pos[0]), float(pos[1])), bool(fl.value)


def trace_pairs3(d: dict, lam_u, q):
    """(bins, ts, status, nan_roots, toric_calls) per (lam_u[i], q[i]) ray."""
    s = make_spec3(d)
    lam_u = np.ascontiguousarray(lam_u, dtype=np.float64)
    q = np.ascontiguousarray(q, dtype=np.float64).reshape(-1, 4)
    n = lam_u.size
    bins = np.zeros(n, dtype=np.uint32)
    ts = np.zeros(n)
    st = np.zeros(n, dtype=np.int32)
    nan = np.zeros(n, dtype=np.uint32)
    calls = np.zeros(n, dtype=np.uint32)
    u32 = C.POINTER(C.c_uint32)
    e = _lib3().orc3_trace_pairs(C.byref(s), _dp(lam_u), _dp(q), n, bins.ctypes.data_as(u32), _dp(ts),
                                 st.ctypes.data_as(C.POINTER(C.c_int32)), nan.ctypes.data_as(u32),
                                 calls.ctypes.data_as(u32))
    assert e == OK, e
    return bins, ts, st, nan, calls


def fitness_points3(d: dict, lam_u, q):
    s = make_spec3(d)
    lam_u = np.ascontiguousarray(lam_u, dtype=np.float64)
    q = np.ascontiguousarray(q, dtype=np.float64).reshape(-1, 4)
    W, R, B = lam_u.size, q.shape[0], int(d["bin_count"])
    p = np.zeros((W, B))
    st = np.zeros(4)
    hits = C.c_uint64(0)
    e = _lib3().orc3_fitness_points(C.byref(s), _dp(lam_u), W, _dp(q), R, _dp(p), _dp(st), C.byref(hits))
    assert e == OK, e
    return p, {"info": float(st[0]), "h_cond": float(st[1]), "h_det": float(st[2]), "size": float(st[3]),
               "hits": int(hits.value)}
