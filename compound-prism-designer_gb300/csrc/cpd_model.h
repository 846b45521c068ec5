// cpd_model.h -- the spectrometer model shared by host C++ and device CUDA code.
//
// Three layers:
//  * Exact f64 model (namespace cpd::x): the reference's per-ray trace
//    (src/spectrometer/ray.rs:309-499, geometry.rs:124-216, spectrometer.rs:265-303)
//    with every rounding step made explicit. On the device the arithmetic uses
//    the _rn intrinsics (no contraction); on the host this header is compiled with
//    -ffp-contract=off. Both therefore give the reference's own f64 results bit
//    for bit, given the same tables. Transcendentals (log in the inverse normal
//    CDF, sin/cos in design construction) are evaluated on the host only.
//  * Per-wavelength setup (lambda_setup): all rays of one wavelength leave the
//    Gaussian beam with direction (1,0) (Ray::new_from_start, ray.rs:277-279), and
//    every face before the curved exit face is flat, so the direction and the s/p
//    transmittances after each flat face are the same for every ray of that
//    wavelength (the same f64 operations on the same operands). Positions on the
//    flat faces are affine in the start height y, so the set of rays that clears
//    every flat face is an interval of y, and, with the ray table sorted by
//    z = norminv(u), a contiguous range of ray indices.
//  * FP32 fast path (fast_ray): per ray, only the exit face and the detector,
//    with a guard margin on every decision; a ray inside any guard band is
//    reported FLAG and re-traced with the exact model.
#pragma once

#include <cstdint>
#include <cmath>
#include <cstring>

#include "../../include/cpd.h"

#if defined(__CUDACC__)
#define CPD_HD __host__ __device__ __forceinline__
#define CPD_HDN __host__ __device__
#else
#define CPD_HD inline
#define CPD_HDN
#endif

namespace cpd {

// 1/phi, the 1-D R1 sequence step (qrng.rs:156-158, kernel.rs:107-108).
constexpr double kAlpha = 1.0 / 1.61803398874989484820458683436563;
// Fixed-point scale of a ray's transmittance t in [0, 1]: one u32 per ray (2^31 t,
// truncated), summed into u64 per (wavelength, bin) cell and per bin over wavelengths.
// The sums are integers, so they do not depend on the order rays are accumulated in.
// A cell holds at most R 2^31 <= 2^53; a per-bin sum over W rows at most W R 2^31,
// which stays below 2^63 while W R <= 2^32 (checked on the host).
constexpr double kTScale = 2147483648.0;             // 2^31
constexpr double kTScaleInv = 1.0 / 2147483648.0;
// Fixed-point scales of the per-design accumulators of p^2 and -p log2 p.
constexpr double kPScale = 70368744177664.0;         // 2^46, sum over wavelengths of p^2
constexpr double kPScaleInv = 1.0 / 70368744177664.0;
constexpr double kHScale = 1099511627776.0;          // 2^40, sum of -p log2 p
constexpr double kHScaleInv = 1.0 / 1099511627776.0;

// 2^31 t for t in [0, 1], rounded to nearest (ties up), with integer operations only
// (no conversion instruction): t = 1.m x 2^(e-127) so 2^31 t = (1.m 2^23) x 2^(e-119).
CPD_HD uint32_t t_fixed(float t)
{
#if defined(__CUDA_ARCH__)
    const uint32_t b = __float_as_uint(t);
#else
    uint32_t b;
    std::memcpy(&b, &t, 4);
#endif
    const int e = (int)(b >> 23) - 119;
    const uint32_t m = (b & 0x7fffffu) | 0x800000u;
    if (e >= 0) return m << (e > 8 ? 8 : e);
    return e > -25 ? (m + (1u << (-e - 1))) >> (-e) : 0u;
}

// The same quantization of an f64 transmittance (exact re-trace path).
CPD_HD uint32_t t_fixed64(double t) { return (uint32_t)(t * kTScale + 0.5); }

// Outcome of a ray.
enum : int { RAY_LOST = 0, RAY_HIT = 1, RAY_FLAG = 2 };

// ----------------------------------------------------------------- device tables

// FP32 constants of the fast path (per design).
struct alignas(16) FastConst {
    float inv_rc;      // 1 / exit-face radius
    float rho;         // exit-face bound radius
    float rho2;        // bound radius^2
    float dnfx, dnfy, dufx, dufy;  // detector normal and direction
    float min_ci, L, c0, slope, inv_slope, bin_size;
    float bw;          // beam width
    int32_t ar;
    uint32_t B;
};

// Per design, on the device: the exact f64 tables plus the FP32 constants.
struct alignas(16) DevDesign {
    int32_t G;
    uint32_t B;
    int32_t ar;
    int32_t pad0;
    double glass[CPD_MAX_GLASS][6];
    double ppx[CPD_MAX_GLASS], ppy[CPD_MAX_GLASS], pnx[CPD_MAX_GLASS], pny[CPD_MAX_GLASS];
    double height;
    double ccx, ccy, crad, cbx, cby, cbr2;
    double bin_size, slope, intercept, min_ci, L;
    double dnx, dny, dpx, dpy, dux, duy;
    double wmin, wmax, bw, bym;
    FastConst fc;
};

// Per (design, wavelength), written by lambda_setup. The FP32 fast path works in
// differences from one reference ray of the wavelength, traced in f64 through the
// exit face and onto the detector: every per-ray quantity is the reference value
// plus a difference computed with a cancellation-free identity, so the FP32 error
// scales with the (small) difference, not with the absolute coordinates or the
// distance to the detector.
struct alignas(16) LamParams {
    float zref_hi, zref_lo;     // z of the reference ray (f32 hi + lo parts)
    float w1x, w1y;             // d(position on the last flat face)/dy
    float dx, dy;               // direction entering the exit face (same for every ray)
    float ts, tp;               // s/p transmittance entering the exit face
    float dlx2, dly2;           // 2 (w_ref - c): ray point on the last face relative to the centre
    float ud2, disc, sd;        // reference: 2 d.(w - c), discriminant, its square root
    float sigma;                // root sign: s = -ud + sigma*sd
    float s, px2, py2, mb;      // reference root, 2 p_ref (rel. bound centre), |p|^2 - rho^2
    float nx, ny;               // reference exit-face normal (c - p)/Rc
    float ci, ci2, crsq, cr;    // reference cosines (ci2 = 2 ci)
    float r, r2, kk;            // n_last, n_last^2, r ci - cr
    float cid, gn, T, du, pos;  // reference detector cosine, (p - P).N, gn/cid, d'.u, position
    uint32_t core_lo, core_hi;  // sorted-ray range that clears every flat face (fast path)
    uint32_t band_lo, band_hi;  // [band_lo, core_lo) and [core_hi, band_hi): guard bands
    uint32_t all_exact;         // no usable reference ray: every core ray is re-traced exactly
    uint32_t pad[3];
};

// Exact per-face data of one wavelength, written by lambda_setup for the re-trace. The
// sequential f64 trace computes these from the same operands for every ray of the
// wavelength, so they are the values it would compute for any one ray.
struct ExactLam {
    double dx[CPD_MAX_GLASS], dy[CPD_MAX_GLASS];  // direction after face k
    double ci[CPD_MAX_GLASS];                     // dot(direction entering face k, N_k)
    double cr[CPD_MAX_GLASS];                     // refraction cosine at face k
    double n[CPD_MAX_GLASS];                      // index of glass k
    double ts, tp;                                // s/p transmittance after the last flat face
};

// ----------------------------------------------------------------- exact f64 ops

namespace x {
CPD_HD double add(double a, double b)
{
#if defined(__CUDA_ARCH__)
    return __dadd_rn(a, b);
#else
    return a + b;
#endif
}
CPD_HD double sub(double a, double b)
{
#if defined(__CUDA_ARCH__)
    return __dsub_rn(a, b);
#else
    return a - b;
#endif
}
CPD_HD double mul(double a, double b)
{
#if defined(__CUDA_ARCH__)
    return __dmul_rn(a, b);
#else
    return a * b;
#endif
}
CPD_HD double div(double a, double b)
{
#if defined(__CUDA_ARCH__)
    return __ddiv_rn(a, b);
#else
    return a / b;
#endif
}
CPD_HD double sqrt_(double a)
{
#if defined(__CUDA_ARCH__)
    return __dsqrt_rn(a);
#else
    return std::sqrt(a);
#endif
}
CPD_HD double fma_(double a, double b, double c)
{
#if defined(__CUDA_ARCH__)
    return __fma_rn(a, b, c);
#else
    return std::fma(a, b, c);
#endif
}
CPD_HD double sqr(double a) { return mul(a, a); }

// f64 reciprocal and square root to ~2^-44 relative, for quantities that only seed the
// FP32 fast path or sit inside a guard band (never for a value the exact trace
// reproduces): an FP32 hardware estimate refined by one Newton-Raphson step in f64
// (y' = y + y(1 - xy); g' = g + (x - g^2) y/2 with y ~ 1/sqrt x). Outside the FP32
// range they fall back to the IEEE operations. On the host both are the IEEE ones.
CPD_HD double rcp_approx(double a)
{
#if defined(__CUDA_ARCH__)
    const double m = fabs(a);
    if (!(m > 1e-30 && m < 1e30)) return __ddiv_rn(1.0, a);
    float s;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(s) : "f"((float)a));
    const double y = (double)s;
    return fma(y, fma(-a, y, 1.0), y);
#else
    return 1.0 / a;
#endif
}
CPD_HD double sqrt_approx(double a)
{
#if defined(__CUDA_ARCH__)
    if (!(a > 1e-30 && a < 1e30)) return __dsqrt_rn(a);
    float s;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(s) : "f"((float)a));
    const double y = (double)s;
    const double g = a * y;
    return fma(0.5 * y, fma(-g, g, a), g);
#else
    return std::sqrt(a);
#endif
}

CPD_HD double trunc_(double a)
{
#if defined(__CUDA_ARCH__)
    return ::trunc(a);
#else
    return std::trunc(a);
#endif
}
CPD_HD bool sign_positive(double a)
{
#if defined(__CUDA_ARCH__)
    return !signbit(a);
#else
    return !std::signbit(a);
#endif
}

// Horner with fused multiply-add from the highest-degree coefficient
// (Glass::calc_n, glasscat.rs:17-22).
CPD_HD double calc_n(const double *c, double w)
{
    double s = c[0];
#pragma unroll
    for (int i = 1; i < 6; i++) s = fma_(s, w, c[i]);
    return s;
}

// UniformDistribution::inverse_cdf (distribution.rs:32-34).
CPD_HD double wavelength(const DevDesign &D, double u) { return add(D.wmin, mul(sub(D.wmax, D.wmin), u)); }

// GaussianBeam 2-D inverse_cdf (spectrometer.rs:26-30) given z = norminv(u).
CPD_HD double beam_y(const DevDesign &D, double z) { return sub(D.bym, mul(D.bw, z)); }

struct Ray {
    double ox, oy, dx, dy, ts, tp;
};

CPD_HD double dot(double ax, double ay, double bx, double by) { return add(mul(ax, bx), mul(ay, by)); }

// Ray::refract (ray.rs:309-367). Returns false on total internal reflection.
CPD_HD bool refract(Ray &r, double nx, double ny, double n1, double n2, bool ar)
{
    double ci = -dot(r.dx, r.dy, nx, ny);
    double rr = n2 == 1.0 ? n1 : div(n1, n2);  // x / 1 == x in IEEE arithmetic: no division for air
    double cr_sq = sub(1.0, mul(sqr(rr), sub(1.0, sqr(ci))));
    if (cr_sq < 0.0) return false;
    double cr = sqrt_(cr_sq);
    double k = sub(mul(rr, ci), cr);
    double vx = add(mul(r.dx, rr), mul(nx, k));
    double vy = add(mul(r.dy, rr), mul(ny, k));
    if (ar && ci > 0.5) {
        r.ts = mul(r.ts, 0.99);
        r.tp = mul(r.tp, 0.99);
    } else {
        double a = mul(n1, ci), b = mul(n2, cr);
        double rs = sqr(div(sub(a, b), add(a, b)));
        double c = mul(n1, cr), e = mul(n2, ci);
        double rp = sqr(div(sub(c, e), add(c, e)));
        r.ts = mul(r.ts, sub(1.0, rs));
        r.tp = mul(r.tp, sub(1.0, rp));
    }
    r.dx = vx;
    r.dy = vy;
    return true;
}

// Error codes of the exact trace: 0 or a CPD_RAYTRACE_* status.
constexpr int kNoHit = CPD_RAYTRACE_NO_SURFACE_INTERSECTION;
constexpr int kTIR = CPD_RAYTRACE_TOTAL_INTERNAL_REFLECTION;
constexpr int kWeak = CPD_RAYTRACE_ANGULAR_RESPONSE_TOO_WEAK;

// Flat face k: HyperPlane::intersection with PrismBounds (geometry.rs:124-145, 62-67),
// translate (ray.rs:281-294), refract. On error the ray is left unchanged.
CPD_HD int flat_face(const DevDesign &D, int k, Ray &r, double n1, double n2)
{
    double nx = D.pnx[k], ny = D.pny[k];
    double ci = dot(r.dx, r.dy, nx, ny);
    if (ci == 0.0) return kNoHit;
    double d = div(dot(sub(D.ppx[k], r.ox), sub(D.ppy[k], r.oy), nx, ny), ci);
    if (!(d >= 0.0)) return kNoHit;
    double hy = fma_(r.dy, d, r.oy);
    if (!(0.0 <= hy && hy <= D.height)) return kNoHit;
    Ray n = r;
    n.ox = fma_(r.dx, d, r.ox);
    n.oy = hy;
    if (!refract(n, nx, ny, n1, n2, D.ar != 0)) return kTIR;
    r = n;
    return 0;
}

CPD_HD bool in_bound(const DevDesign &D, double px, double py)
{
    double ex = sub(px, D.cbx), ey = sub(py, D.cby);
    return dot(ex, ey, ex, ey) <= D.cbr2;
}

// Curved exit face: SphericalLikeSurface::intersection + RadialBounds
// (geometry.rs:161-216, 85-91), translate, refract into air. On error the ray is
// left unchanged.
CPD_HD int exit_face(const DevDesign &D, Ray &r, double n1)
{
    double deltax = sub(r.ox, D.ccx), deltay = sub(r.oy, D.ccy);
    double ud = dot(r.dx, r.dy, deltax, deltay);
    double disc = add(sub(sqr(ud), dot(deltax, deltay, deltax, deltay)), sqr(D.crad));
    if (!(disc > 0.0)) return kNoHit;
    double sd = sqrt_(disc);
    double d1 = sub(-ud, sd), d2 = add(-ud, sd);
    double p1x = fma_(r.dx, d1, r.ox), p1y = fma_(r.dy, d1, r.oy);
    double px, py;
    if (sign_positive(d1) && in_bound(D, p1x, p1y)) {
        px = p1x;
        py = p1y;
    } else {
        double p2x = fma_(r.dx, d2, r.ox), p2y = fma_(r.dy, d2, r.oy);
        if (sign_positive(d2) && in_bound(D, p2x, p2y)) {
            px = p2x;
            py = p2y;
        } else {
            return kNoHit;
        }
    }
    double nx = div(sub(D.ccx, px), D.crad), ny = div(sub(D.ccy, py), D.crad);
    Ray n = r;
    n.ox = px;
    n.oy = py;
    if (!refract(n, nx, ny, n1, 1.0, D.ar != 0)) return kTIR;
    r = n;
    return 0;
}

// Detector: Ray::intersect_detector_array + LinearDetectorArray::{intersection,
// bin_index} (ray.rs:390-402, spectrometer.rs:265-303), euclid_div_rem and the
// saturating f64->u32 cast (utils.rs:177-192).
CPD_HD int detector(const DevDesign &D, const Ray &r, uint32_t &bin, double &t, double *hx = nullptr,
                    double *hy = nullptr)
{
    double ci = -dot(r.dx, r.dy, D.dnx, D.dny);
    if (ci <= D.min_ci) return kWeak;
    double d = div(dot(sub(r.ox, D.dpx), sub(r.oy, D.dpy), D.dnx, D.dny), ci);
    double px = fma_(r.dx, d, r.ox), py = fma_(r.dy, d, r.oy);
    if (hx) {
        *hx = px;
        *hy = py;
    }
    double pos = dot(sub(px, D.dpx), sub(py, D.dpy), D.dux, D.duy);
    if (pos < 0.0 || D.L < pos) return kNoHit;
    double a = sub(pos, D.intercept);
    double q = trunc_(div(a, D.slope));
    double rem = sub(a, mul(q, D.slope));
    if (rem < 0.0) {
        q = D.slope > 0.0 ? sub(q, 1.0) : add(q, 1.0);
        rem = add(rem, D.slope < 0.0 ? -D.slope : D.slope);
    }
    uint32_t b;
    if (!(q == q) || q <= 0.0) b = 0;
    else if (q >= 4294967295.0) b = 4294967295u;
    else b = (uint32_t)q;
    if (b < D.B && rem < D.bin_size) {
        bin = b;
        t = mul(add(r.ts, r.tp), 0.5);
        return 0;
    }
    return kNoHit;
}

// CompoundPrism::propagate (ray.rs:485-499). `faces` counts the faces the ray
// passed (for the propagation path); returns 0 or the first error.
CPD_HD int prism(const DevDesign &D, double lambda, Ray &r, int *faces = nullptr)
{
    double n1 = calc_n(D.glass[0], lambda);
    int e = flat_face(D, 0, r, 1.0, n1);
    if (e) return e;
    if (faces) *faces = 1;
    for (int k = 1; k < D.G; k++) {
        double n2 = calc_n(D.glass[k], lambda);
        e = flat_face(D, k, r, n1, n2);
        if (e) return e;
        if (faces) *faces = k + 1;
        n1 = n2;
    }
    e = exit_face(D, r, n1);
    if (!e && faces) *faces = D.G + 1;
    return e;
}

// Spectrometer::propagate (spectrometer.rs:421-427): exact f64 trace of one ray.
// Returns 0 (hit: bin, t) or the RayTraceError code.
CPD_HD int trace(const DevDesign &D, double lambda, double y, uint32_t &bin, double &t)
{
    Ray r{0.0, y, 1.0, 0.0, 1.0, 1.0};
    int e = prism(D, lambda, r);
    if (e) return e;
    return detector(D, r, bin, t);
}

// The same exact trace with the wavelength's flat-face directions, cosines and glass
// indices taken from E (written by lambda_setup): every operation whose operands differ
// between rays -- the face intersections, the transmittance products, the exit face and
// the detector -- is still done with the reference's operations, so the result is
// bit-identical to trace(). The wavelength's flat faces do not reflect totally (else
// lambda_setup drops it).
template <int G>
CPD_HD int trace_lam_g(const DevDesign &D, const ExactLam &E, double y, uint32_t &bin, double &t)
{
    Ray r{0.0, y, 1.0, 0.0, 1.0, 1.0};
    double n1 = 1.0;
    _Pragma("unroll") for (int k = 0; k < G; k++) {
        const double nx = D.pnx[k], ny = D.pny[k];
        const double ci = E.ci[k];
        if (ci == 0.0) return kNoHit;
        const double d = div(dot(sub(D.ppx[k], r.ox), sub(D.ppy[k], r.oy), nx, ny), ci);
        if (!(d >= 0.0)) return kNoHit;
        const double hy = fma_(r.dy, d, r.oy);
        if (!(0.0 <= hy && hy <= D.height)) return kNoHit;
        r.ox = fma_(r.dx, d, r.ox);
        r.oy = hy;
        // Ray::refract (ray.rs:309-367) with the wavelength's direction and cosines; the
        // transmittance products are the wavelength's too (E.ts, E.tp)
        r.dx = E.dx[k];
        r.dy = E.dy[k];
        n1 = E.n[k];
    }
    r.ts = E.ts;
    r.tp = E.tp;
    const int e = exit_face(D, r, n1);
    if (e) return e;
    return detector(D, r, bin, t);
}
CPD_HD int trace_lam(const DevDesign &D, const ExactLam &E, double y, uint32_t &bin, double &t)
{
    switch (D.G) {
    case 1: return trace_lam_g<1>(D, E, y, bin, t);
    case 2: return trace_lam_g<2>(D, E, y, bin, t);
    case 3: return trace_lam_g<3>(D, E, y, bin, t);
    case 4: return trace_lam_g<4>(D, E, y, bin, t);
    case 5: return trace_lam_g<5>(D, E, y, bin, t);
    default: return trace_lam_g<6>(D, E, y, bin, t);
    }
}
}  // namespace x

// ----------------------------------------------------------------- per-wavelength setup

// Guard widths of the fast path. A decision whose FP32 margin is inside its guard
// is not trusted: the ray is re-traced with the exact model. The widths are
// upper bounds on the FP32 error of each margin measured over random designs,
// times a safety factor ("guard bands").
struct Guards {
    float pos;      // mm, detector coordinate vs 0, L and every bin edge
    float cosine;   // exit-face cr^2, AR threshold 0.5, detector min_ci
    float dist;     // mm, exit-face root sign
    float rel;      // relative: discriminant, radial bound
    float pos_rel;  // detector coordinate, relative to the terms it is summed from
};
// Measured over 40 random designs x 131k rays (host emulation of this code against
// the exact trace): no wrong decision at 0.1x these widths, the first at 0.03x.
// pos_rel (2^-20, 16 FP32 ulps of the largest term) covers designs whose reference
// ray lands far (metres) from the detector, where the absolute 1e-4 mm is below one
// ulp of the summed terms.
CPD_HD Guards default_guards() { return Guards{1.0e-4f, 1.0e-5f, 1.0e-4f, 1.0e-5f, 9.5367431640625e-07f}; }
// The FP32-only study mode: no guard band, nothing flagged.
CPD_HD Guards no_guards() { return Guards{0.f, 0.f, 0.f, 0.f, 0.f}; }

// Relative guard of the y-interval ends: both sides are f64, so a few ulps suffice.
constexpr double kYGuardRel = 1e-11;

// Splits an f64 into f32 hi + lo parts (hi + lo == v to about 2^-48 relative).
CPD_HD void split_f32(double v, float &hi, float &lo)
{
    hi = (float)v;
    lo = (float)(v - (double)hi);
}

// Traces candidate reference rays of the core range in f64 through the exit face and
// onto the detector line, and stores the first one for which every quantity the fast
// path differentiates is defined: a secant exit intersection inside the bound, no total
// internal reflection and a detector cosine above 0.05. (ax, ay) + (bx, by)*y is the
// position on the last flat face, (dx, dy) the direction entering the exit face,
// r the index of the last glass. Returns false if no candidate qualifies.
CPD_HDN inline bool reference_ray(const DevDesign &D, const double *zs, LamParams &P, double ax, double ay,
                                  double bx, double by, double dx, double dy, double r)
{
    const uint32_t lo = P.core_lo, n = P.core_hi - P.core_lo;
    const double vx = D.cbx - D.ccx, vy = D.cby - D.ccy;  // bound centre m minus sphere centre c
    const double rc = D.crad, rho2 = D.cbr2, irc = x::rcp_approx(rc);
    const double qx = D.dpx - D.cbx, qy = D.dpy - D.cby;  // detector position minus m
    const unsigned char at16[9] = {8, 4, 12, 2, 6, 10, 14, 1, 15};
    for (int c = 0; c < 9; c++) {
        uint32_t j = lo + (uint32_t)(((uint64_t)n * at16[c]) / 16u);
        if (j >= P.core_hi) j = P.core_hi - 1;
        const double z = zs[j];
        const double y = D.bym - D.bw * z;
        const double wx = ax + bx * y - D.cbx, wy = ay + by * y - D.cby;  // relative to m
        const double ex_ = wx + vx, ey_ = wy + vy;                         // relative to c
        const double ud = dx * ex_ + dy * ey_;
        const double cq = (ex_ * ex_ + ey_ * ey_) - rc * rc;
        const double disc = ud * ud - cq;
        if (!(disc > 0.0)) continue;
        const double sd = x::sqrt_approx(disc);
        const double d1 = -ud - sd, d2 = -ud + sd;
        double sigma, s;
        const double p1x = wx + dx * d1, p1y = wy + dy * d1;
        const double p2x = wx + dx * d2, p2y = wy + dy * d2;
        if (d1 >= 0.0 && p1x * p1x + p1y * p1y <= rho2) {
            sigma = -1.0;
            s = d1;
        } else if (d2 >= 0.0 && p2x * p2x + p2y * p2y <= rho2) {
            sigma = 1.0;
            s = d2;
        } else {
            continue;
        }
        const double px = wx + dx * s, py = wy + dy * s;
        const double mb = (px * px + py * py) - rho2;
        const double nx = -(vx + px) * irc, ny = -(vy + py) * irc;
        const double ci = -(dx * nx + dy * ny);
        const double crsq = 1.0 - r * r * (1.0 - ci * ci);
        if (!(crsq > 1e-6)) continue;
        const double cr = x::sqrt_approx(crsq);
        const double kk = r * ci - cr;
        const double ox = r * dx + kk * nx, oy = r * dy + kk * ny;
        const double cid = -(ox * D.dnx + oy * D.dny);
        if (!(cid > 0.05)) continue;
        const double gx = px - qx, gy = py - qy;
        const double gn = gx * D.dnx + gy * D.dny, gu = gx * D.dux + gy * D.duy;
        const double T = gn * x::rcp_approx(cid);
        const double du = ox * D.dux + oy * D.duy;
        const double pos = gu + du * T;
        split_f32(z, P.zref_hi, P.zref_lo);
        P.dlx2 = (float)(2.0 * ex_);
        P.dly2 = (float)(2.0 * ey_);
        P.ud2 = (float)(2.0 * ud);
        P.disc = (float)disc;
        P.sd = (float)sd;
        P.sigma = (float)sigma;
        P.s = (float)s;
        P.px2 = (float)(2.0 * px);
        P.py2 = (float)(2.0 * py);
        P.mb = (float)mb;
        P.nx = (float)nx;
        P.ny = (float)ny;
        P.ci = (float)ci;
        P.ci2 = (float)(2.0 * ci);
        P.crsq = (float)crsq;
        P.cr = (float)cr;
        P.r = (float)r;
        P.r2 = (float)(r * r);
        P.kk = (float)kk;
        P.cid = (float)cid;
        P.gn = (float)gn;
        P.T = (float)T;
        P.du = (float)du;
        P.pos = (float)pos;
        return true;
    }
    return false;
}

// Computes the per-wavelength parameters from the exact f64 flat-face chain, given
// the sorted ray table zs[0..R) (ascending z = norminv(u)). Returns false if no ray of
// this wavelength clears the flat faces (all lost); band ranges may still be non-empty.
// If E is given it receives the exact per-face data for the re-trace.
//
// f64 costs about 80 FP32 operations here (70-cycle DFMA latency, ~700-cycle divide
// and square root), so only the direction chain -- which the exact re-trace and every
// per-wavelength decision reuse bit for bit -- is formed with the reference's exact
// operations; the y interval is accurate to ~1e-14 and guarded at 1e-11.
template <int G>
CPD_HDN inline bool lambda_setup_g(const DevDesign &D, double lambda, const double *zs, uint32_t R, LamParams &P,
                                   double yguard_rel, ExactLam *E)
{
    using namespace x;
    {
        // zero every field (the struct is plain data)
        uint32_t *w = reinterpret_cast<uint32_t *>(&P);
        for (unsigned i = 0; i < sizeof(LamParams) / 4; i++) w[i] = 0u;
    }
    double nk[CPD_MAX_GLASS], rr[CPD_MAX_GLASS];
    _Pragma("unroll") for (int k = 0; k < G; k++) nk[k] = calc_n(D.glass[k], lambda);  // independent chains
    // Ray::refract's n1/n2 of every face: independent IEEE divisions, issued ahead of the
    // direction chain instead of on it
    _Pragma("unroll") for (int k = 0; k < G; k++) rr[k] = div(k ? nk[k - 1] : 1.0, nk[k]);
    double ets = 1.0, etp = 1.0;  // exact s/p transmittance products for the re-trace
    // direction/transmittance, exactly as the sequential trace computes them
    double dx = 1.0, dy = 0.0, ts = 1.0, tp = 1.0;
    // position affine in y: o(y) = (ax + bx*y, ay + by*y)
    double ax = 0.0, ay = 0.0, bx = 0.0, by = 1.0;
    double n1 = 1.0;
    // Tightest bounds y >= -L0/L1 (L1 > 0) and y <= U0/U1 (U1 > 0), kept as fractions and
    // compared by cross-multiplication so that only the two winners are divided.
    double L0 = 0.0, L1 = 0.0, Lg = 0.0, U0 = 0.0, U1 = 0.0, Ug = 0.0;
    bool all_band = false;  // a y-independent constraint sits inside its guard: every ray is re-traced
    bool ok = true;
    auto constrain = [&](double c0, double c1, double scale) {
        // c0 + c1*y >= 0 (up to rounding)
        const double g = yguard_rel * (scale + 1.0);
        if (c1 == 0.0) {
            if (c0 < g && c0 > -g) all_band = true;
            if (!(c0 > -g)) ok = false;
        } else if (c1 > 0.0) {
            if (L1 == 0.0 || c0 * L1 < L0 * c1) {
                L0 = c0;
                L1 = c1;
                Lg = g;
            }
        } else {
            const double u1 = -c1;
            if (U1 == 0.0 || c0 * U1 < U0 * u1) {
                U0 = c0;
                U1 = u1;
                Ug = g;
            }
        }
    };
    _Pragma("unroll") for (int k = 0; k < G; k++) {
        const double n2 = nk[k];
        const double nx = D.pnx[k], ny = D.pny[k];
        const double ci = dot(dx, dy, nx, ny);
        if (ci == 0.0) return false;
        // dist(y) = ((P - o(y)).N)/ci = e0 + e1*y (guarded: an approximate reciprocal)
        const double inv = rcp_approx(ci);
        const double e0 = ((D.ppx[k] - ax) * nx + (D.ppy[k] - ay) * ny) * inv;
        const double e1 = -(bx * nx + by * ny) * inv;
        const double sc = (e0 < 0 ? -e0 : e0) + 30.0 * (e1 < 0 ? -e1 : e1) + D.height;
        constrain(e0, e1, sc);                                   // dist >= 0
        const double hy0 = ay + dy * e0, hy1 = by + dy * e1;     // hit y = hy0 + hy1*y
        constrain(hy0, hy1, sc);                                 // 0 <= hit y
        constrain(D.height - hy0, -hy1, sc);                     // hit y <= height
        ax = ax + dx * e0;
        ay = hy0;
        bx = bx + dx * e1;
        by = hy1;
        // Ray::refract's direction with its exact operations (the TIR and AR decisions and
        // every later face depend on it); the s/p transmittances feed only the FP32 fast
        // path, so they are formed in FP32 (1 - R without cancellation).
        const double ci_r = -ci;  // -dot(d, N) of Ray::refract: the same dot product
        const double rk = rr[k];
        const double cr_sq = sub(1.0, mul(sqr(rk), sub(1.0, sqr(ci_r))));
        if (cr_sq < 0.0) return false;  // TIR: the same for every ray
        const double cr = sqrt_(cr_sq);
        const double kq = sub(mul(rk, ci_r), cr);
        const double vx = add(mul(dx, rk), mul(nx, kq));
        const double vy = add(mul(dy, rk), mul(ny, kq));
        if (D.ar && ci_r > 0.5) {
            ts *= 0.99;
            tp *= 0.99;
        } else {
            const float f1 = (float)n1, f2 = (float)n2, fc = (float)ci_r, fr = (float)cr;
            const float a = f1 * fc + f2 * fr, b = f1 * fr + f2 * fc;
            const float k4 = 4.f * f1 * f2 * fc * fr;
            ts *= (double)(k4 / (a * a));
            tp *= (double)(k4 / (b * b));
        }
        if (E) {
            E->dx[k] = vx;
            E->dy[k] = vy;
            E->ci[k] = ci;
            E->cr[k] = cr;
            E->n[k] = n2;
            // the sequential trace's transmittance update at this face, same operations
            if (D.ar && ci_r > 0.5) {
                ets = mul(ets, 0.99);
                etp = mul(etp, 0.99);
            } else {
                const double a = mul(n1, ci_r), b = mul(n2, cr);
                const double rs = sqr(div(sub(a, b), add(a, b)));
                const double c = mul(n1, cr), e = mul(n2, ci_r);
                const double rp = sqr(div(sub(c, e), add(c, e)));
                ets = mul(ets, sub(1.0, rs));
                etp = mul(etp, sub(1.0, rp));
            }
        }
        dx = vx;
        dy = vy;
        n1 = n2;
    }
    if (E) {
        E->ts = ets;
        E->tp = etp;
    }
    if (!ok) return false;
    const double iL = L1 > 0.0 ? rcp_approx(L1) : 0.0, iU = U1 > 0.0 ? rcp_approx(U1) : 0.0;
    const double ylo = L1 > 0.0 ? -L0 * iL : -INFINITY, glo = Lg * iL;
    const double yhi = U1 > 0.0 ? U0 * iU : INFINITY, ghi = Ug * iU;
    // Sorted-ray index ranges. y_j = bym - bw z_j is monotone in z, so the index of a
    // height threshold T is the number of z_j below (bym - T)/bw. The guard widths are
    // many orders above the f64 rounding of that inversion, so the count is taken on
    // the z table with integer-ordered keys (no f64 arithmetic per search step).
    auto zkey = [](double v) -> int64_t {
        int64_t b;
#if defined(__CUDA_ARCH__)
        b = __double_as_longlong(v);
#else
        std::memcpy(&b, &v, 8);
#endif
        return b >= 0 ? b : (int64_t)(0x8000000000000000ull - (uint64_t)b);
    };
    // The four counts of a wavelength, searched in lockstep: the table is read by four
    // independent chains of dependent loads instead of one chain four times as long.
    auto ycount4 = [&](const double thr[4], uint32_t out[4]) {
        int64_t key[4];
        uint32_t lo[4], hi[4];
        const double ibw = rcp_approx(D.bw);
        for (int i = 0; i < 4; i++) {
            const double zt = (D.bym - thr[i]) * ibw;
            key[i] = zkey(zt);
            lo[i] = 0;
            hi[i] = zt != zt ? 0u : R;
        }
        while (lo[0] < hi[0] || lo[1] < hi[1] || lo[2] < hi[2] || lo[3] < hi[3]) {
            for (int i = 0; i < 4; i++) {
                if (lo[i] < hi[i]) {
                    const uint32_t mid = (lo[i] + hi[i]) >> 1;
                    if (zkey(zs[mid]) < key[i]) lo[i] = mid + 1;
                    else hi[i] = mid;
                }
            }
        }
        for (int i = 0; i < 4; i++) out[i] = lo[i];
    };
    if (all_band) {
        P.band_lo = P.core_lo = P.core_hi = 0;
        P.band_hi = R;
    } else if (D.bw == 0.0) {
        // every ray starts at the same height
        double y = D.bym;
        if (y < ylo - glo || y > yhi + ghi) return false;
        if ((y < ylo + glo) || (y > yhi - ghi)) {
            P.band_lo = 0;
            P.core_lo = P.core_hi = 0;
            P.band_hi = R;
        } else {
            P.band_lo = P.core_lo = 0;
            P.core_hi = P.band_hi = R;
        }
    } else {
        // bw > 0: j increasing <=> y decreasing: [yhi+g .. yhi-g] band first, core,
        // [ylo+g .. ylo-g] band; bw < 0 the other way round
        const double thr[4] = {D.bw > 0.0 ? yhi + ghi : ylo - glo, D.bw > 0.0 ? yhi - ghi : ylo + glo,
                               D.bw > 0.0 ? ylo + glo : yhi - ghi, D.bw > 0.0 ? ylo - glo : yhi + ghi};
        uint32_t c[4];
        ycount4(thr, c);
        P.band_lo = c[0];
        P.core_lo = c[1];
        P.core_hi = c[2];
        P.band_hi = c[3];
    }
    if (P.core_hi < P.core_lo) P.core_hi = P.core_lo;
    if (P.band_hi < P.core_hi) P.band_hi = P.core_hi;
    if (P.band_lo > P.core_lo) P.band_lo = P.core_lo;
    P.w1x = (float)bx;
    P.w1y = (float)by;
    P.dx = (float)dx;
    P.dy = (float)dy;
    P.ts = (float)ts;
    P.tp = (float)tp;
    if (P.core_hi > P.core_lo && !reference_ray(D, zs, P, ax, ay, bx, by, dx, dy, n1)) P.all_exact = 1;
    return P.band_hi > P.band_lo;
}

// lambda_setup for a prism count known at compile time: the face loops unroll, so the
// independent work of one face (positions, constraints, transmittances) is scheduled
// into the latency of the next face's exact direction step.
CPD_HDN inline bool lambda_setup(const DevDesign &D, double lambda, const double *zs, uint32_t R, LamParams &P,
                                 double yguard_rel = kYGuardRel, ExactLam *E = nullptr)
{
    switch (D.G) {
    case 1: return lambda_setup_g<1>(D, lambda, zs, R, P, yguard_rel, E);
    case 2: return lambda_setup_g<2>(D, lambda, zs, R, P, yguard_rel, E);
    case 3: return lambda_setup_g<3>(D, lambda, zs, R, P, yguard_rel, E);
    case 4: return lambda_setup_g<4>(D, lambda, zs, R, P, yguard_rel, E);
    case 5: return lambda_setup_g<5>(D, lambda, zs, R, P, yguard_rel, E);
    default: return lambda_setup_g<6>(D, lambda, zs, R, P, yguard_rel, E);
    }
}

// ----------------------------------------------------------------- FP32 fast path

CPD_HD float fabs_f(float a) { return a < 0.f ? -a : a; }

CPD_HD float sqrt_fast(float a)
{
#if defined(__CUDA_ARCH__)
    // the hardware approximation (a couple of ulps): every decision that uses it sits
    // behind a guard band thousands of ulps wide
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(a));
    return r;
#else
    return std::sqrt(a);
#endif
}
CPD_HD float div_fast(float a, float b)
{
#if defined(__CUDA_ARCH__)
    return __fdividef(a, b);
#else
    return a / b;
#endif
}

// One ray through the exit face and onto the detector in FP32, as differences from
// the wavelength's reference ray. (zhi, zlo) is the ray's z = norminv(u) split into
// f32 parts; the ray is known to clear every flat face. Returns RAY_HIT with (bin, t),
// RAY_LOST, or RAY_FLAG when any decision is inside its guard band.
CPD_HD int fast_ray(const FastConst &D, const LamParams &P, const Guards &g, float zhi, float zlo, uint32_t &bin,
                    float &t)
{
    // start-height difference from the reference ray: y = bym - bw z
    const float dz = (P.zref_hi - zhi) + (P.zref_lo - zlo);
    const float dyy = D.bw * dz;
    const float dwx = P.w1x * dyy, dwy = P.w1y * dyy;
    // exit face: s^2 + 2 ud s + cq = 0, ud = d.(w - c), cq = |w - c|^2 - Rc^2
    const float dud = fmaf(P.dx, dwx, P.dy * dwy);
    const float dcq = fmaf(dwx, P.dlx2 + dwx, dwy * (P.dly2 + dwy));
    const float ddisc = fmaf(dud, P.ud2 + dud, -dcq);
    const float disc = P.disc + ddisc;
    if (disc <= g.rel * P.disc) return disc > -g.rel * P.disc ? RAY_FLAG : RAY_LOST;
    const float sd = sqrt_fast(disc);
    // the other root is 2 sd away along the ray: outside the bound when sd > rho
    bool flag = sd < 1.01f * D.rho;
    const float dsd = div_fast(ddisc, sd + P.sd);
    const float ds = fmaf(P.sigma, dsd, -dud);
    const float s = P.s + ds;
    flag |= fabs_f(s) < g.dist;
    const float dpx = fmaf(P.dx, ds, dwx), dpy = fmaf(P.dy, ds, dwy);
    const float mb = P.mb + fmaf(dpx, P.px2 + dpx, dpy * (P.py2 + dpy));
    flag |= fabs_f(mb) < g.rel * D.rho2;
    if (s < 0.f || mb > 0.f) return flag ? RAY_FLAG : RAY_LOST;
    // refraction into air at the exit face, normal n = (c - p)/Rc
    const float dnx = -dpx * D.inv_rc, dny = -dpy * D.inv_rc;
    const float dci = -fmaf(P.dx, dnx, P.dy * dny);
    const float ci = P.ci + dci;
    const float dcr2 = P.r2 * dci * (P.ci2 + dci);
    const float crsq = P.crsq + dcr2;
    if (crsq < g.cosine) return crsq > -g.cosine ? RAY_FLAG : RAY_LOST;
    const float cr = sqrt_fast(crsq);
    const float dcr = div_fast(dcr2, cr + P.cr);
    const float dkk = fmaf(P.r, dci, -dcr);
    const float nx = P.nx + dnx, ny = P.ny + dny;
    const float dex = fmaf(P.kk, dnx, dkk * nx), dey = fmaf(P.kk, dny, dkk * ny);
    float ts = P.ts, tp = P.tp;
    if (D.ar) flag |= fabs_f(ci - 0.5f) < g.cosine;
    if (D.ar && ci > 0.5f) {
        ts *= 0.99f;
        tp *= 0.99f;
    } else {
        // 1 - Rs = 4 n1 n2 ci cr / (n1 ci + n2 cr)^2, 1 - Rp likewise with ci<->cr (n2 = 1)
        const float r = P.r;
        const float a = fmaf(r, ci, cr), b = fmaf(r, cr, ci);
        const float a2 = a * a, b2 = b * b;
        const float inv = div_fast(4.f * r * ci * cr, a2 * b2);
        ts *= b2 * inv;
        tp *= a2 * inv;
    }
    // detector line
    const float dcid = -fmaf(dex, D.dnfx, dey * D.dnfy);
    const float cid = P.cid + dcid;
    if (cid <= D.min_ci + g.cosine) return cid > D.min_ci - g.cosine ? RAY_FLAG : RAY_LOST;
    const float dgn = fmaf(dpx, D.dnfx, dpy * D.dnfy);
    const float dgu = fmaf(dpx, D.dufx, dpy * D.dufy);
    const float ddu = fmaf(dex, D.dufx, dey * D.dufy);
    const float dT = div_fast(fmaf(dgn, P.cid, -P.gn * dcid), cid * P.cid);
    const float tu = ddu * (P.T + dT), tt = P.du * dT;
    const float dpos = tu + (tt + dgu);
    const float pos = P.pos + dpos;
    // The position is the one unbounded quantity (a reference ray can land metres from
    // the detector): its guard grows with the magnitudes it was summed from.
    const float gp = fmaf(g.pos_rel, fabs_f(P.pos) + fabs_f(tu) + fabs_f(tt) + fabs_f(dgu), g.pos);
    if (pos < -gp || pos > D.L + gp) return RAY_LOST;
    flag |= pos < gp || pos > D.L - gp;
    const float xx = pos - D.c0;
    float qf = floorf(xx * D.inv_slope);
    float rem = fmaf(-qf, D.slope, xx);
    if (rem < 0.f) {
        qf -= 1.f;
        rem += D.slope;
    } else if (rem >= D.slope) {
        qf += 1.f;
        rem -= D.slope;
    }
    flag |= rem < gp || rem > D.slope - gp || fabs_f(rem - D.bin_size) < gp;
    if (flag) return RAY_FLAG;
    const uint32_t b = qf <= 0.f ? 0u : (uint32_t)qf;
    if (b < D.B && rem < D.bin_size) {
        bin = b;
        t = (ts + tp) * 0.5f;
        return RAY_HIT;
    }
    return RAY_LOST;
}

}  // namespace cpd
