// cpd_model.h -- the spectrometer model shared by host C++ and device CUDA code.
//
// Three layers:
//  * Exact f64 model (namespace cpd::x): the reference's per-ray trace
//    (src/spectrometer/ray.rs:309-499, geometry.rs:124-216, spectrometer.rs:265-303)
//    with every rounding step made explicit. On the device the arithmetic uses
//    the _rn intrinsics (no contraction); on the host this header is compiled with
//    -ffp-contract=off. Both therefore give the reference's own f64 results bit
//    for bit, given the same tables. The log of the inverse normal CDF is evaluated
//    on the host only; the sin/cos of design construction on the host, or with CUDA's
//    f64 functions when the device builds the design (cpd_build.h).
//  * Per-wavelength setup (lambda_setup_df, cpd_df.h): all rays of one wavelength
//    leave the Gaussian beam with direction (1,0) (Ray::new_from_start,
//    ray.rs:277-279), and every face before the curved exit face is flat, so the
//    direction and the s/p transmittances after each flat face are the same for every
//    ray of that wavelength. Positions on the flat faces are affine in the start
//    height y, so the set of rays that clears every flat face is an interval of y,
//    and, with the ray table sorted by z = norminv(u), a contiguous range of ray
//    indices.
//  * FP32 fast path (fast_ray): per ray, only the exit face and the detector,
//    with a guard margin on every decision; a ray inside any guard band is
//    reported FLAG and re-traced in float-float (trace_df, cpd_df.h).
#pragma once

#include <cstdint>
#include <cmath>
#include <cstring>

#include "../../include/cpd.h"
#include "cpd_ff.h"

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

// 2^31 t for t in [0, 1], rounded to nearest even: one FP32-to-u32 conversion (the
// conversion unit; a 64-bit conversion would go to the FP64 unit).
CPD_HD uint32_t t_fixed(float t)
{
#if defined(__CUDA_ARCH__)
    return __float2uint_rn(t * 2147483648.0f);
#else
    return (uint32_t)std::nearbyint((double)t * 2147483648.0);
#endif
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
    float hL;          // L / 2
    int32_t ar;
    uint32_t B;
};

// Float-float copies of the design tables (split on the host), for the per-wavelength
// setup and the guard-band re-trace (cpd_df.h).
struct alignas(16) DFConst {
    ff::F2 glass[CPD_MAX_GLASS][6];
    ff::F2 ppx[CPD_MAX_GLASS], ppy[CPD_MAX_GLASS], pnx[CPD_MAX_GLASS], pny[CPD_MAX_GLASS];
    ff::F2 height;
    ff::F2 ccx, ccy, rc2, irc;            // exit-face centre, radius^2, 1/radius
    ff::F2 cbx, cby, cbr2, vx, vy;        // bound centre, bound radius^2, bound centre - centre
    ff::F2 bin_size, slope, islope, intercept, min_ci, L;
    ff::F2 dnx, dny, dpx, dpy, dux, duy;  // detector normal, position, direction
    ff::F2 qx, qy;                        // detector position - bound centre
    ff::F2 wmin, wspan, bw, bym;          // wavelength range, beam width and centre
};

// Per design, on the device: the exact f64 tables, their float-float copies and the
// FP32 constants.
struct alignas(16) DevDesign {
    int32_t G;
    uint32_t B;
    int32_t ar;
    int32_t status;  // 0, or the error of a design built on the device (its rays are all lost)
    double glass[CPD_MAX_GLASS][6];
    double ppx[CPD_MAX_GLASS], ppy[CPD_MAX_GLASS], pnx[CPD_MAX_GLASS], pny[CPD_MAX_GLASS];
    double height;
    double ccx, ccy, crad, cbx, cby, cbr2;
    double bin_size, slope, intercept, min_ci, L;
    double dnx, dny, dpx, dpy, dux, duy;
    double wmin, wmax, bw, bym;
    double size, deviation;  // size_and_deviation (spectrometer.rs:429-437)
    FastConst fc;
    DFConst dc;
};

// Per (design, wavelength), written by lambda_setup_df. The FP32 fast path works in
// differences from one reference ray of the wavelength, traced in f64 through the
// exit face and onto the detector: every per-ray quantity is the reference value
// plus a difference computed with a cancellation-free identity, so the FP32 error
// scales with the (small) difference, not with the absolute coordinates or the
// distance to the detector.
struct alignas(16) LamParams {
    float zref_hi, zref_lo;     // z of the reference ray (f32 hi + lo parts)
    float wzx, wzy;             // d(position on the last flat face)/d(zref - z) = (dw/dy) bw
    float dx, dy;               // direction entering the exit face (same for every ray)
    float ts, tp;               // s/p transmittance entering the exit face
    float ca, cb;               // d(cq) = dz (ca + cb dz): ca = 2 (w_ref - c).wz, cb = |wz|^2
    float ud2, disc, sd;        // reference: 2 d.(w - c), discriminant, its square root
    float sigma;                // root sign: s = -ud + sigma*sd
    float s, px2, py2, mb;      // reference root, 2 p_ref (rel. bound centre), |p|^2 - rho^2
    float nf, nu;               // reference exit-face normal (c - p)/Rc . detector normal, . direction
    float ci, ci2, crsq, cr;    // reference cosines (ci2 = 2 ci)
    float r, r2, kk;            // n_last, n_last^2, r ci - cr
    float cid, T, du, pos;      // reference detector cosine, distance (p - P).N / cid, d'.u, position
    uint32_t core_lo, core_hi;  // sorted-ray range that clears every flat face (fast path)
    uint32_t band_lo, band_hi;  // [band_lo, core_lo) and [core_hi, band_hi): guard bands
    uint32_t all_exact;         // no usable reference ray: every core ray is re-traced exactly
    float uz;                   // d(ud) = uz dz: d.wz
    uint32_t pad[3];
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
    if ((b < D.B) & (rem < D.bin_size)) {
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

}  // namespace x

// ----------------------------------------------------------------- per-wavelength setup

// Guard widths of the fast path. A decision whose FP32 margin is inside its guard
// is not trusted: the ray is re-traced with the exact model. The widths are
// upper bounds on the FP32 error of each margin measured over random designs,
// times a safety factor.
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

// ----------------------------------------------------------------- adaptive sampling
//
// The stop rule of the reference GPU kernel (src/spectrometer/kernel.rs:127-178): the
// rays of one wavelength are taken in index order, 32 per round. After each round, every
// bin that the round's rays hit merges the round into its Welford state (32 samples: the
// hits' t and zeros for the round's other rays), and the wavelength stops when the round
// hit some bin and every bin it hit passes the SEM test (welford.rs:80-84,
// SEM^2 <= (5e-3)^2). p(d|lambda) is then the bin's sum of t over all rays consumed.
//
// Here the Welford states are exact integer sums, so the test is exact arithmetic on
// quantized transmittances, the same on the host and the device:
//   t_q = t_fixed >> 11 (t in 2^-20 units), N = samples (32 per round in which the bin was
//   hit), q1 = sum t_q, q2 = sum t_q^2 over its h hits,
//   M2 = (q2 - q1^2 / N) 2^-40 < (5e-3)^2 N (N - 1)
//   <=>  40000 (N q2 - q1^2) < N^2 (N - 1) 2^40.
// N <= 2^22 rays keeps every term below 2^107 (unsigned 128-bit arithmetic).
constexpr uint32_t kRoundRays = 32;
constexpr int kTqShift = 11;
// Bound on |t_q(FP32 fast path) - t_q(exact)| for a fast-path hit: it holds while the
// fast path's transmittance error stays below 2^-19 (~1.9e-6; measured: below 3e-7).
constexpr uint32_t kTqDelta = 2;

enum : int { SEM_FAIL = 0, SEM_PASS = 1, SEM_UNSURE = 2 };

// The SEM test of one bin. With delta > 0 the sums are those of FP32 transmittances,
// each t_q within delta of its exact value: the test is SEM_UNSURE when those errors
// could change its outcome, i.e. when |40000 (N q2 - q1^2) - N^2 (N - 1) 2^40| is within
// 40000 (N h delta (2^21 + delta) + h delta (2 q1 + h delta)).
CPD_HD int sem_test(uint64_t N, uint64_t h, uint64_t q1, uint64_t q2, uint32_t delta)
{
    typedef unsigned __int128 u128;
    // N q2 >= q1^2: Cauchy-Schwarz over the N samples (hits and zeros)
    const u128 lhs = (u128)40000u * ((u128)N * q2 - (u128)q1 * q1);
    const u128 rhs = ((u128)N * N * (N - 1u)) << 40;
    if (delta == 0u) return lhs < rhs ? SEM_PASS : SEM_FAIL;
    const u128 hd = (u128)h * delta;
    const u128 err =
        (u128)40000u * ((u128)N * h * ((u128)delta * ((1u << 21) + delta)) + hd * (2u * (u128)q1 + hd));
    if (lhs + err < rhs) return SEM_PASS;
    if (lhs >= rhs + err) return SEM_FAIL;
    return SEM_UNSURE;
}

// Integers to float with integer-unit and FP32 instructions only: below 2^23 exactly (the
// float of exponent 23 whose mantissa is v, minus 2^23); below 2^63 in 21-bit pieces,
// within 2^-23 relative (two roundings).
CPD_HD float f32_small(uint32_t v)
{
    const uint32_t b = 0x4B000000u | v;
    float f;
#if defined(__CUDA_ARCH__)
    f = __uint_as_float(b);
#else
    std::memcpy(&f, &b, 4);
#endif
    return f - 8388608.f;
}
CPD_HD float f32_wide(uint64_t v)
{
    const float a = f32_small((uint32_t)(v >> 42)), b = f32_small((uint32_t)(v >> 21) & 0x1fffffu);
    return (a * 0x1p42f + b * 0x1p21f) + f32_small((uint32_t)v & 0x1fffffu);
}

// An FP32 screen of sem_test (same arguments, N <= 2^22, q2 < 2^63): SEM_PASS or SEM_FAIL
// when float arithmetic with error bounds settles the test, else -1 (run sem_test). With
// A = N q2 and Q = q1^2 in float, every product and sum rounds by at most 2^-24 relative
// and each conversion by 2^-23, so the computed 40000 (A - Q) is within 8 2^-24 40000 (A + Q)
// of lhs and the computed N^2 (N - 1) 2^40 within 3 2^-24 of rhs; the margins (2^-18 of the
// terms, and of the err bound) exceed those errors and the rounding of the comparisons'
// own sums.
CPD_HD int sem_quick(uint32_t N, uint32_t h, uint64_t q1, uint64_t q2, uint32_t delta)
{
    const float n = f32_small(N), f1 = f32_wide(q1), f2 = f32_wide(q2);
    const float A = n * f2, Q = f1 * f1;
    const float L = 40000.f * (A - Q), eL = 40000.f * 0x1p-18f * (A + Q);
    const float Y = n * n * (n - 1.f) * 0x1p40f, eY = Y * 0x1p-18f;
    float E = 0.f;
    if (delta) {
        const float d = (float)delta, hd = f32_small(h) * d;
        E = 40000.f * (n * f32_small(h) * (d * (0x1p21f + d)) + hd * (2.f * f1 + hd)) * (1.f + 0x1p-18f);
    }
    if (L + eL + E < Y - eY) return SEM_PASS;
    if (L - eL >= Y + eY + E) return SEM_FAIL;
    return -1;
}

// A cell's sum of t over `count` rays rescaled to the pass's common divisor R:
// round(s1 R / count), so that p = cell 2^-31 / R everywhere downstream.
CPD_HD uint64_t rescale_cell(uint64_t s1, uint32_t R, uint32_t count)
{
    if (count == R || s1 == 0u) return s1;
    typedef unsigned __int128 u128;
    return (uint64_t)(((u128)s1 * R + count / 2u) / count);
}

// Splits an f64 into f32 hi + lo parts (hi + lo == v to about 2^-48 relative).
CPD_HD void split_f32(double v, float &hi, float &lo)
{
    hi = (float)v;
    lo = (float)(v - (double)hi);
}



// ----------------------------------------------------------------- FP32 fast path

// |a|: an operand modifier of the consuming instruction on the device. It differs from
// (a < 0 ? -a : a) only in the sign of -0 and of NaN, which no comparison or sum below sees.
CPD_HD float fabs_f(float a)
{
#if defined(__CUDA_ARCH__)
    return fabsf(a);
#else
    return std::fabs(a);
#endif
}

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
// Every operation of the fast path is written out (mulr, addr, subr: rounded, never
// fused; fmaf: fused), so that each inlined copy of it -- the trace kernel steps two rays
// at a time -- gives the same bits for the same ray, and the host build computes what
// the device computes (up to the hardware square root and reciprocal estimates).
CPD_HD float mulr(float a, float b) { return ff::mul_rn(a, b); }
CPD_HD float addr(float a, float b) { return ff::add_rn(a, b); }
CPD_HD float subr(float a, float b) { return ff::sub_rn(a, b); }

// The fast path's thresholds that combine a design constant with a guard, rounded once
// (the same operations wherever they are formed: per work item on the device, or on the
// host for a pass whose design constants are kernel parameters).
struct FastLimits {
    float rho101;  // 1.01 rho: a root whose other root may lie inside the bound
    float rho2g;   // guard on |p|^2 - rho^2
    float ci_lo;   // min_ci - cosine guard
    float ci_hi;   // min_ci + cosine guard
};
CPD_HD FastLimits fast_limits(const FastConst &D, const Guards &g)
{
    return FastLimits{mulr(1.01f, D.rho), mulr(g.rel, D.rho2), subr(D.min_ci, g.cosine), addr(D.min_ci, g.cosine)};
}

CPD_HD int fast_ray(const FastConst &D, const FastLimits &Lm, const LamParams &P, const Guards &g, float zhi,
                    float zlo, uint32_t &bin, float &t)
{
    // start-height difference from the reference ray (y = bym - bw z): the point on the
    // last flat face moves by dw = wz dz
    const float dz = addr(subr(P.zref_hi, zhi), subr(P.zref_lo, zlo));
    const float dwx = mulr(P.wzx, dz), dwy = mulr(P.wzy, dz);
    // exit face: s^2 + 2 ud s + cq = 0, ud = d.(w - c), cq = |w - c|^2 - Rc^2; both change
    // by polynomials in dz whose coefficients the setup formed in float-float
    const float dud = mulr(P.uz, dz);
    const float dcq = mulr(dz, fmaf(P.cb, dz, P.ca));
    const float ddisc = fmaf(dud, addr(P.ud2, dud), -dcq);
    const float disc = addr(P.disc, ddisc);
    const float gdisc = mulr(g.rel, P.disc);
    if (disc <= gdisc) return disc > -gdisc ? RAY_FLAG : RAY_LOST;
    const float sd = sqrt_fast(disc);
    // the other root is 2 sd away along the ray: outside the bound when sd > rho
    bool flag = sd < Lm.rho101;
    const float dsd = div_fast(ddisc, addr(sd, P.sd));
    const float ds = fmaf(P.sigma, dsd, -dud);
    const float s = addr(P.s, ds);
    flag |= fabs_f(s) < g.dist;
    const float dpx = fmaf(P.dx, ds, dwx), dpy = fmaf(P.dy, ds, dwy);
    const float mb = addr(P.mb, fmaf(dpx, addr(P.px2, dpx), mulr(dpy, addr(P.py2, dpy))));
    flag |= fabs_f(mb) < Lm.rho2g;
    if ((s < 0.f) | (mb > 0.f)) return flag ? RAY_FLAG : RAY_LOST;
    // refraction into air at the exit face, normal n = (c - p)/Rc, so dn = -dp/Rc and
    // dci = -d.dn = (d.dp)/Rc = (ds + dud)/Rc (|d| = 1)
    const float dci = mulr(addr(ds, dud), D.inv_rc);
    const float ci = addr(P.ci, dci);
    const float dcr2 = mulr(mulr(P.r2, dci), addr(P.ci2, dci));
    const float crsq = addr(P.crsq, dcr2);
    if (crsq < g.cosine) return crsq > -g.cosine ? RAY_FLAG : RAY_LOST;
    const float cr = sqrt_fast(crsq);
    const float dcr = div_fast(dcr2, addr(cr, P.cr));
    const float dkk = fmaf(P.r, dci, -dcr);
    // the ray's transmittance t = (ts + tp) / 2 after the exit face
    float tr;
    if (D.ar) flag |= fabs_f(subr(ci, 0.5f)) < g.cosine;
    if (D.ar && ci > 0.5f) {
        tr = mulr(addr(P.ts, P.tp), 0.495f);  // 0.99 (ts + tp) / 2
    } else {
        // 1 - Rs = 4 n1 n2 ci cr / a^2, 1 - Rp = 4 n1 n2 ci cr / b^2 (n2 = 1), a = r ci + cr,
        // b = r cr + ci: t = 2 r ci cr (ts b^2 + tp a^2) / (a^2 b^2)
        const float r = P.r;
        const float a = fmaf(r, ci, cr), b = fmaf(r, cr, ci);
        const float a2 = mulr(a, a), b2 = mulr(b, b);
        const float q = div_fast(mulr(mulr(mulr(2.f, r), ci), cr), mulr(a2, b2));
        tr = mulr(q, fmaf(P.ts, b2, mulr(P.tp, a2)));
    }
    // detector line (normal N, direction U). The exit direction e = r d + kk n changes by
    // de = kk_ref dn + dkk n; with dn = -dp/Rc its components along N and U follow from
    // dgn = dp.N and dgu = dp.U: de.N = dkk nf - (kk_ref + dkk) dgn/Rc, likewise for U
    const float dgn = fmaf(dpx, D.dnfx, mulr(dpy, D.dnfy));
    const float dgu = fmaf(dpx, D.dufx, mulr(dpy, D.dufy));
    const float kn = mulr(addr(P.kk, dkk), D.inv_rc);
    const float dcid = fmaf(dgn, kn, -mulr(dkk, P.nf));  // cid = -e.N
    const float cid = addr(P.cid, dcid);
    if (cid <= Lm.ci_hi) return cid > Lm.ci_lo ? RAY_FLAG : RAY_LOST;
    const float ddu = fmaf(-dgu, kn, mulr(dkk, P.nu));
    // T = gn / cid: dT = (dgn - T_ref dcid) / cid
    const float dT = div_fast(fmaf(-P.T, dcid, dgn), cid);
    const float tu = mulr(ddu, addr(P.T, dT)), tt = mulr(P.du, dT);
    const float dpos = addr(tu, addr(tt, dgu));
    const float pos = addr(P.pos, dpos);
    // The position is the one unbounded quantity (a reference ray can land metres from
    // the detector): its guard grows with the magnitudes it was summed from.
    const float gp = fmaf(g.pos_rel, addr(addr(fabs_f(tu), fabs_f(tt)), fabs_f(dgu)),
                          fmaf(g.pos_rel, fabs_f(P.pos), g.pos));
    // 0 <= pos <= L, as a distance from the detector's middle
    const float dm = fabs_f(subr(pos, D.hL));
    if (dm > addr(D.hL, gp)) return RAY_LOST;
    flag |= dm > subr(D.hL, gp);
    const float xx = subr(pos, D.c0);
    const float qf = floorf(mulr(xx, D.inv_slope));
    // within an ulp of a bin boundary the rounded quotient can be one off; such a
    // remainder falls outside [gp, slope - gp] and the ray is flagged
    const float rem = fmaf(-qf, D.slope, xx);
    flag |= (rem < gp) | (rem > subr(D.slope, gp)) | (fabs_f(subr(rem, D.bin_size)) < gp);
    if (flag) return RAY_FLAG;
#if defined(__CUDA_ARCH__)
    const uint32_t b = __float2uint_rz(qf);  // saturating: negative -> 0
#else
    const uint32_t b = qf <= 0.f ? 0u : (qf >= 4294967295.f ? 4294967295u : (uint32_t)qf);
#endif
    if ((b < D.B) & (rem < D.bin_size)) {
        bin = b;
        t = tr;
        return RAY_HIT;
    }
    return RAY_LOST;
}
CPD_HD int fast_ray(const FastConst &D, const LamParams &P, const Guards &g, float zhi, float zlo, uint32_t &bin,
                    float &t)
{
    return fast_ray(D, fast_limits(D, g), P, g, zhi, zlo, bin, t);
}

}  // namespace cpd
