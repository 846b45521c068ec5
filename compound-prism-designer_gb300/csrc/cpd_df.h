// cpd_df.h -- the per-wavelength setup and the guard-band re-trace in float-float.
//
// On this GPU one f64 warp instruction occupies its SM sub-partition's FP64 unit for
// ~64 cycles whatever the number of active lanes, so a per-wavelength program written
// in f64 is bound by its f64 instruction count. Everything here runs instead on the
// FP32 pipe in float-float arithmetic: a value is an unevaluated sum hi + lo of two
// floats, ~2^-46 relative after each operation (Knuth's two-sum, the FMA two-product,
// and one Newton step in float-float on a hardware FP32 estimate for 1/x and sqrt x).
// That is ~60x coarser than f64 but 10^6 times finer than the 1e-4 mm and 1e-5 guard
// bands of the FP32 fast path, so:
//  * lambda_setup_df gives the fast path its per-wavelength constants and the sorted-
//    ray ranges (the same role and the same operations as the reference's f64 trace,
//    ray.rs:309-499, with float-float rounding);
//  * trace_df decides every ray the fast path flags. It agrees with the exact f64 trace
//    of the reference on bin and loss except for rays within ~1e-11 mm (or ~1e-13 in a
//    cosine) of a decision threshold.
// The exact f64 model (cpd_model.h, namespace x) remains the FP64 study mode, the host
// methods and the oracle comparison.
#pragma once

#include "cpd_ff.h"
#include "cpd_model.h"

namespace cpd {
namespace df {

using ff::F2;

// add and mul are ff::add and ff::mul (found by argument-dependent lookup)
using ff::add;
using ff::mul;
CPD_HD F2 c(float h) { return F2{h, 0.f}; }
CPD_HD F2 neg(F2 a) { return F2{-a.hi, -a.lo}; }
CPD_HD F2 sub(F2 a, F2 b) { return ff::add(a, neg(b)); }
CPD_HD F2 sqr(F2 a) { return ff::mul(a, a); }
// a * f for a float f
CPD_HD F2 mulf(F2 a, float f)
{
    const float p = ff::mul_rn(a.hi, f);
    const float e = ff::fmaf_(a.hi, f, -p);
    return ff::fast_two_sum(p, ff::fmaf_(a.lo, f, e));
}
CPD_HD F2 dot(F2 ax, F2 ay, F2 bx, F2 by) { return add(mul(ax, bx), mul(ay, by)); }

// hardware estimates (a couple of ulps) of 1/x and 1/sqrt(x); exact IEEE on the host
CPD_HD float rcp_est(float x)
{
#if defined(__CUDA_ARCH__)
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
#else
    return 1.0f / x;
#endif
}
CPD_HD float rsqrt_est(float x)
{
#if defined(__CUDA_ARCH__)
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
#else
    return 1.0f / std::sqrt(x);
#endif
}
// a / b: q0 = a y, then one correction q1 = (a - b q0) y with the residual in float-float
CPD_HD F2 div(F2 a, F2 b)
{
    const float y = rcp_est(b.hi);
    const float q0 = ff::mul_rn(a.hi, y);
    const F2 r = sub(a, mulf(b, q0));
    const float q1 = ff::mul_rn(r.hi, y);
    const F2 q = ff::fast_two_sum(q0, q1);
    // second correction: the estimate y is only good to a couple of ulps
    const F2 r2 = sub(a, mul(b, q));
    return ff::add_f(q, ff::mul_rn(r2.hi, y));
}
CPD_HD F2 rcp(F2 b) { return div(c(1.f), b); }
// sqrt a for a >= 0 (0 for a <= 0): s0 = a/sqrt(a) from the estimate, then two Heron
// corrections s + (a - s^2)/(2 s) with the residual in float-float
CPD_HD F2 sqrt(F2 a)
{
    if (!(a.hi > 0.f)) return c(0.f);
    const float y = rsqrt_est(a.hi);
    const float s0 = ff::mul_rn(a.hi, y);
    const float h = 0.5f * y;
    const float p = ff::mul_rn(s0, s0);
    const F2 r0 = sub(a, F2{p, ff::fmaf_(s0, s0, -p)});  // a - s0^2, s0^2 exactly
    const F2 s = ff::fast_two_sum(s0, ff::mul_rn(r0.hi, h));
    return ff::add_f(s, ff::mul_rn(sub(a, sqr(s)).hi, h));
}
CPD_HD F2 addf(F2 a, float b) { return ff::add_f(a, b); }
CPD_HD bool lt(F2 a, F2 b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
CPD_HD bool le(F2 a, F2 b) { return a.hi < b.hi || (a.hi == b.hi && a.lo <= b.lo); }
CPD_HD bool pos(F2 a) { return a.hi > 0.f || (a.hi == 0.f && a.lo > 0.f); }
CPD_HD bool neg_(F2 a) { return a.hi < 0.f || (a.hi == 0.f && a.lo < 0.f); }
CPD_HD F2 abs_(F2 a) { return neg_(a) ? neg(a) : a; }

// an f64 as float-float (FP64 pipe: use for inputs only)
CPD_HD F2 from_d(double v)
{
    const float h = (float)v;
    return F2{h, (float)(v - (double)h)};
}
CPD_HD double to_d(F2 a) { return (double)a.hi + (double)a.lo; }

constexpr float kBig = 3.0e38f;  // an unbounded end of the y interval

}  // namespace df

// Per (design, wavelength row): what the float-float re-trace needs.
struct alignas(16) LamDF {
    ff::F2 ylo, yhi;    // the start heights that clear every flat face
    ff::F2 ax, ay, bx, by;  // position on the last flat face: (ax + bx y, ay + by y)
    ff::F2 dx, dy;      // direction entering the exit face
    ff::F2 n;           // index of the last glass
    float ts, tp;       // s/p transmittance entering the exit face
    uint32_t lost;      // no ray of this wavelength reaches the exit face
    float ts_lo, tp_lo; // low words: ts, tp as float-float
    uint32_t pad;
};

// The fast path's reference ray (see LamParams) in float-float: the first candidate of
// the core range for which every differentiated quantity is defined.
CPD_HDN inline bool reference_ray_df(const DevDesign &D, const float *z32, LamParams &P, ff::F2 ax, ff::F2 ay,
                                     ff::F2 bx, ff::F2 by, ff::F2 dx, ff::F2 dy, ff::F2 r)
{
    using namespace df;
    const DFConst &C = D.dc;
    const uint32_t lo = P.core_lo, n = P.core_hi - P.core_lo;
    const unsigned char at16[9] = {8, 4, 12, 2, 6, 10, 14, 1, 15};
    for (int k = 0; k < 9; k++) {
        uint32_t j = lo + (uint32_t)(((uint64_t)n * at16[k]) / 16u);
        if (j >= P.core_hi) j = P.core_hi - 1;
        const F2 z{z32[2 * j], z32[2 * j + 1]};
        const F2 y = sub(C.bym, mul(C.bw, z));
        const F2 wx = sub(add(ax, mul(bx, y)), C.cbx), wy = sub(add(ay, mul(by, y)), C.cby);  // relative to m
        const F2 ex = add(wx, C.vx), ey = add(wy, C.vy);                                         // relative to c
        const F2 ud = dot(dx, dy, ex, ey);
        const F2 cq = sub(dot(ex, ey, ex, ey), C.rc2);
        const F2 disc = sub(sqr(ud), cq);
        if (!pos(disc)) continue;
        const F2 sd = sqrt(disc);
        const F2 d1 = sub(neg(ud), sd), d2 = sub(sd, ud);
        const F2 p1x = add(wx, mul(dx, d1)), p1y = add(wy, mul(dy, d1));
        const F2 p2x = add(wx, mul(dx, d2)), p2y = add(wy, mul(dy, d2));
        float sigma;
        F2 s;
        if (!neg_(d1) && le(dot(p1x, p1y, p1x, p1y), C.cbr2)) {
            sigma = -1.f;
            s = d1;
        } else if (!neg_(d2) && le(dot(p2x, p2y, p2x, p2y), C.cbr2)) {
            sigma = 1.f;
            s = d2;
        } else {
            continue;
        }
        const F2 px = add(wx, mul(dx, s)), py = add(wy, mul(dy, s));
        const F2 mb = sub(dot(px, py, px, py), C.cbr2);
        const F2 nx = neg(mul(add(C.vx, px), C.irc)), ny = neg(mul(add(C.vy, py), C.irc));
        const F2 ci = neg(dot(dx, dy, nx, ny));
        const F2 crsq = sub(c(1.f), mul(sqr(r), sub(c(1.f), sqr(ci))));
        if (!(crsq.hi > 1e-6f)) continue;
        const F2 cr = sqrt(crsq);
        const F2 kk = sub(mul(r, ci), cr);
        const F2 ox = add(mul(r, dx), mul(kk, nx)), oy = add(mul(r, dy), mul(kk, ny));
        const F2 cid = neg(dot(ox, oy, C.dnx, C.dny));
        if (!(cid.hi > 0.05f)) continue;
        const F2 gx = sub(px, C.qx), gy = sub(py, C.qy);
        const F2 gn = dot(gx, gy, C.dnx, C.dny), gu = dot(gx, gy, C.dux, C.duy);
        const F2 T = div(gn, cid);
        const F2 du = dot(ox, oy, C.dux, C.duy);
        const F2 ps = add(gu, mul(du, T));
        P.zref_hi = z.hi;
        P.zref_lo = z.lo;
        // the exit-face terms as polynomials in dz = zref - z: the point on the last flat
        // face moves by wz dz, wz = (bx, by) bw
        const F2 wzx = mul(bx, C.bw), wzy = mul(by, C.bw);
        P.wzx = wzx.hi;
        P.wzy = wzy.hi;
        P.uz = dot(dx, dy, wzx, wzy).hi;
        P.ca = 2.f * dot(ex, ey, wzx, wzy).hi;
        P.cb = dot(wzx, wzy, wzx, wzy).hi;
        P.ud2 = 2.f * ud.hi;
        P.disc = disc.hi;
        P.sd = sd.hi;
        P.sigma = sigma;
        P.s = s.hi;
        P.px2 = 2.f * px.hi;
        P.py2 = 2.f * py.hi;
        P.mb = mb.hi;
        P.nf = dot(nx, ny, C.dnx, C.dny).hi;
        P.nu = dot(nx, ny, C.dux, C.duy).hi;
        P.ci = ci.hi;
        P.ci2 = 2.f * ci.hi;
        P.crsq = crsq.hi;
        P.cr = cr.hi;
        P.r = r.hi;
        P.r2 = sqr(r).hi;
        P.kk = kk.hi;
        P.cid = cid.hi;
        P.T = T.hi;
        P.du = du.hi;
        P.pos = ps.hi;
        return true;
    }
    return false;
}

// The state a wavelength's setup carries through the flat faces. Direction part: the
// direction d entering the next face, the index n1 of the glass it leaves, the s/p
// transmittance products. Position part: the affine point a + b y on the last face, and
// the tightest bounds y >= -L0/L1 (L1 > 0) and y <= U0/U1 (U1 > 0), compared by
// cross-multiplication so that only the two winners are divided.
struct SetupDir {
    ff::F2 dx, dy, n1, ts, tp;
};
struct SetupPos {
    ff::F2 ax, ay, bx, by, L0, L1, U0, U1;
    float Lg, Ug;
    bool lost;  // a bound independent of y excludes every ray
};
CPD_HD SetupDir setup_dir_init()
{
    return SetupDir{df::c(1.f), df::c(0.f), df::c(1.f), df::c(1.f), df::c(1.f)};
}
CPD_HD SetupPos setup_pos_init()
{
    using df::c;
    return SetupPos{c(0.f), c(0.f), c(0.f), c(1.f), c(0.f), c(0.f), c(0.f), c(0.f), 0.f, 0.f, false};
}
// The wavelength of u-point u.
CPD_HDN inline ff::F2 setup_lambda(const DevDesign &D, double u)
{
    return df::add(D.dc.wmin, df::mul(D.dc.wspan, df::from_d(u)));
}
// The cosine d.N at flat face k (the same value for both parts of the face).
CPD_HDN inline ff::F2 face_cos(const DevDesign &D, int k, ff::F2 dx, ff::F2 dy)
{
    return df::dot(dx, dy, D.dc.pnx[k], D.dc.pny[k]);
}

// The position part of flat face k (ci = its cosine, nonzero; dx, dy = the direction that
// enters it): the distance to the face e0 + e1 y, the three bounds it puts on y, and the
// point on the face.
CPD_HDN inline void face_position(const DevDesign &D, int k, ff::F2 ci, ff::F2 dx, ff::F2 dy, SetupPos &S,
                                  float yg)
{
    using namespace df;
    const DFConst &C = D.dc;
    auto constrain = [&](F2 c0, F2 c1, float scale) {
        // c0 + c1 y >= 0
        const float g = yg * (scale + 1.f);
        if (c1.hi == 0.f) {
            if (neg_(c0)) S.lost = true;  // independent of y: decided here for every ray
        } else if (c1.hi > 0.f) {
            if (S.L1.hi == 0.f || lt(mul(c0, S.L1), mul(S.L0, c1))) {
                S.L0 = c0;
                S.L1 = c1;
                S.Lg = g;
            }
        } else {
            const F2 u1 = neg(c1);
            if (S.U1.hi == 0.f || lt(mul(c0, S.U1), mul(S.U0, u1))) {
                S.U0 = c0;
                S.U1 = u1;
                S.Ug = g;
            }
        }
    };
    const F2 nx = C.pnx[k], ny = C.pny[k];
    // dist(y) = ((P - o(y)).N)/ci = e0 + e1 y; hit y = hy0 + hy1 y
    const F2 inv = rcp(ci);
    const F2 e0 = mul(dot(sub(C.ppx[k], S.ax), sub(C.ppy[k], S.ay), nx, ny), inv);
    const F2 e1 = neg(mul(dot(S.bx, S.by, nx, ny), inv));
    const float sc = fabsf(e0.hi) + 30.f * fabsf(e1.hi) + C.height.hi;
    constrain(e0, e1, sc);
    const F2 hy0 = add(S.ay, mul(dy, e0)), hy1 = add(S.by, mul(dy, e1));
    constrain(hy0, hy1, sc);
    constrain(sub(C.height, hy0), neg(hy1), sc);
    S.ax = add(S.ax, mul(dx, e0));
    S.ay = hy0;
    S.bx = add(S.bx, mul(dx, e1));
    S.by = hy1;
}

// The direction part of flat face k: Ray::refract (ray.rs:309-367), the same for every ray
// of the wavelength, and the face's Fresnel factors. Returns false on total internal
// reflection (the state is then left as it was).
CPD_HDN inline bool face_direction(const DevDesign &D, int k, ff::F2 lambda, ff::F2 ci, SetupDir &S,
                                   bool df_fresnel)
{
    using namespace df;
    const DFConst &C = D.dc;
    const F2 ar99{0.99f, -9.5367431640625e-09f};  // 0.99 = hi + lo to ~1e-17
    F2 n2 = C.glass[k][0];  // Glass::calc_n (Horner, glasscat.rs:17-22)
#pragma unroll
    for (int i = 1; i < 6; i++) n2 = add(mul(n2, lambda), C.glass[k][i]);
    const F2 nx = C.pnx[k], ny = C.pny[k];
    const F2 ci_r = neg(ci);
    const F2 n1 = S.n1;
    const F2 rr = div(n1, n2);
    const F2 cr_sq = sub(c(1.f), mul(sqr(rr), sub(c(1.f), sqr(ci_r))));
    if (neg_(cr_sq)) return false;  // total internal reflection
    const F2 cr = sqrt(cr_sq);
    const F2 kq = sub(mul(rr, ci_r), cr);
    const F2 vx = add(mul(S.dx, rr), mul(nx, kq)), vy = add(mul(S.dy, rr), mul(ny, kq));
    // s/p transmittance products in float-float: the AR factor 0.99 is not a float, and
    // six float roundings would bias every ray of the wavelength by ~6e-8
    if (D.ar && lt(c(0.5f), ci_r)) {
        S.ts = mul(S.ts, ar99);
        S.tp = mul(S.tp, ar99);
    } else if (df_fresnel) {
        const F2 a = add(mul(n1, ci_r), mul(n2, cr)), b = add(mul(n1, cr), mul(n2, ci_r));
        const F2 k4 = mulf(mul(mul(n1, n2), mul(ci_r, cr)), 4.f);
        S.ts = mul(S.ts, div(k4, sqr(a)));
        S.tp = mul(S.tp, div(k4, sqr(b)));
    } else {
        // 1 - R without cancellation: 4 n1 n2 ci cr / (n1 ci + n2 cr)^2 (s), ci <-> cr (p)
        const float f1 = n1.hi, f2 = n2.hi, fc = ci_r.hi, fr = cr.hi;
        const float a = f1 * fc + f2 * fr, b = f1 * fr + f2 * fc;
        const float k4 = 4.f * f1 * f2 * fc * fr;
        S.ts = mulf(S.ts, k4 / (a * a));
        S.tp = mulf(S.tp, k4 / (b * b));
    }
    S.dx = vx;
    S.dy = vy;
    S.n1 = n2;
    return true;
}

// After the flat faces: the y interval, E, the sorted-ray ranges and the reference ray.
CPD_HDN inline bool setup_tail(const DevDesign &D, const float *z32, uint32_t R, LamParams &P, LamDF *E,
                               const SetupDir &Sd, const SetupPos &Sp, bool lost)
{
    using namespace df;
    const DFConst &C = D.dc;
    const F2 L0 = Sp.L0, L1 = Sp.L1, U0 = Sp.U0, U1 = Sp.U1;
    const F2 ylo = L1.hi > 0.f ? neg(div(L0, L1)) : c(-kBig), yhi = U1.hi > 0.f ? div(U0, U1) : c(kBig);
    const float glo = L1.hi > 0.f ? Sp.Lg / L1.hi : 0.f, ghi = U1.hi > 0.f ? Sp.Ug / U1.hi : 0.f;
    auto write_e = [&]() {
        if (!E) return;
        E->ylo = ylo;
        E->yhi = yhi;
        E->ax = Sp.ax;
        E->ay = Sp.ay;
        E->bx = Sp.bx;
        E->by = Sp.by;
        E->dx = Sd.dx;
        E->dy = Sd.dy;
        E->n = Sd.n1;
        E->ts = Sd.ts.hi;
        E->tp = Sd.tp.hi;
        E->lost = lost ? 1u : 0u;
        E->ts_lo = Sd.ts.lo;
        E->tp_lo = Sd.tp.lo;
        E->pad = 0u;
    };
    if (lost) {
        write_e();
        return false;
    }
    // Sorted-ray index ranges: y_j = bym - bw z_j is monotone in z, so the index of a
    // height threshold T is the number of z_j below (bym - T)/bw, counted on the (hi,
    // lo) table. The four counts are branch-free lower bounds stepping together: the
    // interval lengths depend on R alone, so every lane runs the same iterations and the
    // four table reads of an iteration are independent (a branchy bisection per key took
    // ~6k cycles at R = 1024, its steps serialised behind their branches).
    auto ycount4 = [&](const F2 thr[4], uint32_t out[4]) {
        F2 key[4];
        const F2 ibw = rcp(C.bw);
#pragma unroll
        for (int i = 0; i < 4; i++) {
            key[i] = fabsf(thr[i].hi) >= kBig ? c(((thr[i].hi > 0.f) == (C.bw.hi > 0.f)) ? -INFINITY : INFINITY)
                                              : mul(sub(C.bym, thr[i]), ibw);
            out[i] = 0u;
        }
        if (R == 0u) return;
        // invariant: the count lies in [base, base + n]; z[base + n/2] < key moves base up
        uint32_t base[4] = {0u, 0u, 0u, 0u};
        for (uint32_t n = R; n > 1u;) {
            const uint32_t half = n >> 1;
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const uint32_t m = base[i] + half;
                base[i] = lt(F2{z32[2 * m], z32[2 * m + 1]}, key[i]) ? m : base[i];
            }
            n -= half;
        }
#pragma unroll
        for (int i = 0; i < 4; i++)
            out[i] = base[i] + (lt(F2{z32[2 * base[i]], z32[2 * base[i] + 1]}, key[i]) ? 1u : 0u);
    };
    if (C.bw.hi == 0.f) {
        // every ray starts at the same height
        const F2 y = C.bym;
        if (lt(y, addf(ylo, -glo)) || lt(addf(yhi, ghi), y)) {
            write_e();
            return false;
        }
        if (lt(y, addf(ylo, glo)) || lt(addf(yhi, -ghi), y)) {
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
        const bool up = C.bw.hi > 0.f;
        const F2 thr[4] = {up ? addf(yhi, ghi) : addf(ylo, -glo), up ? addf(yhi, -ghi) : addf(ylo, glo),
                           up ? addf(ylo, glo) : addf(yhi, -ghi), up ? addf(ylo, -glo) : addf(yhi, ghi)};
        uint32_t cnt[4];
        ycount4(thr, cnt);
        P.band_lo = cnt[0];
        P.core_lo = cnt[1];
        P.core_hi = cnt[2];
        P.band_hi = cnt[3];
    }
    if (P.core_hi < P.core_lo) P.core_hi = P.core_lo;
    if (P.band_hi < P.core_hi) P.band_hi = P.core_hi;
    if (P.band_lo > P.core_lo) P.band_lo = P.core_lo;
    P.dx = Sd.dx.hi;
    P.dy = Sd.dy.hi;
    P.ts = Sd.ts.hi;
    P.tp = Sd.tp.hi;
    if (P.core_hi > P.core_lo &&
        !reference_ray_df(D, z32, P, Sp.ax, Sp.ay, Sp.bx, Sp.by, Sd.dx, Sd.dy, Sd.n1))
        P.all_exact = 1;
    // the re-trace's record last: its scattered stores (one line per row and field) would
    // otherwise queue ahead of the ray-range searches' loads
    write_e();
    return P.band_hi > P.band_lo;
}

CPD_HD void zero_lam_params(LamParams &P)
{
    uint32_t *w = reinterpret_cast<uint32_t *>(&P);
    for (unsigned i = 0; i < sizeof(LamParams) / 4; i++) w[i] = 0u;
}

// Per-wavelength setup in float-float. u is the wavelength's u-point (lambda = wmin +
// (wmax - wmin) u); z32 the sorted ray table as (hi, lo) float pairs, R entries. Fills P
// (fast-path constants and the band / core ranges of sorted rays) and, if given, E.
// Returns false if no ray of this wavelength clears the flat faces. The face loop is
// kept rolled: one warp runs this program once per wavelength, so instruction fetch,
// not scheduling freedom, is what a longer unrolled body would cost.
// With df_fresnel the Fresnel factors of the flat faces are formed in float-float too,
// so that E's transmittances match the f64 trace to ~2^-44 (the adaptive mode's exact
// path needs them); otherwise each factor is an FP32 value (~1e-7).
CPD_HDN inline bool lambda_setup_df(const DevDesign &D, double u, const float *z32, uint32_t R, LamParams &P,
                                    double yguard_rel = kYGuardRel, LamDF *E = nullptr, bool df_fresnel = false)
{
    const int G = D.G;
    zero_lam_params(P);
    const ff::F2 lambda = setup_lambda(D, u);
    SetupDir Sd = setup_dir_init();
    SetupPos Sp = setup_pos_init();
    const float yg = (float)yguard_rel;
    bool lost = false;
#pragma unroll 1
    for (int k = 0; k < G; k++) {
        if (Sp.lost) break;
        const ff::F2 ci = face_cos(D, k, Sd.dx, Sd.dy);
        if (ci.hi == 0.f) {  // parallel to the face: no ray meets it
            lost = true;
            break;
        }
        face_position(D, k, ci, Sd.dx, Sd.dy, Sp, yg);
        if (!face_direction(D, k, lambda, ci, Sd, df_fresnel)) {
            lost = true;
            break;
        }
    }
    return setup_tail(D, z32, R, P, E, Sd, Sp, lost || Sp.lost);
}

// The float-float re-trace of one ray (start height from z = zh + zl): the flat faces
// through the wavelength's y interval and affine position, then the curved exit face
// (SphericalLikeSurface::intersection + RadialBounds, geometry.rs:161-216, 85-91;
// Ray::refract into air, ray.rs:309-367) and the detector (ray.rs:390-402,
// spectrometer.rs:265-303). Returns true and (bin, t) on a hit.
// One ray in float-float from the wavelength's LamDF. kExactT: the transmittance too
// (exit-face Fresnel factors in float-float from E's float-float flat-face products),
// returned as tfix = 2^31 t rounded as t_fixed64 does; otherwise t is an FP32 value.
template <bool kExactT>
CPD_HDN inline bool trace_df_(const DevDesign &D, const LamDF &E, float zh, float zl, uint32_t &bin, float &t,
                              uint32_t &tfix)
{
    using namespace df;
    const DFConst &C = D.dc;
    if (E.lost) return false;
    const F2 y = sub(C.bym, mul(C.bw, F2{zh, zl}));
    if (lt(y, E.ylo) || lt(E.yhi, y)) return false;
    const F2 ox = add(E.ax, mul(E.bx, y)), oy = add(E.ay, mul(E.by, y));
    // exit face
    const F2 ex = sub(ox, C.ccx), ey = sub(oy, C.ccy);
    const F2 ud = dot(E.dx, E.dy, ex, ey);
    const F2 disc = add(sub(sqr(ud), dot(ex, ey, ex, ey)), C.rc2);
    if (!pos(disc)) return false;
    const F2 sd = sqrt(disc);
    const F2 d1 = sub(neg(ud), sd), d2 = sub(sd, ud);
    const F2 p1x = add(ox, mul(E.dx, d1)), p1y = add(oy, mul(E.dy, d1));
    auto in_bound = [&](F2 px, F2 py) {
        const F2 qx = sub(px, C.cbx), qy = sub(py, C.cby);
        return le(dot(qx, qy, qx, qy), C.cbr2);
    };
    F2 px, py;
    if (!neg_(d1) && in_bound(p1x, p1y)) {
        px = p1x;
        py = p1y;
    } else {
        const F2 p2x = add(ox, mul(E.dx, d2)), p2y = add(oy, mul(E.dy, d2));
        if (!neg_(d2) && in_bound(p2x, p2y)) {
            px = p2x;
            py = p2y;
        } else {
            return false;
        }
    }
    const F2 nx = mul(sub(C.ccx, px), C.irc), ny = mul(sub(C.ccy, py), C.irc);
    const F2 ci = neg(dot(E.dx, E.dy, nx, ny));
    const F2 rr = E.n;  // n1 / 1
    const F2 cr_sq = sub(c(1.f), mul(sqr(rr), sub(c(1.f), sqr(ci))));
    if (neg_(cr_sq)) return false;  // total internal reflection
    const F2 cr = sqrt(cr_sq);
    const F2 k = sub(mul(rr, ci), cr);
    const F2 vx = add(mul(E.dx, rr), mul(nx, k)), vy = add(mul(E.dy, rr), mul(ny, k));
    float ts = E.ts, tp = E.tp;
    F2 tsd{E.ts, E.ts_lo}, tpd{E.tp, E.tp_lo};
    if (D.ar && lt(c(0.5f), ci)) {
        if (kExactT) {
            const F2 ar99{0.99f, -9.5367431640625e-09f};  // 0.99 = hi + lo to ~1e-17
            tsd = mul(tsd, ar99);
            tpd = mul(tpd, ar99);
        } else {
            ts *= 0.99f;
            tp *= 0.99f;
        }
    } else if (kExactT) {
        // 1 - R_s = 4 n ci cr / (n ci + cr)^2, 1 - R_p = 4 n ci cr / (n cr + ci)^2 (n2 = 1)
        const F2 a = add(mul(rr, ci), cr), b = add(mul(rr, cr), ci);
        const F2 k4 = mulf(mul(rr, mul(ci, cr)), 4.f);
        tsd = mul(tsd, div(k4, sqr(a)));
        tpd = mul(tpd, div(k4, sqr(b)));
    } else {
        const float f1 = rr.hi, fc = ci.hi, fr = cr.hi;
        const float a = f1 * fc + fr, b = f1 * fr + fc;
        const float k4 = 4.f * f1 * fc * fr;
        ts *= k4 / (a * a);
        tp *= k4 / (b * b);
    }
    // detector
    const F2 cid = neg(dot(vx, vy, C.dnx, C.dny));
    if (!lt(C.min_ci, cid)) return false;
    const F2 dist = div(dot(sub(px, C.dpx), sub(py, C.dpy), C.dnx, C.dny), cid);
    const F2 hx = add(px, mul(vx, dist)), hy = add(py, mul(vy, dist));
    const F2 ps = dot(sub(hx, C.dpx), sub(hy, C.dpy), C.dux, C.duy);
    if (neg_(ps) || lt(C.L, ps)) return false;
    const F2 a = sub(ps, C.intercept);
    // euclid_div_rem (utils.rs:177-192) with a positive slope
    float q = floorf(mul(a, C.islope).hi);
    F2 rem = sub(a, mulf(C.slope, q));
    if (neg_(rem)) {
        q -= 1.f;
        rem = add(rem, C.slope);
    } else if (le(C.slope, rem)) {
        q += 1.f;
        rem = sub(rem, C.slope);
    }
    const uint32_t b = q <= 0.f ? 0u : (q >= 4294967295.f ? 4294967295u : (uint32_t)q);
    if (b < D.B && lt(rem, C.bin_size)) {
        bin = b;
        if (kExactT) {
            const F2 s = add(tsd, tpd);  // t = s / 2, exactly
            t = 0.5f * s.hi;
            tfix = t_fixed64(0.5 * ((double)s.hi + (double)s.lo));
        } else {
            t = (ts + tp) * 0.5f;
        }
        return true;
    }
    return false;
}

// The re-trace of a flagged ray: bin and an FP32 transmittance.
CPD_HDN inline bool trace_df(const DevDesign &D, const LamDF &E, float zh, float zl, uint32_t &bin, float &t)
{
    uint32_t tfix = 0;
    return trace_df_<false>(D, E, zh, zl, bin, t, tfix);
}

// The adaptive mode's exact path: bin and tfix = 2^31 t (t to ~2^-44), for E filled by
// lambda_setup_df with df_fresnel.
CPD_HDN inline bool trace_df_exact(const DevDesign &D, const LamDF &E, float zh, float zl, uint32_t &bin,
                                   uint32_t &tfix)
{
    float t = 0.f;
    return trace_df_<true>(D, E, zh, zl, bin, t, tfix);
}

}  // namespace cpd
