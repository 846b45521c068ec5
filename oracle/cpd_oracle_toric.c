/*
 * cpd_oracle_toric.c -- TEST INFRASTRUCTURE ONLY (see cpd_oracle.h).
 *
 * Double-precision restatement of the reference's 3-D spectrometer: a fiber beam
 * (FiberBeam, src/spectrometer/spectrometer.rs:75-125) through a compound prism whose
 * first and last faces are toric lenses (CulminatingToricCompoundPrism,
 * src/spectrometer/ray.rs:112-118; ToricLens, src/spectrometer/toric.rs:204-262), with
 * flat inner faces bounded in height and width (PrismBounds 3-D, geometry.rs:69-77), onto
 * the linear detector (spectrometer.rs:265-303). The ray-torus intersection is the
 * reference's closed-form quartic solution (sympy_soln, toric.rs:41-141) with its cube root
 * (approx_cbrt, cbrt.rs:49-68), restated operation for operation, so that the oracle
 * reproduces the reference's own results, including where that closed form yields NaN.
 *
 * Vectors are 3-D; a dot product is the un-fused sum x + y + z of the lane products
 * (the ordered reduction of the 4-lane SIMD vector whose fourth lane is 0), mul_add is
 * fused per lane. Build with -ffp-contract=off. Citations are paths inside the reference
 * project.
 */
#include "cpd_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

typedef double real;
#define ORC_D(x) (x)
#include "cpd_oracle_model.h"

typedef struct { double x, y, z; } v3;

static v3 v3_make(double x, double y, double z) { v3 r = {x, y, z}; return r; }
static v3 v3_add(v3 a, v3 b) { return v3_make(a.x + b.x, a.y + b.y, a.z + b.z); }
static v3 v3_sub(v3 a, v3 b) { return v3_make(a.x - b.x, a.y - b.y, a.z - b.z); }
static v3 v3_scale(v3 a, double s) { return v3_make(a.x * s, a.y * s, a.z * s); }
static v3 v3_div(v3 a, double s) { return v3_make(a.x / s, a.y / s, a.z / s); }
static v3 v3_neg(v3 a) { return v3_make(-a.x, -a.y, -a.z); }
static double v3_dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static v3 v3_fma(v3 a, double b, v3 c) { return v3_make(fma(a.x, b, c.x), fma(a.y, b, c.y), fma(a.z, b, c.z)); }
/* angled_xy / rot_180_xy / rot_90_xy / rot_90_ccw_xy on a 3-D vector (vector.rs:336-378). */
static v3 v3_angled(double th) { return v3_make(cos(th), sin(th), 0.0); }
static v3 v3_rot180(v3 a) { return v3_make(-a.x, -a.y, a.z); }
static v3 v3_rot90(v3 a) { return v3_make(-a.y, a.x, a.z); }
static v3 v3_rot90ccw(v3 a) { return v3_make(a.y, -a.x, a.z); }

/* ------------------------------------------------------------ cube root, quartic */

/* bit_magic + approx_cbrt (cbrt.rs:8-10, 49-68): Moroz et al.'s magic-constant cube
 * root; the magic step runs on the f32 value of x, the two refinements in f64 with the
 * f32 constants widened. */
static float cbrt_magic(float x)
{
    uint32_t b;
    memcpy(&b, &x, 4);
    b = 0x548c2b4bu - b / 3u;
    float y;
    memcpy(&y, &b, 4);
    return y;
}

double orc_approx_cbrt(double x)
{
    const double k1 = (double)1.752319676f, k2 = (double)1.2509524245f, k3 = (double)0.5093818292f;
    const double one_third = (double)0.333333333333f;
    int s = !signbit(x);
    x = fabs(x);
    double y = (double)cbrt_magic((float)x);
    double c = x * y * y * y;
    y = y * (k1 - c * (k2 - k3 * c));
    double d = x * y * y;
    c = 1.0 - d * y;
    double res = d * (1.0 + one_third * c);
    return s ? res : -res;
}

static double sqrd(double v) { return v * v; }
static double cube(double v) { return v * v * v; }

/* sympy_soln (toric.rs:41-141): the four roots of the ray-torus quartic, in the
 * reference's operation order. */
void orc_toric_roots(double r_2, double R_2, double dp_magn_sq, double dp_v, double dp_n, double n_v,
                     double roots[4])
{
    const double _2 = 2, _3 = 3, _4 = 4, _6 = 6, _8 = 8, _12 = 12, _16 = 16, _27 = 27, _108 = 108, _216 = 216;
    double x0 = R_2 * dp_v;
    double x1 = dp_magn_sq * dp_v;
    double x2 = dp_v * r_2;
    double x3 = dp_n * n_v;
    double x4 = R_2 * x3;
    double x5 = sqrd(n_v);
    double x6 = _2 * R_2;
    double x7 = R_2 - dp_magn_sq + r_2 - x5 * x6;
    double x8 = _8 * dp_v * x7 - _8 * x0 + _8 * x1 - _8 * x2 + _16 * x4;
    double x9 = _2 * r_2;
    double x10 = sqrd(dp_v);
    double x11 = R_2 * x5;
    double x12 = _2 * dp_magn_sq - _2 * x10 + _4 * x11 - x6 - x9;
    double x13 = cube(x12);
    double x14 = _4 * dp_v;
    double x15 = sqrd(-_4 * x0 + _4 * x1 + x14 * x7 - _4 * x2 + _8 * x4);
    double x16 = sqrd(R_2);
    double x17 = sqrd(dp_magn_sq);
    double x18 = sqrd(r_2);
    double x19 = dp_magn_sq * x6;
    double x20 = r_2 * x6;
    double x21 = dp_magn_sq * x9;
    double x22 = _4 * R_2 * sqrd(dp_n);
    double x23 = x14 * (-x0 + x1 + x14 * (R_2 / _8 - dp_magn_sq / _8 + r_2 / _8 - x10 / _16 - x11 / _4) - x2 +
                        x3 * x6);
    double x24 = x16 + x17 + x18 - x19 - x20 - x21 + x22 - x23;
    double x25 = x12 * x24;
    double x26 = -x13 / _108 - x15 / _8 + x25 / _3;
    double x27 = _2 * orc_approx_cbrt(x26);
    double x28 = _8 * R_2 / _3;
    double x29 = _4 * R_2 / _3 - _4 * dp_magn_sq / _3 + _4 * r_2 / _3 + _4 * x10 / _3 - x28 * x5;
    double x30 = sqrt(-x27 + x29);
    double x31 = x8 / x30;
    double x32 = -_8 * dp_magn_sq / _3 + _8 * r_2 / _3 + _8 * x10 / _3 - _16 * x11 / _3 + x28;
    double x33 = x27 + x32;
    double x34 = sqrt(x31 + x33) / _2;
    double x35 = -dp_v;
    double x36 = x30 / _2;
    double x37 = x35 - x36;
    double x38 = sqrd(x12) / _12;
    int x39 = x24 + x38 == 0.0;
    double x40 = -x16 - x17 - x18 + x19 + x20 + x21 - x22 + x23 - x38;
    double x41 = orc_approx_cbrt(x13 / _216 + x15 / _16 - x25 / _6 + sqrt(sqrd(x26) / _4 + cube(x40) / _27));
    double x42 = _2 * x41;
    double x43 = _2 * x40 / (_3 * x41);
    double x44 = sqrt(x29 + x42 - x43);
    double x45 = x8 / x44;
    double x46 = x32 - x42 + x43;
    double x47 = sqrt(x45 + x46) / _2;
    double x48 = x44 / _2;
    double x49 = x35 - x48;
    double x50 = sqrt(-x31 + x33) / _2;
    double x51 = x35 + x36;
    double x52 = sqrt(-x45 + x46) / _2;
    double x53 = x35 + x48;
    roots[3] = x39 ? x34 + x37 : x47 + x49;
    roots[2] = x39 ? x50 + x51 : x52 + x53;
    roots[1] = x39 ? -x34 + x37 : -x47 + x49;
    roots[0] = x39 ? -x50 + x51 : -x52 + x53;
}

/* ------------------------------------------------------------ geometry */

typedef struct { v3 point, normal; } plane3;

/* ToricLens: ToricSurface + SandwichBounds (toric.rs:14-27, 146-201; geometry.rs:94-109). */
typedef struct {
    v3 center, tnormal;           /* torus centre, toroidal normal */
    double tradius, pradius;      /* toroidal and poloidal radii */
    v3 bcenter, bnormal;          /* sandwich bounds */
    double bheight;
} toric;

typedef struct {
    int nglass, ar_coated;
    double glass[ORC_MAX_GLASS][6];
    double height, half_width;
    toric first;
    plane3 inner[ORC_MAX_GLASS];  /* inner faces 1..G-1 */
    toric last;
} prism3;

typedef struct {
    uint32_t bin_count;
    double bin_size, slope, intercept, min_ci, length;
    v3 normal, position, direction;
} detector3;

typedef struct {
    prism3 cp;
    detector3 det;
    double wmin, wmax;
    double fiber_radius, fiber_min_cos, fiber_center_y;
} spectrometer3;

/* ToricLens::from_hyperplane (toric.rs:221-262). */
static toric toric_from_plane(plane3 hp, double spc, double ntc, double height, double width)
{
    toric t;
    double chord = fabs(height / hp.normal.x); /* sec_xy */
    double pr = chord * 0.5 / fabs(spc);
    double tr = width * 0.5 / ntc;
    double apothem = sqrt(sqrd(pr) - sqrd(chord) * 0.25);
    double sagitta = pr - apothem;
    t.center = v3_fma(hp.normal, copysign(apothem + tr, spc), hp.point);
    t.tnormal = v3_rot90(hp.normal);
    t.tradius = tr;
    t.pradius = pr;
    t.bcenter = hp.point;
    t.bnormal = !signbit(spc) ? v3_neg(hp.normal) : hp.normal;
    t.bheight = sagitta;
    return t;
}

/* create_joined_trapezoids (geometry.rs:430-489) with 3-D vectors (z = 0), then
 * CompoundPrism::new (ray.rs:137-183) with toric first and last faces. */
static int build_prism3(const orc_spec3 *s3, prism3 *cp)
{
    const orc_spec *s = &s3->base;
    int G = s->nglass;
    if (G < 1 || G > ORC_MAX_GLASS) return ORC_INVALID;
    memset(cp, 0, sizeof(*cp));
    cp->nglass = G;
    cp->ar_coated = s->ar_coated;
    cp->height = s->height;
    cp->half_width = s->width * 0.5;
    memcpy(cp->glass, s->glass, sizeof(cp->glass));
    double h2 = s->height * 0.5;
    v3 normal = v3_rot180(v3_angled(s->angles[0]));
    plane3 first = {v3_make(fabs(normal.y / normal.x) * h2, h2, 0.0), normal};
    int prev_sign = !signbit(normal.y);
    double d1 = first.point.x;
    double mx = first.point.x;
    plane3 last = {{0, 0, 0}, {0, 0, 0}};
    for (int k = 1; k <= G; k++) {
        double angle = s->angles[k];
        double sep_len = s->lengths[k - 1];
        v3 n = v3_rot180(v3_angled(angle));
        int sign = !signbit(n.y);
        double d2 = fabs(n.y / n.x) * h2;
        double sep_dist = sep_len + (prev_sign != sign ? d1 + d2 : fabs(d1 - d2));
        prev_sign = sign;
        d1 = d2;
        mx += sep_dist;
        plane3 hp = {v3_make(mx, h2, 0.0), n};
        if (k < G) cp->inner[k] = hp;
        else last = hp;
    }
    cp->first = toric_from_plane(first, s3->curv0[0], s3->curv0[1], s->height, s->width);
    cp->last = toric_from_plane(last, s3->curv1[0], s3->curv1[1], s->height, s->width);
    return ORC_OK;
}

/* LinearDetectorArray::new in 3-D (spectrometer.rs:183-219). */
static void build_detector3(const orc_spec *s, detector3 *d)
{
    d->bin_count = s->bin_count;
    d->bin_size = s->bin_size;
    d->slope = s->linear_slope;
    d->intercept = s->linear_intercept;
    d->min_ci = cos(s->max_incident_angle);
    d->length = s->det_length;
    d->normal = v3_rot180(v3_angled(s->det_angle));
    d->direction = s->det_flipped ? v3_rot90(d->normal) : v3_rot90ccw(d->normal);
    d->position = v3_make(s->det_position[0], s->det_position[1], 0.0);
}

static int build_spectrometer3(const orc_spec3 *s, spectrometer3 *sp)
{
    int e = build_prism3(s, &sp->cp);
    if (e) return e;
    if (s->base.bin_count == 0) return ORC_INVALID;
    build_detector3(&s->base, &sp->det);
    sp->wmin = s->base.wmin;
    sp->wmax = s->base.wmax;
    /* FiberBeam::new (spectrometer.rs:85-94) */
    sp->fiber_radius = s->fiber_radius;
    sp->fiber_min_cos = sqrt(1.0 - sqrd(s->fiber_na));
    sp->fiber_center_y = s->fiber_center_y;
    return ORC_OK;
}

/* ------------------------------------------------------------ ray trace */

typedef struct { v3 origin, dir; double ts, tp; } ray3;

/* FiberBeam 3-D inverse_cdf (spectrometer.rs:108-125) with UniformDiscDistribution
 * (distribution.rs:57-66). */
static ray3 fiber_ray(const spectrometer3 *sp, const double q[4])
{
    const double tau = 6.283185307179586476925286766559;
    double st = sin(q[1] * tau), ct = cos(q[1] * tau);
    double r = sp->fiber_radius * sqrt(q[0]);
    double y = r * ct, z = r * st;
    double ux = sp->fiber_min_cos + q[2] * (1.0 - sp->fiber_min_cos);
    double s_ux = sqrt(1.0 - sqrd(ux));
    double sr = sin(q[3] * tau), cr = cos(q[3] * tau);
    ray3 ray = {v3_make(0.0, y + sp->fiber_center_y, z), v3_make(ux, s_ux * cr, s_ux * sr), 1.0, 1.0};
    return ray;
}

/* HyperPlane::intersection with PrismBounds 3-D (geometry.rs:124-145, 69-77). */
static int plane3_intersect(const plane3 *p, double height, double half_width, const ray3 *r, double *dist)
{
    double ci = v3_dot(r->dir, p->normal);
    if (ci == 0.0) return 0;
    double d = v3_dot(v3_sub(p->point, r->origin), p->normal) / ci;
    if (d >= 0.0) {
        v3 h = v3_fma(r->dir, d, r->origin);
        if (0.0 <= h.y && h.y <= height && -half_width <= h.z && h.z <= half_width) {
            *dist = d;
            return 1;
        }
    }
    return 0;
}

static int sandwich_in(const toric *t, v3 p)
{
    double dp = v3_dot(t->bnormal, v3_sub(p, t->bcenter));
    return 0.0 <= dp && dp <= t->bheight;
}

/* ToricSurface::intersection (toric.rs:146-201): the first root in r0..r3 that is not
 * negative and lies within the bounds; NaN roots fail both tests. */
static int toric_intersect(const toric *t, const ray3 *r, double *dist, v3 *normal, uint32_t *nan_roots)
{
    v3 dp = v3_sub(r->origin, t->center);
    double dp_magn_sq = v3_dot(dp, dp);
    double dp_v = v3_dot(dp, r->dir);
    double dp_n = v3_dot(dp, t->tnormal);
    double n_v = v3_dot(t->tnormal, r->dir);
    double R_2 = sqrd(t->tradius);
    double r_2 = sqrd(t->pradius);
    double roots[4];
    orc_toric_roots(r_2, R_2, dp_magn_sq, dp_v, dp_n, n_v, roots);
    if (nan_roots)
        for (int i = 0; i < 4; i++) *nan_roots += isnan(roots[i]) ? 1u : 0u;
    for (int i = 0; i < 4; i++) {
        double d = roots[i];
        if (d < 0.0) continue;
        v3 p = v3_fma(r->dir, d, r->origin);
        if (!sandwich_in(t, p)) continue;
        /* t_center = normalize(oproj(p - c, n)) * R + c; normal = (t_center - p) / r */
        v3 u = v3_sub(p, t->center);
        v3 op = v3_sub(u, v3_scale(t->tnormal, v3_dot(u, t->tnormal)));
        v3 on = v3_div(op, sqrt(v3_dot(op, op)));
        v3 tc = v3_fma(on, t->tradius, t->center);
        *normal = v3_div(v3_sub(tc, p), t->pradius);
        *dist = d;
        return 1;
    }
    return 0;
}

/* Ray::refract (ray.rs:309-367) in 3-D. */
static int refract3(ray3 *r, v3 normal, double n1, double n2, int ar_coated)
{
    double ci = -v3_dot(r->dir, normal);
    double rr = n1 / n2;
    double cr_sq = 1.0 - sqrd(rr) * (1.0 - sqrd(ci));
    if (cr_sq < 0.0) return ORC_TOTAL_INTERNAL_REFLECTION;
    double cr = sqrt(cr_sq);
    v3 v = v3_add(v3_scale(r->dir, rr), v3_scale(normal, rr * ci - cr));
    double ts, tp;
    if (ar_coated && ci > 0.5) {
        ts = r->ts * 0.99;
        tp = r->tp * 0.99;
    } else {
        double rs = sqrd((n1 * ci - n2 * cr) / (n1 * ci + n2 * cr));
        double rp = sqrd((n1 * cr - n2 * ci) / (n1 * cr + n2 * ci));
        ts = r->ts * (1.0 - rs);
        tp = r->tp * (1.0 - rp);
    }
    r->dir = v;
    r->ts = ts;
    r->tp = tp;
    return ORC_OK;
}

/* Per-ray counters of the toric faces (for the failure-rate measurement). */
typedef struct {
    uint32_t nan_roots;   /* roots that came out NaN at the faces this ray reached */
    int toric_calls;      /* toric faces this ray reached */
} toric_stats;

static int toric_propagate(ray3 *r, const toric *t, double n1, double n2, int ar, toric_stats *ts)
{
    double d;
    v3 normal;
    if (ts) ts->toric_calls++;
    if (!toric_intersect(t, r, &d, &normal, ts ? &ts->nan_roots : NULL)) return ORC_NO_SURFACE_INTERSECTION;
    r->origin = v3_fma(r->dir, d, r->origin);
    return refract3(r, normal, n1, n2, ar);
}

static int plane3_propagate(ray3 *r, const plane3 *p, const prism3 *cp, double n1, double n2)
{
    double d;
    if (!plane3_intersect(p, cp->height, cp->half_width, r, &d)) return ORC_NO_SURFACE_INTERSECTION;
    r->origin = v3_fma(r->dir, d, r->origin);
    return refract3(r, p->normal, n1, n2, cp->ar_coated);
}

/* CompoundPrism::propagate (ray.rs:485-499) with the toric first and last faces. */
static int prism3_propagate(const prism3 *cp, ray3 *r, double w, toric_stats *ts)
{
    double n1 = orc_calc_n(cp->glass[0], w);
    int e = toric_propagate(r, &cp->first, 1.0, n1, cp->ar_coated, ts);
    if (e) return e;
    for (int k = 1; k < cp->nglass; k++) {
        double n2 = orc_calc_n(cp->glass[k], w);
        e = plane3_propagate(r, &cp->inner[k], cp, n1, n2);
        if (e) return e;
        n1 = n2;
    }
    return toric_propagate(r, &cp->last, n1, 1.0, cp->ar_coated, ts);
}

/* Ray::intersect_detector_array + LinearDetectorArray (ray.rs:390-402,
 * spectrometer.rs:265-303) in 3-D. */
static int detector3_hit(const detector3 *dt, const ray3 *r, uint32_t *bin, double *t)
{
    double ci = -v3_dot(r->dir, dt->normal);
    if (ci <= dt->min_ci) return ORC_ANGULAR_RESPONSE_TOO_WEAK;
    double d = v3_dot(v3_sub(r->origin, dt->position), dt->normal) / ci;
    v3 p = v3_fma(r->dir, d, r->origin);
    double pos = v3_dot(v3_sub(p, dt->position), dt->direction);
    if (pos < 0.0 || dt->length < pos) return ORC_NO_SURFACE_INTERSECTION;
    double q, rem;
    euclid_div_rem(pos - dt->intercept, dt->slope, &q, &rem);
    uint32_t b = sat_u32(q);
    if (b < dt->bin_count && rem < dt->bin_size) {
        *bin = b;
        *t = (r->ts + r->tp) * 0.5;
        return ORC_OK;
    }
    return ORC_NO_SURFACE_INTERSECTION;
}

static double sample_wavelength3(const spectrometer3 *sp, double u) { return sp->wmin + (sp->wmax - sp->wmin) * u; }

static int spec3_propagate(const spectrometer3 *sp, const double q[4], double w, uint32_t *bin, double *t,
                           toric_stats *ts)
{
    ray3 r = fiber_ray(sp, q);
    int e = prism3_propagate(&sp->cp, &r, w, ts);
    if (e) return e;
    return detector3_hit(&sp->det, &r, bin, t);
}

/* ------------------------------------------------------------ API */

/* Qrng<[f64; 4]> from [seed; 4]: state_i = fract(state_i + alpha_i) (qrng.rs:157-255, with
 * ALPHA_4 = 1/phi_4^k, phi_4 the positive root of x^5 = x + 1). */
void orc3_qrng_points(double seed, size_t n, double *out)
{
    const double phi4 = 1.167303978261418684256045899854842180720560371525489039140082449275651903429527;
    const double alpha[4] = {1.0 / phi4, 1.0 / (phi4 * phi4), 1.0 / (phi4 * phi4 * phi4),
                             1.0 / (phi4 * phi4 * phi4 * phi4)};
    double st[4] = {seed, seed, seed, seed};
    for (size_t i = 0; i < n; i++)
        for (int k = 0; k < 4; k++) {
            st[k] = fractd(st[k] + alpha[k]);
            out[4 * i + k] = st[k];
        }
}

int orc3_position_detector(const orc_spec3 *s, double acceptance, double pos_out[2], int32_t *flipped_out)
{
    prism3 cp;
    int e = build_prism3(s, &cp);
    if (e) return e;
    /* detector_array_positioning (spectrometer.rs:322-364): Ray::new_from_start(median y) */
    ray3 r0 = {v3_make(0.0, s->fiber_center_y, 0.0), v3_make(1.0, 0.0, 0.0), 1.0, 1.0};
    double unaccepted_halved = fmax(1.0 - acceptance, 0.0) * 0.5;
    double wmin = s->base.wmin + (s->base.wmax - s->base.wmin) * unaccepted_halved;
    double wmax = s->base.wmin + (s->base.wmax - s->base.wmin) * (1.0 - unaccepted_halved);
    ray3 lower = r0, upper = r0;
    e = prism3_propagate(&cp, &lower, wmin, NULL);
    if (e) return e;
    e = prism3_propagate(&cp, &upper, wmax, NULL);
    if (e) return e;
    if ((lower.ts + lower.tp) * 0.5 <= 1e-3 || (upper.ts + upper.tp) * 0.5 <= 1e-3)
        return ORC_ANGULAR_RESPONSE_TOO_WEAK;
    /* fit_ray_difference_surface (geometry.rs:495-542) on the x/y components */
    v3 spec = v3_scale(v3_rot90(v3_angled(s->base.det_angle)), s->base.det_length);
    double a = upper.dir.x, b = -lower.dir.x, c = upper.dir.y, d = -lower.dir.y;
    double det = a * d - b * c;
    if (det == 0.0) return ORC_NO_SURFACE_INTERSECTION;
    double i10 = -c / det, i11 = a / det;
    v3 temp = v3_add(v3_sub(spec, upper.origin), lower.origin);
    double d2 = i10 * temp.x + i11 * temp.y;
    v3 vtx;
    if (d2 > 0.0) {
        vtx = v3_fma(lower.dir, d2, lower.origin);
        *flipped_out = 0;
    } else {
        temp = v3_add(v3_sub(v3_neg(spec), upper.origin), lower.origin);
        d2 = i10 * temp.x + i11 * temp.y;
        if (d2 < 0.0) return ORC_NO_SURFACE_INTERSECTION;
        vtx = v3_fma(lower.dir, d2, lower.origin);
        *flipped_out = 1;
    }
    pos_out[0] = vtx.x;
    pos_out[1] = vtx.y;
    return ORC_OK;
}

int orc3_trace_pairs(const orc_spec3 *s, const double *lam_u, const double *q, size_t n, uint32_t *bins,
                     double *ts, int32_t *status, uint32_t *nan_roots, uint32_t *toric_calls)
{
    spectrometer3 sp;
    int e = build_spectrometer3(s, &sp);
    if (e) return e;
    for (size_t i = 0; i < n; i++) {
        toric_stats st = {0, 0};
        uint32_t b = sp.det.bin_count;
        double t = 0.0;
        int r = spec3_propagate(&sp, q + 4 * i, sample_wavelength3(&sp, lam_u[i]), &b, &t, &st);
        bins[i] = r == ORC_OK ? b : sp.det.bin_count;
        ts[i] = r == ORC_OK ? t : 0.0;
        if (status) status[i] = r;
        if (nan_roots) nan_roots[i] = st.nan_roots;
        if (toric_calls) toric_calls[i] = (uint32_t)st.toric_calls;
    }
    return ORC_OK;
}

int orc3_fitness_points(const orc_spec3 *s, const double *lam_u, size_t W, const double *q, size_t R,
                        double *p_out, double stats[4], uint64_t *hits_out)
{
    spectrometer3 sp;
    int e = build_spectrometer3(s, &sp);
    if (e) return e;
    if (W == 0 || R == 0) return ORC_INVALID;
    uint32_t B = sp.det.bin_count;
    double *p = p_out ? p_out : (double *)malloc(sizeof(double) * W * B);
    double *pbar = (double *)calloc(B, sizeof(double));
    uint64_t hits = 0;
    double h_cond = 0.0;
    for (size_t k = 0; k < W; k++) {
        double w = sample_wavelength3(&sp, lam_u[k]);
        double *row = p + k * B;
        for (uint32_t b = 0; b < B; b++) row[b] = 0.0;
        for (size_t r = 0; r < R; r++) {
            uint32_t bin;
            double t;
            if (spec3_propagate(&sp, q + 4 * r, w, &bin, &t, NULL) == ORC_OK) {
                row[bin] += t;
                hits++;
            }
        }
        double h = 0.0;
        for (uint32_t b = 0; b < B; b++) {
            row[b] = row[b] / (double)R;
            h += plog2p(row[b]);
            pbar[b] += row[b];
        }
        h_cond += h;
    }
    h_cond /= (double)W;
    double h_det = 0.0;
    for (uint32_t b = 0; b < B; b++) h_det += plog2p(pbar[b] / (double)W);
    if (stats) {
        v3 mid = v3_fma(sp.det.direction, sp.det.length * 0.5, sp.det.position);
        double dx = mid.x, dy = mid.y - sp.fiber_center_y;
        stats[0] = h_cond - h_det;
        stats[1] = h_cond;
        stats[2] = h_det;
        stats[3] = sqrt(dx * dx + dy * dy + 0.0 * 0.0);
    }
    if (hits_out) *hits_out = hits;
    free(pbar);
    if (!p_out) free(p);
    return ORC_OK;
}
