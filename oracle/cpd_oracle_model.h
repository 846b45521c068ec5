/*
 * cpd_oracle_model.h -- TEST INFRASTRUCTURE ONLY (see cpd_oracle.h).
 *
 * The per-ray model of the oracle: the reference's 2-D spectrometer geometry, ray
 * trace and detector (src/spectrometer/{vector,utils,erf,geometry,ray,spectrometer}.rs),
 * written over the scalar type `real`. cpd_oracle.c includes it with real = double (the
 * oracle itself); the op-counting build (ops_count.cpp) includes it with a scalar that
 * counts every operation, so the work per ray is measured on this very code. Build with
 * -ffp-contract=off: every fused multiply-add is an explicit fma() at a site where the
 * Rust source calls `mul_add`. ORC_D(x) is the double value of a real.
 * Citations are paths inside the reference project.
 */
#ifndef CPD_ORACLE_MODEL_H
#define CPD_ORACLE_MODEL_H

typedef struct { real x, y; } v2;

static v2 v2_make(real x, real y) { v2 r = {x, y}; return r; }
static v2 v2_add(v2 a, v2 b) { return v2_make(a.x + b.x, a.y + b.y); }
static v2 v2_sub(v2 a, v2 b) { return v2_make(a.x - b.x, a.y - b.y); }
static v2 v2_scale(v2 a, real s) { return v2_make(a.x * s, a.y * s); }
static v2 v2_div(v2 a, real s) { return v2_make(a.x / s, a.y / s); }
static v2 v2_neg(v2 a) { return v2_make(-a.x, -a.y); }
/* Vector::dot = hadamard_product + reduce_sum (vector.rs:281-283, 489-495). */
static real v2_dot(v2 a, v2 b) { return a.x * b.x + a.y * b.y; }
/* SimdVector::mul_add: self * b + c fused per lane (vector.rs:497-503). */
static v2 v2_fma(v2 a, real b, v2 c) { return v2_make(fma(a.x, b, c.x), fma(a.y, b, c.y)); }
/* angled_xy / rot_180_xy / rot_90_xy / rot_90_ccw_xy (vector.rs:336-378). */
static v2 v2_angled(real th) { return v2_make(cos(th), sin(th)); }
static v2 v2_rot180(v2 a) { return v2_make(-a.x, -a.y); }
static v2 v2_rot90(v2 a) { return v2_make(-a.y, a.x); }
static v2 v2_rot90ccw(v2 a) { return v2_make(a.y, -a.x); }
static real sqr(real x) { return x * x; }
/* num_traits Float::fract = self - self.trunc(). */
static real fractd(real x) { return x - trunc(x); }
/* Float::is_sign_positive: true for +0 and positive values. */
static int sign_positive(real x) { return !signbit(x); }

/* ---------------------------------------------------------------- numerics */

/* Shaw's rational inverse normal CDF, src/spectrometer/erf.rs:27-73.
 * `polynomial` (erf.rs:8-16) is a Horner reduce with mul_add from the first
 * (highest-degree) coefficient. */
static const double SHAW_P[8] = {
    4.3304513840364031401e-8, 0.000036313870818023761224, 0.0034424140686962222423,
    0.085838533424158257377, 0.73176759583280610539, 2.3884158540184385711,
    3.0333178251950406994, 1.2533141359896652729};
static const double SHAW_Q[8] = {
    1.3141263119543315917e-6, 0.00030617264753008793976, 0.014494272424798068406,
    0.2168237095066675527, 1.2356513216582148689, 2.9373357991677046357,
    2.9202373175993672857, 1.0};

static real horner_k(const double *c, int n, real z)
{
    real s = c[0];
    for (int i = 1; i < n; i++) s = fma(s, z, c[i]);
    return s;
}

static real norminv_r(real x)
{
    real u = x > 0.5 ? 1.0 - x : x;
    real v = -log(2.0 * u);
    real p = horner_k(SHAW_P, 8, v);
    real q = horner_k(SHAW_Q, 8, v);
    return copysign(v * p / q, x - 0.5);
}

/* Glass::calc_n, src/spectrometer/glasscat.rs:17-22, on the prism's coefficients. The
 * reference evaluates it per ray and surface (ray.rs:490,494); it depends on the
 * wavelength alone, so the op-counting build books it as per-wavelength work
 * (ORC_PER_LAMBDA_BEGIN/END switch its counters; empty otherwise). */
#ifndef ORC_PER_LAMBDA_BEGIN
#define ORC_PER_LAMBDA_BEGIN
#define ORC_PER_LAMBDA_END
#endif
static real calc_n_r(const real *c, real w)
{
    ORC_PER_LAMBDA_BEGIN;
    real s = c[0];
    for (int i = 1; i < 6; i++) s = fma(s, w, c[i]);
    ORC_PER_LAMBDA_END;
    return s;
}

/* Welford, src/spectrometer/welford.rs:5-57. */
typedef struct { real count, mean, m2; } welford;

static void wf_next(welford *w, real x)
{
    w->count += 1.0;
    real delta = x - w->mean;
    w->mean += delta / w->count;
    real delta2 = x - w->mean;
    w->m2 += delta * delta2;
}

static void wf_skip(welford *w, real new_count)
{
    if (w->count < new_count) {
        real zero_count = new_count - w->count;
        real count = new_count;
        w->mean = (w->count * w->mean) / count;
        w->m2 += sqr(w->mean) * w->count * zero_count / count;
        w->count = count;
    }
}

static int wf_sem_le(const welford *w, real err2)
{
    return w->m2 < err2 * (w->count * (w->count - 1.0));
}

/* FloatExt::plog2p, src/spectrometer/utils.rs:196-202. */
static real plog2p(real p) { return p > 0.0 ? p * log2(p) : 0.0; }

/* FloatExt::euclid_div_rem, utils.rs:177-192. */
static void euclid_div_rem(real a, real b, real *q, real *r)
{
    real qq = trunc(a / b);
    real rr = a - qq * b;
    if (rr < 0.0) {
        *q = b > 0.0 ? qq - 1.0 : qq + 1.0;
        *r = rr + fabs(b);
    } else {
        *q = qq;
        *r = rr;
    }
}

/* Rust `f64 as u32`: saturating, NaN -> 0 (utils.rs:55-74 `v as $to`). */
static uint32_t sat_u32(real q)
{
    if (!(q == q)) return 0;
    if (q <= 0.0) return 0;
    if (q >= 4294967295.0) return 4294967295u;
    return (uint32_t)ORC_D(q);
}

/* ---------------------------------------------------------------- geometry */

typedef struct { v2 point, normal; } hyperplane;

typedef struct {
    int nglass, ar_coated;
    real glass[ORC_MAX_GLASS][6];
    real height;
    hyperplane planes[ORC_MAX_GLASS]; /* surface 0 .. G-1 (entry face + inner faces) */
    /* CurvedPlane exit face: SphericalLikeSurface + RadialBounds (geometry.rs:280-315) */
    v2 center;
    real radius;
    v2 bound_center;
    real bound_r2;
} prism;

typedef struct {
    uint32_t bin_count;
    real bin_size, slope, intercept, min_ci, length;
    v2 normal, position, direction;
} detector;

typedef struct {
    prism cp;
    detector det;
    real wmin, wmax, beam_width, beam_y_mean;
} spectrometer;

/* create_joined_trapezoids, src/spectrometer/geometry.rs:430-489, and
 * CompoundPrism::new (src/spectrometer/ray.rs:137-183) with the 2-D surface
 * types of the pyo3 CompoundPrism (src/pylib.rs:690-754). */
static int build_prism(const orc_spec *s, prism *cp)
{
    int G = s->nglass;
    if (G < 1 || G > ORC_MAX_GLASS) return ORC_INVALID;
    memset((void *)cp, 0, sizeof(*cp));
    cp->nglass = G;
    cp->ar_coated = s->ar_coated;
    cp->height = s->height;
    for (int g = 0; g < ORC_MAX_GLASS; g++)
        for (int i = 0; i < 6; i++) cp->glass[g][i] = s->glass[g][i];
    real h2 = s->height * 0.5;
    /* first face */
    v2 normal = v2_rot180(v2_angled(s->angles[0]));
    cp->planes[0].point = v2_make(fabs(normal.y / normal.x) * h2, h2);
    cp->planes[0].normal = normal;
    int prev_sign = sign_positive(normal.y);
    real d1 = cp->planes[0].point.x;
    real mx = cp->planes[0].point.x;
    /* array_prepend(first_sep_length, sep_lengths) (utils.rs:5-12): inner face i uses
     * lengths[i], the last face uses lengths[G-1]. Angles: inner faces angles[1..G-1],
     * last face angles[G]. */
    hyperplane last = {{0, 0}, {0, 0}};
    for (int k = 1; k <= G; k++) {
        real angle = s->angles[k];
        real sep_len = s->lengths[k - 1];
        v2 n = v2_rot180(v2_angled(angle));
        int sign = sign_positive(n.y);
        real d2 = fabs(n.y / n.x) * h2;
        real sep_dist = sep_len + (prev_sign != sign ? d1 + d2 : fabs(d1 - d2));
        prev_sign = sign;
        d1 = d2;
        mx += sep_dist;
        hyperplane hp = {v2_make(mx, h2), n};
        if (k < G) cp->planes[k] = hp;
        else last = hp;
    }
    /* CurvedPlane::from_hyperplane, geometry.rs:283-314. */
    real k_curv = s->curvature;
    real chord = fabs(s->height / last.normal.x); /* sec_xy (vector.rs:392-397) */
    real radius = chord * 0.5 / fabs(k_curv);
    real apothem = sqrt(sqr(radius) - sqr(chord) * 0.25);
    real sagitta = radius - apothem;
    cp->center = v2_fma(last.normal, copysign(apothem, k_curv), last.point);
    cp->radius = radius;
    cp->bound_center = v2_fma(last.normal, -copysign(sagitta, k_curv), last.point);
    cp->bound_r2 = sqr(sagitta) + sqr(chord) * 0.25;
    return ORC_OK;
}

/* LinearDetectorArray::new, src/spectrometer/spectrometer.rs:183-219, with
 * min_ci = cos(max_incident_angle) (src/pylib.rs:886). */
static void build_detector(const orc_spec *s, detector *d)
{
    d->bin_count = s->bin_count;
    d->bin_size = s->bin_size;
    d->slope = s->linear_slope;
    d->intercept = s->linear_intercept;
    d->min_ci = cos(s->max_incident_angle);
    d->length = s->det_length;
    d->normal = v2_rot180(v2_angled(s->det_angle));
    d->direction = s->det_flipped ? v2_rot90(d->normal) : v2_rot90ccw(d->normal);
    d->position = v2_make(s->det_position[0], s->det_position[1]);
}

static int build_spectrometer(const orc_spec *s, spectrometer *sp)
{
    int e = build_prism(s, &sp->cp);
    if (e) return e;
    if (s->bin_count == 0) return ORC_INVALID;
    build_detector(s, &sp->det);
    sp->wmin = s->wmin;
    sp->wmax = s->wmax;
    sp->beam_width = s->beam_width;
    sp->beam_y_mean = s->beam_y_mean;
    return ORC_OK;
}

/* ---------------------------------------------------------------- ray trace */

typedef struct { v2 origin, dir; real ts, tp; } ray;

/* Ray::new_from_start (ray.rs:277-279). */
static ray ray_start(real y)
{
    ray r = {{0.0, y}, {1.0, 0.0}, 1.0, 1.0};
    return r;
}

/* HyperPlane::intersection with PrismBounds 2-D (geometry.rs:124-145, 62-67). */
static int plane_intersect(const hyperplane *p, real height, const ray *r, real *dist)
{
    real ci = v2_dot(r->dir, p->normal);
    if (ci == 0.0) return 0;
    real d = v2_dot(v2_sub(p->point, r->origin), p->normal) / ci;
    if (d >= 0.0) {
        v2 h = v2_fma(r->dir, d, r->origin);
        if (0.0 <= h.y && h.y <= height) {
            *dist = d;
            return 1;
        }
    }
    return 0;
}

/* SphericalLikeSurface::intersection + RadialBounds (geometry.rs:161-216, 85-91). */
static int curved_intersect(const prism *cp, const ray *r, real *dist, v2 *normal)
{
    v2 delta = v2_sub(r->origin, cp->center);
    real ud = v2_dot(r->dir, delta);
    real disc = sqr(ud) - v2_dot(delta, delta) + sqr(cp->radius);
    if (!(disc > 0.0)) return 0; /* tangent and none are misses */
    real sd = sqrt(disc);
    real d1 = -ud - sd, d2 = -ud + sd;
    v2 p1 = v2_fma(r->dir, d1, r->origin);
    v2 p2 = v2_fma(r->dir, d2, r->origin);
    real dd;
    v2 p;
    if (sign_positive(d1) && v2_dot(v2_sub(p1, cp->bound_center), v2_sub(p1, cp->bound_center)) <= cp->bound_r2) {
        dd = d1;
        p = p1;
    } else if (sign_positive(d2) &&
               v2_dot(v2_sub(p2, cp->bound_center), v2_sub(p2, cp->bound_center)) <= cp->bound_r2) {
        dd = d2;
        p = p2;
    } else {
        return 0;
    }
    *dist = dd;
    *normal = v2_div(v2_sub(cp->center, p), cp->radius);
    return 1;
}

/* Ray::refract (ray.rs:309-367). */
static int refract(ray *r, v2 normal, real n1, real n2, int ar_coated)
{
    real ci = -v2_dot(r->dir, normal);
    real rr = n1 / n2;
    real cr_sq = 1.0 - sqr(rr) * (1.0 - sqr(ci));
    if (cr_sq < 0.0) return ORC_TOTAL_INTERNAL_REFLECTION;
    real cr = sqrt(cr_sq);
    v2 v = v2_add(v2_scale(r->dir, rr), v2_scale(normal, rr * ci - cr));
    real ts, tp;
    if (ar_coated && ci > 0.5) {
        ts = r->ts * 0.99;
        tp = r->tp * 0.99;
    } else {
        real rs = sqr((n1 * ci - n2 * cr) / (n1 * ci + n2 * cr));
        real rp = sqr((n1 * cr - n2 * ci) / (n1 * cr + n2 * ci));
        ts = r->ts * (1.0 - rs);
        tp = r->tp * (1.0 - rp);
    }
    r->dir = v;
    r->ts = ts;
    r->tp = tp;
    return ORC_OK;
}

/* surface_propagate (ray.rs:370-382): intersect, translate (ray.rs:281-294, a
 * fused mul_add), refract. */
static int plane_propagate(ray *r, const hyperplane *p, real height, real n1, real n2, int ar)
{
    real d;
    if (!plane_intersect(p, height, r, &d)) return ORC_NO_SURFACE_INTERSECTION;
    r->origin = v2_fma(r->dir, d, r->origin);
    return refract(r, p->normal, n1, n2, ar);
}

static int curved_propagate(ray *r, const prism *cp, real n1, real n2, int ar)
{
    real d;
    v2 normal;
    if (!curved_intersect(cp, r, &d, &normal)) return ORC_NO_SURFACE_INTERSECTION;
    r->origin = v2_fma(r->dir, d, r->origin);
    return refract(r, normal, n1, n2, ar);
}

/* CompoundPrism::propagate (ray.rs:485-499): air -> glass0 -> ... -> glass(G-1) -> air. */
static int prism_propagate(const prism *cp, ray *r, real w)
{
    real n1 = calc_n_r(cp->glass[0], w);
    int e = plane_propagate(r, &cp->planes[0], cp->height, 1.0, n1, cp->ar_coated);
    if (e) return e;
    for (int k = 1; k < cp->nglass; k++) {
        real n2 = calc_n_r(cp->glass[k], w);
        e = plane_propagate(r, &cp->planes[k], cp->height, n1, n2, cp->ar_coated);
        if (e) return e;
        n1 = n2;
    }
    return curved_propagate(r, cp, n1, 1.0, cp->ar_coated);
}

/* Ray::intersect_detector_array (ray.rs:390-402) with
 * LinearDetectorArray::{intersection, bin_index} (spectrometer.rs:265-303). */
static int detector_hit(const detector *dt, const ray *r, v2 *pos_out, uint32_t *bin, real *t)
{
    real ci = -v2_dot(r->dir, dt->normal);
    if (ci <= dt->min_ci) return ORC_ANGULAR_RESPONSE_TOO_WEAK;
    real d = v2_dot(v2_sub(r->origin, dt->position), dt->normal) / ci;
    v2 p = v2_fma(r->dir, d, r->origin);
    if (pos_out) *pos_out = p;
    real pos = v2_dot(v2_sub(p, dt->position), dt->direction);
    if (pos < 0.0 || dt->length < pos) return ORC_NO_SURFACE_INTERSECTION;
    real q, rem;
    euclid_div_rem(pos - dt->intercept, dt->slope, &q, &rem);
    uint32_t b = sat_u32(q);
    if (b < dt->bin_count && rem < dt->bin_size) {
        *bin = b;
        *t = (r->ts + r->tp) * 0.5; /* average_transmittance (ray.rs:297-299) */
        return ORC_OK;
    }
    return ORC_NO_SURFACE_INTERSECTION;
}

/* GaussianBeam 2-D inverse_cdf (spectrometer.rs:26-30). */
static real beam_y(const spectrometer *sp, real u)
{
    return sp->beam_y_mean - sp->beam_width * norminv_r(u);
}

/* UniformDistribution::inverse_cdf (distribution.rs:32-34). */
static real sample_wavelength(const spectrometer *sp, real u)
{
    return sp->wmin + (sp->wmax - sp->wmin) * u;
}

/* Spectrometer::propagate (spectrometer.rs:421-427). */
static int spec_propagate(const spectrometer *sp, real y, real w, uint32_t *bin, real *t)
{
    ray r = ray_start(y);
    int e = prism_propagate(&sp->cp, &r, w);
    if (e) return e;
    return detector_hit(&sp->det, &r, NULL, bin, t);
}

/* size_and_deviation + mid_pt (spectrometer.rs:429-437, 305-308). */
static void size_and_deviation(const spectrometer *sp, real *size, real *dev)
{
    v2 mid = v2_fma(sp->det.direction, sp->det.length * 0.5, sp->det.position);
    real dx = mid.x;
    real dy = mid.y - sp->beam_y_mean;
    v2 dv = v2_make(dx, dy);
    real sz = sqrt(v2_dot(dv, dv));
    *size = sz;
    *dev = fabs(dv.y / sz);
}

/* ------------------------------------------------------ detector positioning */

/* fit_ray_difference_surface (geometry.rs:495-542). */
static int fit_ray_difference_surface(const ray *lower, const ray *upper, real d_length,
                                      real d_angle, v2 *vertex, int32_t *flipped)
{
    v2 spec_dir = v2_rot90(v2_angled(d_angle));
    v2 spec = v2_scale(spec_dir, d_length);
    real a = upper->dir.x, b = -lower->dir.x, c = upper->dir.y, d = -lower->dir.y;
    real det = a * d - b * c;
    if (det == 0.0) return 0;
    real i10 = -c / det, i11 = a / det;
    v2 temp = v2_add(v2_sub(spec, upper->origin), lower->origin);
    real d2 = i10 * temp.x + i11 * temp.y;
    if (d2 > 0.0) {
        *vertex = v2_fma(lower->dir, d2, lower->origin);
        *flipped = 0;
        return 1;
    }
    temp = v2_add(v2_sub(v2_neg(spec), upper->origin), lower->origin);
    d2 = i10 * temp.x + i11 * temp.y;
    if (d2 < 0.0) return 0;
    *vertex = v2_fma(lower->dir, d2, lower->origin);
    *flipped = 1;
    return 1;
}


#endif
