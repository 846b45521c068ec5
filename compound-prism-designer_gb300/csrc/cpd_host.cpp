// cpd_host.cpp -- host side of the C ABI: design construction, detector
// positioning, the device-table conversion and the reference API's host methods
// (cpu_fitness, ray_trace, exit_ray). Compiled with -ffp-contract=off so the exact
// model in cpd_model.h gives the reference's f64 results.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "cpd_ff.h"
#include "cpd_host.h"
#include "cpd_model.h"

namespace cpd {

namespace {
struct V2 {
    double x, y;
};
V2 angled(double th) { return V2{std::cos(th), std::sin(th)}; }  // Vector::angled_xy (vector.rs:336-343)
V2 rot180(V2 a) { return V2{-a.x, -a.y}; }
V2 rot90(V2 a) { return V2{-a.y, a.x}; }
V2 rot90ccw(V2 a) { return V2{a.y, -a.x}; }
V2 vfma(V2 a, double b, V2 c) { return V2{std::fma(a.x, b, c.x), std::fma(a.y, b, c.y)}; }
}  // namespace

// create_joined_trapezoids (geometry.rs:430-489) and CurvedPlane::from_hyperplane
// (geometry.rs:283-314), into the cpd_design tables.
int build_prism(const cpd_spectrometer_params &p, cpd_design &d)
{
    const int G = p.nglass;
    if (G < 1 || G > CPD_MAX_GLASS) return CPD_INVALID_ARGUMENT;
    if (!(p.height > 0.0) || !(std::fabs(p.curvature) > 0.0) || !(std::fabs(p.curvature) <= 1.0))
        return CPD_INVALID_ARGUMENT;
    d.nglass = G;
    d.ar_coated = p.ar_coated ? 1 : 0;
    std::memcpy(d.glass, p.glass, sizeof(d.glass));
    d.height = p.height;
    const double h2 = p.height * 0.5;
    V2 n0 = rot180(angled(p.angles[0]));
    V2 pt0{std::fabs(n0.y / n0.x) * h2, h2};
    d.face_point[0][0] = pt0.x;
    d.face_point[0][1] = pt0.y;
    d.face_normal[0][0] = n0.x;
    d.face_normal[0][1] = n0.y;
    bool prev_sign = !std::signbit(n0.y);
    double d1 = pt0.x, mx = pt0.x;
    V2 last_pt{0, 0}, last_n{0, 0};
    // array_prepend (utils.rs:5-12): face k (1..G-1) uses lengths[k-1], the exit face lengths[G-1]
    for (int k = 1; k <= G; k++) {
        V2 n = rot180(angled(p.angles[k]));
        bool sign = !std::signbit(n.y);
        double d2 = std::fabs(n.y / n.x) * h2;
        double sep = p.lengths[k - 1] + (prev_sign != sign ? d1 + d2 : std::fabs(d1 - d2));
        prev_sign = sign;
        d1 = d2;
        mx += sep;
        if (k < G) {
            d.face_point[k][0] = mx;
            d.face_point[k][1] = h2;
            d.face_normal[k][0] = n.x;
            d.face_normal[k][1] = n.y;
        } else {
            last_pt = V2{mx, h2};
            last_n = n;
        }
    }
    const double kc = p.curvature;
    const double chord = std::fabs(p.height / last_n.x);
    const double radius = chord * 0.5 / std::fabs(kc);
    const double apothem = std::sqrt(radius * radius - chord * chord * 0.25);
    const double sagitta = radius - apothem;
    V2 c = vfma(last_n, std::copysign(apothem, kc), last_pt);
    V2 m = vfma(last_n, -std::copysign(sagitta, kc), last_pt);
    d.exit_center[0] = c.x;
    d.exit_center[1] = c.y;
    d.exit_radius = radius;
    d.exit_bound_center[0] = m.x;
    d.exit_bound_center[1] = m.y;
    d.exit_bound_r2 = sagitta * sagitta + chord * chord * 0.25;
    for (int k = 0; k < G; k++)
        if (!std::isfinite(d.face_point[k][0]) || !std::isfinite(d.face_normal[k][0])) return CPD_INVALID_ARGUMENT;
    if (!std::isfinite(radius) || !std::isfinite(apothem)) return CPD_INVALID_ARGUMENT;
    return CPD_OK;
}

void fill_source(const cpd_spectrometer_params &p, cpd_design &d)
{
    d.wavelength_bounds[0] = p.wavelength_bounds[0];
    d.wavelength_bounds[1] = p.wavelength_bounds[1];
    d.beam_width = p.beam_width;
    d.beam_y_mean = p.beam_y_mean;
}

// f64 tables -> device record (exact part copied, FP32 fast-path constants derived in f64).
void design_to_dev(const cpd_design &d, DevDesign &D)
{
    std::memset(&D, 0, sizeof(D));
    D.G = d.nglass;
    D.B = d.bin_count;
    D.ar = d.ar_coated;
    std::memcpy(D.glass, d.glass, sizeof(D.glass));
    for (int k = 0; k < CPD_MAX_GLASS; k++) {
        D.ppx[k] = d.face_point[k][0];
        D.ppy[k] = d.face_point[k][1];
        D.pnx[k] = d.face_normal[k][0];
        D.pny[k] = d.face_normal[k][1];
    }
    D.height = d.height;
    D.ccx = d.exit_center[0];
    D.ccy = d.exit_center[1];
    D.crad = d.exit_radius;
    D.cbx = d.exit_bound_center[0];
    D.cby = d.exit_bound_center[1];
    D.cbr2 = d.exit_bound_r2;
    D.bin_size = d.bin_size;
    D.slope = d.linear_slope;
    D.intercept = d.linear_intercept;
    D.min_ci = d.min_ci;
    D.L = d.det_length;
    D.dnx = d.det_normal[0];
    D.dny = d.det_normal[1];
    D.dpx = d.det_position[0];
    D.dpy = d.det_position[1];
    D.dux = d.det_direction[0];
    D.duy = d.det_direction[1];
    D.wmin = d.wavelength_bounds[0];
    D.wmax = d.wavelength_bounds[1];
    D.bw = d.beam_width;
    D.bym = d.beam_y_mean;
    FastConst &f = D.fc;
    f.inv_rc = (float)(1.0 / D.crad);
    f.rho = (float)std::sqrt(D.cbr2);
    f.rho2 = (float)D.cbr2;
    f.dnfx = (float)D.dnx;
    f.dnfy = (float)D.dny;
    f.dufx = (float)D.dux;
    f.dufy = (float)D.duy;
    f.min_ci = (float)D.min_ci;
    f.L = (float)D.L;
    f.c0 = (float)D.intercept;
    f.slope = (float)D.slope;
    f.inv_slope = (float)(1.0 / D.slope);
    f.bin_size = (float)D.bin_size;
    f.bw = (float)D.bw;
    f.hL = (float)(0.5 * D.L);
    f.ar = D.ar;
    f.B = D.B;
    DFConst &c = D.dc;
    auto sp = [](double v) {
        ff::F2 r;
        ff::split(v, r.hi, r.lo);
        return r;
    };
    for (int k = 0; k < CPD_MAX_GLASS; k++) {
        for (int i = 0; i < 6; i++) c.glass[k][i] = sp(D.glass[k][i]);
        c.ppx[k] = sp(D.ppx[k]);
        c.ppy[k] = sp(D.ppy[k]);
        c.pnx[k] = sp(D.pnx[k]);
        c.pny[k] = sp(D.pny[k]);
    }
    c.height = sp(D.height);
    c.ccx = sp(D.ccx);
    c.ccy = sp(D.ccy);
    c.rc2 = sp(D.crad * D.crad);
    c.irc = sp(1.0 / D.crad);
    c.cbx = sp(D.cbx);
    c.cby = sp(D.cby);
    c.cbr2 = sp(D.cbr2);
    c.vx = sp(D.cbx - D.ccx);
    c.vy = sp(D.cby - D.ccy);
    c.bin_size = sp(D.bin_size);
    c.slope = sp(D.slope);
    c.islope = sp(1.0 / D.slope);
    c.intercept = sp(D.intercept);
    c.min_ci = sp(D.min_ci);
    c.L = sp(D.L);
    c.dnx = sp(D.dnx);
    c.dny = sp(D.dny);
    c.dpx = sp(D.dpx);
    c.dpy = sp(D.dpy);
    c.dux = sp(D.dux);
    c.duy = sp(D.duy);
    c.qx = sp(D.dpx - D.cbx);
    c.qy = sp(D.dpy - D.cby);
    c.wmin = sp(D.wmin);
    c.wspan = sp(D.wmax - D.wmin);
    c.bw = sp(D.bw);
    c.bym = sp(D.bym);
}

// Shaw's inverse normal CDF (erf.rs:27-73), host-side: the ray tables are built here
// so that the device never evaluates a logarithm on the exact path.
double norminv(double x)
{
    static const double P[8] = {4.3304513840364031401e-8, 0.000036313870818023761224,
                                0.0034424140686962222423, 0.085838533424158257377,
                                0.73176759583280610539,   2.3884158540184385711,
                                3.0333178251950406994,    1.2533141359896652729};
    static const double Q[8] = {1.3141263119543315917e-6, 0.00030617264753008793976,
                                0.014494272424798068406,  0.2168237095066675527,
                                1.2356513216582148689,    2.9373357991677046357,
                                2.9202373175993672857,    1.0};
    const double u = x > 0.5 ? 1.0 - x : x;
    const double v = -std::log(2.0 * u);
    double p = P[0], q = Q[0];
    for (int i = 1; i < 8; i++) {
        p = std::fma(p, v, P[i]);
        q = std::fma(q, v, Q[i]);
    }
    return std::copysign(v * p / q, x - 0.5);
}

void ray_table(const double *ray_u, uint32_t R, std::vector<double> &z64, std::vector<float> &z32,
               std::vector<uint32_t> *rank)
{
    std::vector<std::pair<double, uint32_t>> zj;
    zj.reserve(R);
    for (uint32_t j = 0; j < R; j++) {
        double z = norminv(ray_u[j]);
        if (std::isfinite(z)) zj.emplace_back(z, j);  // a non-finite start height never reaches a face
    }
    std::sort(zj.begin(), zj.end());
    z64.resize(zj.size());
    z32.resize(2 * zj.size());
    if (rank) rank->assign(R, 0xffffffffu);
    for (size_t i = 0; i < zj.size(); i++) {
        z64[i] = zj[i].first;
        split_f32(z64[i], z32[2 * i], z32[2 * i + 1]);
        if (rank) (*rank)[zj[i].second] = (uint32_t)i;
    }
}

// The GPU point policy: u_i = fract(fma(i0 + i, 1/phi, seed)) (kernel.rs:128-130 in f64).
void seed_points(double seed, uint32_t first, uint32_t n, double *out)
{
    for (uint32_t i = 0; i < n; i++) {
        double v = std::fma((double)(first + i), kAlpha, seed);
        out[i] = v - std::trunc(v);
    }
}

}  // namespace cpd

using namespace cpd;

extern "C" {

int cpd_abi_version(void) { return CPD_ABI_VERSION; }

const char *cpd_status_string(int s)
{
    switch (s) {
    case CPD_OK: return "OK";
    case CPD_NOT_CONVERGED: return "NotConverged";
    case CPD_RAYTRACE_NO_SURFACE_INTERSECTION: return "NoSurfaceIntersection";
    case CPD_RAYTRACE_OUT_OF_BOUNDS: return "OutOfBounds";
    case CPD_RAYTRACE_TOTAL_INTERNAL_REFLECTION: return "TotalInternalReflection";
    case CPD_RAYTRACE_ANGULAR_RESPONSE_TOO_WEAK: return "SpectrometerAngularResponseTooWeak";
    case CPD_INVALID_ARGUMENT: return "InvalidArgument";
    case CPD_CUDA_ERROR: return "CudaError";
    case CPD_TIMEOUT: return "Timeout";
    case CPD_NO_CAPACITY: return "NoCapacity";
    case CPD_NOT_IMPLEMENTED: return "NotImplemented";
    default: return "Unknown";
    }
}

double cpd_norminv(double u) { return cpd::norminv(u); }

double cpd_glass_index(const double coeffs[6], double w) { return x::calc_n(coeffs, w); }

int cpd_entropy_log2(uint64_t count, double out[2])
{
    if (!out || count == 0) return CPD_INVALID_ARGUMENT;
    static float tab[4 * ff::kLogTable];
    static bool ready = [] {
        ff::make_log_table(tab);
        return true;
    }();
    (void)ready;
    const ff::F2 l = ff::log2_u64(count, tab);
    out[0] = l.hi;
    out[1] = l.lo;
    return CPD_OK;
}

int cpd_position_detector_array(const cpd_spectrometer_params *p, double acceptance, double position_out[2],
                                int32_t *flipped_out)
{
    if (!p || !position_out || !flipped_out) return CPD_INVALID_ARGUMENT;
    if (!(acceptance > 0.0) || !(acceptance <= 1.0)) return CPD_INVALID_ARGUMENT;
    cpd_design d;
    std::memset(&d, 0, sizeof(d));
    int e = build_prism(*p, d);
    if (e) return e;
    fill_source(*p, d);
    DevDesign D;
    design_to_dev(d, D);
    // detector_array_positioning (spectrometer.rs:322-364)
    const double uh = std::max(1.0 - acceptance, 0.0) * 0.5;
    const double wmin = x::wavelength(D, uh);
    const double wmax = x::wavelength(D, 1.0 - uh);
    x::Ray lo{0.0, D.bym, 1.0, 0.0, 1.0, 1.0}, up = lo;
    e = x::prism(D, wmin, lo);
    if (e) return e;
    e = x::prism(D, wmax, up);
    if (e) return e;
    if ((lo.ts + lo.tp) * 0.5 <= 1e-3 || (up.ts + up.tp) * 0.5 <= 1e-3) return CPD_RAYTRACE_ANGULAR_RESPONSE_TOO_WEAK;
    // fit_ray_difference_surface (geometry.rs:495-542)
    V2 spec_dir = rot90(angled(p->det_angle));
    V2 spec{spec_dir.x * p->det_length, spec_dir.y * p->det_length};
    const double a = up.dx, b = -lo.dx, c = up.dy, dd = -lo.dy;
    const double det = a * dd - b * c;
    if (det == 0.0) return CPD_RAYTRACE_NO_SURFACE_INTERSECTION;
    const double i10 = -c / det, i11 = a / det;
    double tx = (spec.x - up.ox) + lo.ox, ty = (spec.y - up.oy) + lo.oy;
    double d2 = i10 * tx + i11 * ty;
    int32_t flipped = 0;
    if (!(d2 > 0.0)) {
        tx = (-spec.x - up.ox) + lo.ox;
        ty = (-spec.y - up.oy) + lo.oy;
        d2 = i10 * tx + i11 * ty;
        if (d2 < 0.0) return CPD_RAYTRACE_NO_SURFACE_INTERSECTION;
        flipped = 1;
    }
    position_out[0] = std::fma(lo.dx, d2, lo.ox);
    position_out[1] = std::fma(lo.dy, d2, lo.oy);
    *flipped_out = flipped;
    return CPD_OK;
}

int cpd_design_build(const cpd_spectrometer_params *p, cpd_design *out)
{
    if (!p || !out) return CPD_INVALID_ARGUMENT;
    if (p->bin_count == 0 || p->bin_count > CPD_MAX_BINS) return CPD_INVALID_ARGUMENT;
    if (!(p->linear_slope > 0.0) || !(p->bin_size > 0.0) || !(p->det_length > 0.0)) return CPD_INVALID_ARGUMENT;
    if (!(p->wavelength_bounds[1] >= p->wavelength_bounds[0])) return CPD_INVALID_ARGUMENT;
    cpd_design d;
    std::memset(&d, 0, sizeof(d));
    int e = build_prism(*p, d);
    if (e) return e;
    fill_source(*p, d);
    // LinearDetectorArray::new (spectrometer.rs:183-219), min_ci = cos (src/pylib.rs:886)
    d.bin_count = p->bin_count;
    d.bin_size = p->bin_size;
    d.linear_slope = p->linear_slope;
    d.linear_intercept = p->linear_intercept;
    d.min_ci = std::cos(p->max_incident_angle);
    d.det_length = p->det_length;
    V2 n = rot180(angled(p->det_angle));
    V2 u = p->det_flipped ? rot90(n) : rot90ccw(n);
    d.det_normal[0] = n.x;
    d.det_normal[1] = n.y;
    d.det_direction[0] = u.x;
    d.det_direction[1] = u.y;
    d.det_position[0] = p->det_position[0];
    d.det_position[1] = p->det_position[1];
    // size_and_deviation + mid_pt (spectrometer.rs:429-437, 305-308)
    V2 mid = vfma(u, p->det_length * 0.5, V2{d.det_position[0], d.det_position[1]});
    const double dx = mid.x, dy = mid.y - p->beam_y_mean;
    const double size = std::sqrt(dx * dx + dy * dy);
    d.size = size;
    d.deviation = std::fabs(dy / size);
    *out = d;
    return CPD_OK;
}

int cpd_design_build_batch(const cpd_spectrometer_params *p, uint32_t n, double acceptance, cpd_design *out,
                           int32_t *status)
{
    if ((!p || !out || !status) && n) return CPD_INVALID_ARGUMENT;
    if (acceptance != 0.0 && !(acceptance > 0.0 && acceptance <= 1.0)) return CPD_INVALID_ARGUMENT;
    for (uint32_t i = 0; i < n; i++) {
        cpd_spectrometer_params q = p[i];
        int e = CPD_OK;
        if (acceptance > 0.0) e = cpd_position_detector_array(&q, acceptance, q.det_position, &q.det_flipped);
        if (!e) e = cpd_design_build(&q, &out[i]);
        if (e) std::memset(&out[i], 0, sizeof(cpd_design));
        status[i] = e;
    }
    return CPD_OK;
}

int cpd_exit_ray(const cpd_design *d, double y, double wavelength, double out[4])
{
    if (!d || !out) return CPD_INVALID_ARGUMENT;
    DevDesign D;
    design_to_dev(*d, D);
    x::Ray r{0.0, y, 1.0, 0.0, 1.0, 1.0};
    int e = x::prism(D, wavelength, r);
    if (e) return e;
    out[0] = r.ox;
    out[1] = r.oy;
    out[2] = r.dx;
    out[3] = r.dy;
    return CPD_OK;
}

int cpd_ray_trace(const cpd_design *d, double wavelength, double initial_y, double *rows, uint32_t *nrows)
{
    if (!d || !rows || !nrows) return CPD_INVALID_ARGUMENT;
    DevDesign D;
    design_to_dev(*d, D);
    // propagate_trace + propagation_path (ray.rs:501-541, spectrometer.rs:439-464)
    uint32_t n = 0;
    auto row = [&](const x::Ray &r) {
        rows[4 * n + 0] = r.ox;
        rows[4 * n + 1] = r.oy;
        rows[4 * n + 2] = r.dx;
        rows[4 * n + 3] = r.dy;
        n++;
    };
    x::Ray r{0.0, initial_y, 1.0, 0.0, 1.0, 1.0};
    row(r);
    double n1 = x::calc_n(D.glass[0], wavelength);
    bool ok = x::flat_face(D, 0, r, 1.0, n1) == 0;
    if (ok) row(r);
    for (int k = 1; ok && k < D.G; k++) {
        double n2 = x::calc_n(D.glass[k], wavelength);
        ok = x::flat_face(D, k, r, n1, n2) == 0;
        if (ok) row(r);
        n1 = n2;
    }
    if (ok && x::exit_face(D, r, n1) == 0) row(r);
    uint32_t bin;
    double t, hx, hy;
    if (x::detector(D, r, bin, t, &hx, &hy) == 0) {
        x::Ray last = r;
        last.ox = hx;
        last.oy = hy;
        row(last);
    }
    *nrows = n;
    return CPD_OK;
}

// Spectrometer.cpu_fitness: the reference's adaptive estimator (fitness.rs:5-147),
// including its Welford `skip` bookkeeping, in f64 on the host.
int cpd_fitness_cpu(const cpd_design *d, uint64_t max_n, uint64_t max_m, cpd_fitness *out)
{
    if (!d || !out || d->bin_count == 0) return CPD_INVALID_ARGUMENT;
    DevDesign D;
    design_to_dev(*d, D);
    const uint32_t B = D.B;
    struct W {
        double count = 0, mean = 0, m2 = 0;
        void next(double x)
        {
            count += 1.0;
            double delta = x - mean;
            mean += delta / count;
            m2 += delta * (x - mean);
        }
        void skip(double c)
        {
            if (count < c) {
                double zc = c - count;
                mean = (count * mean) / c;
                m2 += mean * mean * count * zc / c;
                count = c;
            }
        }
        bool sem_le(double e2) const { return m2 < e2 * (count * (count - 1.0)); }
    };
    const double e2 = 5e-3 * 5e-3;
    std::vector<W> pd(B), row(B);
    W hcond;
    uint64_t rays = 0, hits = 0;
    double st = 0.5;
    uint64_t n_rows = 0;
    for (uint64_t it = 0; it < max_n; it++) {
        st = st + kAlpha;
        st = st - std::trunc(st);
        const double w = x::wavelength(D, st);
        for (auto &v : row) v = W();
        double count = 0.0, sr = 0.5;
        for (uint64_t m = 0; m < max_m; m++) {
            sr = sr + kAlpha;
            sr = sr - std::trunc(sr);
            count += 1.0;
            rays++;
            uint32_t bin;
            double t;
            if (x::trace(D, w, x::beam_y(D, norminv(sr)), bin, t) == 0) {
                hits++;
                row[bin].skip(count);
                row[bin].next(t);
                if (row[bin].sem_le(e2)) break;
            }
        }
        double h = 0.0;
        for (uint32_t b = 0; b < B; b++) {
            row[b].skip(count);
            const double p = row[b].mean;
            pd[b].next(p);
            h += p > 0.0 ? p * std::log2(p) : 0.0;
        }
        hcond.next(h);
        n_rows++;
        bool all = true;
        for (uint32_t b = 0; b < B && all; b++) all = pd[b].sem_le(e2);
        if (all) break;
    }
    double hdet = 0.0, max_sem = 0.0;
    for (uint32_t b = 0; b < B; b++) {
        const double p = pd[b].mean;
        hdet = hdet + (p > 0.0 ? p * std::log2(p) : 0.0);
        const double sem = std::sqrt(pd[b].m2 / (pd[b].count - 1.0) / pd[b].count);
        if (std::isfinite(sem)) max_sem = std::max(max_sem, sem);
    }
    std::memset(out, 0, sizeof(*out));
    out->size = d->size;
    out->deviation = d->deviation;
    out->info = hcond.mean - hdet;
    out->h_cond = hcond.mean;
    out->h_det = hdet;
    out->max_sem = max_sem;
    out->rays = rays;
    out->hits = hits;
    out->wavelengths = (uint32_t)n_rows;
    out->status = CPD_OK;
    return CPD_OK;
}

}  // extern "C"
