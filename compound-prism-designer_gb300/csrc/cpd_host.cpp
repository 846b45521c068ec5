// cpd_host.cpp -- host side of the C ABI: design construction, detector
// positioning, the device-table conversion and the reference API's host methods
// (cpu_fitness, ray_trace, exit_ray). Compiled with -ffp-contract=off so the exact
// model in cpd_model.h gives the reference's f64 results.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "cpd_build.h"
#include "cpd_ff.h"
#include "cpd_host.h"
#include "cpd_model.h"

namespace cpd {

// f64 tables -> device record (cpd_build.h).
void design_to_dev(const cpd_design &d, DevDesign &D) { build::to_dev(d, D); }

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
    return build::position(*p, acceptance, position_out, *flipped_out);
}

int cpd_design_build(const cpd_spectrometer_params *p, cpd_design *out)
{
    if (!p || !out) return CPD_INVALID_ARGUMENT;
    cpd_design d;
    const int e = build::design(*p, d);
    if (e) return e;
    *out = d;
    return CPD_OK;
}

int cpd_design_build_batch(const cpd_spectrometer_params *p, uint32_t n, double acceptance, cpd_design *out,
                           int32_t *status)
{
    if ((!p || !out || !status) && n) return CPD_INVALID_ARGUMENT;
    if (acceptance != 0.0 && !(acceptance > 0.0 && acceptance <= 1.0)) return CPD_INVALID_ARGUMENT;
    for (uint32_t i = 0; i < n; i++) status[i] = build::design_positioned(p[i], acceptance, out[i]);
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
