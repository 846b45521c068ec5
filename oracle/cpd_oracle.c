/*
 * cpd_oracle.c -- TEST INFRASTRUCTURE ONLY (see cpd_oracle.h).
 *
 * Double-precision restatement of the reference's 2-D compound-prism
 * spectrometer model and CPU fitness estimator. Build with -ffp-contract=off:
 * every fused multiply-add below is an explicit fma() at a site where the Rust
 * source calls `mul_add` (scalar mul_add, or the std SimdVector mul_add which is
 * `Simd::mul_add`, fused, src/spectrometer/vector.rs:497-503). Dot products are
 * the un-fused `hadamard_product(..).reduce_sum()` of vector.rs:281-283.
 * Citations are paths inside the reference project.
 */
#include "cpd_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

typedef double real;
#define ORC_D(x) (x)
#include "cpd_oracle_model.h"

/* ---------------------------------------------------------------- numerics */

/* Shaw's inverse normal CDF (src/spectrometer/erf.rs:62-73). */
double orc_norminv(double x) { return norminv_r(x); }

/* Glass::calc_n, src/spectrometer/glasscat.rs:17-22. */
double orc_calc_n(const double coeffs[6], double w) { return horner_k(coeffs, 6, w); }

/* Qrng 1-D: alpha = 1/phi (qrng.rs:156-158); next() = state.iadd_mod_1(alpha)
 * = fract(state + alpha) (qrng.rs:217-219, 248-254). */
static const double ORC_ALPHA = 1.0 / 1.61803398874989484820458683436563;

void orc_qrng_points(double seed, size_t n, double *out)
{
    double st = seed;
    for (size_t i = 0; i < n; i++) {
        st = fractd(st + ORC_ALPHA);
        out[i] = st;
    }
}

/* The GPU seed policy of the library under test (u_i = fract(fma(first + i, 1/phi, seed)),
 * the golden-ratio points of src/spectrometer/kernel.rs:128-130 computed in f64 from the
 * index), so that a check runs on the very points the GPU call used. */
void orc_gpu_points(double seed, uint64_t first, size_t n, double *out)
{
    for (size_t i = 0; i < n; i++) out[i] = fractd(fma((double)(first + i), ORC_ALPHA, seed));
}


int orc_position_detector(const orc_spec *s, double acceptance, double pos_out[2], int32_t *flipped_out)
{
    prism cp;
    int e = build_prism(s, &cp);
    if (e) return e;
    spectrometer sp;
    sp.wmin = s->wmin;
    sp.wmax = s->wmax;
    /* detector_array_positioning, spectrometer.rs:322-364 */
    ray r0 = ray_start(s->beam_y_mean);
    double unaccepted_halved = fmax(1.0 - acceptance, 0.0) * 0.5;
    double wmin = sample_wavelength(&sp, unaccepted_halved);
    double wmax = sample_wavelength(&sp, 1.0 - unaccepted_halved);
    ray lower = r0, upper = r0;
    e = prism_propagate(&cp, &lower, wmin);
    if (e) return e;
    e = prism_propagate(&cp, &upper, wmax);
    if (e) return e;
    if ((lower.ts + lower.tp) * 0.5 <= 1e-3 || (upper.ts + upper.tp) * 0.5 <= 1e-3)
        return ORC_ANGULAR_RESPONSE_TOO_WEAK;
    v2 vtx;
    if (!fit_ray_difference_surface(&lower, &upper, s->det_length, s->det_angle, &vtx, flipped_out))
        return ORC_NO_SURFACE_INTERSECTION;
    pos_out[0] = vtx.x;
    pos_out[1] = vtx.y;
    return ORC_OK;
}

/* ---------------------------------------------------------------- API */

int orc_propagate(const orc_spec *s, double wavelength, double ray_u, uint32_t *bin, double *t)
{
    spectrometer sp;
    int e = build_spectrometer(s, &sp);
    if (e) return e;
    return spec_propagate(&sp, beam_y(&sp, ray_u), wavelength, bin, t);
}

int orc_design_dump(const orc_spec *s, double *out)
{
    spectrometer sp;
    int e = build_spectrometer(s, &sp);
    if (e) return e;
    int G = sp.cp.nglass, k = 0;
    for (int i = 0; i < G; i++) {
        out[k++] = sp.cp.planes[i].point.x;
        out[k++] = sp.cp.planes[i].point.y;
        out[k++] = sp.cp.planes[i].normal.x;
        out[k++] = sp.cp.planes[i].normal.y;
    }
    out[k++] = sp.cp.center.x;
    out[k++] = sp.cp.center.y;
    out[k++] = sp.cp.radius;
    out[k++] = sp.cp.bound_center.x;
    out[k++] = sp.cp.bound_center.y;
    out[k++] = sp.cp.bound_r2;
    out[k++] = sp.det.normal.x;
    out[k++] = sp.det.normal.y;
    out[k++] = sp.det.direction.x;
    out[k++] = sp.det.direction.y;
    out[k++] = sp.det.min_ci;
    size_and_deviation(&sp, &out[k], &out[k + 1]);
    return ORC_OK;
}

int orc_propagation_path(const orc_spec *s, double wavelength, double initial_y, double *rows)
{
    spectrometer sp;
    int e = build_spectrometer(s, &sp);
    if (e) return -e;
    const prism *cp = &sp.cp;
    ray r = ray_start(initial_y);
    int n = 0;
#define ORC_ROW(rr)                  \
    do {                             \
        rows[4 * n + 0] = (rr).origin.x; \
        rows[4 * n + 1] = (rr).origin.y; \
        rows[4 * n + 2] = (rr).dir.x;    \
        rows[4 * n + 3] = (rr).dir.y;    \
        n++;                         \
    } while (0)
    /* propagate_trace (ray.rs:501-541) yields the start ray and each refracted ray
     * until the first error; propagation_path (spectrometer.rs:439-464) then tries
     * the detector with the last ray it yielded, whether or not the prism trace
     * reached the exit face. */
    ORC_ROW(r);
    double n1 = orc_calc_n(cp->glass[0], wavelength);
    ray nr0 = r;
    int ok = plane_propagate(&nr0, &cp->planes[0], cp->height, 1.0, n1, cp->ar_coated) == ORC_OK;
    if (ok) {
        r = nr0;
        ORC_ROW(r);
    }
    for (int k = 1; ok && k < cp->nglass; k++) {
        double n2 = orc_calc_n(cp->glass[k], wavelength);
        ray nr = r;
        ok = plane_propagate(&nr, &cp->planes[k], cp->height, n1, n2, cp->ar_coated) == ORC_OK;
        if (ok) {
            r = nr;
            ORC_ROW(r);
        }
        n1 = n2;
    }
    if (ok) {
        ray nr = r;
        if (curved_propagate(&nr, cp, n1, 1.0, cp->ar_coated) == ORC_OK) {
            r = nr;
            ORC_ROW(r);
        }
    }
    v2 p;
    uint32_t b;
    double t;
    if (detector_hit(&sp.det, &r, &p, &b, &t) == ORC_OK) {
        ray last = r;
        last.origin = p;
        ORC_ROW(last);
    }
#undef ORC_ROW
    return n;
}

int orc_stop_face(const orc_spec *s, double wavelength, double initial_y, int *status)
{
    spectrometer sp;
    int e = build_spectrometer(s, &sp);
    if (e) return -(100 + e);
    const prism *cp = &sp.cp;
    ray r = ray_start(initial_y);
    double n1 = orc_calc_n(cp->glass[0], wavelength);
    *status = plane_propagate(&r, &cp->planes[0], cp->height, 1.0, n1, cp->ar_coated);
    if (*status != ORC_OK) return 0;
    for (int k = 1; k < cp->nglass; k++) {
        double n2 = orc_calc_n(cp->glass[k], wavelength);
        *status = plane_propagate(&r, &cp->planes[k], cp->height, n1, n2, cp->ar_coated);
        if (*status != ORC_OK) return k;
        n1 = n2;
    }
    *status = curved_propagate(&r, cp, n1, 1.0, cp->ar_coated);
    return *status != ORC_OK ? cp->nglass : -1;
}

/* vector_quasi_monte_carlo_integration + p_dets_l_wavelength (fitness.rs:5-34, 48-69).
 * Returns the rays consumed (the integration's final `count`). */
static size_t p_dets_adaptive(const spectrometer *sp, double w, size_t max_m, welford *stats)
{
    uint32_t nbin = sp->det.bin_count;
    const double max_err = 5e-3;
    const double max_err_sq = max_err * max_err;
    for (uint32_t i = 0; i < nbin; i++) stats[i].count = stats[i].mean = stats[i].m2 = 0.0;
    double count = 0.0;
    double st = 0.5;
    for (size_t it = 0; it < max_m; it++) {
        st = fractd(st + ORC_ALPHA);
        count += 1.0;
        uint32_t bin;
        double t;
        if (spec_propagate(sp, beam_y(sp, st), w, &bin, &t) == ORC_OK) {
            wf_skip(&stats[bin], count);
            wf_next(&stats[bin], t);
            if (wf_sem_le(&stats[bin], max_err_sq)) break;
        }
    }
    for (uint32_t i = 0; i < nbin; i++) wf_skip(&stats[i], count);
    return (size_t)count;
}

int orc_p_dets_l_wavelength_count(const orc_spec *s, double wavelength, size_t max_m, double *out,
                                  uint64_t *rays_out)
{
    spectrometer sp;
    int e = build_spectrometer(s, &sp);
    if (e) return e;
    welford *stats = (welford *)calloc(sp.det.bin_count, sizeof(welford));
    if (!stats) return ORC_INVALID;
    size_t c = p_dets_adaptive(&sp, wavelength, max_m, stats);
    for (uint32_t i = 0; i < sp.det.bin_count; i++) out[i] = stats[i].mean;
    if (rays_out) *rays_out = c;
    free(stats);
    return ORC_OK;
}

int orc_p_dets_l_wavelength(const orc_spec *s, double wavelength, size_t max_m, double *out)
{
    return orc_p_dets_l_wavelength_count(s, wavelength, max_m, out, NULL);
}

/* mutual_information + fitness (fitness.rs:79-147). */
int orc_fitness_adaptive(const orc_spec *s, size_t max_n, size_t max_m, double out[3])
{
    return orc_fitness_adaptive_work(s, max_n, max_m, out, NULL, NULL);
}

int orc_fitness_adaptive_work(const orc_spec *s, size_t max_n, size_t max_m, double out[3], uint64_t *wavelengths_out,
                              uint64_t *rays_out)
{
    uint64_t n_w = 0, n_r = 0;
    spectrometer sp;
    int e = build_spectrometer(s, &sp);
    if (e) return e;
    uint32_t nbin = sp.det.bin_count;
    welford *p_dets = (welford *)calloc(nbin, sizeof(welford));
    welford *row = (welford *)calloc(nbin, sizeof(welford));
    if (!p_dets || !row) {
        free(p_dets);
        free(row);
        return ORC_INVALID;
    }
    welford h_det_l_w = {0, 0, 0};
    const double max_err_sqr = 5e-3 * 5e-3;
    double st = 0.5;
    for (size_t it = 0; it < max_n; it++) {
        st = fractd(st + ORC_ALPHA);
        double w = sample_wavelength(&sp, st);
        n_r += p_dets_adaptive(&sp, w, max_m, row);
        n_w++;
        double h = 0.0;
        for (uint32_t i = 0; i < nbin; i++) {
            wf_next(&p_dets[i], row[i].mean);
            h += plog2p(row[i].mean);
        }
        wf_next(&h_det_l_w, h);
        int all = 1;
        for (uint32_t i = 0; i < nbin; i++)
            if (!wf_sem_le(&p_dets[i], max_err_sqr)) {
                all = 0;
                break;
            }
        if (all) break;
    }
    double h_det = 0.0;
    for (uint32_t i = 0; i < nbin; i++) h_det = h_det + plog2p(p_dets[i].mean);
    double size, dev;
    size_and_deviation(&sp, &size, &dev);
    out[0] = size;
    out[1] = h_det_l_w.mean - h_det;
    out[2] = dev;
    if (wavelengths_out) *wavelengths_out = n_w;
    if (rays_out) *rays_out = n_r;
    free(p_dets);
    free(row);
    return ORC_OK;
}

/* --------------------------------------------- fixed-N on explicit point sets */

typedef struct {
    const spectrometer *sp;
    const double *lam_u, *ys;
    size_t W, R;
    double *p;          /* W*B */
    uint64_t hits;
    size_t k0, k1;
    int adaptive;
    uint32_t *counts;   /* W (adaptive): rays consumed per wavelength */
} fixed_job;

/* ------------------------------------ adaptive sampling on explicit point sets
 *
 * The per-wavelength stop of the reference GPU kernel (src/spectrometer/kernel.rs:
 * 127-178): rays in the given order, 32 per round (the last round may be shorter; the
 * reference rounds max_evals down to a multiple of 32, kernel.rs:137). After a round,
 * each bin the round hit merges a Welford state of the round's samples (its hits' t, zeros
 * for the other rays; kernel.rs:147-170, welford.rs:59-91); the wavelength stops after
 * a round that hit some bin and after which every bin it hit passes
 * sem_le_error_threshold with (5e-3)^2 (welford.rs:80-84, kernel.rs:170-178), and
 * p(d|lambda) is the bin's mean over every ray consumed (Welford::skip, kernel.rs:181-189).
 *
 * The merges are done in exact arithmetic, on t quantized as the GPU quantizes it:
 * t_fixed = round(2^31 t), t_q = t_fixed >> 11, so that M2 N = N sum t_q^2 - (sum t_q)^2
 * and the test 40000 (N q2 - q1^2) < N^2 (N - 1) 2^40 are exact integers (the reference's
 * f32 merges round; parity with that rounding is unpinned). */
typedef unsigned __int128 orc_u128;

static uint32_t orc_t_fixed(double t) { return (uint32_t)(t * 2147483648.0 + 0.5); }

static int orc_sem_pass(uint64_t n, uint64_t q1, uint64_t q2)
{
    orc_u128 lhs = (orc_u128)40000u * ((orc_u128)n * q2 - (orc_u128)q1 * q1);
    orc_u128 rhs = ((orc_u128)n * n * (n - 1u)) << 40;
    return lhs < rhs;
}

typedef struct {
    uint64_t s1, q1, q2, n;
    size_t stamp;       /* last round that merged this bin, plus one */
} orc_bin;

static uint32_t adaptive_wavelength(const spectrometer *sp, double w, const double *ys, size_t R, orc_bin *st,
                                    double *row, uint64_t *hits)
{
    uint32_t B = sp->det.bin_count;
    for (uint32_t b = 0; b < B; b++) st[b].s1 = st[b].q1 = st[b].q2 = st[b].n = st[b].stamp = 0;
    size_t count = 0;
    size_t round = 0;
    for (size_t r0 = 0; r0 < R; r0 += 32, round++) {
        size_t nr = R - r0 < 32 ? R - r0 : 32;
        uint32_t bins[32], tf[32];
        int hit[32], any = 0;
        count += nr;
        for (size_t l = 0; l < nr; l++) {
            double t;
            hit[l] = spec_propagate(sp, ys[r0 + l], w, &bins[l], &t) == ORC_OK;
            if (hit[l]) {
                tf[l] = orc_t_fixed(t);
                any = 1;
                (*hits)++;
            }
        }
        if (!any) continue;
        /* every bin the round hit: merge, then test */
        for (size_t l = 0; l < nr; l++)
            if (hit[l]) {
                orc_bin *bs = &st[bins[l]];
                if (bs->stamp != round + 1) {
                    bs->stamp = round + 1;
                    bs->n += nr;
                }
                uint64_t q = tf[l] >> 11;
                bs->s1 += tf[l];
                bs->q1 += q;
                bs->q2 += q * q;
            }
        int finished = 1;
        for (size_t l = 0; l < nr; l++)
            if (hit[l] && !orc_sem_pass(st[bins[l]].n, st[bins[l]].q1, st[bins[l]].q2)) finished = 0;
        if (finished) break;
    }
    for (uint32_t b = 0; b < B; b++) row[b] = (double)st[b].s1 / ((double)count * 2147483648.0);
    return (uint32_t)count;
}

static void *fixed_worker(void *arg)
{
    fixed_job *j = (fixed_job *)arg;
    uint32_t B = j->sp->det.bin_count;
    uint64_t hits = 0;
    if (j->adaptive) {
        orc_bin *st = calloc(B, sizeof(orc_bin));
        for (size_t k = j->k0; k < j->k1; k++) {
            double w = sample_wavelength(j->sp, j->lam_u[k]);
            uint32_t c = adaptive_wavelength(j->sp, w, j->ys, j->R, st, j->p + k * B, &hits);
            if (j->counts) j->counts[k] = c;
        }
        free(st);
        j->hits = hits;
        return NULL;
    }
    for (size_t k = j->k0; k < j->k1; k++) {
        double w = sample_wavelength(j->sp, j->lam_u[k]);
        double *row = j->p + k * B;
        for (uint32_t b = 0; b < B; b++) row[b] = 0.0;
        for (size_t r = 0; r < j->R; r++) {
            uint32_t bin;
            double t;
            if (spec_propagate(j->sp, j->ys[r], w, &bin, &t) == ORC_OK) {
                row[bin] += t;
                hits++;
            }
        }
        for (uint32_t b = 0; b < B; b++) row[b] = row[b] / (double)j->R;
    }
    j->hits = hits;
    return NULL;
}

static int fitness_points_impl(const orc_spec *s, const double *lam_u, size_t W, const double *ray_u, size_t R,
                               int nthreads, double *p_out, double stats[4], uint64_t *hits_out, int adaptive,
                               uint32_t *counts_out);

int orc_fitness_points(const orc_spec *s, const double *lam_u, size_t W, const double *ray_u,
                       size_t R, int nthreads, double *p_out, double stats[4], uint64_t *hits_out)
{
    return fitness_points_impl(s, lam_u, W, ray_u, R, nthreads, p_out, stats, hits_out, 0, NULL);
}

int orc_fitness_adaptive_points(const orc_spec *s, const double *lam_u, size_t W, const double *ray_u, size_t R,
                                int nthreads, double *p_out, double stats[4], uint64_t *hits_out,
                                uint32_t *counts_out)
{
    return fitness_points_impl(s, lam_u, W, ray_u, R, nthreads, p_out, stats, hits_out, 1, counts_out);
}

static int fitness_points_impl(const orc_spec *s, const double *lam_u, size_t W, const double *ray_u, size_t R,
                               int nthreads, double *p_out, double stats[4], uint64_t *hits_out, int adaptive,
                               uint32_t *counts_out)
{
    spectrometer sp;
    int e = build_spectrometer(s, &sp);
    if (e) return e;
    if (W == 0 || R == 0) return ORC_INVALID;
    uint32_t B = sp.det.bin_count;
    double *p = p_out ? p_out : malloc(sizeof(double) * W * B);
    double *ys = malloc(sizeof(double) * R);
    if (!p || !ys) {
        if (!p_out) free(p);
        free(ys);
        return ORC_INVALID;
    }
    for (size_t r = 0; r < R; r++) ys[r] = beam_y(&sp, ray_u[r]);
    if (nthreads < 1) nthreads = 1;
    if ((size_t)nthreads > W) nthreads = (int)W;
    fixed_job *jobs = calloc((size_t)nthreads, sizeof(fixed_job));
    pthread_t *th = calloc((size_t)nthreads, sizeof(pthread_t));
    for (int i = 0; i < nthreads; i++) {
        jobs[i].sp = &sp;
        jobs[i].lam_u = lam_u;
        jobs[i].ys = ys;
        jobs[i].W = W;
        jobs[i].R = R;
        jobs[i].p = p;
        jobs[i].k0 = W * (size_t)i / (size_t)nthreads;
        jobs[i].k1 = W * (size_t)(i + 1) / (size_t)nthreads;
        jobs[i].adaptive = adaptive;
        jobs[i].counts = counts_out;
    }
    for (int i = 1; i < nthreads; i++) pthread_create(&th[i], NULL, fixed_worker, &jobs[i]);
    fixed_worker(&jobs[0]);
    uint64_t hits = jobs[0].hits;
    for (int i = 1; i < nthreads; i++) {
        pthread_join(th[i], NULL);
        hits += jobs[i].hits;
    }
    /* mutual information over the W rows, in row order (fitness.rs:95-122). */
    if (stats) {
        double h_cond = 0.0;
        double *pbar = calloc(B, sizeof(double));
        for (size_t k = 0; k < W; k++) {
            double h = 0.0;
            for (uint32_t b = 0; b < B; b++) {
                h += plog2p(p[k * B + b]);
                pbar[b] += p[k * B + b];
            }
            h_cond += h;
        }
        h_cond /= (double)W;
        double h_det = 0.0;
        for (uint32_t b = 0; b < B; b++) h_det += plog2p(pbar[b] / (double)W);
        double size, dev;
        size_and_deviation(&sp, &size, &dev);
        stats[0] = h_cond - h_det;
        stats[1] = h_cond;
        stats[2] = h_det;
        stats[3] = size;
        free(pbar);
    }
    if (hits_out) *hits_out = hits;
    free(jobs);
    free(th);
    free(ys);
    if (!p_out) free(p);
    return ORC_OK;
}

int orc_trace_pairs(const orc_spec *s, const double *lam_u, const double *ray_u, size_t n,
                    uint32_t *bins, double *ts)
{
    spectrometer sp;
    int e = build_spectrometer(s, &sp);
    if (e) return e;
    for (size_t i = 0; i < n; i++) {
        double w = sample_wavelength(&sp, lam_u[i]);
        uint32_t b;
        double t;
        if (spec_propagate(&sp, beam_y(&sp, ray_u[i]), w, &b, &t) == ORC_OK) {
            bins[i] = b;
            ts[i] = t;
        } else {
            bins[i] = sp.det.bin_count;
            ts[i] = 0.0;
        }
    }
    return ORC_OK;
}
