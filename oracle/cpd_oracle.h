/*
 * cpd_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C, double-precision restatement of the compound-prism spectrometer
 * fitness path of jdtatz/compound-prism-designer (Rust crate `src/`). It is the
 * parity reference of the CUDA implementation's tests and the timed CPU baseline. Only
 * tests, the smoke check and the benchmark's CPU-baseline / reference legs may
 * load it; the product library never links or calls it.
 *
 * Every function cites the reference file:line it restates. Arithmetic is
 * compiled with -ffp-contract=off, and fma() is called exactly where the Rust
 * source calls `mul_add` (Rust never contracts a*b+c on its own), so the
 * results are the reference's own f64 results up to the last-ulp differences of
 * libm's log/sin/cos.
 *
 * Parity pin: the known-design golden values of src/fitness.rs:250-257
 * (size 41.3, info 0.7407, deviation 0.377159) and the Shaw inverse-normal
 * accuracy points of src/spectrometer/erf.rs:142-161 (tests/test_oracle_golden.py).
 */
#ifndef CPD_ORACLE_H
#define CPD_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_MAX_GLASS 6

/* Error codes: the four RayTraceError variants of src/spectrometer/ray.rs:10-16. */
enum {
    ORC_OK = 0,
    ORC_NO_SURFACE_INTERSECTION = 1,
    ORC_OUT_OF_BOUNDS = 2,
    ORC_TOTAL_INTERNAL_REFLECTION = 3,
    ORC_ANGULAR_RESPONSE_TOO_WEAK = 4,
    ORC_INVALID = 10
};

/* Flat spectrometer description, field for field what the pyo3 constructors take
 * (src/pylib.rs: CompoundPrism 690-754, DetectorArray 864-902,
 * UniformWavelengthDistribution 298-309, GaussianBeam 347-356). */
typedef struct orc_spec {
    int32_t nglass;                       /* G, 1..6 */
    int32_t ar_coated;
    double glass[ORC_MAX_GLASS][6];       /* Horner coefficients, highest degree first */
    double angles[ORC_MAX_GLASS + 1];     /* G+1 face angles (radians) */
    double lengths[ORC_MAX_GLASS];        /* G separation lengths */
    double curvature;                     /* signed normalized curvature of the exit face */
    double height, width;
    /* detector array */
    uint32_t bin_count;
    int32_t det_flipped;
    double bin_size, linear_slope, linear_intercept, det_length, max_incident_angle, det_angle;
    double det_position[2];
    /* source */
    double wmin, wmax;                    /* UniformDistribution bounds (micrometres) */
    double beam_width, beam_y_mean;       /* GaussianBeam */
} orc_spec;

/* Shaw inverse normal CDF (src/spectrometer/erf.rs:62-73). */
double orc_norminv(double x);
/* Horner glass polynomial (src/spectrometer/glasscat.rs:300-305). */
double orc_calc_n(const double coeffs[6], double w);
/* The reference CPU point set: Qrng::new_from_scalar(seed).take(n), i.e. the
 * incremental R1 sequence state = fract(state + 1/phi) (src/spectrometer/qrng.rs:526-563). */
void orc_qrng_points(double seed, size_t n, double *out);

/* The GPU seed policy's points: u_i = fract(fma(first + i, 1/phi, seed)). */
void orc_gpu_points(double seed, uint64_t first, size_t n, double *out);

/* detector_array_positioning (src/spectrometer/spectrometer.rs:322-364). Uses
 * only the prism fields, the source fields and det_length/det_angle of `s`. */
int orc_position_detector(const orc_spec *s, double acceptance, double pos_out[2],
                          int32_t *flipped_out);

/* One ray: Spectrometer::propagate (spectrometer.rs:421-427) for the ray
 * GaussianBeam::inverse_cdf([ray_u]) at wavelength `wavelength` (micrometres).
 * Returns ORC_OK and (bin, t) or a RayTraceError code. */
int orc_propagate(const orc_spec *s, double wavelength, double ray_u, uint32_t *bin, double *t);

/* Geometry dump for table-equality tests: 2*(G) plane values (point x,y; normal x,y per plane),
 * then curved (center x,y, radius, bound center x,y, bound radius^2),
 * then detector (normal x,y, direction x,y, min_ci), then (size, deviation).
 * Writes 4*G + 6 + 5 + 2 doubles. */
int orc_design_dump(const orc_spec *s, double *out);

/* Spectrometer::propagation_path (spectrometer.rs:439-464): writes up to
 * (G+3) rows of (origin x, origin y, dir x, dir y); returns the row count. */
int orc_propagation_path(const orc_spec *s, double wavelength, double initial_y, double *rows);

/* The face at which the prism trace of propagate_trace (ray.rs:501-541) stops for this
 * wavelength and start height: 0..G-1 for the flat faces (0 = entrance), G for the curved
 * exit face, -1 when the ray leaves through the exit face; *status = the stopping error
 * (ORC_OK when it leaves). Negative build errors are returned as -(100 + e). */
int orc_stop_face(const orc_spec *s, double wavelength, double initial_y, int *status);

/* fitness() (src/fitness.rs:130-147) with the reference's adaptive SEM stops.
 * out = {size, info, deviation}. */
int orc_fitness_adaptive(const orc_spec *s, size_t max_n, size_t max_m, double out[3]);
/* The same, also writing the wavelengths the outer SEM stop let through and the rays
 * traced over them (the work the reference's estimator did). */
int orc_fitness_adaptive_work(const orc_spec *s, size_t max_n, size_t max_m, double out[3], uint64_t *wavelengths_out,
                              uint64_t *rays_out);

/* p_dets_l_wavelength (src/fitness.rs:48-69) for one wavelength: writes bin_count means. */
int orc_p_dets_l_wavelength(const orc_spec *s, double wavelength, size_t max_m, double *out);
/* The same, also writing the rays consumed (the integration's final count: the ray at
 * which the SEM stop fired, or max_m). */
int orc_p_dets_l_wavelength_count(const orc_spec *s, double wavelength, size_t max_m, double *out,
                                  uint64_t *rays_out);

/* Fixed-N estimator on explicit point sets: wavelength u-points lam_u[W]
 * (lambda = wmin + (wmax-wmin)*u) and ray u-points ray_u[R]. p(d|lambda) = sum(t)/R over
 * all R rays (misses count as zeros, as the Welford `skip` of fitness.rs:30-32 does).
 * p_out (optional, W*B), stats (optional, 4): {info, h_cond_mean, h_det, size}.
 * hits_out (optional): total count of rays that reached a bin.
 * nthreads <= 0 uses one thread. */
int orc_fitness_points(const orc_spec *s, const double *lam_u, size_t W, const double *ray_u,
                       size_t R, int nthreads, double *p_out, double stats[4], uint64_t *hits_out);

/* Adaptive sampling on explicit point sets: the per-wavelength SEM stop of the
 * reference GPU kernel (src/spectrometer/kernel.rs:127-178) with exact Welford merges on
 * t_q = round(2^31 t) >> 11 (cpd_oracle.c states the rule). Rays are taken in the given
 * order, 32 per round; p(d|lambda) = sum of t over the rays consumed / their number.
 * counts_out (optional, W): rays consumed per wavelength. Other arguments as
 * orc_fitness_points. */
int orc_fitness_adaptive_points(const orc_spec *s, const double *lam_u, size_t W, const double *ray_u,
                                size_t R, int nthreads, double *p_out, double stats[4], uint64_t *hits_out,
                                uint32_t *counts_out);

/* Per-ray twin of propagation_test_kernel (src/spectrometer/kernel.rs:195-224) in f64:
 * lambda = wmin + (wmax-wmin)*lam_u[i]; bin_count marks a lost ray. */
int orc_trace_pairs(const orc_spec *s, const double *lam_u, const double *ray_u, size_t n,
                    uint32_t *bins, double *ts);

/* ------------------------------------------------ 3-D: fiber beam, toric lenses
 * (cpd_oracle_toric.c). The reference's Dim3 spectrometer: FiberBeam
 * (src/spectrometer/spectrometer.rs:75-125), CulminatingToricCompoundPrism
 * (src/spectrometer/ray.rs:112-118, toric.rs:204-262), the 3-D linear detector. */
typedef struct orc_spec3 {
    orc_spec base;          /* prism, detector and wavelength fields; base.curvature and the
                               beam fields are unused */
    double curv0[2];        /* first toric lens: signed normalized poloidal curvature,
                               normalized toroidal curvature */
    double curv1[2];        /* last toric lens */
    double fiber_radius, fiber_na, fiber_center_y;
} orc_spec3;

/* approx_cbrt (src/spectrometer/cbrt.rs:49-68). */
double orc_approx_cbrt(double x);
/* sympy_soln (src/spectrometer/toric.rs:41-141): roots[0..3] of the ray-torus quartic. */
void orc_toric_roots(double r_2, double R_2, double dp_magn_sq, double dp_v, double dp_n, double n_v,
                     double roots[4]);
/* Qrng<[f64; 4]> from [seed; 4] (qrng.rs:157-255): n points, out[4 i + k]. */
void orc3_qrng_points(double seed, size_t n, double *out);
/* detector_array_positioning (spectrometer.rs:322-364) for the 3-D spectrometer. */
int orc3_position_detector(const orc_spec3 *s, double acceptance, double pos_out[2], int32_t *flipped_out);
/* One ray per (lam_u[i], q[4 i .. 4 i + 3]): bins[i] (bin_count when lost), ts[i], and optionally
 * the RayTraceError code, the NaN roots met at the toric faces and the toric faces reached. */
int orc3_trace_pairs(const orc_spec3 *s, const double *lam_u, const double *q, size_t n, uint32_t *bins,
                     double *ts, int32_t *status, uint32_t *nan_roots, uint32_t *toric_calls);
/* Fixed-N estimator on explicit points (W wavelength u-points, R 4-D ray points), as
 * orc_fitness_points; stats[3] = size. */
int orc3_fitness_points(const orc_spec3 *s, const double *lam_u, size_t W, const double *q, size_t R,
                        double *p_out, double stats[4], uint64_t *hits_out);

#ifdef __cplusplus
}
#endif
#endif
