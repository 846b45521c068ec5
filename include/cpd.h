/*
 * cpd.h -- C ABI of the GB300 compound-prism spectrometer fitness library.
 *
 * This is the drop-in boundary for the fitness path of
 * jdtatz/compound-prism-designer. Every entry point takes plain pointers and
 * sizes and returns a cpd_status; nothing throws across the ABI. Each
 * declaration names the reference interface it replaces (paths inside the
 * reference project). A Rust -sys crate, a ctypes stub or a pyo3 shim binds
 * this header unchanged.
 *
 * Units: lengths in millimetres, wavelengths in micrometres, angles in radians.
 */
#ifndef CPD_H
#define CPD_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CPD_ABI_VERSION 1
#define CPD_MAX_GLASS 6            /* MAX_GLASS, src/pylib.rs:458 */
#define CPD_MAX_BINS 1024
#define CPD_MAX_WAVELENGTHS 65536  /* per design per call (max_n) */
#define CPD_MAX_RAYS (1u << 22)    /* per wavelength (max_eval / max_m) */

/* Status codes. The four RAYTRACE_* values are the variants of
 * RayTraceError (src/spectrometer/ray.rs:10-16); NOT_CONVERGED is the `None`
 * that cuda_fitness returns when the SEM stop is not met
 * (src/cuda_fitness.rs:403-422). */
typedef enum cpd_status {
    CPD_OK = 0,
    CPD_NOT_CONVERGED = 1,
    CPD_RAYTRACE_NO_SURFACE_INTERSECTION = 2,
    CPD_RAYTRACE_OUT_OF_BOUNDS = 3,
    CPD_RAYTRACE_TOTAL_INTERNAL_REFLECTION = 4,
    CPD_RAYTRACE_ANGULAR_RESPONSE_TOO_WEAK = 5,
    CPD_INVALID_ARGUMENT = 6,
    CPD_CUDA_ERROR = 7,
    CPD_TIMEOUT = 8,
    CPD_NO_CAPACITY = 9,
    CPD_NOT_IMPLEMENTED = 10
} cpd_status;

/* Everything the reference's pyo3 constructors take for one 2-D spectrometer:
 * CompoundPrism (src/pylib.rs:690-754), DetectorArray (src/pylib.rs:870-902),
 * UniformWavelengthDistribution (src/pylib.rs:306-316), GaussianBeam
 * (src/pylib.rs:365-372). */
typedef struct cpd_spectrometer_params {
    int32_t nglass;                        /* G, 1..6 (len(glasses)) */
    int32_t ar_coated;
    double glass[CPD_MAX_GLASS][6];        /* Glass coefficients, highest degree first */
    double angles[CPD_MAX_GLASS + 1];      /* G+1 face angles */
    double lengths[CPD_MAX_GLASS];         /* G separation lengths */
    double curvature;                      /* signed normalized curvature of the exit face */
    double height, width;
    uint32_t bin_count;
    int32_t det_flipped;
    double bin_size, linear_slope, linear_intercept, det_length, max_incident_angle, det_angle;
    double det_position[2];
    double wavelength_bounds[2];
    double beam_width, beam_y_mean;
} cpd_spectrometer_params;

/* A built design: the f64 surface and detector tables the fitness kernels read.
 * Plain data; copy it freely. Built by cpd_design_build. */
typedef struct cpd_design {
    int32_t nglass;
    uint32_t bin_count;
    int32_t ar_coated;
    int32_t reserved;
    double glass[CPD_MAX_GLASS][6];
    double face_point[CPD_MAX_GLASS][2];   /* entry face and inner faces */
    double face_normal[CPD_MAX_GLASS][2];
    double height;
    double exit_center[2], exit_radius;    /* CurvedPlane exit face */
    double exit_bound_center[2], exit_bound_r2;
    double bin_size, linear_slope, linear_intercept, min_ci, det_length;
    double det_normal[2], det_position[2], det_direction[2];
    double wavelength_bounds[2];
    double beam_width, beam_y_mean;
    double size, deviation;                /* size_and_deviation (spectrometer.rs:429-437) */
} cpd_design;

/* Result of one fitness evaluation: DesignFitness (src/fitness.rs:36-41) plus
 * diagnostics. */
typedef struct cpd_fitness {
    double size, info, deviation;
    double h_cond;          /* mean over wavelengths of sum_d p log2 p  (= -H(D|L)) */
    double h_det;           /* sum_d pbar log2 pbar                     (= -H(D))   */
    double max_sem;         /* max over bins of the SEM of p(d|lambda) across wavelengths */
    uint64_t rays;          /* rays evaluated */
    uint64_t hits;          /* rays that reached a detector bin */
    uint64_t retraced;      /* rays re-traced in exact f64 (guard band) */
    uint64_t fast_rays;     /* rays evaluated by the FP32 fast path (exit face + detector) */
    uint32_t wavelengths;   /* wavelength rows accumulated */
    int32_t status;         /* CPD_OK or CPD_NOT_CONVERGED */
} cpd_fitness;

/* Trace precision of the GPU estimator. */
enum {
    CPD_TRACE_HYBRID = 0,   /* FP32 trace; rays within a guard band of any decision
                               threshold are re-traced in exact f64 (default) */
    CPD_TRACE_FP32 = 1,     /* FP32 trace only, no re-trace (precision study) */
    CPD_TRACE_FP64 = 2      /* every ray in exact f64 (precision study reference) */
};

/* Sampling flag, OR-ed into a trace mode (CPD_TRACE_HYBRID only) or passed as
 * cpd_fitness_gpu_ex's `sampling`: the per-wavelength SEM stop of the reference GPU
 * kernel (src/spectrometer/kernel.rs:127-178). Each wavelength takes its rays in index
 * order, 32 per round, and stops after the first round that hit some bin and after which
 * every bin it hit has SEM <= 5e-3 (welford.rs:80-84); p(d|lambda) is the bin's sum of t
 * over the rays consumed. The Welford state of each bin is kept as exact integer sums
 * (t quantized to 2^-20 for the test), so the decisions are those of exact arithmetic
 * and the same on every launch shape. Without the flag every wavelength uses all rays
 * (fixed N). cpd_fitness.rays then counts the rays consumed. */
#define CPD_SAMPLING_ADAPTIVE 0x10u
/* With CPD_SAMPLING_ADAPTIVE: every wavelength on the exact path (float-float trace and
 * transmittances, exact test) instead of the FP32 fast path with the exact path as
 * fallback. For verification: the stop rounds are those of CPD_SAMPLING_ADAPTIVE. */
#define CPD_SAMPLING_EXACT 0x20u

typedef struct cpd_context cpd_context;

/* ---------------------------------------------------------------- host side */

int cpd_abi_version(void);
const char *cpd_status_string(int status);

/* position_detector_array (src/pylib.rs:815-838 -> detector_array_positioning,
 * src/spectrometer/spectrometer.rs:322-364). Reads the prism, source, det_length
 * and det_angle fields of `p`. */
int cpd_position_detector_array(const cpd_spectrometer_params *p, double acceptance,
                                double position_out[2], int32_t *flipped_out);

/* Builds the design tables: CompoundPrism::new (src/spectrometer/ray.rs:137-183),
 * LinearDetectorArray::new (src/spectrometer/spectrometer.rs:183-219) and the
 * argument checks of SizedCompoundPrism::new (src/pylib.rs:514-561). */
int cpd_design_build(const cpd_spectrometer_params *p, cpd_design *out);

/* No reference counterpart: cpd_design_build over n parameter records, for an
 * optimizer that builds a whole generation at once (designer.py:203-265 builds one
 * Spectrometer per call). With acceptance in (0, 1] each detector is first placed by
 * cpd_position_detector_array (its det_position/det_flipped inputs are ignored); with
 * acceptance 0 they are used as given. status[i] is design i's cpd_design_build or
 * positioning status; a failed design is zero-filled. Returns CPD_OK unless the
 * arguments are invalid. */
int cpd_design_build_batch(const cpd_spectrometer_params *p, uint32_t n, double acceptance,
                           cpd_design *out, int32_t *status);

/* CompoundPrism.exit_ray (src/pylib.rs:563-573): out = {x, y, dir x, dir y}. */
int cpd_exit_ray(const cpd_design *d, double y, double wavelength, double out[4]);

/* Spectrometer.ray_trace / propagation_path (src/pylib.rs:1061-1083,
 * spectrometer.rs:439-464): rows of (x, y, dir x, dir y), at most G+3. */
int cpd_ray_trace(const cpd_design *d, double wavelength, double initial_y, double *rows,
                  uint32_t *nrows);

/* Spectrometer.cpu_fitness (src/pylib.rs:1010-1026 -> src/fitness.rs:130-147):
 * the reference's adaptive f64 estimator on the host. An explicit CPU method of
 * the reference API; the GPU entry points never call it. */
int cpd_fitness_cpu(const cpd_design *d, uint64_t max_n, uint64_t max_m, cpd_fitness *out);

/* The f64 inverse normal CDF the ray tables use (src/spectrometer/erf.rs:62-73). */
double cpd_norminv(double u);

/* No reference counterpart: the float-float log2 of an integer count that the GPU
 * entropy sums use (FP32-pipe arithmetic, table-driven), evaluated on the host with the
 * same code, for accuracy checks. out = {hi, lo}; log2(count) ~= hi + lo. */
int cpd_entropy_log2(uint64_t count, double out[2]);

/* Glass.__call__ -> Glass::calc_n (src/pylib.rs:76-78, src/spectrometer/glasscat.rs:17-22):
 * index of refraction at wavelength w (micrometres) from the 6 Horner coefficients. */
double cpd_glass_index(const double coeffs[6], double w);

/* ---------------------------------------------------------------- GPU side */

/* CudaFitnessContext::new / quick_init / set_cached_cuda_context
 * (src/cuda_fitness.rs:187-197, 324-329, 362-363): one context per GPU; owns a
 * stream, pooled device buffers and captured CUDA graphs. Thread-safe. */
int cpd_context_create(int device, cpd_context **out);
void cpd_context_destroy(cpd_context *ctx);

/* cuda_fitness (src/cuda_fitness.rs:347-423), Spectrometer.gpu_fitness
 * (src/pylib.rs:1088-1135): for each seed, max_n wavelengths
 * u_i = fract(seed + i/phi) and max_eval rays u_j = fract(seed + (j+1)/phi);
 * p(d|lambda) accumulated in FP64; stops at the first seed after which every
 * bin's SEM across wavelengths is <= 5e-3 (status CPD_OK), else
 * CPD_NOT_CONVERGED with the estimate of all seeds. nwarp is the block-shape
 * hint of the reference (warps per CTA). */
int cpd_fitness_gpu(cpd_context *ctx, const cpd_design *d, const double *seeds, uint32_t nseeds,
                    uint32_t max_n, uint32_t nwarp, uint32_t max_eval, cpd_fitness *out);

/* cpd_fitness_gpu with a sampling choice: 0 (fixed N, what cpd_fitness_gpu does) or
 * CPD_SAMPLING_ADAPTIVE, the reference kernel's per-wavelength SEM stop
 * (src/spectrometer/kernel.rs:127-178) inside the same seed loop. */
int cpd_fitness_gpu_ex(cpd_context *ctx, const cpd_design *d, const double *seeds, uint32_t nseeds,
                       uint32_t max_n, uint32_t nwarp, uint32_t max_eval, uint32_t sampling,
                       cpd_fitness *out);

/* Fixed-N estimator on explicit point sets (the parity entry point): W wavelength
 * u-points and R ray u-points, every wavelength traced with all R rays
 * (prob_dets_given_wavelengths, src/spectrometer/kernel.rs:89-193, on given
 * points). p_out (optional, W*B, row-major) receives p(d|lambda). trace_mode is a
 * CPD_TRACE_* value, optionally with CPD_SAMPLING_ADAPTIVE (then R is the ray budget
 * and the rays are taken in the given order). */
int cpd_fitness_gpu_points(cpd_context *ctx, const cpd_design *d, const double *lam_u, uint32_t W,
                           const double *ray_u, uint32_t R, uint32_t trace_mode, cpd_fitness *out,
                           double *p_out);

/* No counterpart in the reference. The same fixed-N estimator as
 * cpd_fitness_gpu_points, for callers that cannot allocate device memory: a host
 * application that owns the GPU's memory budget and forbids plug-in libraries to
 * allocate, or a latency-critical loop that must not pay the device-wide
 * synchronisation a cudaMalloc/cudaFree can bring. It calls no allocator: every
 * intermediate buffer lives in one file-scope device array of about 3 MiB, which every
 * GPU that loads the library holds until the process exits. Inputs and outputs are host
 * pointers; no context is used; the work runs on the legacy default stream of the
 * current device and the call returns when it is done. Each call resolves the array's
 * address in the current context and uploads every table it needs with its inputs, so
 * it stays valid after a cudaDeviceReset and from another driver context on the same
 * GPU. Limits per call: W <= 1024 wavelengths, R <= 4096 rays, bin_count <= 128;
 * larger requests return CPD_NO_CAPACITY. CPD_NO_CAPACITY also depends on the data: at
 * most 32768 guard-band rays are re-traced per call (about 0.8% of the rays at the
 * largest W and R), so a design with many rays near a decision threshold (near-critical
 * exit faces) can exceed it at sizes within the limits, and CPD_TRACE_FP64, which
 * re-traces every ray that clears the flat faces, needs W*R <= 32768; the allocating
 * entry points grow their queue instead. Every call on a device shares the array, which keeps the previous
 * call's contents; each call clears what must start at zero. Calls that overlapped on the
 * GPU would race on the array: calls from threads of one process are therefore serialised
 * per device, and each returns only when its work is done. */
int cpd_fitness_gpu_points_static(const cpd_design *d, const double *lam_u, uint32_t W, const double *ray_u,
                                  uint32_t R, uint32_t trace_mode, cpd_fitness *out, double *p_out);

/* Spectrometer.transmission_probability (src/pylib.rs:1028-1058): p(d|lambda) for
 * explicit wavelengths by the reference's estimator, p_dets_l_wavelength
 * (src/fitness.rs:5-34,48-69): the reference's ray points (the R1 sequence from 0.5,
 * fitness.rs:19) in order, at most max_m per wavelength; each hit pads its bin's Welford
 * state with zeros up to the ray count and adds its t, and the wavelength stops at the
 * first hit after which its bin's SEM <= 5e-3; p is each bin's mean after padding every bin
 * to the final count. Each ray is traced in exact f64 and the Welford updates follow the
 * reference's f64 operation order, so the results are the reference's own. out is n*B
 * row-major. */
int cpd_transmission_probability(cpd_context *ctx, const cpd_design *d, const double *wavelengths,
                                 uint32_t n, uint32_t max_m, double *out);

/* Flag of cpd_transmission_probability_ex: every wavelength uses all max_m rays (fixed N,
 * p = sum of t / max_m, the estimator of cpd_fitness_gpu_points) instead of the reference's
 * SEM stop. */
#define CPD_TP_FIXED_N 0x1u

/* cpd_transmission_probability with flags (0 or CPD_TP_FIXED_N) and, optionally, the rays
 * each wavelength consumed (rays_out, n entries: the ray at which the stop fired, or
 * max_m). */
int cpd_transmission_probability_ex(cpd_context *ctx, const cpd_design *d, const double *wavelengths,
                                    uint32_t n, uint32_t max_m, uint32_t flags, double *out,
                                    uint32_t *rays_out);

/* launch_propagation_test / propagation_test_kernel (src/cuda_fitness.rs:247-317,
 * src/spectrometer/kernel.rs:195-224): one ray per (lam_u[i], ray_u[i]) pair.
 * bins[i] = bin index or bin_count for a lost ray; ts[i] = transmittance;
 * flags[i] (optional) = 1 where the ray was re-traced in exact f64. */
int cpd_trace_rays(cpd_context *ctx, const cpd_design *d, const double *lam_u, const double *ray_u,
                   uint32_t n, uint32_t trace_mode, uint32_t *bins, double *ts, uint8_t *flags);

/* Per-design sampling plan of a batched launch. */
typedef struct cpd_batch_item {
    double seed;        /* point-set seed, as cpd_fitness_gpu */
    uint32_t max_n;     /* W, wavelengths */
    uint32_t max_eval;  /* R, rays per wavelength */
} cpd_batch_item;

/* Batched form (no reference counterpart; the reference evaluates one design per
 * call, designer.py:267-300): n designs of mixed G, B, W, R in one captured
 * launch sequence. outs[i].status is CPD_OK or CPD_NOT_CONVERGED per design. trace_mode
 * may carry CPD_SAMPLING_ADAPTIVE (then the autotuner is not used: the adaptive kernels
 * have no launch shape). */
int cpd_fitness_gpu_batch(cpd_context *ctx, const cpd_design *designs, const cpd_batch_item *items,
                          uint32_t n, uint32_t trace_mode, cpd_fitness *outs);

/* Design construction on the device (no reference counterpart; the reference builds each
 * Spectrometer on the host, src/pylib.rs:690-1170). The batched form with parameter records
 * instead of built designs: the pass's first kernel builds each design on the GPU (the
 * f64 construction of cpd_design_build, the detector positioned first by
 * cpd_position_detector_array when acceptance is in (0, 1]; acceptance 0 takes
 * det_position/det_flipped as given) and the fitness follows in the same launch sequence.
 * The construction's sin/cos are CUDA's f64 functions, so a design may differ from the
 * host-built one in the last bit of its tables. outs[i].status is the build error of a
 * design that could not be built (a CPD_RAYTRACE_* or CPD_INVALID_ARGUMENT value; its
 * other fields are zero), else CPD_OK or CPD_NOT_CONVERGED. */
int cpd_fitness_gpu_batch_params(cpd_context *ctx, const cpd_spectrometer_params *params,
                                 const cpd_batch_item *items, uint32_t n, double acceptance,
                                 uint32_t trace_mode, cpd_fitness *outs);

/* cpd_design_build_batch on the GPU: the same records and status codes (up to the last-bit
 * differences of CUDA's sin/cos), one thread per design. */
int cpd_design_build_device(cpd_context *ctx, const cpd_spectrometer_params *params, uint32_t n,
                            double acceptance, cpd_design *out, int32_t *status);

/* Launch-shape tuning of the batched/plain kernels (ray tile = rays per lane per
 * work item, warps per CTA). 0 leaves a value unchanged. */
int cpd_set_launch_shape(cpd_context *ctx, uint32_t ray_tile, uint32_t warps_per_cta);
int cpd_get_launch_shape(cpd_context *ctx, uint32_t *ray_tile, uint32_t *warps_per_cta);

/* The project's launch-shape autotuner (no reference counterpart; the reference takes
 * a fixed nwarp hint, src/pylib.rs:1088). Times the batch with every ray tile in
 * {4, 8, 16, 32, 64, 128, 256}, plus the tiles that split the work into 2..6 whole rounds of
 * the resident warps, and warps per CTA in {2, 4, 8} (captured graph, minimum of two
 * timed passes each), sets the fastest on the context and remembers it for the batch's
 * class: trace mode and the binary orders of magnitude of its design count, wavelength
 * rows, rays and widest detector. Results do not depend on the shape. Fixed-N passes
 * only (a trace mode without CPD_SAMPLING_ADAPTIVE). */
int cpd_autotune_batch(cpd_context *ctx, const cpd_design *designs, const cpd_batch_item *items,
                       uint32_t n, uint32_t trace_mode, uint32_t *ray_tile, uint32_t *warps_per_cta,
                       double *best_ms);
/* When on, cpd_fitness_gpu_batch and cpd_fitness_gpu use the remembered shape of the
 * pass's class, and run the autotuner first for a class they have not seen
 * (cpd_fitness_gpu then ignores its nwarp hint). Off by default. */
int cpd_set_autotune(cpd_context *ctx, int on);

/* Device time of the last GPU call's kernels (CUDA events on the context stream), ms,
 * and the number of kernel launches it issued. */
int cpd_last_timing(cpd_context *ctx, double *kernel_ms, uint32_t *launches);

/* Per-kernel timing: when on, each pass is launched without graph replay and CUDA
 * events bracket every kernel; cpd_last_kernel_times then returns the last pass's
 * {setup, trace, retrace, entropy} device times in ms. */
int cpd_set_profiling(cpd_context *ctx, int on);
int cpd_last_kernel_times(cpd_context *ctx, double ms[4]);

/* Host->device and device->host bytes the last GPU call copied. */
int cpd_last_transfer_bytes(cpd_context *ctx, uint64_t *h2d, uint64_t *d2h);

/* FP32 FMA throughput probe: runs a dependent-chain-free FMA kernel for `iters`
 * iterations on every SM and returns the achieved TFLOP/s (roofline peak). */
int cpd_measure_fp32_peak(cpd_context *ctx, uint32_t iters, double *tflops);

/* SFU throughput probe: independent chains of the reciprocal-square-root estimate
 * (the special-function unit that the trace's square roots and reciprocals use) on
 * every SM for `iters` iterations; returns the achieved results per second, in G/s (the
 * SFU roofline's peak). */
int cpd_measure_sfu_peak(cpd_context *ctx, uint32_t iters, double *gops);

/* ---------------------------------------------------------------- serving */

/* Continuous-batching fitness server (no reference counterpart: the reference's
 * optimizer, designer.py:267-300, calls gpu_fitness once per design and waits).
 * Requests of any size arrive from any thread; a worker thread admits their designs
 * first-come first-served into passes while the device bytes of the designs in flight
 * (histogram, per-wavelength tables and ray tables; about W*(8B+400) + 16R bytes each)
 * stay within mem_budget_bytes, and keeps up to `slots` passes in flight on separate
 * streams. A design larger than the budget runs alone. max_designs_per_pass caps one
 * pass (0 = 256). Each design's result is bitwise the one it gets alone
 * (cpd_fitness_gpu_batch with n = 1): the accumulation is integer and
 * order-independent. */
typedef struct cpd_server cpd_server;
int cpd_server_create(cpd_context *ctx, uint64_t mem_budget_bytes, uint32_t slots,
                      uint32_t max_designs_per_pass, cpd_server **out);
/* Queues n designs (one trace mode per request, optionally with
 * CPD_SAMPLING_ADAPTIVE; a pass holds requests of one mode); returns a request id at
 * once. */
int cpd_server_submit(cpd_server *sv, const cpd_design *designs, const cpd_batch_item *items,
                      uint32_t n, uint32_t trace_mode, uint64_t *request_id);
/* cpd_server_submit with parameter records: the designs are built on the device inside
 * their pass (as cpd_fitness_gpu_batch_params), so an optimizer that produces parameters
 * needs no host build step. A pass holds requests of one trace mode, one kind (designs or
 * parameter records) and one acceptance. */
int cpd_server_submit_params(cpd_server *sv, const cpd_spectrometer_params *params,
                             const cpd_batch_item *items, uint32_t n, double acceptance,
                             uint32_t trace_mode, uint64_t *request_id);
/* Waits up to timeout_ms for a request. On completion writes its n results, the time
 * from submit to completion (latency_ms, optional), forgets the request and returns
 * CPD_OK (or the error a pass met); on timeout returns CPD_TIMEOUT and the request
 * stays queued. */
int cpd_server_wait(cpd_server *sv, uint64_t request_id, cpd_fitness *outs, double timeout_ms,
                    double *latency_ms);
int cpd_server_stats(cpd_server *sv, uint64_t *designs_done, uint64_t *passes,
                     uint64_t *max_passes_in_flight, uint64_t *pending_designs);
/* Finishes every queued design, then stops the worker and frees the slots. */
void cpd_server_destroy(cpd_server *sv);

/* ---------------------------------------------------------------- device-resident loop */

/* No reference counterpart (the reference's optimizer calls gpu_fitness once per design,
 * designer.py:267-300, through a process-wide lock, src/cuda_fitness.rs:322-362): a
 * serving loop that lives on the GPU. One persistent kernel; each of its CTAs owns a
 * histogram slab and evaluates whole designs, taking them from a ring of records in
 * mapped host memory, with no host step between designs. The host queues requests and
 * feeds the ring; completions are read from mapped memory. The GPU memory for histograms
 * is hist_budget_bytes split into slabs of max_cells cells (8 bytes each), one per
 * resident CTA: a design is admitted when W * bin_count <= max_cells and W <= max_rows,
 * else cpd_loop_submit returns CPD_NO_CAPACITY. A CTA with no work waits at most idle_ms,
 * then leaves; the loop relaunches the kernel when new work arrives. Fixed N with the
 * hybrid trace (CPD_TRACE_HYBRID) only. Each design's result is bitwise its result from
 * cpd_fitness_gpu_batch with n = 1 (integer accumulation, the same device code). */
typedef struct cpd_loop cpd_loop;
typedef struct cpd_loop_config {
    uint64_t hist_budget_bytes;  /* 0: 4 GiB */
    uint32_t max_cells;          /* W * bin_count a slab holds; 0: 2^20 */
    uint32_t max_rows;           /* wavelengths a slab holds; 0: 8192 */
    uint32_t ring_capacity;      /* designs published and not yet completed; 0: 16384 */
    uint32_t ctas_per_sm;        /* 0: as many as fit */
    uint32_t idle_ms;            /* a CTA's longest wait for work; 0: 200 */
    uint32_t ray_tile;           /* rays per lane per trace work item; 0: 64 */
} cpd_loop_config;
typedef struct cpd_loop_report {
    uint64_t designs_done;           /* completions read by the host */
    uint64_t device_designs;         /* designs the CTAs evaluated */
    uint64_t kernel_launches;        /* launches of the loop kernel (after idle exits) */
    uint64_t max_designs_in_flight;  /* published and not yet completed, at most */
    uint64_t pending_designs;        /* queued on the host, not yet published */
    uint64_t table_resets;           /* times the device table arena was emptied */
    uint64_t inline_retraced;        /* flagged rays re-traced inline (a slab queue was full) */
    uint64_t slab_bytes;             /* device bytes per CTA */
    uint32_t ctas;                   /* CTAs of the loop kernel */
    uint32_t idle_exits;             /* CTAs that left after idle_ms without work */
    uint32_t stop_exits;             /* CTAs that left on cpd_loop_destroy */
    uint32_t reserved;
} cpd_loop_report;
int cpd_loop_create(cpd_context *ctx, const cpd_loop_config *cfg, cpd_loop **out);
/* Queues n designs (trace mode CPD_TRACE_HYBRID); returns a request id at once. */
int cpd_loop_submit(cpd_loop *loop, const cpd_design *designs, const cpd_batch_item *items, uint32_t n,
                    uint32_t trace_mode, uint64_t *request_id);
/* As cpd_server_wait. */
int cpd_loop_wait(cpd_loop *loop, uint64_t request_id, cpd_fitness *outs, double timeout_ms, double *latency_ms);
int cpd_loop_stats(cpd_loop *loop, cpd_loop_report *out);
/* Finishes every queued design, lets the CTAs leave, frees the loop. */
void cpd_loop_destroy(cpd_loop *loop);

#ifdef __cplusplus
}
#endif
#endif
