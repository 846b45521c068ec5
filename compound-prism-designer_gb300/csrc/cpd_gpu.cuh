// cpd_gpu.cuh -- device-side job descriptors and kernel launchers.
#pragma once

#include <cuda_runtime.h>

#include "cpd_df.h"
#include "cpd_ff.h"
#include "cpd_model.h"

#ifndef CPD_TILE_CELLS_BATCH
#define CPD_TILE_CELLS_BATCH 2048
#endif

namespace cpd {

// One design in a launch sequence. Offsets index the launch's shared buffers.
struct alignas(16) DesignJob {
    uint32_t W;          // wavelength rows this pass
    uint32_t R;          // rays per wavelength (estimator divisor)
    uint32_t Rz;         // rays in the sorted table (R minus non-finite start heights)
    uint32_t B;          // detector bins
    uint64_t row_off;    // first global wavelength row (LamParams index)
    uint64_t hist_off;   // first histogram cell (rows x B, u64)
    uint64_t lam_off;    // first wavelength u-point
    uint64_t ray_off;    // first entry of the sorted ray tables
    uint64_t rank_off;   // first entry of the rank table (adaptive sampling)
    uint64_t acc_off;    // first per-bin accumulator (B cells in each of S1, S2)
    uint64_t item_off;   // first trace work item
    uint64_t tile_off;   // first entropy tile
    uint32_t nchunk;     // ray chunks per 32-wavelength block
    uint32_t tile_rows;  // wavelength rows per entropy tile
    uint32_t ntiles;
    uint32_t pad;
    float unit_hi, unit_lo;  // p per count unit, 2^-31 / R, float-float
    float lu_hi, lu_lo;      // log2 of that unit, float-float
    double pscale;           // 2^-31 / R in f64, for the optional p(d|lambda) output (set on the host:
                             // an f64 division on the device issues to the slow FP64 unit)
    double pad2;
};

// A ray whose FP32 result fell inside a guard band: (design, wavelength row, ray). In
// adaptive sampling: a wavelength row whose stop decision needs the exact path (j unused).
struct alignas(16) QEntry {
    uint32_t design, k, j, pad;
};

// Sorted-ray tables up to this many rays can be staged in shared memory by the setup.
constexpr uint32_t kStageRays = 2048;

// Per-launch control words (zeroed before every pass).
struct Control {
    unsigned long long item_counter;
    unsigned long long queue_count;
    unsigned int overflow;
    unsigned int tiles_done;  // entropy tiles finished (single-design passes)
};

// What the host reads of a pass's Control words, written by the re-trace kernel (the
// last kernel to change them) into mapped host memory.
struct HostStatus {
    unsigned long long queue_count;
    unsigned int overflow;
    unsigned int pad;
};

// Copies of each per-design ray counter: thousands of warps add to the counters of one
// design, and same-address atomics serialize in L2, so each warp adds to one of
// kSpread copies and the finalize sums them.
constexpr int kSpread = 16;

// Per-design accumulators that persist across the seeds of one call.
struct DesignAcc {
    unsigned long long H;                  // sum over rows and bins of -p log2 p, 2^-40 units
    unsigned long long rows;               // wavelength rows accumulated
    unsigned long long hits[kSpread];      // rays that reached a bin
    unsigned long long retraced[kSpread];  // rays re-traced
    unsigned long long fast[kSpread];      // rays evaluated by the FP32 fast path
};

// Per-design result of the fused finalize (cumulative over passes).
struct DesignOut {
    double info, h_cond, h_det, max_sem;
    double size, deviation;  // from the design record (built on the host or the device)
    unsigned long long hits, retraced, rows, fast;
    int32_t converged;
    int32_t status;          // the design record's status (a device build's error)
};

// Cells per entropy tile: a design's tile is max(1, cells / B) rows, kTileCells for a
// single-design pass (one CTA per tile: more tiles, more SMs busy on its short tail) and
// kTileCellsBatch for passes of several designs (one warp per tile, many tiles: fewer,
// larger tiles spend less on each tile's job lookup and per-bin atomics).
constexpr uint32_t kTileCells = 512;
constexpr uint32_t kTileCellsBatch = CPD_TILE_CELLS_BATCH;

struct LaunchArgs {
    const DevDesign *designs;
    const DesignJob *jobs;
    uint32_t njobs;
    uint64_t total_rows;
    uint64_t total_items;
    uint64_t total_tiles;
    const double *lam_u;
    const double *z64;
    const float *z32;     // (hi, lo) f32 pairs of the sorted z table
    const uint32_t *rank; // adaptive sampling: ray index -> sorted position (~0u: no start height)
    LamParams *lp;
    LamDF *lx;            // per row: float-float data for the re-trace
    unsigned long long *hist;
    unsigned long long *S1;
    unsigned long long *S2;
    DesignAcc *acc;
    DesignOut *out;       // results (mapped host memory in the context's passes)
    Control *ctl;
    HostStatus *status;   // optional (mapped host memory)
    uint32_t clear_acc;   // the setup kernel zeroes S1, S2 (acc_cells) and acc (njobs) first
    uint64_t acc_cells;
    QEntry *queue;
    uint32_t qcap;
    uint32_t ray_tile;
    // Single-design passes: per 32-row block, [min core_lo, max core_hi) over its rows,
    // written by the setup (which also adds the block's length to ctl->item_counter). The
    // trace then splits the sum of those lengths into equal shares, one per resident warp,
    // instead of handing out work items from the counter. nullptr: work items.
    uint2 *spans;
    // The design's fast-path constants and thresholds when `spans` is set: read by the
    // trace as kernel parameters (constant-bank operands), which leaves their registers to
    // the ray loop.
    FastConst fc;
    FastLimits fl;
    // The design's job record when `spans` is set (jobs[0]), a kernel parameter: the
    // setup's first loads (the wavelength point, the design record, the z table) then
    // do not wait for a load of the job.
    DesignJob one;
    // The setup stages a design's sorted z table in shared memory when it has at most
    // stage_cap rays (at most kStageRays; 0: none); the setup's blocks get
    // 8 * even(stage_cap) bytes, so a pass whose tables are small or not staged at all does
    // not hold shared memory it does not use.
    uint32_t stage_cap;
    uint32_t mode;        // CPD_TRACE_*
    uint32_t adaptive;    // per-wavelength SEM stop: 1, or 2 with every row on the exact path
    uint32_t max_B;       // widest detector of the launch
    Guards guards;
    double yguard_rel;
    double *p_out;        // optional W x B for the single design of the launch
    // designs built on the device (CPD_BUILD_ON_DEVICE): parameter records, written into
    // the design records by the build kernel before the setup
    const cpd_spectrometer_params *params;
    double build_acceptance;
    const float *logtab;  // float-float log2 table (cpd_ff.h), 4 x 256 floats
};

// Most warps that trace (and decide) one wavelength's rounds at once under adaptive
// sampling: one round per warp.
constexpr uint32_t kMaxAdaptWarps = 16;

// Per-bin state of one wavelength under adaptive sampling: shared memory, one array per
// field (consecutive bins in consecutive words), carved from B-sized slices.
struct BinStates {
    // Within one group of rounds: byte v of lanes[b] holds 1 + the lane of round v that
    // carries the round's sums for bin b (0: round v missed b); bit v of rounds[b] is set
    // when round v hit b.
    uint4 *lanes;
    unsigned long long *s1;  // sum of t_fixed over the bin's hits
    unsigned long long *q1;  // sum of t_q
    unsigned long long *q2;  // sum of t_q^2
    uint32_t *n;             // Welford samples: the sizes of the rounds that hit the bin
    uint32_t *h;             // hits
    uint32_t *rounds;
    __device__ BinStates(void *base, uint32_t B)
    {
        lanes = static_cast<uint4 *>(base);
        s1 = reinterpret_cast<unsigned long long *>(lanes + B);
        q1 = s1 + B;
        q2 = q1 + B;
        n = reinterpret_cast<uint32_t *>(q2 + B);
        h = n + B;
        rounds = h + B;
    }
};
// Bytes of shared memory the bin states of a B-bin detector take.
constexpr size_t bin_state_bytes(uint32_t B) { return (size_t)B * (16 + 3 * 8 + 3 * 4); }

// Once per device, before the first pass: the adaptive kernels' shared-memory limit
// (above the default 48 KB).
cudaError_t configure_kernels();

// ------------------------------------------------------------ device-resident serving loop
//
// A persistent kernel whose CTAs take designs from a ring in mapped host memory and
// evaluate each one whole (setup, FP32 trace, re-trace of the guard bands and the flagged
// rays, entropy, finalize) with no host step between designs. The host publishes records
// and reads completions; nothing on the device waits for anything but new work, and that
// wait gives up after an idle limit.

// One design of the ring (mapped host memory), written by the host before it publishes
// the index: the design, its job (W, R, Rz, B, tables' offsets in the table arena,
// fixed-point units) and the trace mode.
struct alignas(16) LoopWork {
    DevDesign d;
    DesignJob j;
    uint32_t mode;
    uint32_t ray_tile;
    uint32_t pad[2];
};
static_assert(sizeof(LoopWork) % 16 == 0, "ring records are copied in 16-byte words");

// The result slot of a ring entry (mapped host memory): written by the CTA that evaluated
// the entry, then `seq` = index + 1 after a system-scope fence.
struct alignas(16) LoopDone {
    DesignOut o;
    unsigned long long seq;
    uint32_t status;   // 0, or the design exceeded the CTA's queue (never: it re-traces inline)
    uint32_t pad;
};

// Control words (mapped host memory), written by the host.
struct alignas(16) LoopCtl {
    unsigned long long published;  // ring entries published (monotone)
    unsigned int stop;             // the CTAs leave once no published entry is left
    unsigned int pad;
};

struct LoopArgs {
    const LoopWork *ring;         // capacity entries (mapped)
    LoopDone *done;               // capacity entries (mapped)
    LoopCtl *ctl;                 // mapped
    unsigned long long *claimed;  // device: ring entries claimed by CTAs
    uint32_t capacity;
    uint32_t max_cells;           // histogram cells of a slab (W B)
    uint32_t max_rows;            // wavelength rows of a slab
    uint32_t qcap;                // flagged rays a slab's queue holds (more are re-traced inline)
    unsigned char *slabs;         // per-CTA scratch, slab_bytes each
    size_t slab_bytes;
    const double *lam;            // table arena: wavelength u-points
    const double *z64;            // table arena: sorted z, f64
    const float *z32;             // table arena: sorted z, (hi, lo) float pairs
    const float *logtab;
    unsigned long long idle_ns;   // a CTA leaves after this long without work
    struct LoopCounters *cnt;     // device
    uint32_t max_B;               // widest detector a slab holds
    uint32_t pad;
};

// Device-side counters of the loop kernel.
struct LoopCounters {
    unsigned long long claimed;     // ring entries claimed by CTAs
    unsigned long long designs;     // designs evaluated
    unsigned long long inline_retraced;  // flagged rays re-traced inline (the queue was full)
    unsigned int idle_exits;        // CTAs that left after the idle limit
    unsigned int stop_exits;        // CTAs that left on the host's stop word
};

// A DesignOut as the cpd_fitness of a fixed-N evaluation of `rays` rays (with the SEM
// convergence status), as every synchronous entry point fills it.
void fitness_from_out(const DesignOut &o, uint64_t rays, cpd_fitness &f);

// Bytes of one CTA's slab for designs of up to max_rows rows and max_cells cells.
size_t loop_slab_bytes(uint32_t max_rows, uint32_t max_cells, uint32_t max_B, uint32_t qcap);
// Launches the loop kernel with `grid` CTAs on `stream`.
void launch_loop(const LoopArgs &a, uint32_t grid, cudaStream_t stream);
// CTAs of the loop kernel resident per SM.
int loop_ctas_per_sm();

// Launches setup -> trace -> retrace -> entropy -> finalize on `stream` (adaptive
// sampling: setup -> adaptive rounds -> exact rounds of the unsure rows -> entropy ->
// finalize). Returns the
// number of kernel launches issued. If `ev` is given (5 events), ev[0..3] are recorded
// before setup, trace, retrace and entropy, and ev[4] after finalize. With `pdl` (and no
// events) each kernel after the setup is a programmatic dependent launch: its blocks
// become resident while its predecessor runs and wait for its results.
int launch_pass(const LaunchArgs &a, int num_sms, uint32_t warps_per_cta, cudaStream_t stream,
                cudaEvent_t *ev = nullptr, bool pdl = false);

// Warps of the trace kernel resident at once with this block shape.
// The kernel of a single-design pass's trace (its graph node's parameters carry the
// design's constants and are updated per call).
const void *trace_spans_kernel_fn();

uint64_t trace_resident_warps(int num_sms, uint32_t warps_per_cta);

// cpd_design records built on the device from n parameter records (one thread each).
void launch_build_records(const cpd_spectrometer_params *p, uint32_t n, double acceptance, cpd_design *out,
                          int32_t *status, cudaStream_t stream);

// One thread per (lam_u[i], z[i]) pair: the twin of propagation_test_kernel.
void launch_trace_pairs(const DevDesign *d, const double *lam_u, const double *z64, uint32_t n, uint32_t mode,
                        uint32_t *bins, double *ts, uint8_t *flags, cudaStream_t stream);

// The reference CPU estimator of p(d|lambda) (p_dets_l_wavelength, src/fitness.rs:5-69) for
// n explicit wavelengths, one block each: out[n x B] and the rays each consumed. z64 holds
// norminv of the reference's ray points in ray order (max_m of them).
void launch_tp_adaptive(const DevDesign *d, uint32_t B, const double *lambdas, uint32_t n, const double *z64,
                        uint32_t max_m, double *out, uint32_t *rays_out, cudaStream_t stream);

// FP32 FMA throughput probe.
void launch_fma_peak(float *out, uint32_t iters, int blocks, int threads, cudaStream_t stream);
// SFU (MUFU) throughput probe: 8 x 16 reciprocal-square-root estimates per thread and iteration.
void launch_mufu_peak(float *out, uint32_t iters, int blocks, int threads, cudaStream_t stream);

}  // namespace cpd
