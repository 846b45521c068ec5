// cpd_kernels.cu -- the GB300 kernels of the fitness path.
//
// A pass over a set of designs runs five kernels on one stream:
//   setup    one thread per (design, wavelength): the flat-face chain in float-float
//            (cpd_df.h) -> LamParams for the fast path and LamDF for the re-trace;
//            guard-band rays of the y interval go to the re-trace queue
//   trace    persistent warps over work items (design, 32-wavelength block, ray
//            chunk); lane = wavelength; FP32 exit face + detector per ray; hits
//            accumulate per lane as run-length fixed-point sums (rays are sorted by
//            start height, so consecutive rays mostly share a bin) flushed with one
//            64-bit atomic per run; guard-band rays go to the warp's list, which the warp
//            re-traces itself (the global queue once the list is full)
//   retrace  every queued ray: float-float re-trace (exact f64 in the FP64 study mode,
//            bit-identical to the reference's f64 CPU trace)
//   entropy  one warp (many tiles) or one block (few) per (design, row tile): p = sum/R,
//            p log2 p, per-bin sums of p and p^2 in float-float with fixed-point
//            accumulation (order independent)
//   finalize one warp per design: H(D), MI, SEM convergence (in a single-design pass the
//            entropy block that completes the last tile runs it).
// A single-design pass with a fixed ray count (the plain call) runs setup_pair_kernel (two
// warps per 32 rows) and trace_spans_kernel (equal shares of the ray slots per warp, the
// design's constants as kernel parameters) in place of the first two. Adaptive sampling
// replaces trace and retrace with adaptive1_kernel / adaptive_kernel and
// adaptive_exact_kernel.
#include <cuda_runtime.h>

#include "cpd_build.h"
#include "cpd_df.h"
#include "cpd_gpu.cuh"

namespace cpd {

namespace {

enum Field { F_ROW = 0, F_ITEM = 1, F_TILE = 2 };

template <int FIELD>
__device__ __forceinline__ uint64_t job_field(const DesignJob &j)
{
    return FIELD == F_ROW ? j.row_off : FIELD == F_ITEM ? j.item_off : j.tile_off;
}

// Largest i with field(jobs[i]) <= v.
template <int FIELD>
__device__ __forceinline__ uint32_t find_job(const DesignJob *__restrict__ jobs, uint32_t n, uint64_t v)
{
    uint32_t lo = 0, hi = n;
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if (job_field<FIELD>(jobs[mid]) <= v) lo = mid;
        else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ void push_ray(const LaunchArgs &a, uint32_t d, uint32_t k, uint32_t j)
{
    unsigned long long pos = atomicAdd(&a.ctl->queue_count, 1ull);
    if (pos < a.qcap) a.queue[pos] = QEntry{d, k, j, 0u};
    else atomicOr(&a.ctl->overflow, 1u);
}

// The rays [j0, j1) and [j2, j3) of row k, queued with one atomic for the whole run (a row's
// guard bands can hold dozens of rays; one round trip to the queue counter per ray made a
// serial chain on the setup's critical path).
__device__ __forceinline__ void push_ranges(const LaunchArgs &a, uint32_t d, uint32_t k, uint32_t j0, uint32_t j1,
                                            uint32_t j2, uint32_t j3)
{
    const uint32_t na = j1 > j0 ? j1 - j0 : 0u, nb = j3 > j2 ? j3 - j2 : 0u;
    if (na + nb == 0u) return;
    const unsigned long long pos = atomicAdd(&a.ctl->queue_count, (unsigned long long)(na + nb));
    if (pos + na + nb > a.qcap) atomicOr(&a.ctl->overflow, 1u);
    for (uint32_t i = 0; i < na + nb; i++) {
        if (pos + i >= a.qcap) break;
        a.queue[pos + i] = QEntry{d, k, i < na ? j0 + i : j2 + (i - na), 0u};
    }
}

// Designs built on the device from parameter records (CPD_BUILD_ON_DEVICE): one thread
// per design, the f64 construction of cpd_build.h (positioning first when the pass's
// acceptance is positive), written straight into the pass's design records. A design whose
// construction fails keeps its status in the record; the setup then loses all its rays.
__global__ void __launch_bounds__(32) build_kernel(const LaunchArgs a)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.njobs) return;
    cpd_design d;
    const int e = build::design_positioned(a.params[i], a.build_acceptance, d);
    DevDesign D;
    build::to_dev(d, D);
    D.status = e;
    if (e) D.B = a.jobs[i].B;
    const_cast<DevDesign *>(a.designs)[i] = D;
}

// cpd_design records from parameter records, for the host (cpd_design_build_device).
__global__ void __launch_bounds__(32) build_records_kernel(const cpd_spectrometer_params *p, uint32_t n,
                                                           double acceptance, cpd_design *out, int32_t *status)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    cpd_design d;
    status[i] = build::design_positioned(p[i], acceptance, d);
    out[i] = d;
}


__device__ __forceinline__ void cp_async16(void *smem, const void *gmem)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gmem) : "memory");
}

// The setup of one wavelength row (below): LamParams and LamDF, and the row's guard-band
// rays queued. Returns the row's fast-path range [core_lo, core_hi) (empty: hi <= lo).
// A row whose design failed its device build: every ray of it is lost.
__device__ __forceinline__ uint2 setup_failed_row(const LaunchArgs &a, uint64_t row)
{
    LamParams P;
    zero_lam_params(P);
    LamDF *E = a.lx + row;
    memset(E, 0, sizeof(LamDF));
    E->lost = 1u;
    a.lp[row] = P;
    return make_uint2(0u, 0u);
}

// A row's LamParams after lambda_setup_df: its guard-band rays queued as the mode asks, the
// record written. Returns the row's fast-path range [core_lo, core_hi) (empty: hi <= lo).
__device__ __forceinline__ uint2 setup_finish(const LaunchArgs &a, uint32_t d, uint32_t k, uint64_t row, LamParams &P)
{
    if (a.adaptive) {
        // the adaptive rounds trace every ray of the band themselves
    } else if (a.mode == CPD_TRACE_FP64 || (P.all_exact && a.mode == CPD_TRACE_HYBRID)) {
        push_ranges(a, d, k, P.band_lo, P.band_hi, 0u, 0u);
        P.core_lo = P.core_hi = 0;
    } else if (P.all_exact) {
        // FP32-only study mode without a reference ray: these rays are counted as lost
        P.core_lo = P.core_hi = 0;
    } else {
        push_ranges(a, d, k, P.band_lo, P.core_lo, P.core_hi, P.band_hi);
    }
    a.lp[row] = P;
    return make_uint2(P.core_lo, P.core_hi);
}

// The setup of one wavelength row (below): LamParams and LamDF, and the row's guard-band
// rays queued. Returns the row's fast-path range [core_lo, core_hi) (empty: hi <= lo).
__device__ __forceinline__ uint2 setup_row(const LaunchArgs &a, uint64_t row, uint32_t d, double u,
                                           const DevDesign &sD, uint32_t d0, bool stage_z, const float *sz)
{
    const DesignJob &J = a.jobs[d];
    const uint32_t k = (uint32_t)(row - J.row_off);
    const bool staged = d == d0;
    const DevDesign &D = staged ? sD : a.designs[d];
    const float *z32 = staged && stage_z ? sz : a.z32 + 2 * J.ray_off;
    if (D.status) return setup_failed_row(a, row);
    LamParams P;
    lambda_setup_df(D, u, z32, J.Rz, P, a.yguard_rel, a.lx + row, a.adaptive != 0);
    return setup_finish(a, d, k, row, P);
}

// One warp per block of 32 rows. The block first copies its design record and, for
// tables of up to a.stage_cap rays, its sorted z table into shared memory with
// asynchronous 16-byte copies that are all in flight at once (one memory latency
// instead of a chain of dependent loads), so the per-wavelength program and its binary
// searches run on shared-memory operands. Ray tables start 16-byte aligned (the host
// pads each to an even number of rays).
__global__ void __launch_bounds__(32) setup_kernel(const LaunchArgs a)
{
    // lets the trace kernel's blocks become resident now; they wait for this grid's
    // results in cudaGridDependencySynchronize
    cudaTriggerProgrammaticLaunchCompletion();
    if (a.clear_acc) {
        // a fresh pass: zero the per-bin and per-design accumulators (the kernels that add
        // to them wait for this grid to complete)
        const uint64_t gt = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
        const uint64_t nt = (uint64_t)gridDim.x * blockDim.x;
        for (uint64_t i = gt; i < a.acc_cells; i += nt) a.S1[i] = a.S2[i] = 0ull;
        unsigned long long *acc = reinterpret_cast<unsigned long long *>(a.acc);
        const uint64_t words = (uint64_t)a.njobs * (sizeof(DesignAcc) / sizeof(unsigned long long));
        for (uint64_t i = gt; i < words; i += nt) acc[i] = 0ull;
    }
    __shared__ __align__(16) DevDesign sD;
    extern __shared__ __align__(16) float sz[];  // 2 even(stage_cap) floats
    const uint64_t row0 = blockIdx.x * (uint64_t)blockDim.x;
    const uint64_t row = row0 + threadIdx.x;
    const uint32_t d0 = find_job<F_ROW>(a.jobs, a.njobs, row0);
    const DesignJob &J0 = a.jobs[d0];
    const bool stage_z = J0.Rz <= a.stage_cap;
    // the row's design and wavelength point, loaded while the copies below are in flight
    // (the point is not in L2 when the previous pass's tables were evicted)
    uint32_t d = 0;
    double u = 0.0;
    if (row < a.total_rows) {
        d = find_job<F_ROW>(a.jobs, a.njobs, row);
        const DesignJob &J = a.jobs[d];
        u = a.lam_u[J.lam_off + (row - J.row_off)];
    }
    {
        const char *src = reinterpret_cast<const char *>(a.designs + d0);
        char *dst = reinterpret_cast<char *>(&sD);
        for (uint32_t i = threadIdx.x; i < sizeof(DevDesign) / 16; i += blockDim.x) cp_async16(dst + 16 * i, src + 16 * i);
        if (stage_z) {
            const char *zs = reinterpret_cast<const char *>(a.z32 + 2 * J0.ray_off);
            char *zd = reinterpret_cast<char *>(sz);
            const uint32_t n16 = (J0.Rz + 1u) / 2u;  // 16-byte chunks (two rays each)
            for (uint32_t i = threadIdx.x; i < n16; i += blockDim.x) cp_async16(zd + 16 * i, zs + 16 * i);
        }
        asm volatile("cp.async.wait_all;" ::: "memory");
    }
    __syncthreads();
    uint2 core = make_uint2(0u, 0u);
    if (row < a.total_rows) core = setup_row(a, row, d, u, sD, d0, stage_z, sz);
    if (a.spans) {
        // single-design pass: this block's 32 rows are the trace's block blockIdx.x
        const bool any = core.y > core.x;
        const uint32_t lo = __reduce_min_sync(0xffffffffu, any ? core.x : 0xffffffffu);
        const uint32_t hi = __reduce_max_sync(0xffffffffu, any ? core.y : 0u);
        if (threadIdx.x == 0) {
            const uint2 s = hi > lo ? make_uint2(lo, hi) : make_uint2(0u, 0u);
            a.spans[blockIdx.x] = s;
            if (s.y > s.x) atomicAdd(&a.ctl->item_counter, (unsigned long long)(s.y - s.x));
        }
    }
}


// The rays [j0, j1) of the 32-row block blk of design d (lane = row), each lane clamped
// to its row's fast-path range: FP32 fast path, hits as run-length fixed-point sums
// flushed with one 64-bit atomic per run, guard-band rays queued for the re-trace.
// The setup of a single-design pass (a.spans set) by two warps per block of 32 rows. Each
// row's flat-face chain splits into two halves that depend on each other only through the
// direction entering each face: warp 0 runs the direction part of every face (the glass
// index, the refraction, the Fresnel factors), warp 1 the position part (the distance to
// the face, the bounds it puts on y, the point on it), face by face in step: at face k warp
// 1 reads the direction d_k that warp 0 published at face k - 1, one block barrier per face.
// Each warp stops where lambda_setup_df's loop would stop (a face parallel to the ray, which
// both see from the same cosine; total internal reflection, which warp 0 reports; a bound
// independent of y, which warp 1 reports), and warp 0 then finishes the row alone (y
// interval, ray ranges, reference ray). The functions are lambda_setup_df's own, so every
// output is bit-identical to the one-warp setup; the chain that is one warp per SM in the
// plain call is about half as long.
__global__ void __launch_bounds__(64) setup_pair_kernel(const LaunchArgs a)
{
    cudaTriggerProgrammaticLaunchCompletion();
    if (a.clear_acc) {
        const uint64_t gt = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
        const uint64_t nt = (uint64_t)gridDim.x * blockDim.x;
        for (uint64_t i = gt; i < a.acc_cells; i += nt) a.S1[i] = a.S2[i] = 0ull;
        unsigned long long *acc = reinterpret_cast<unsigned long long *>(a.acc);
        const uint64_t words = (uint64_t)a.njobs * (sizeof(DesignAcc) / sizeof(unsigned long long));
        for (uint64_t i = gt; i < words; i += nt) acc[i] = 0ull;
    }
    __shared__ __align__(16) DevDesign sD;
    extern __shared__ __align__(16) float sz[];  // 2 even(stage_cap) floats
    __shared__ ff::F2 s_dir[CPD_MAX_GLASS + 1][2][32];  // direction entering face k (x, y)
    __shared__ uint32_t s_tir[32], s_bound[32];          // stops reported at the last face
    __shared__ SetupPos s_pos[32];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint64_t row = blockIdx.x * 32ull + lane;
    const DesignJob &J = a.one;
    const bool have = row < a.total_rows;
    const bool stage_z = J.Rz <= a.stage_cap;
    const double u = have && warp == 0 ? a.lam_u[J.lam_off + row] : 0.0;
    {
        // two groups of copies: the design record, which the face loop needs, and the z
        // table, which only the ray ranges after the loop read (its copies land while the
        // faces run)
        const char *src = reinterpret_cast<const char *>(a.designs);
        char *dst = reinterpret_cast<char *>(&sD);
        for (uint32_t i = threadIdx.x; i < sizeof(DevDesign) / 16; i += blockDim.x) cp_async16(dst + 16 * i, src + 16 * i);
        asm volatile("cp.async.commit_group;" ::: "memory");
        if (stage_z) {
            const char *zs = reinterpret_cast<const char *>(a.z32 + 2 * J.ray_off);
            char *zd = reinterpret_cast<char *>(sz);
            const uint32_t n16 = (J.Rz + 1u) / 2u;  // 16-byte chunks (two rays each)
            for (uint32_t i = threadIdx.x; i < n16; i += blockDim.x) cp_async16(zd + 16 * i, zs + 16 * i);
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
        asm volatile("cp.async.wait_group 1;" ::: "memory");
    }
    __syncthreads();
    const DevDesign &D = sD;
    const int G = D.G;
    const float yg = (float)a.yguard_rel;
    SetupDir Sd = setup_dir_init();
    SetupPos Sp = setup_pos_init();
    const ff::F2 lambda = warp == 0 ? setup_lambda(D, u) : ff::F2{0.f, 0.f};
    bool stop = !have || D.status != 0;
    bool lost = false;  // warp 0: a face parallel to the ray, or total internal reflection
#pragma unroll 1
    for (int k = 0; k < G; k++) {
        bool tir = false;
        if (!stop) {
            if (warp == 0) {
                const ff::F2 ci = face_cos(D, k, Sd.dx, Sd.dy);
                if (ci.hi == 0.f) {
                    lost = stop = true;
                } else if (!face_direction(D, k, lambda, ci, Sd, false)) {
                    lost = stop = tir = true;
                } else {
                    s_dir[k + 1][0][lane] = Sd.dx;
                    s_dir[k + 1][1][lane] = Sd.dy;
                }
            } else {
                const ff::F2 dx = k == 0 ? df::c(1.f) : s_dir[k][0][lane];
                const ff::F2 dy = k == 0 ? df::c(0.f) : s_dir[k][1][lane];
                const ff::F2 ci = face_cos(D, k, dx, dy);
                if (ci.hi == 0.f) stop = true;  // warp 0 sees the same cosine
                else face_position(D, k, ci, dx, dy, Sp, yg);
                if (Sp.lost) stop = true;
            }
        }
        if (warp == 0) s_tir[lane] = tir ? 1u : 0u;
        else s_bound[lane] = Sp.lost ? 1u : 0u;
        __syncthreads();
        // lambda_setup_df breaks after a face's direction part that found total internal
        // reflection, and before the face after one whose position part found a bound
        // independent of y
        if (warp == 0 && s_bound[lane]) stop = true;
        if (warp == 1 && s_tir[lane]) stop = true;
        __syncthreads();  // the flags are written again at the next face
    }
    if (warp == 1) s_pos[lane] = Sp;
    asm volatile("cp.async.wait_all;" ::: "memory");  // this thread's share of the z table
    __syncthreads();
    if (warp == 1) return;
    uint2 core = make_uint2(0u, 0u);
    if (have) {
        if (D.status) {
            core = setup_failed_row(a, row);
        } else {
            Sp = s_pos[lane];
            const float *z32 = stage_z ? sz : a.z32 + 2 * J.ray_off;
            LamParams P;
            zero_lam_params(P);
            setup_tail(D, z32, J.Rz, P, a.lx + row, Sd, Sp, lost || Sp.lost);
            core = setup_finish(a, 0u, (uint32_t)row, row, P);
        }
    }
    // this block's 32 rows are the trace's block blockIdx.x
    const bool any = core.y > core.x;
    const uint32_t lo = __reduce_min_sync(0xffffffffu, any ? core.x : 0xffffffffu);
    const uint32_t hi = __reduce_max_sync(0xffffffffu, any ? core.y : 0u);
    if (lane == 0) {
        const uint2 sp = hi > lo ? make_uint2(lo, hi) : make_uint2(0u, 0u);
        a.spans[blockIdx.x] = sp;
        if (sp.y > sp.x) atomicAdd(&a.ctl->item_counter, (unsigned long long)(sp.y - sp.x));
    }
}

// Flagged rays a warp of the single-design trace keeps for its own re-trace.
constexpr uint32_t kWarpFlags = 32;

// The float-float re-trace of one queued ray (k, j) of design d, counted in copy sp of
// the design's counters.
__device__ __forceinline__ void retrace_ray(const LaunchArgs &a, uint32_t d, uint32_t k, uint32_t j, uint32_t sp)
{
    const DesignJob &J = a.jobs[d];
    const float *z = a.z32 + 2 * (J.ray_off + j);
    uint32_t bin = 0;
    float t = 0.f;
    if (trace_df(a.designs[d], a.lx[J.row_off + k], z[0], z[1], bin, t)) {
        atomicAdd(a.hist + J.hist_off + (uint64_t)k * J.B + bin, (unsigned long long)t_fixed(t));
        atomicAdd(&a.acc[d].hits[sp], 1ull);
    }
    atomicAdd(&a.acc[d].retraced[sp], 1ull);
}

// PARAM_FC: the single-design trace, whose constants are kernel parameters. Flagged rays
// go to the warp's list (wlist, *wcount: design, row, ray), the global queue once it is full.
template <bool PARAM_FC>
__device__ __forceinline__ void trace_block_rays(const LaunchArgs &a, uint32_t d, const DesignJob &J, uint32_t blk,
                                                 uint32_t j0, uint32_t j1, uint32_t lane, uint3 *wlist,
                                                 uint32_t *wcount)
{
    const uint32_t k = blk * 32u + lane;
    // the design's constants: kernel parameters (constant-bank operands, no registers)
    // for a single-design pass, else a copy in registers
    const FastConst Cd = PARAM_FC ? FastConst{} : a.designs[d].fc;
    const FastConst &C = PARAM_FC ? a.fc : Cd;
    const FastLimits Ld = PARAM_FC ? FastLimits{} : fast_limits(Cd, a.guards);
    const FastLimits &Lm = PARAM_FC ? a.fl : Ld;
    LamParams P;
    uint32_t lo = 0, hi = 0;
    if (k < J.W) {
        P = a.lp[J.row_off + k];
        lo = max(j0, P.core_lo);
        hi = min(j1, P.core_hi);
    }
    const float2 *__restrict__ zt = reinterpret_cast<const float2 *>(a.z32) + J.ray_off;
    unsigned long long *hrow = a.hist + J.hist_off + (uint64_t)k * J.B;
    uint32_t cur = 0xffffffffu;
    unsigned long long sum = 0ull;
    uint32_t nhit = 0;
    for (uint32_t j = lo; j < hi; ++j) {
        const float2 z = __ldg(zt + j);
        uint32_t bin = 0;
        float t = 0.f;
        const int r = fast_ray(C, Lm, P, a.guards, z.x, z.y, bin, t);
        if (r == RAY_HIT) {
            if (bin != cur) {
                if (sum) atomicAdd(hrow + cur, sum);
                cur = bin;
                sum = 0ull;
            }
            sum += t_fixed(t);
            nhit++;
        } else if (r == RAY_FLAG) {
            const uint32_t pos = atomicAdd(wcount, 1u);
            if (pos < kWarpFlags) wlist[pos] = make_uint3(d, k, j);
            else push_ray(a, d, k, j);
        }
    }
    if (sum) atomicAdd(hrow + cur, sum);
    nhit = __reduce_add_sync(0xffffffffu, nhit);
    const uint32_t nfast = __reduce_add_sync(0xffffffffu, hi > lo ? hi - lo : 0u);
    const uint32_t sp = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) % (uint32_t)kSpread;
    if (lane == 0 && nhit) atomicAdd(&a.acc[d].hits[sp], (unsigned long long)nhit);
    if (lane == 0 && nfast) atomicAdd(&a.acc[d].fast[sp], (unsigned long long)nfast);
}

// The trace of a single-design pass whose setup wrote the blocks' spans (a.spans). Its
// design constants are kernel parameters (constant-bank operands), which frees the ~17
// registers a copy of them takes (75 registers with the re-trace list, no spill). Measured
// on the 4096 x 1024 plain pass: at 64 registers
// (4 blocks of 256 per SM, 32 warps, no spill) the trace issues 68% of the slots against
// 62%, but fills the register file, so the re-trace and entropy blocks can no longer
// become resident while it runs, and the pass is ~1.5 us slower than at 3 blocks per SM.
#ifndef CPD_TRACE_SPANS_MIN_BLOCKS
#define CPD_TRACE_SPANS_MIN_BLOCKS 3
#endif
__global__ void __launch_bounds__(256, CPD_TRACE_SPANS_MIN_BLOCKS) trace_spans_kernel(const LaunchArgs a)
{
    cudaTriggerProgrammaticLaunchCompletion();
    cudaGridDependencySynchronize();  // setup's LamParams and queue
    const uint32_t lane = threadIdx.x & 31u;
    // Equal shares of the design's fast-path ray slots: the blocks' spans laid end to
    // end (U slots in all), warp w taking [U w / nw, U (w + 1) / nw). A warp's lanes
    // step through a block's span together, so a span costs its length whatever the
    // rows' own ranges; every warp gets the same work and no warp waits on a counter.
    // Nothing stays live in registers across a segment's ray loop (which needs every
    // register it can get): the cursor waits in shared memory, and the share's end and the
    // prefix over the spans are found again from the pass's words for each segment.
    // A warp's flagged rays wait in its list and are re-traced by the warp after its share
    // (rays past kWarpFlags go to the global queue and the re-trace kernel): the re-trace
    // of the pass then overlaps the trace instead of following it.
    __shared__ volatile unsigned long long s_cur[8];  // per warp of the block (<= 256 threads)
    __shared__ uint3 s_flags[8][kWarpFlags];
    __shared__ uint32_t s_nflags[8];
    const uint32_t wib = threadIdx.x >> 5;
    {
        const uint64_t w = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
        const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
        s_cur[wib] = a.ctl->item_counter * w / nw;  // the next slot of this warp's share
        if (lane == 0) s_nflags[wib] = 0u;
    }
    for (;;) {
        __syncwarp();
        uint64_t cur = s_cur[threadIdx.x >> 5];
        const uint64_t end = a.ctl->item_counter * (((blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5) + 1u) /
                             (((uint64_t)gridDim.x * blockDim.x) >> 5);
        if (cur >= end) break;
        const uint32_t nb = (a.jobs[0].W + 31u) / 32u;
        uint64_t pre = 0;  // slots of the blocks before group c
        uint32_t c = 0, sx, len, incl;
        for (;;) {
            const uint32_t b = c + lane;
            const uint2 s = b < nb ? a.spans[b] : make_uint2(0u, 0u);
            sx = s.x;
            len = s.y - s.x;
            incl = len;  // inclusive scan over the group
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= (uint32_t)o) incl += v;
            }
            const uint32_t tot = __shfl_sync(0xffffffffu, incl, 31);
            if (pre + tot > cur) break;
            pre += tot;
            c += 32u;
        }
        // the block holding the cursor: the first whose end lies past it (nonempty)
        const int l = __ffs(__ballot_sync(0xffffffffu, pre + incl > cur)) - 1;
        const uint32_t bx = __shfl_sync(0xffffffffu, sx, l);
        const uint32_t ln = __shfl_sync(0xffffffffu, len, l);
        const uint64_t e0 = pre + __shfl_sync(0xffffffffu, incl, l) - ln;
        const uint64_t rem = end - e0;
        const uint32_t stop = rem < ln ? (uint32_t)rem : ln;
        const uint32_t r0 = bx + (uint32_t)(cur - e0);
        __syncwarp();
        s_cur[threadIdx.x >> 5] = e0 + stop;
        const DesignJob J = a.jobs[0];
        trace_block_rays<true>(a, 0u, J, c + (uint32_t)l, r0, bx + stop, lane, s_flags[wib], &s_nflags[wib]);
    }
    __syncwarp();
    const uint32_t nf = min(s_nflags[wib], kWarpFlags);
    const uint32_t sp = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) % (uint32_t)kSpread;
    for (uint32_t i = lane; i < nf; i += 32u) retrace_ray(a, 0u, s_flags[wib][i].y, s_flags[wib][i].z, sp);
}

// 72 registers: 28 resident warps per SM (blocks of 2 or 4 warps) against 24 at 80, for a
// 24-byte spill; measured on the 1024-design batched pass: 12.82 -> 12.33 ms (64 registers
// spill 88 bytes: 16.4 ms)
#ifndef CPD_TRACE_MAXNREG
#define CPD_TRACE_MAXNREG 72
#endif
__global__ void __maxnreg__(CPD_TRACE_MAXNREG) trace_kernel(const LaunchArgs a)
{
    cudaTriggerProgrammaticLaunchCompletion();
    cudaGridDependencySynchronize();  // setup's LamParams and queue
    const uint32_t lane = threadIdx.x & 31u;
    // a warp's flagged rays wait in its list; the warp re-traces them once half of the
    // list is taken, and at its end (rays past kWarpFlags go to the global queue)
    __shared__ uint3 s_flags[8][kWarpFlags];
    __shared__ uint32_t s_nflags[8];
    const uint32_t wib = threadIdx.x >> 5;
    const uint32_t sp = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) % (uint32_t)kSpread;
    if (lane == 0) s_nflags[wib] = 0u;
    for (;;) {
        unsigned long long item = 0;
        if (lane == 0) item = atomicAdd(&a.ctl->item_counter, 1ull);
        item = __shfl_sync(0xffffffffu, item, 0);
        if (item >= a.total_items) break;
        const uint32_t d = find_job<F_ITEM>(a.jobs, a.njobs, item);
        const DesignJob J = a.jobs[d];
        const uint64_t local = item - J.item_off;
        const uint32_t blk = (uint32_t)(local / J.nchunk);
        const uint32_t chunk = (uint32_t)(local - (uint64_t)blk * J.nchunk);
        const uint32_t j0 = chunk * a.ray_tile;
        trace_block_rays<false>(a, d, J, blk, j0, min(j0 + a.ray_tile, J.Rz), lane, s_flags[wib], &s_nflags[wib]);
        __syncwarp();
        const uint32_t nf = s_nflags[wib];
        if (nf >= kWarpFlags / 2u) {
            const uint32_t n = min(nf, kWarpFlags);
            if (lane < n) retrace_ray(a, s_flags[wib][lane].x, s_flags[wib][lane].y, s_flags[wib][lane].z, sp);
            __syncwarp();
            if (lane == 0) s_nflags[wib] = 0u;
            __syncwarp();
        }
    }
    __syncwarp();
    const uint32_t n = min(s_nflags[wib], kWarpFlags);
    if (lane < n) retrace_ray(a, s_flags[wib][lane].x, s_flags[wib][lane].y, s_flags[wib][lane].z, sp);
}

// The queued rays, hybrid mode: the float-float re-trace.
// The pass's final queue state for the host (no later kernel changes it).
__device__ __forceinline__ void publish_status(const LaunchArgs &a)
{
    if (a.status && blockIdx.x == 0 && threadIdx.x == 0) {
        a.status->queue_count = a.ctl->queue_count;
        a.status->overflow = a.ctl->overflow;
        a.status->pad = 0u;
    }
}

__global__ void __launch_bounds__(32) retrace_kernel(const LaunchArgs a)
{
    cudaTriggerProgrammaticLaunchCompletion();
    cudaGridDependencySynchronize();  // the queue of the setup and trace kernels
    publish_status(a);
    const unsigned long long qn = a.ctl->queue_count;
    const uint64_t n = qn < a.qcap ? qn : a.qcap;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const QEntry e = a.queue[i];
        retrace_ray(a, e.design, e.k, e.j, (uint32_t)(i % kSpread));
    }
}

// The queued rays, FP64 study mode: the exact f64 trace of the reference
// (bit-identical to its CPU path). A kernel of its own, so that the hybrid re-trace
// does not carry this code.
__global__ void __launch_bounds__(32) retrace_exact_kernel(const LaunchArgs a)
{
    cudaTriggerProgrammaticLaunchCompletion();
    cudaGridDependencySynchronize();  // the queue of the setup and trace kernels
    publish_status(a);
    const unsigned long long qn = a.ctl->queue_count;
    const uint64_t n = qn < a.qcap ? qn : a.qcap;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const QEntry e = a.queue[i];
        const DevDesign &D = a.designs[e.design];
        const DesignJob &J = a.jobs[e.design];
        uint32_t bin = 0;
        double t = 0.0;
        if (x::trace(D, x::wavelength(D, a.lam_u[J.lam_off + e.k]), x::beam_y(D, a.z64[J.ray_off + e.j]), bin, t) ==
            0) {
            atomicAdd(a.hist + J.hist_off + (uint64_t)e.k * J.B + bin, (unsigned long long)t_fixed64(t));
            atomicAdd(&a.acc[e.design].hits[i % kSpread], 1ull);
        }
        atomicAdd(&a.acc[e.design].retraced[i % kSpread], 1ull);
    }
}

// ------------------------------------------------------------------ adaptive sampling

// The float-float exact trace of one ray as (bin or ~0u, t_fixed).
__device__ __forceinline__ uint2 trace_df_exact_packed(const DevDesign &D, const LamDF &E, float zh, float zl)
{
    uint32_t b = 0, tx = 0;
    return trace_df_exact(D, E, zh, zl, b, tx) ? make_uint2(b, tx) : make_uint2(0xffffffffu, 0u);
}

// The same, out of line: the fast kernel takes it for ~0.1% of its rays, and inlined its
// float-float code would set the register budget of the whole kernel.
__device__ __noinline__ uint2 trace_df_exact_call(const DevDesign &D, const LamDF &E, float zh, float zl)
{
    return trace_df_exact_packed(D, E, zh, zl);
}

// Per-warp scratch of the adaptive kernels (dynamic shared memory, one slot per warp,
// before the bin states). A group of KW rounds is traced by KW warps, warp w taking round
// w of the group; each warp sums its round's hits per bin into its slot, and the group's
// stop decisions are then taken by all warps at once, each from its round's exact Welford
// states (the states at the group's start plus the sums of the group's rounds up to its
// own). The first round that stops, or that the FP32 sums cannot settle, ends the row.
struct RoundSlot {
    // indexed by the leader lane of a bin the round hit: the round's sums there, in 32-bit
    // pieces (t_fixed = q 2^11 + low, q = qh 2^10 + ql, q <= 2^20): sum q, sum low,
    // sum qh^2, sum qh ql, sum ql^2, and the hits
    uint32_t p[6][32];
    uint32_t df;       // ballot of the rays traced in float-float
    uint32_t nh;       // hits of the round
    uint32_t verdict;  // 0 go on, 1 stop, 2 unsure
    uint32_t pad;
};
static_assert(sizeof(RoundSlot) % 16 == 0, "bin states follow the slots 16-byte aligned");
// Dynamic shared memory of an adaptive block of KW warps over B-bin detectors.
constexpr size_t adapt_smem_bytes(uint32_t KW, uint32_t B) { return KW * sizeof(RoundSlot) + bin_state_bytes(B); }
static_assert(adapt_smem_bytes(kMaxAdaptWarps, CPD_MAX_BINS) <= 227u * 1024u, "shared memory per block");

// Dynamic shared memory of the one-warp form (adaptive_row1): the row's LamParams and
// FastConst, one slot, the bin states.
constexpr size_t adapt1_smem_bytes(uint32_t B)
{
    return sizeof(LamParams) + sizeof(FastConst) + adapt_smem_bytes(1, B);
}

// Byte v of a bin's group lane table (v = the round within the group).
__device__ __forceinline__ uint32_t lane_entry(const uint4 &w, uint32_t v)
{
    const uint32_t word = v < 8u ? (v < 4u ? w.x : w.y) : (v < 12u ? w.z : w.w);
    return (word >> (8u * (v & 3u))) & 0xffu;
}

// One wavelength row under adaptive sampling (the stop rule of src/spectrometer/
// kernel.rs:127-178, restated with exact integer Welford sums: cpd_model.h, sem_test)
// by one block of KW warps; the bin states live in shared memory after the KW slots.
// Tracing: lane l of warp w takes ray g0 + 32 w + l in index order; `rank` maps it to its
// place in the sorted z table, whose band / core ranges (from the setup) say how to trace
// it: lost outside the band, the FP32 fast path inside the core, the float-float trace
// (exact transmittance) otherwise or when the fast path flags it.
// Deciding: each bin a round hit is led by the lowest lane that hit it; the leader sums
// the round's hits there, and the bin's group lane table records which lane of which round
// holds those sums. A round's leaders then add the sums of the group's rounds up to theirs
// to the states at the group's start, run the SEM test, and vote: the round stops the row
// when it hit some bin and every bin it hit passes. Rounds after the first one that stops
// were traced for nothing and are dropped; the states through that round are written back
// by the leader of each bin's latest round. Everything is integer, so the result equals
// the one-round-at-a-time order bit for bit.
// kExact: every ray by the float-float trace and the exact test. Otherwise a row whose
// stop decision the FP32 transmittances cannot settle (sem_test: SEM_UNSURE) leaves
// nothing behind and returns true: the caller redoes it on the exact path. (In the
// verification mode every row is queued for adaptive_exact_kernel instead.)
template <bool kExact>
__device__ bool adaptive_row(const LaunchArgs &a, uint64_t row, unsigned long long *smem, uint32_t KW,
                             uint32_t warp, uint32_t lane)
{
    const uint32_t d = find_job<F_ROW>(a.jobs, a.njobs, row);
    const DesignJob &J = a.jobs[d];
    const uint32_t k = (uint32_t)(row - J.row_off);
    const uint32_t B = J.B, R = J.R;
    const DevDesign &D = a.designs[d];
    const uint32_t tid = warp * 32u + lane, nthr = KW * 32u;
    if (!kExact && a.adaptive == 2u) {
        // verification mode: every row on the exact path
        if (tid == 0) {
            const unsigned long long pos = atomicAdd(&a.ctl->queue_count, 1ull);
            if (pos < a.qcap) a.queue[pos] = QEntry{d, k, 0u, 0u};
            else atomicOr(&a.ctl->overflow, 1u);
        }
        return false;
    }
    RoundSlot *slots = reinterpret_cast<RoundSlot *>(smem);
    RoundSlot &my = slots[warp];
    const FastConst C = D.fc;
    const LamParams P = a.lp[row];
    const LamDF &E = a.lx[row];
    const BinStates st(slots + KW, B);
    for (uint32_t b = tid; b < B; b += nthr) {
        st.s1[b] = st.q1[b] = st.q2[b] = 0ull;
        st.n[b] = st.h[b] = 0u;
        st.lanes[b] = make_uint4(0u, 0u, 0u, 0u);
        st.rounds[b] = 0u;
    }
    __syncthreads();
    const uint32_t *rank = a.rank + J.rank_off;
    const float2 *zt = reinterpret_cast<const float2 *>(a.z32) + J.ray_off;
    const uint32_t lt_mask = (1u << lane) - 1u;
    uint32_t count = 0, flag = 0;  // the same in every thread
    uint32_t hits = 0, ndf = 0;    // thread 0
    // no ray clears the flat faces: every round runs without a hit
    const uint32_t g_start = P.band_lo >= P.band_hi ? R : 0u;
    if (g_start == R) count = R;
    // the ray a lane traces in the next group, loaded while the current group is decided:
    // its sorted position (~0u: none, or no finite start height; outside the band either
    // way) and its start height
    uint32_t s_nx = 0xffffffffu;
    float2 z_nx = make_float2(0.f, 0.f);
    const auto fetch = [&](uint32_t g) {
        const uint32_t j = g + warp * kRoundRays + lane;
        s_nx = j < R ? rank[j] : 0xffffffffu;
        if (s_nx >= P.band_lo && s_nx < P.band_hi) z_nx = zt[s_nx];
    };
    if (g_start < R) fetch(g_start);
    for (uint32_t g0 = g_start; g0 < R; g0 += KW * kRoundRays) {
        // 1. trace round `warp` of the group; each bin's leader sums the round's hits there
        uint32_t bin = 0xffffffffu, tf = 0u;
        bool used_df = false;
        {
            const uint32_t s = s_nx;
            if (s >= P.band_lo && s < P.band_hi) {
                const float2 z = z_nx;
                int res = RAY_FLAG;
                if (!kExact && !P.all_exact && s >= P.core_lo && s < P.core_hi) {
                    uint32_t b = 0;
                    float t = 0.f;
                    res = fast_ray(C, P, a.guards, z.x, z.y, b, t);
                    if (res == RAY_HIT) {
                        bin = b;
                        tf = t_fixed(t);
                    }
                }
                if (res == RAY_FLAG) {
                    const uint2 r = trace_df_exact_call(D, E, z.x, z.y);
                    bin = r.x;
                    tf = r.y;
                    used_df = true;
                }
            }
        }
        if (g0 + KW * kRoundRays < R) fetch(g0 + KW * kRoundRays);
        const bool hit = bin != 0xffffffffu;
        const uint32_t hm = __ballot_sync(0xffffffffu, hit);
        const uint32_t dfb = __ballot_sync(0xffffffffu, used_df);
        const uint32_t grp = __match_any_sync(0xffffffffu, bin);
        const bool leader = hit && (grp & lt_mask) == 0u;
        if (lane == 0) {
            my.df = dfb;
            my.nh = (uint32_t)__popc(hm);
        }
        {
            // the bin's sums over its lanes: shared-memory adds into the leader's slot
            my.p[0][lane] = my.p[1][lane] = my.p[2][lane] = my.p[3][lane] = my.p[4][lane] = 0u;
            __syncwarp();
            if (hit) {
                const uint32_t ld = (uint32_t)__ffs(grp) - 1u, q = tf >> kTqShift;
                const uint32_t qh = q >> 10, ql = q & 0x3ffu;
                atomicAdd(&my.p[0][ld], q);
                atomicAdd(&my.p[1][ld], tf & 0x7ffu);
                atomicAdd(&my.p[2][ld], qh * qh);
                atomicAdd(&my.p[3][ld], qh * ql);
                atomicAdd(&my.p[4][ld], ql * ql);
            }
        }
        if (leader) {
            my.p[5][lane] = (uint32_t)__popc(grp);
            atomicOr(reinterpret_cast<uint32_t *>(st.lanes + bin) + (warp >> 2), (lane + 1u) << (8u * (warp & 3u)));
            atomicOr(st.rounds + bin, 1u << warp);
        }
        __syncthreads();
        // 2. every round's decision at once, from the states through that round
        uint4 lw = make_uint4(0u, 0u, 0u, 0u);
        uint32_t rmask = 0u;  // leader: the group's rounds that hit its bin
        unsigned long long cs1 = 0, cq1 = 0, cq2 = 0;
        uint32_t cn = 0, ch = 0;
        int verdict = SEM_PASS;
        if (leader) {
            lw = st.lanes[bin];
            rmask = st.rounds[bin];
            cs1 = st.s1[bin];
            cq1 = st.q1[bin];
            cq2 = st.q2[bin];
            cn = st.n[bin];
            ch = st.h[bin];
            for (uint32_t m = rmask & ((2u << warp) - 1u); m; m &= m - 1u) {  // rounds <= warp
                const uint32_t v = (uint32_t)__ffs(m) - 1u, l = lane_entry(lw, v);
                const RoundSlot &o = slots[v];
                const uint32_t sq = o.p[0][l - 1u];
                cs1 += ((unsigned long long)sq << kTqShift) + o.p[1][l - 1u];
                cq1 += sq;
                cq2 += ((unsigned long long)o.p[2][l - 1u] << 20) + ((unsigned long long)o.p[3][l - 1u] << 11) +
                       o.p[4][l - 1u];
                ch += o.p[5][l - 1u];
                cn += min(kRoundRays, R - (g0 + v * kRoundRays));
            }
            verdict = sem_quick(cn, ch, cq1, cq2, kExact ? 0u : kTqDelta);
        }
        if (__any_sync(0xffffffffu, verdict < 0) && verdict < 0)
            verdict = sem_test(cn, ch, cq1, cq2, kExact ? 0u : kTqDelta);
        const bool fail = __any_sync(0xffffffffu, verdict == SEM_FAIL);
        const bool unsure = __any_sync(0xffffffffu, verdict == SEM_UNSURE);
        if (lane == 0) my.verdict = (!hm || fail) ? 0u : (!kExact && unsure) ? 2u : 1u;
        __syncthreads();
        // 3. the first round that stops ends the row; the states through it are kept
        // (lane v reads round v's verdict)
        const uint32_t vv = lane < KW ? slots[lane].verdict : 0u;
        const uint32_t vb = __ballot_sync(0xffffffffu, vv != 0u);
        const uint32_t last = vb ? (uint32_t)__ffs(vb) - 1u : KW - 1u;
        if (vb) flag = __shfl_sync(0xffffffffu, vv, last);
        for (uint32_t v = 0; v <= last && g0 + v * kRoundRays < R; v++) {
            count += min(kRoundRays, R - (g0 + v * kRoundRays));
            if (tid == 0) {  // the row's totals, published by thread 0
                hits += slots[v].nh;
                ndf += (uint32_t)__popc(slots[v].df);
            }
        }
        if (leader) {
            const uint32_t later = rmask & ((2u << last) - 1u) & ~((2u << warp) - 1u);
            const uint32_t earlier = rmask & ((1u << warp) - 1u);
            if (warp <= last && !later) {  // the bin's latest round through `last`
                st.s1[bin] = cs1;
                st.q1[bin] = cq1;
                st.q2[bin] = cq2;
                st.n[bin] = cn;
                st.h[bin] = ch;
            }
            if (!earlier) {  // the bin's first round of the group clears its lane table
                st.lanes[bin] = make_uint4(0u, 0u, 0u, 0u);
                st.rounds[bin] = 0u;
            }
        }
        if (!flag && g0 + KW * kRoundRays >= R) flag = 1u;  // out of rays
        __syncthreads();
        if (flag) break;
    }
    if (flag == 2u) {
        // the caller redoes the row on the exact path at once
        __syncthreads();
        return true;
    } else {
        unsigned long long *hrow = a.hist + J.hist_off + (uint64_t)k * B;
        for (uint32_t b = tid; b < B; b += nthr) {
            const unsigned long long s1 = st.s1[b];
            if (s1) hrow[b] = rescale_cell(s1, R, count);
        }
        if (tid == 0) {
            const uint32_t sp = (uint32_t)(row % (uint64_t)kSpread);
            atomicAdd(&a.acc[d].fast[sp], (unsigned long long)count);
            if (hits) atomicAdd(&a.acc[d].hits[sp], (unsigned long long)hits);
            if (ndf) atomicAdd(&a.acc[d].retraced[sp], (unsigned long long)ndf);
        }
    }
    __syncthreads();  // the slots and bin states are reused by the block's next row
    return false;
}

// One wavelength row under adaptive sampling by a single warp (the form for passes with
// many rows, where the rows themselves fill the GPU): the same rounds and decisions as
// adaptive_row, one round after another. Each bin's exact integer Welford sums are kept
// cumulatively in shared memory; a round's hit lanes add their sums into the slot of their
// bin's leader (the lowest lane that hit it), the leader adds them to the bin's state and
// tests the state through the round, and the round stops the row when it hit some bin and
// every bin it hit passes. No lane tables, no barriers: one warp decides each round alone.
template <bool kExact>
__device__ bool adaptive_row1(const LaunchArgs &a, uint64_t row, unsigned long long *smem, uint32_t lane)
{
    const uint32_t d = find_job<F_ROW>(a.jobs, a.njobs, row);
    const DesignJob &J = a.jobs[d];
    const uint32_t k = (uint32_t)(row - J.row_off);
    const uint32_t B = J.B, R = J.R;
    const DevDesign &D = a.designs[d];
    if (!kExact && a.adaptive == 2u) {
        // verification mode: every row on the exact path
        if (lane == 0) {
            const unsigned long long pos = atomicAdd(&a.ctl->queue_count, 1ull);
            if (pos < a.qcap) a.queue[pos] = QEntry{d, k, 0u, 0u};
            else atomicOr(&a.ctl->overflow, 1u);
        }
        return false;
    }
    // the row's constants are the same in every lane: they live in shared memory (read
    // where they are used), which leaves the registers to more resident warps
    LamParams &P = *reinterpret_cast<LamParams *>(smem);
    FastConst &C = *reinterpret_cast<FastConst *>(reinterpret_cast<char *>(smem) + sizeof(LamParams));
    RoundSlot &my = *reinterpret_cast<RoundSlot *>(reinterpret_cast<char *>(smem) + sizeof(LamParams) + sizeof(FastConst));
    const LamDF &E = a.lx[row];
    const BinStates st(&my + 1, B);
    static_assert(sizeof(LamParams) % 16 == 0 && sizeof(FastConst) % 16 == 0, "16-byte copies");
    if (lane < sizeof(LamParams) / 16)
        reinterpret_cast<uint4 *>(&P)[lane] = reinterpret_cast<const uint4 *>(a.lp + row)[lane];
    else if (lane < (sizeof(LamParams) + sizeof(FastConst)) / 16)
        reinterpret_cast<uint4 *>(&C)[lane - sizeof(LamParams) / 16] =
            reinterpret_cast<const uint4 *>(&D.fc)[lane - sizeof(LamParams) / 16];
    for (uint32_t b = lane; b < B; b += 32u) {
        st.s1[b] = st.q1[b] = st.q2[b] = 0ull;
        st.n[b] = st.h[b] = 0u;
    }
    __syncwarp();
    const uint32_t *rank = a.rank + J.rank_off;
    const float2 *zt = reinterpret_cast<const float2 *>(a.z32) + J.ray_off;
    const uint32_t lt_mask = (1u << lane) - 1u;
    uint32_t count = 0, flag = 0, hits = 0, ndf = 0;  // the same in every lane
    // no ray clears the flat faces: every round runs without a hit
    const uint32_t g_start = P.band_lo >= P.band_hi ? R : 0u;
    if (g_start == R) count = R;
    // the ray this lane traces in the next round, loaded while the current one is decided
    uint32_t s_nx = 0xffffffffu;
    float2 z_nx = make_float2(0.f, 0.f);
    const auto fetch = [&](uint32_t g) {
        const uint32_t j = g + lane;
        s_nx = j < R ? rank[j] : 0xffffffffu;
        if (s_nx >= P.band_lo && s_nx < P.band_hi) z_nx = zt[s_nx];
    };
    if (g_start < R) fetch(g_start);
    for (uint32_t g0 = g_start; g0 < R; g0 += kRoundRays) {
        uint32_t bin = 0xffffffffu, tf = 0u;
        bool used_df = false;
        {
            const uint32_t s = s_nx;
            if (s >= P.band_lo && s < P.band_hi) {
                const float2 z = z_nx;
                int res = RAY_FLAG;
                if (!kExact && !P.all_exact && s >= P.core_lo && s < P.core_hi) {
                    uint32_t b = 0;
                    float t = 0.f;
                    res = fast_ray(C, P, a.guards, z.x, z.y, b, t);
                    if (res == RAY_HIT) {
                        bin = b;
                        tf = t_fixed(t);
                    }
                }
                if (res == RAY_FLAG) {
                    const uint2 r = trace_df_exact_call(D, E, z.x, z.y);
                    bin = r.x;
                    tf = r.y;
                    used_df = true;
                }
            }
        }
        if (g0 + kRoundRays < R) fetch(g0 + kRoundRays);
        const bool hit = bin != 0xffffffffu;
        const uint32_t hm = __ballot_sync(0xffffffffu, hit);
        const uint32_t dfb = __ballot_sync(0xffffffffu, used_df);
        const uint32_t grp = __match_any_sync(0xffffffffu, bin);
        const bool leader = hit && (grp & lt_mask) == 0u;
        const uint32_t rn = min(kRoundRays, R - g0);  // samples of this round
        // the round's sums per bin, in 32-bit pieces (as adaptive_row): into the leader's slot
        my.p[0][lane] = my.p[1][lane] = my.p[2][lane] = my.p[3][lane] = my.p[4][lane] = 0u;
        __syncwarp();
        if (hit) {
            const uint32_t ld = (uint32_t)__ffs(grp) - 1u, q = tf >> kTqShift;
            const uint32_t qh = q >> 10, ql = q & 0x3ffu;
            atomicAdd(&my.p[0][ld], q);
            atomicAdd(&my.p[1][ld], tf & 0x7ffu);
            atomicAdd(&my.p[2][ld], qh * qh);
            atomicAdd(&my.p[3][ld], qh * ql);
            atomicAdd(&my.p[4][ld], ql * ql);
        }
        __syncwarp();
        int verdict = SEM_PASS;
        uint32_t cn = 0, ch = 0;
        unsigned long long cq1 = 0, cq2 = 0;
        if (leader) {
            const uint32_t sq = my.p[0][lane];
            st.s1[bin] += ((unsigned long long)sq << kTqShift) + my.p[1][lane];
            cq1 = st.q1[bin] + sq;
            cq2 = st.q2[bin] + ((unsigned long long)my.p[2][lane] << 20) +
                  ((unsigned long long)my.p[3][lane] << 11) + my.p[4][lane];
            cn = st.n[bin] + rn;
            ch = st.h[bin] + (uint32_t)__popc(grp);
            st.q1[bin] = cq1;
            st.q2[bin] = cq2;
            st.n[bin] = cn;
            st.h[bin] = ch;
            verdict = sem_quick(cn, ch, cq1, cq2, kExact ? 0u : kTqDelta);
        }
        if (__any_sync(0xffffffffu, verdict < 0) && verdict < 0)
            verdict = sem_test(cn, ch, cq1, cq2, kExact ? 0u : kTqDelta);
        const bool fail = __any_sync(0xffffffffu, verdict == SEM_FAIL);
        const bool unsure = __any_sync(0xffffffffu, verdict == SEM_UNSURE);
        count += rn;
        hits += (uint32_t)__popc(hm);
        ndf += (uint32_t)__popc(dfb);
        if (hm && !fail) {
            flag = (!kExact && unsure) ? 2u : 1u;
            break;
        }
        if (g0 + kRoundRays >= R) {
            flag = 1u;  // out of rays
            break;
        }
    }
    __syncwarp();
    if (flag == 2u) return true;  // the caller redoes the row on the exact path at once
    unsigned long long *hrow = a.hist + J.hist_off + (uint64_t)k * B;
    for (uint32_t b = lane; b < B; b += 32u) {
        const unsigned long long s1 = st.s1[b];
        if (s1) hrow[b] = rescale_cell(s1, R, count);
    }
    if (lane == 0) {
        const uint32_t sp = (uint32_t)(row % (uint64_t)kSpread);
        atomicAdd(&a.acc[d].fast[sp], (unsigned long long)count);
        if (hits) atomicAdd(&a.acc[d].hits[sp], (unsigned long long)hits);
        if (ndf) atomicAdd(&a.acc[d].retraced[sp], (unsigned long long)ndf);
    }
    __syncwarp();  // the slot and bin states are reused by the next row
    return false;
}

#ifndef CPD_ADAPT_KW_MANY
#define CPD_ADAPT_KW_MANY 1  // warps per row when at least 8 rows per SM (1: adaptive1_kernel)
#endif
#ifndef CPD_ADAPT_KW_SOME
#define CPD_ADAPT_KW_SOME 4  // warps per row at 2 to 7 rows per SM
#endif
#ifndef CPD_ADAPT_MIN_BLOCKS
#define CPD_ADAPT_MIN_BLOCKS 2  // 64 registers at kMaxAdaptWarps warps per block
#endif
// One row per block of KW = blockDim.x / 32 warps: rows differ widely in length (a single
// round to all R / 32), and one row per block lets the block scheduler balance them.
__global__ void __launch_bounds__(32 * kMaxAdaptWarps, CPD_ADAPT_MIN_BLOCKS) adaptive_kernel(const LaunchArgs a)
{
    extern __shared__ __align__(16) unsigned long long adapt_smem[];
    cudaTriggerProgrammaticLaunchCompletion();
    cudaGridDependencySynchronize();  // the setup's LamParams and LamDF
    const uint32_t kw = blockDim.x >> 5, warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    // a row whose stop decision the FP32 transmittances cannot settle is redone here, on
    // the float-float path from its first round, while other blocks go on with theirs
    if (adaptive_row<false>(a, blockIdx.x, adapt_smem, kw, warp, lane))
        adaptive_row<true>(a, blockIdx.x, adapt_smem, kw, warp, lane);
}

#ifndef CPD_ADAPT1_MIN_BLOCKS
#define CPD_ADAPT1_MIN_BLOCKS 32
#endif
// The many-rows form: one row per one-warp block (adaptive_row1).
__global__ void __launch_bounds__(32, CPD_ADAPT1_MIN_BLOCKS) adaptive1_kernel(const LaunchArgs a)
{
    extern __shared__ __align__(16) unsigned long long adapt_smem[];
    cudaTriggerProgrammaticLaunchCompletion();
    cudaGridDependencySynchronize();  // the setup's LamParams and LamDF
    if (adaptive_row1<false>(a, blockIdx.x, adapt_smem, threadIdx.x))
        adaptive_row1<true>(a, blockIdx.x, adapt_smem, threadIdx.x);
}

// The queued rows: the float-float path from the first round on, one row per block of
// blockDim.x / 32 warps (as many as the rounds kernel used: a queued row of a plain call
// is on the pass's critical path).
__global__ void __launch_bounds__(32 * kMaxAdaptWarps, 1) adaptive_exact_kernel(const LaunchArgs a)
{
    extern __shared__ __align__(16) unsigned long long adapt_smem[];
    cudaTriggerProgrammaticLaunchCompletion();
    cudaGridDependencySynchronize();  // the adaptive kernel's queue
    publish_status(a);
    const unsigned long long qn = a.ctl->queue_count;
    const uint64_t n = qn < a.qcap ? qn : a.qcap;
    for (uint64_t i = blockIdx.x; i < n; i += gridDim.x) {
        const QEntry e = a.queue[i];
        const uint64_t row = a.jobs[e.design].row_off + e.k;
        if (blockDim.x == 32u) adaptive_row1<true>(a, row, adapt_smem, threadIdx.x);
        else adaptive_row<true>(a, row, adapt_smem, blockDim.x >> 5, threadIdx.x >> 5, threadIdx.x & 31u);
    }
}

__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

constexpr int kEntropyThreads = 256;

// A non-negative float-float value in fixed point with `scale` units, its hi and lo
// words rounded separately: one rounding per cell, so that the sums over cells are integer
// sums whose value does not depend on how the cells are grouped.
// The conversions are 32-bit or exact bit arithmetic: 64-bit float-to-integer conversions
// issue to the FP64 unit, ~64 cycles per warp instruction on this GPU.
__device__ __forceinline__ unsigned long long df_to_fixed(ff::F2 v, float scale)
{
    const float x = v.hi * scale;  // >= 0, below 2^47
    unsigned long long q;
    if (x < 2147483648.0f) {
        q = __float2uint_rn(x);
    } else {
        // at or above 2^31 a float is an integer: its significand shifted by its exponent
        const uint32_t bits = __float_as_uint(x);
        q = (unsigned long long)((bits & 0x7fffffu) | 0x800000u) << (((bits >> 23) & 0xffu) - 150u);
    }
    // |lo| is below half an ulp of hi: |lo scale| < 2^23
    const long long r = (long long)q + __float2int_rn(v.lo * scale);
    return r > 0 ? (unsigned long long)r : 0ull;
}

// Per-design finalize: H(D) from the per-bin sums, MI, and the SEM stop of cuda_fitness
// (src/cuda_fitness.rs:392-422), by nthr threads (one warp, or the 256 threads of an entropy
// block; red: nthr / 32 scratch records in shared memory when nthr > 32). f64 costs ~64
// cycles per warp instruction here (a division or square root ~700 cycles of latency), and
// this runs on the tail of the plain call, so everything is float-float on the FP32 pipe:
// pbar = S1 / (n R 2^31), log2 pbar = log2 S1 - log2(n R) - 31 (logs of integers,
// ff::log2_u64, absolute error < 1e-12), each bin's pbar log2 pbar rounded once to 2^-50
// fixed point (so the sum over bins is the same integer for any number of threads), and
// each bin's Welford M2, S2 - S1^2 / n, against (5e-3)^2 n (n - 1). Only the conversion of
// the three results to double is f64.
struct FinalizeRed {
    long long hdet;
    float m2max;
    int conv;
};
constexpr float kHdetScale = 1125899906842624.0f;  // 2^50

__device__ void finalize_design(const LaunchArgs &a, uint32_t d, const DesignJob &J, uint32_t tid, uint32_t nthr,
                                const float *tab, FinalizeRed *red)
{
    using ff::F2;
    const uint32_t lane = tid & 31u;
    // every load first, so that their L2 round trips overlap one another and the
    // float-float prologue: the design's sums, its ray counters and this thread's first bin
    const unsigned long long rows = __ldcg(&a.acc[d].rows) + J.W;
    const unsigned long long Hsum = __ldcg(&a.acc[d].H);
    const bool cp = lane < (uint32_t)kSpread;
    const unsigned long long hits_l = cp ? __ldcg(&a.acc[d].hits[lane]) : 0ull;
    const unsigned long long retraced_l = cp ? __ldcg(&a.acc[d].retraced[lane]) : 0ull;
    const unsigned long long fast_l = cp ? __ldcg(&a.acc[d].fast[lane]) : 0ull;
    unsigned long long c1n = 0ull, c2n = 0ull;
    if (tid < J.B) {
        c1n = __ldcg(&a.S1[J.acc_off + tid]);
        c2n = __ldcg(&a.S2[J.acc_off + tid]);
    }
    const F2 n = ff::from_u64(rows);
    const F2 inv_n = df::rcp(n);
    const F2 unit{J.unit_hi, J.unit_lo};  // p per count unit, 2^-31 / R
    const F2 inv_nr = ff::mul(unit, inv_n);
    const unsigned long long nR = rows * (unsigned long long)J.R;
    const F2 lnr = ff::add_f(ff::log2_u64(nR, tab), 31.f);
    const F2 thr = df::div(ff::mul(n, ff::from_u64(rows - 1ull)), df::c(40000.f));  // (5e-3)^2 n (n - 1)
    const F2 s2unit{(float)kPScaleInv, 0.f};
    long long hdet = 0;  // sum of pbar log2 pbar (<= 0), 2^-50 units
    float m2max = 0.f;
    int conv = 1;
    for (uint32_t b = tid; b < J.B; b += nthr) {
        const unsigned long long c1 = c1n, c2 = c2n;
        if (b + nthr < J.B) {  // the next bin's sums
            c1n = __ldcg(&a.S1[J.acc_off + b + nthr]);
            c2n = __ldcg(&a.S2[J.acc_off + b + nthr]);
        }
        const F2 sc1 = ff::from_u64(c1);
        if (c1) {
            const F2 pbar = ff::mul(sc1, inv_nr);
            const F2 lg = ff::add(ff::log2_u64(c1, tab), F2{-lnr.hi, -lnr.lo});
            const F2 pl = ff::mul(pbar, lg);
            hdet -= (long long)df_to_fixed(F2{-pl.hi, -pl.lo}, kHdetScale);
        }
        // Welford M2 of the per-wavelength p(d|lambda) (welford.rs:26-57)
        const F2 s1 = ff::mul(sc1, unit);  // sum over rows of p
        const F2 s2 = ff::mul(ff::from_u64(c2), s2unit);
        F2 m2 = df::sub(s2, ff::mul(ff::mul(s1, s1), inv_n));
        if (df::neg_(m2)) m2 = F2{0.f, 0.f};
        conv &= df::lt(m2, thr) ? 1 : 0;
        m2max = fmaxf(m2max, m2.hi);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        hdet += (long long)__shfl_xor_sync(0xffffffffu, (unsigned long long)hdet, o);
        m2max = fmaxf(m2max, __shfl_xor_sync(0xffffffffu, m2max, o));
    }
    conv = __all_sync(0xffffffffu, conv);
    if (nthr > 32u) {
        if (lane == 0) red[tid >> 5] = FinalizeRed{hdet, m2max, conv};
        __syncthreads();
        if (tid >= 32u) return;
        const uint32_t nw = nthr >> 5;
        FinalizeRed r = lane < nw ? red[lane] : FinalizeRed{0, 0.f, 1};
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            r.hdet += (long long)__shfl_xor_sync(0xffffffffu, (unsigned long long)r.hdet, o);
            r.m2max = fmaxf(r.m2max, __shfl_xor_sync(0xffffffffu, r.m2max, o));
        }
        hdet = r.hdet;
        m2max = r.m2max;
        conv = __all_sync(0xffffffffu, r.conv);
    }
    const unsigned long long hits = warp_sum_u64(hits_l);
    const unsigned long long retraced = warp_sum_u64(retraced_l);
    const unsigned long long fast = warp_sum_u64(fast_l);
    if (lane == 0) {
        const F2 H = ff::mul(ff::from_u64(Hsum), F2{(float)kHScaleInv, 0.f});
        const F2 hc = ff::mul(H, inv_n);
        const double h_cond = -((double)hc.hi + (double)hc.lo);
        const double h_det = (double)hdet * (1.0 / 1125899906842624.0);
        DesignOut o;
        o.h_cond = h_cond;
        o.h_det = h_det;
        o.info = h_cond - h_det;
        const float fn = (float)rows;
        o.max_sem = rows > 1ull ? (double)sqrtf(m2max / (fn - 1.f) / fn) : (double)INFINITY;
        const DevDesign &D = a.designs[d];
        o.size = D.size;
        o.deviation = D.deviation;
        o.hits = hits;
        o.retraced = retraced;
        o.rows = rows;
        o.fast = fast;
        o.converged = conv;
        o.status = D.status;
        a.out[d] = o;
        a.acc[d].rows = rows;
    }
}

// One nonzero cell of the histogram: -p log2 p (2^-40 units) and p^2 (2^-46 units) in
// fixed point, p = c 2^-31 / R in float-float on the FP32 pipe.
__device__ __forceinline__ void entropy_cell(unsigned long long cv, ff::F2 unit, ff::F2 lu, const float *tab,
                                             unsigned long long &hq, unsigned long long &pq)
{
    const ff::F2 p = ff::mul(ff::from_u64(cv), unit);
    const ff::F2 lp = ff::add(ff::log2_u64(cv, tab), lu);
    const ff::F2 plp = ff::mul(p, lp);  // p log2 p <= 0
    hq = df_to_fixed(ff::F2{-plp.hi, -plp.lo}, (float)kHScale);
    pq = df_to_fixed(ff::mul(p, p), (float)kPScale);
}

// The finalize of a single-design pass, folded into the entropy kernel: the warp that
// accounts the design's last tile runs it (after the fences that publish every tile's sums).
__device__ __forceinline__ bool last_tile_of_design(const LaunchArgs &a, const DesignJob &J, uint32_t lane)
{
    __threadfence();
    unsigned last = 0;
    if (lane == 0) last = atomicAdd(&a.ctl->tiles_done, 1u) == J.ntiles - 1u ? 1u : 0u;
    last = __shfl_sync(0xffffffffu, last, 0);
    if (last) __threadfence();
    return last != 0u;
}

// Entropy sums of the rows [r0, r1) of one design by one warp (the form for passes with
// many tiles: no block-level synchronization). Lane -> (bin, row phase): for B <= 32 the
// lanes split into 32/B row phases of one bin each; for wider detectors a lane owns bins
// lane, lane+32, ... of every row, NB of them per sweep. Each step reads 8/NB rows x NB
// bins, so eight loads per lane are in flight.
template <int NB, bool WITH_P>
__device__ __forceinline__ void entropy_tile(const LaunchArgs &a, const DesignJob &J, uint32_t r0, uint32_t r1,
                                             uint32_t lane, const float *tab, unsigned long long &hl)
{
    constexpr uint32_t RS = 8u / NB;
    const uint32_t B = J.B;
    const uint32_t groups = B <= 32u ? 32u / B : 1u;
    const uint32_t grp = B <= 32u ? lane / B : 0u;
    const uint32_t bin0 = B <= 32u ? lane % B : lane;
    const bool active = grp < groups;
    const ff::F2 unit{J.unit_hi, J.unit_lo}, lu{J.lu_hi, J.lu_lo};
    unsigned long long *base = a.hist + J.hist_off;
    const double pscale = J.pscale;  // p per count unit, for the optional p(d|lambda) output
    for (uint32_t bg = 0; bg < B; bg += 32u * NB) {
        unsigned long long c1[NB], q2[NB];
#pragma unroll
        for (int i = 0; i < NB; i++) c1[i] = q2[i] = 0ull;
        for (uint32_t row = r0 + grp; row < r1; row += RS * groups) {
            unsigned long long c[RS * NB];
#pragma unroll
            for (uint32_t rr = 0; rr < RS; rr++) {
                const uint32_t rw = row + rr * groups;
#pragma unroll
                for (int i = 0; i < NB; i++) {
                    const uint32_t b = bg + bin0 + 32u * (uint32_t)i;
                    c[rr * NB + i] = (active && rw < r1 && b < B) ? base[(uint64_t)rw * B + b] : 0ull;
                }
            }
            // one copy of the cell code, not RS x NB (instruction fetch)
#pragma unroll 1
            for (uint32_t q = 0; q < RS * NB; q++) {
                const uint32_t rw = row + (q / NB) * groups;
                const uint32_t i = q % NB;
                const uint32_t b = bg + bin0 + 32u * i;
                const unsigned long long cv = c[q];
                if (cv) {
                    base[(uint64_t)rw * B + b] = 0ull;
                    unsigned long long hq, pq;
                    entropy_cell(cv, unit, lu, tab, hq, pq);
                    hl += hq;
#pragma unroll
                    for (int ii = 0; ii < NB; ii++)
                        if (ii == (int)i) {
                            q2[ii] += pq;
                            c1[ii] += cv;
                        }
                }
                if (WITH_P && active && rw < r1 && b < B) a.p_out[(uint64_t)rw * B + b] = (double)cv * pscale;
            }
        }
#pragma unroll
        for (int i = 0; i < NB; i++) {
            const uint32_t b = bg + bin0 + 32u * (uint32_t)i;
            if (c1[i]) {
                atomicAdd(&a.S1[J.acc_off + b], c1[i]);
                atomicAdd(&a.S2[J.acc_off + b], q2[i]);
            }
        }
    }
}

// One warp per tile.
// WITH_P: the pass also writes p(d|lambda) (a.p_out); a kernel of its own, so that the
// f64 conversion of every cell is not issued when nobody reads it.
template <bool WITH_P>
__global__ void __launch_bounds__(kEntropyThreads, 4) entropy_warp_kernel(const LaunchArgs a)
{
    __shared__ float tab[4 * ff::kLogTable];
    cudaTriggerProgrammaticLaunchCompletion();
    for (uint32_t i = threadIdx.x; i < 4u * ff::kLogTable; i += blockDim.x) tab[i] = a.logtab[i];
    __syncthreads();
    cudaGridDependencySynchronize();  // the histogram of the trace and re-trace kernels
    // A pass whose re-trace queue overflowed is re-run by the host: leave every
    // accumulator untouched.
    if (a.ctl->overflow || a.ctl->queue_count > a.qcap) return;
    const uint32_t lane = threadIdx.x & 31u;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t tile = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; tile < a.total_tiles; tile += nw) {
        const uint32_t d = find_job<F_TILE>(a.jobs, a.njobs, tile);
        const DesignJob J = a.jobs[d];
        const uint32_t r0 = (uint32_t)(tile - J.tile_off) * J.tile_rows;
        const uint32_t r1 = min(r0 + J.tile_rows, J.W);
        const uint32_t nb = (J.B + 31u) / 32u;  // bins per lane
        unsigned long long hl = 0ull;
        if (nb >= 3u) entropy_tile<4, WITH_P>(a, J, r0, r1, lane, tab, hl);
        else if (nb == 2u) entropy_tile<2, WITH_P>(a, J, r0, r1, lane, tab, hl);
        else entropy_tile<1, WITH_P>(a, J, r0, r1, lane, tab, hl);
        hl = warp_sum_u64(hl);
        if (lane == 0 && hl) atomicAdd(&a.acc[d].H, hl);
        if (a.njobs == 1 && last_tile_of_design(a, J, lane)) finalize_design(a, d, J, lane, 32u, tab, nullptr);
    }
}

// One block per entropy tile (tile_rows rows of one design, at most kTileCells cells),
// the form for passes with few tiles (the plain call), where one warp per tile would
// leave most SMs idle: thread t takes cells t, t + 256, ... of the tile in row-major order,
// and the tile's per-bin sums meet in shared memory, then one global atomic per bin and
// sum. In both forms each cell's terms are rounded to fixed point once (entropy_cell), so
// every sum is independent of the grouping of cells into threads, tiles and launches,
// and each nonzero cell is zeroed after it is read, which leaves the histogram clear for
// the next pass.
template <bool WITH_P>
__global__ void __launch_bounds__(kEntropyThreads, 4) entropy_block_kernel(const LaunchArgs a)
{
    __shared__ float tab[4 * ff::kLogTable];
    extern __shared__ __align__(16) unsigned long long ent_smem[];  // per-bin s1, s2 (max_B each)
    __shared__ unsigned long long hsum;
    __shared__ unsigned last_tile;
    __shared__ FinalizeRed fin_red[kEntropyThreads / 32];
    cudaTriggerProgrammaticLaunchCompletion();
    for (uint32_t i = threadIdx.x; i < 4u * ff::kLogTable; i += blockDim.x) tab[i] = a.logtab[i];
    __syncthreads();
    cudaGridDependencySynchronize();  // the histogram of the trace and re-trace kernels
    // A pass whose re-trace queue overflowed is re-run by the host: leave every
    // accumulator untouched.
    if (a.ctl->overflow || a.ctl->queue_count > a.qcap) return;
    const uint32_t t = threadIdx.x, lane = t & 31u;
    for (uint64_t tile = blockIdx.x; tile < a.total_tiles; tile += gridDim.x) {
        const uint32_t d = find_job<F_TILE>(a.jobs, a.njobs, tile);
        const DesignJob J = a.jobs[d];
        const uint32_t B = J.B;
        const uint32_t r0 = (uint32_t)(tile - J.tile_off) * J.tile_rows;
        const uint32_t r1 = min(r0 + J.tile_rows, J.W);
        unsigned long long *s1 = ent_smem, *s2 = ent_smem + B;
        for (uint32_t b = t; b < B; b += kEntropyThreads) s1[b] = s2[b] = 0ull;
        if (t == 0) hsum = 0ull;
        __syncthreads();
        const ff::F2 unit{J.unit_hi, J.unit_lo}, lu{J.lu_hi, J.lu_lo};
        unsigned long long *base = a.hist + J.hist_off;
        const double pscale = J.pscale;
        const uint32_t cells = (r1 - r0) * B;
        const uint32_t db = (uint32_t)kEntropyThreads % B, dr = (uint32_t)kEntropyThreads / B;
        uint32_t b = t % B, row = r0 + t / B;
        unsigned long long hl = 0ull;
        // two cells per step, both loaded before either is processed, so that their
        // memory latencies and their float-float chains overlap
        for (uint32_t i0 = t; i0 < cells; i0 += 2u * kEntropyThreads) {
            uint64_t idx[2];
            uint32_t bc[2];
            unsigned long long cv[2];
#pragma unroll
            for (int k = 0; k < 2; k++) {
                const bool in = i0 + (uint32_t)k * kEntropyThreads < cells;
                idx[k] = (uint64_t)row * B + b;
                bc[k] = b;
                cv[k] = in ? base[idx[k]] : 0ull;
                if (WITH_P && in) a.p_out[idx[k]] = (double)cv[k] * pscale;
                b += db;
                row += dr;
                if (b >= B) {
                    b -= B;
                    row++;
                }
            }
#pragma unroll
            for (int k = 0; k < 2; k++) {
                if (cv[k]) {
                    base[idx[k]] = 0ull;
                    unsigned long long hq, pq;
                    entropy_cell(cv[k], unit, lu, tab, hq, pq);
                    hl += hq;
                    atomicAdd(s1 + bc[k], cv[k]);
                    atomicAdd(s2 + bc[k], pq);
                }
            }
        }
        hl = warp_sum_u64(hl);
        if (lane == 0 && hl) atomicAdd(&hsum, hl);
        __syncthreads();
        for (uint32_t bb = t; bb < B; bb += kEntropyThreads) {
            const unsigned long long v1 = s1[bb];
            if (v1) {
                atomicAdd(&a.S1[J.acc_off + bb], v1);
                atomicAdd(&a.S2[J.acc_off + bb], s2[bb]);
            }
        }
        if (t == 0 && hsum) atomicAdd(&a.acc[d].H, hsum);
        if (a.njobs == 1) {
            // a single design (the plain call): the block that finishes the last tile runs
            // the finalize, which saves a launch; with many designs the per-tile fences
            // would cost more than the separate finalize kernel
            __threadfence();
            __syncthreads();
            if (t == 0) last_tile = atomicAdd(&a.ctl->tiles_done, 1u) == J.ntiles - 1u ? 1u : 0u;
            __syncthreads();
            if (last_tile) {
                __threadfence();
                finalize_design(a, d, J, t, kEntropyThreads, tab, fin_red);
            }
        }
        __syncthreads();  // the shared sums are reused by the block's next tile
    }
}

// One warp per design after the entropy kernel.
__global__ void __launch_bounds__(128) finalize_kernel(const LaunchArgs a)
{
    __shared__ float tab[4 * ff::kLogTable];
    for (uint32_t i = threadIdx.x; i < 4u * ff::kLogTable; i += blockDim.x) tab[i] = a.logtab[i];
    __syncthreads();
    cudaGridDependencySynchronize();  // the entropy kernel's sums
    // A pass whose re-trace queue overflowed is re-run by the host: write nothing.
    if (a.ctl->overflow || a.ctl->queue_count > a.qcap) return;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t d = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; d < a.njobs; d += nw) {
        const DesignJob J = a.jobs[d];
        finalize_design(a, d, J, lane, 32u, tab, nullptr);
    }
}

__global__ void __launch_bounds__(128) trace_pairs_kernel(const DevDesign *__restrict__ dd,
                                                          const double *__restrict__ lam_u,
                                                          const double *__restrict__ z64, uint32_t n,
                                                          uint32_t mode, uint32_t *bins, double *ts,
                                                          uint8_t *flags)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const DevDesign &D = *dd;
    const double z = z64[i];
    uint32_t bin = D.B;
    double t = 0.0;
    uint8_t fl = 0;
    if (isfinite(z)) {
        if (mode == CPD_TRACE_FP64) {
            uint32_t b = 0;
            double te = 0.0;
            if (x::trace(D, x::wavelength(D, lam_u[i]), x::beam_y(D, z), b, te) == 0) {
                bin = b;
                t = te;
            }
        } else {
            float zz[2];
            split_f32(z, zz[0], zz[1]);
            LamParams P;
            LamDF E;
            const double yg = mode == CPD_TRACE_FP32 ? 0.0 : kYGuardRel;
            lambda_setup_df(D, lam_u[i], zz, 1u, P, yg, &E);
            bool retrace = false;
            if (P.core_lo == 0 && P.core_hi == 1 && !P.all_exact) {
                const Guards g = mode == CPD_TRACE_FP32 ? no_guards() : default_guards();
                uint32_t b = 0;
                float tf = 0.f;
                const int r = fast_ray(D.fc, P, g, zz[0], zz[1], b, tf);
                if (r == RAY_HIT) {
                    bin = b;
                    t = tf;
                } else if (r == RAY_FLAG) {
                    retrace = true;
                }
            } else if (P.band_lo == 0 && P.band_hi == 1) {
                // in a y-interval guard band, or its own reference ray without a usable
                // exit/detector geometry
                retrace = mode == CPD_TRACE_HYBRID;
            }
            if (retrace) {
                fl = 1;
                uint32_t b = 0;
                float tf = 0.f;
                if (trace_df(D, E, zz[0], zz[1], b, tf)) {
                    bin = b;
                    t = tf;
                }
            }
        }
    }
    bins[i] = bin;
    ts[i] = t;
    if (flags) flags[i] = fl;
}

// ------------------------------------------------------------------ p_dets_l_wavelength
//
// The reference CPU estimator of p(d|lambda) for one wavelength
// (vector_quasi_monte_carlo_integration + p_dets_l_wavelength, src/fitness.rs:5-34,48-69),
// the one Spectrometer.transmission_probability returns (src/pylib.rs:1028-1058): rays in
// order; a ray that hits bin b pads b's Welford state with zeros up to the ray count
// (Welford::skip), adds its t (next_sample), and the integration stops at the first hit
// after which its bin's SEM^2 <= (5e-3)^2 (sem_le_error_threshold, welford.rs:5-57); every
// bin is then padded to the final count and p = its mean. The bin that fired the stop keeps
// a count one ahead of the rays (skip then next_sample), as the reference does.
//
// One block per wavelength, kTpRays threads. A round traces kTpRays rays in exact f64
// (x::trace, bit-identical to the reference's f64 trace), sorts the round's hits by (bin,
// ray), and the first thread of each bin's run replays the run's Welford updates in the
// reference's f64 operation order, keeping the state after each update and stopping at the
// run's first passing hit. The round's stop is the earliest passing hit over all bins;
// each bin then keeps its state after its last hit before or at that ray. The result is
// the one-ray-at-a-time order of the reference bit for bit: the bins' states are
// independent, and every hit up to the stop is applied in ray order within its bin.
constexpr uint32_t kTpRays = 256;

struct TpWelford {
    double c, m, m2;
};

// Welford::skip (welford.rs:34-42).
__device__ __forceinline__ void tp_skip(TpWelford &w, double n)
{
    if (w.c < n) {
        const double z = x::sub(n, w.c);
        w.m = x::div(x::mul(w.c, w.m), n);
        w.m2 = x::add(w.m2, x::div(x::mul(x::mul(x::sqr(w.m), w.c), z), n));
        w.c = n;
    }
}

// Welford::next_sample (welford.rs:26-32).
__device__ __forceinline__ void tp_next(TpWelford &w, double v)
{
    w.c = x::add(w.c, 1.0);
    const double d = x::sub(v, w.m);
    w.m = x::add(w.m, x::div(d, w.c));
    w.m2 = x::add(w.m2, x::mul(d, x::sub(v, w.m)));
}

__global__ void __launch_bounds__(kTpRays) tp_adaptive_kernel(const DevDesign *__restrict__ dd,
                                                              const double *__restrict__ lambdas,
                                                              const double *__restrict__ z64, uint32_t max_m,
                                                              double *out, uint32_t *rays_out)
{
    __shared__ __align__(16) DevDesign sD;
    __shared__ uint32_t key[kTpRays];   // (bin << 8) | ray within the round; ~0u: no hit
    __shared__ double tv[kTpRays];      // t of the round's ray i
    __shared__ double sc[kTpRays], sm[kTpRays], sm2[kTpRays];  // state after sorted hit k
    __shared__ uint32_t stop_i;
    extern __shared__ __align__(16) double wst[];  // c[B] | m[B] | m2[B]
    const uint32_t tid = threadIdx.x;
    for (uint32_t i = tid; i < sizeof(DevDesign) / 4; i += blockDim.x)
        reinterpret_cast<uint32_t *>(&sD)[i] = reinterpret_cast<const uint32_t *>(dd)[i];
    const uint32_t B = dd->B;
    double *wc = wst, *wm = wst + B, *wm2 = wst + 2 * B;
    for (uint32_t b = tid; b < B; b += blockDim.x) wc[b] = wm[b] = wm2[b] = 0.0;
    __syncthreads();
    const double lambda = lambdas[blockIdx.x];
    const double e2 = x::mul(5e-3, 5e-3);
    uint32_t count = max_m;
    for (uint32_t j0 = 0; j0 < max_m; j0 += kTpRays) {
        const uint32_t j = j0 + tid;
        uint32_t k = ~0u;
        if (j < max_m) {
            uint32_t bin = 0;
            double t = 0.0;
            if (x::trace(sD, lambda, x::beam_y(sD, z64[j]), bin, t) == 0) {
                k = (bin << 8) | tid;
                tv[tid] = t;
            }
        }
        key[tid] = k;
        if (tid == 0) stop_i = ~0u;
        if (!__syncthreads_or(k != ~0u)) continue;  // no hit this round
        // bitonic sort of the keys: hits grouped by bin, in ray order within a bin
        for (uint32_t w = 2; w <= kTpRays; w <<= 1)
            for (uint32_t h = w >> 1; h > 0; h >>= 1) {
                const uint32_t o = tid ^ h;
                if (o > tid) {
                    const uint32_t a = key[tid], b = key[o];
                    if ((a > b) == ((tid & w) == 0)) {
                        key[tid] = b;
                        key[o] = a;
                    }
                }
                __syncthreads();
            }
        const uint32_t kk = key[tid];
        const bool head = kk != ~0u && (tid == 0 || (key[tid - 1] >> 8) != (kk >> 8));
        uint32_t last = tid;  // sorted position of the run's last hit
        if (head) {
            const uint32_t b = kk >> 8;
            TpWelford st{wc[b], wm[b], wm2[b]};
            while (last + 1 < kTpRays && key[last + 1] != ~0u && (key[last + 1] >> 8) == b) last++;
            for (uint32_t q = tid; q <= last; q++) {
                const uint32_t i = key[q] & 0xffu;
                tp_skip(st, (double)(j0 + i + 1u));
                tp_next(st, tv[i]);
                sc[q] = st.c;
                sm[q] = st.m;
                sm2[q] = st.m2;
                if (st.m2 < x::mul(e2, x::mul(st.c, x::sub(st.c, 1.0)))) {
                    atomicMin(&stop_i, i);
                    break;
                }
            }
        }
        __syncthreads();
        const uint32_t si = stop_i;
        if (head) {
            // the bin's state after its last hit at or before the stop
            int q_keep = -1;
            for (uint32_t q = tid; q <= last && (key[q] & 0xffu) <= si; q++) q_keep = (int)q;
            if (q_keep >= 0) {
                const uint32_t b = kk >> 8;
                wc[b] = sc[q_keep];
                wm[b] = sm[q_keep];
                wm2[b] = sm2[q_keep];
            }
        }
        __syncthreads();
        if (si != ~0u) {
            count = j0 + si + 1u;
            break;
        }
    }
    // every bin padded to the final ray count (the reference's closing skip)
    for (uint32_t b = tid; b < B; b += blockDim.x) {
        TpWelford st{wc[b], wm[b], wm2[b]};
        tp_skip(st, (double)count);
        out[(uint64_t)blockIdx.x * B + b] = st.m;
    }
    if (tid == 0 && rays_out) rays_out[blockIdx.x] = count;
}

__global__ void fma_peak_kernel(float *out, uint32_t iters)
{
    float a0 = threadIdx.x * 1e-7f, a1 = a0 + 1e-7f, a2 = a0 + 2e-7f, a3 = a0 + 3e-7f;
    float a4 = a0 + 4e-7f, a5 = a0 + 5e-7f, a6 = a0 + 6e-7f, a7 = a0 + 7e-7f;
    const float b = 0.999999f, c = 1e-7f;
    for (uint32_t i = 0; i < iters; i++) {
#pragma unroll
        for (int u = 0; u < 16; u++) {
            a0 = fmaf(a0, b, c);
            a1 = fmaf(a1, b, c);
            a2 = fmaf(a2, b, c);
            a3 = fmaf(a3, b, c);
            a4 = fmaf(a4, b, c);
            a5 = fmaf(a5, b, c);
            a6 = fmaf(a6, b, c);
            a7 = fmaf(a7, b, c);
        }
    }
    const float s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
    if (s == 12345.0f) out[blockIdx.x] = s;  // keeps the chains live
}

// SFU throughput probe: eight independent chains of the reciprocal-square-root estimate
// (MUFU.RSQ) per thread; the values stay near 1.
__global__ void mufu_peak_kernel(float *out, uint32_t iters)
{
    float a[8];
#pragma unroll
    for (int k = 0; k < 8; k++) a[k] = 1.0f + 1e-3f * (float)k + 1e-7f * (float)threadIdx.x;
    for (uint32_t i = 0; i < iters; i++) {
#pragma unroll
        for (int u = 0; u < 16; u++)
#pragma unroll
            for (int k = 0; k < 8; k++) asm volatile("rsqrt.approx.ftz.f32 %0, %0;" : "+f"(a[k]));
    }
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < 8; k++) s += a[k];
    if (s == 12345.0f) out[blockIdx.x] = s;  // keeps the chains live
}

// ------------------------------------------------------------------ device-resident loop
//
// One CTA evaluates one design at a time, start to finish, with the pass's device code:
// lambda_setup_df per wavelength row, fast_ray over the core rays (lane = wavelength, items
// of 32 rows x a ray chunk claimed from a shared counter), trace_df for the guard-band rays
// of every row and the rays fast_ray flagged, entropy_cell over the W x B cells, then
// finalize_design. Every sum is the same integer as in the pass, so a design's result is
// bitwise its batched result. The CTA then claims the next published ring entry.

constexpr uint32_t kLoopThreads = 256;
#ifndef CPD_LOOP_MIN_BLOCKS
#define CPD_LOOP_MIN_BLOCKS 3
#endif

struct SlabLayout {
    size_t hist, lp, lx, queue, s1, s2, acc, band, bytes;
};

__host__ __device__ inline SlabLayout slab_layout(uint32_t rows, uint32_t cells, uint32_t maxB, uint32_t qcap)
{
    SlabLayout L;
    size_t o = 0;
    L.hist = o;
    o += (8 * (size_t)cells + 255) & ~size_t(255);
    L.lp = o;
    o += (sizeof(LamParams) * (size_t)rows + 255) & ~size_t(255);
    L.lx = o;
    o += (sizeof(LamDF) * (size_t)rows + 255) & ~size_t(255);
    L.queue = o;
    o += (sizeof(QEntry) * (size_t)qcap + 255) & ~size_t(255);
    L.s1 = o;
    o += (8 * (size_t)maxB + 255) & ~size_t(255);
    L.s2 = o;
    o += (8 * (size_t)maxB + 255) & ~size_t(255);
    L.acc = o;
    o += (sizeof(DesignAcc) + 255) & ~size_t(255);
    L.band = o;
    o += (4 * ((size_t)rows + 1) + 255) & ~size_t(255);
    L.bytes = o;
    return L;
}

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ unsigned long long load_acquire_sys(const unsigned long long *p)
{
    unsigned long long v;
    asm volatile("ld.acquire.sys.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void store_release_sys(unsigned long long *p, unsigned long long v)
{
    asm volatile("st.release.sys.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// The float-float re-trace of one ray into the CTA's histogram; returns 1 on a hit.
__device__ __noinline__ uint32_t loop_retrace(const DevDesign &D, const LamDF &E, const float *z32, uint32_t j,
                                              unsigned long long *hrow)
{
    uint32_t bin = 0;
    float t = 0.f;
    if (trace_df(D, E, z32[2 * j], z32[2 * j + 1], bin, t)) {
        atomicAdd(hrow + bin, (unsigned long long)t_fixed(t));
        return 1u;
    }
    return 0u;
}

// The loop's per-wavelength setup: rows t, t + nthr, ... (out of line, so that its
// float-float program does not set the register budget of the trace loop).
__device__ __noinline__ void loop_setup(const DevDesign &D, const double *lam, const float *z32, uint32_t Rz, uint32_t W,
                                        LamParams *lp, LamDF *lx, uint32_t t, uint32_t nthr)
{
    for (uint32_t k = t; k < W; k += nthr) {
        LamParams P;
        lambda_setup_df(D, lam[k], z32, Rz, P, kYGuardRel, lx + k, false);
        if (P.all_exact) {
            // no reference ray: every ray of the band is re-traced
            P.core_lo = P.core_hi = 0;
        }
        lp[k] = P;
    }
}

// Counters of one design in the loop (shared memory).
struct LoopTally {
    unsigned long long hits, retraced, fast, H, inl;
    uint32_t item, qn;
};

// The loop's FP32 trace of the core rays by one warp: items of 32 rows x a ray chunk,
// claimed from the shared counter; hits as run-length fixed-point sums into the slab's
// histogram; flagged rays to the slab's queue, or re-traced here when it is full.
__device__ __noinline__ void loop_trace(const DevDesign &D, const LamParams *lp, const LamDF *lx, const float *z32,
                                        uint32_t W, uint32_t B, uint32_t Rz, uint32_t ray_tile,
                                        unsigned long long *hist, QEntry *queue, uint32_t qcap, LoopTally *tally,
                                        uint32_t lane)
{
    const uint32_t nblk = (W + 31u) / 32u;
    const uint32_t nchunk = Rz ? (Rz + ray_tile - 1u) / ray_tile : 1u;
    const uint32_t total = nblk * nchunk;
    // the design's constants in registers (read from shared memory at every use, they cost
    // more than the registers: loop alone 171 -> 172 k designs/s)
    const FastConst C = D.fc;
    const Guards guards = default_guards();
    const FastLimits Lm = fast_limits(C, guards);
    for (;;) {
        uint32_t item = 0;
        if (lane == 0) item = atomicAdd(&tally->item, 1u);
        item = __shfl_sync(0xffffffffu, item, 0);
        if (item >= total) break;
        const uint32_t blk = item / nchunk, chunk = item - blk * nchunk;
        const uint32_t k = blk * 32u + lane;
        LamParams P;
        uint32_t lo = 0, hi = 0;
        if (k < W) {
            P = lp[k];
            const uint32_t j0 = chunk * ray_tile;
            const uint32_t j1 = min(j0 + ray_tile, Rz);
            lo = max(j0, P.core_lo);
            hi = min(j1, P.core_hi);
        }
        const float2 *__restrict__ zt = reinterpret_cast<const float2 *>(z32);
        unsigned long long *hrow = hist + (uint64_t)k * B;
        uint32_t cur = 0xffffffffu;
        unsigned long long sum = 0ull;
        uint32_t nhit = 0, ninl = 0;
        for (uint32_t j = lo; j < hi; ++j) {
            const float2 z = __ldg(zt + j);
            uint32_t bin = 0;
            float tt = 0.f;
            const int r = fast_ray(C, Lm, P, guards, z.x, z.y, bin, tt);
            if (r == RAY_HIT) {
                if (bin != cur) {
                    if (sum) atomicAdd(hrow + cur, sum);
                    cur = bin;
                    sum = 0ull;
                }
                sum += t_fixed(tt);
                nhit++;
            } else if (r == RAY_FLAG) {
                const uint32_t pos = atomicAdd(&tally->qn, 1u);
                if (pos < qcap) {
                    queue[pos] = QEntry{0u, k, j, 0u};
                } else {
                    // the queue is full: re-trace here (counted as re-traced, as queued)
                    nhit += loop_retrace(D, lx[k], z32, j, hrow);
                    ninl++;
                }
            }
        }
        if (sum) atomicAdd(hrow + cur, sum);
        nhit = __reduce_add_sync(0xffffffffu, nhit);
        ninl = __reduce_add_sync(0xffffffffu, ninl);
        const uint32_t nfast = __reduce_add_sync(0xffffffffu, hi > lo ? hi - lo : 0u);
        if (lane == 0) {
            if (nhit) atomicAdd(&tally->hits, (unsigned long long)nhit);
            if (nfast) atomicAdd(&tally->fast, (unsigned long long)nfast);
            if (ninl) {
                atomicAdd(&tally->retraced, (unsigned long long)ninl);
                atomicAdd(&tally->inl, (unsigned long long)ninl);
            }
        }
    }
}

__global__ void __launch_bounds__(kLoopThreads, CPD_LOOP_MIN_BLOCKS) loop_kernel(const LoopArgs L)
{
    __shared__ __align__(16) LoopWork sW;
    DevDesign &sD = sW.d;
    DesignJob &sJ = sW.j;
    __shared__ float tab[4 * ff::kLogTable];
    __shared__ FinalizeRed fin_red[kLoopThreads / 32];
    __shared__ unsigned long long s_idx;
    __shared__ LoopTally tally;
    extern __shared__ __align__(16) unsigned long long loop_smem[];  // per-bin s1, s2 (max_B each)
    const uint32_t t = threadIdx.x, lane = t & 31u;
    for (uint32_t i = t; i < 4u * ff::kLogTable; i += blockDim.x) tab[i] = L.logtab[i];
    const SlabLayout SL = slab_layout(L.max_rows, L.max_cells, L.max_B, L.qcap);
    unsigned char *slab = L.slabs + (size_t)blockIdx.x * L.slab_bytes;
    unsigned long long *hist = reinterpret_cast<unsigned long long *>(slab + SL.hist);
    LamParams *lp = reinterpret_cast<LamParams *>(slab + SL.lp);
    LamDF *lx = reinterpret_cast<LamDF *>(slab + SL.lx);
    QEntry *queue = reinterpret_cast<QEntry *>(slab + SL.queue);
    unsigned long long *S1 = reinterpret_cast<unsigned long long *>(slab + SL.s1);
    unsigned long long *S2 = reinterpret_cast<unsigned long long *>(slab + SL.s2);
    DesignAcc *acc = reinterpret_cast<DesignAcc *>(slab + SL.acc);
    uint32_t *band = reinterpret_cast<uint32_t *>(slab + SL.band);  // exclusive prefix of band rays per row
    unsigned long long *s1 = loop_smem, *s2 = loop_smem + L.max_B;
    __shared__ uint32_t s_part[kLoopThreads];
    // the idle wait: bounded in time and in polls (a poll sleeps about a microsecond)
    const unsigned long long max_polls = L.idle_ns / 500ull + 1000ull;
    unsigned long long idle_start = global_ns();
    for (;;) {
        // ---- claim the next published ring entry, or leave after the idle limit
        if (t == 0) {
            unsigned long long got = ~0ull;
            for (unsigned long long polls = 0;; polls++) {
                const unsigned long long pub = load_acquire_sys(&L.ctl->published);
                const unsigned long long n = *reinterpret_cast<volatile unsigned long long *>(&L.cnt->claimed);
                if (n < pub) {
                    if (atomicCAS(&L.cnt->claimed, n, n + 1ull) == n) {
                        got = n;
                        break;
                    }
                    continue;
                }
                if (*reinterpret_cast<volatile unsigned int *>(&L.ctl->stop)) {
                    atomicAdd(&L.cnt->stop_exits, 1u);
                    break;
                }
                if (polls >= max_polls || global_ns() - idle_start > L.idle_ns) {
                    atomicAdd(&L.cnt->idle_exits, 1u);
                    break;
                }
                __nanosleep(1000);
            }
            s_idx = got;
            tally = LoopTally{0ull, 0ull, 0ull, 0ull, 0ull, 0u, 0u};
        }
        __syncthreads();
        const unsigned long long idx = s_idx;
        if (idx == ~0ull) break;
        const uint32_t slot = (uint32_t)(idx % L.capacity);
        {
            // the record (after thread 0's acquire of `published` and the barrier), in 16-byte
            // words from mapped host memory
            const uint4 *src = reinterpret_cast<const uint4 *>(&L.ring[slot]);
            uint4 *dst = reinterpret_cast<uint4 *>(&sW);
            for (uint32_t i = t; i < sizeof(LoopWork) / 16; i += blockDim.x) dst[i] = __ldcv(src + i);
        }
        unsigned long long *accw = reinterpret_cast<unsigned long long *>(acc);
        for (uint32_t i = t; i < sizeof(DesignAcc) / 8; i += blockDim.x) accw[i] = 0ull;
        __syncthreads();
        const uint32_t W = sJ.W, B = sJ.B, Rz = sJ.Rz, ray_tile = sW.ray_tile;
        const float *z32 = L.z32 + 2 * sJ.ray_off;
        for (uint32_t b = t; b < B; b += blockDim.x) s1[b] = s2[b] = 0ull;

        // ---- per-wavelength setup
        loop_setup(sD, L.lam + sJ.lam_off, z32, Rz, W, lp, lx, t, blockDim.x);
        __syncthreads();

        // ---- FP32 trace of the core rays
        loop_trace(sD, lp, lx, z32, W, B, Rz, ray_tile, hist, queue, L.qcap, &tally, lane);
        __syncthreads();

        // ---- float-float re-trace of every row's guard bands, spread over all threads (an
        // exclusive prefix sum of the rows' band rays: rows differ widely), then the queue
        {
            // per thread: a contiguous run of rows; its band rays, then a scan over threads
            const uint32_t per = (W + blockDim.x - 1u) / blockDim.x;
            const uint32_t k0 = min(t * per, W), k1 = min(k0 + per, W);
            uint32_t run = 0;
            for (uint32_t k = k0; k < k1; k++) {
                const LamParams &P = lp[k];
                band[k] = run;
                run += P.all_exact ? P.band_hi - P.band_lo : (P.core_lo - P.band_lo) + (P.band_hi - P.core_hi);
            }
            s_part[t] = run;
            __syncthreads();
            if (t == 0) {
                uint32_t acc_n = 0;
                for (uint32_t i = 0; i < blockDim.x; i++) {
                    const uint32_t v = s_part[i];
                    s_part[i] = acc_n;
                    acc_n += v;
                }
                band[W] = acc_n;
            }
            __syncthreads();
            for (uint32_t k = k0; k < k1; k++) band[k] += s_part[t];
            __syncthreads();
        }
        {
            unsigned long long hits = 0ull, ret = 0ull;
            const uint32_t nband = band[W];
            for (uint32_t i = t; i < nband; i += blockDim.x) {
                // the row holding band ray i: the last k with band[k] <= i
                uint32_t lo = 0, hi = W;
                while (hi - lo > 1u) {
                    const uint32_t mid = (lo + hi) >> 1;
                    if (band[mid] <= i) lo = mid;
                    else hi = mid;
                }
                const uint32_t k = lo, r = i - band[k];
                const LamParams &P = lp[k];
                const uint32_t na = P.all_exact ? P.band_hi - P.band_lo : P.core_lo - P.band_lo;
                const uint32_t j = r < na ? P.band_lo + r : P.core_hi + (r - na);
                hits += loop_retrace(sD, lx[k], z32, j, hist + (uint64_t)k * B);
                ret++;
            }
            const uint32_t qn = min(tally.qn, L.qcap);
            for (uint32_t i = t; i < qn; i += blockDim.x) {
                const QEntry e = queue[i];
                hits += loop_retrace(sD, lx[e.k], z32, e.j, hist + (uint64_t)e.k * B);
                ret++;
            }
            hits = warp_sum_u64(hits);
            ret = warp_sum_u64(ret);
            if (lane == 0) {
                if (hits) atomicAdd(&tally.hits, hits);
                if (ret) atomicAdd(&tally.retraced, ret);
            }
        }
        __syncthreads();

        // ---- entropy over the W x B cells; each nonzero cell is cleared for the next design
        {
            const ff::F2 unit{sJ.unit_hi, sJ.unit_lo}, lu{sJ.lu_hi, sJ.lu_lo};
            const uint32_t cells = W * B;
            unsigned long long hl = 0ull;
            for (uint32_t i = t; i < cells; i += blockDim.x) {
                const unsigned long long cv = hist[i];
                if (cv) {
                    hist[i] = 0ull;
                    unsigned long long hq, pq;
                    entropy_cell(cv, unit, lu, tab, hq, pq);
                    hl += hq;
                    const uint32_t b = i % B;
                    atomicAdd(s1 + b, cv);
                    atomicAdd(s2 + b, pq);
                }
            }
            hl = warp_sum_u64(hl);
            if (lane == 0 && hl) atomicAdd(&tally.H, hl);
        }
        __syncthreads();
        for (uint32_t b = t; b < B; b += blockDim.x) {
            S1[b] = s1[b];
            S2[b] = s2[b];
        }
        if (t == 0) {
            acc->H = tally.H;
            acc->rows = 0ull;
            acc->hits[0] = tally.hits;
            acc->retraced[0] = tally.retraced;
            acc->fast[0] = tally.fast;
            if (tally.inl) atomicAdd(&L.cnt->inline_retraced, tally.inl);
        }
        __syncthreads();

        // ---- finalize into the ring entry's result slot (mapped host memory)
        {
            LaunchArgs a;
            memset(&a, 0, sizeof(a));
            a.designs = &sD;
            a.acc = acc;
            a.S1 = S1;
            a.S2 = S2;
            a.out = &L.done[slot].o;
            DesignJob J = sJ;
            J.acc_off = 0;
            finalize_design(a, 0u, J, t, blockDim.x, tab, fin_red);
        }
        __syncthreads();
        if (t == 0) {
            L.done[slot].status = 0u;
            __threadfence_system();
            store_release_sys(&L.done[slot].seq, idx + 1ull);
            atomicAdd(&L.cnt->designs, 1ull);
        }
        idle_start = global_ns();
    }
}

}  // namespace

// A launch that, with `pdl`, may start before the previous kernel on the stream has
// finished (programmatic dependent launch): the kernel waits for its predecessor's
// results in cudaGridDependencySynchronize.
void launch_k(void (*k)(const LaunchArgs), unsigned grid, unsigned block, size_t smem, cudaStream_t st, bool pdl,
              const LaunchArgs &a)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = pdl ? attr : nullptr;
    cfg.numAttrs = pdl ? 1 : 0;
    cudaLaunchKernelEx(&cfg, k, a);
}

int launch_pass(const LaunchArgs &a, int num_sms, uint32_t warps_per_cta, cudaStream_t stream, cudaEvent_t *ev,
                bool pdl)
{
    // per-kernel events would stand between the kernels
    pdl = pdl && ev == nullptr;
    int launches = 0;
    if (ev) cudaEventRecord(ev[0], stream);
    if (a.params) {
        launch_k(build_kernel, (a.njobs + 31u) / 32u, 32, 0, stream, false, a);
        launches++;
    }
    if (a.total_rows) {
        // one warp per block: each row is one thread's latency-bound float-float chain,
        // so spreading the rows over every SM matters
        const uint32_t blocks = (uint32_t)((a.total_rows + 31) / 32);
        const uint32_t cap = a.stage_cap < kStageRays ? a.stage_cap : kStageRays;
        // a single-design pass (spans) splits each row's chain over two warps
        launch_k(a.spans ? setup_pair_kernel : setup_kernel, blocks, a.spans ? 64 : 32,
                 2 * ((cap + 1u) & ~1u) * sizeof(float), stream, false, a);
        launches++;
    }
    if (a.adaptive) {
        const uint32_t maxB = a.max_B ? a.max_B : (uint32_t)CPD_MAX_BINS;
        if (ev) cudaEventRecord(ev[1], stream);
        if (a.total_rows) {
            // enough rows to fill the GPU: few warps per row (rounds traced past a row's
            // stop are wasted); fewer rows: up to kMaxAdaptWarps warps per row trace and
            // decide that many rounds at once
            const uint64_t per_sm = a.total_rows / (uint64_t)num_sms;
            const uint32_t kw = per_sm >= 8 ? CPD_ADAPT_KW_MANY : per_sm >= 2 ? CPD_ADAPT_KW_SOME : kMaxAdaptWarps;
            launch_k(kw == 1u ? adaptive1_kernel : adaptive_kernel, (unsigned)a.total_rows, 32 * kw,
                     kw == 1u ? adapt1_smem_bytes(maxB) : adapt_smem_bytes(kw, maxB), stream, pdl, a);
            launches++;
        }
        if (ev) cudaEventRecord(ev[2], stream);
        const uint32_t kwe = a.total_rows / (uint64_t)num_sms >= 8 ? 1u : kMaxAdaptWarps;
        launch_k(adaptive_exact_kernel, (unsigned)(num_sms * (kwe == 1u ? 8 : 1)), 32 * kwe,
                 kwe == 1u ? adapt1_smem_bytes(maxB) : adapt_smem_bytes(kwe, maxB), stream, pdl, a);
        launches++;
    } else {
    if (ev) cudaEventRecord(ev[1], stream);
    if (a.mode != CPD_TRACE_FP64 && a.total_items) {
        int per_sm = 0;
        const int threads = (int)warps_per_cta * 32;
        auto k = a.spans ? trace_spans_kernel : trace_kernel;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, threads, 0);
        if (per_sm < 1) per_sm = 1;
        uint64_t grid = (uint64_t)num_sms * per_sm;
        // equal shares: every resident warp; work items: no more warps than items
        const uint64_t need = (a.total_items + warps_per_cta - 1) / warps_per_cta;
        if (!a.spans && grid > need) grid = need;
        launch_k(k, (unsigned)grid, threads, 0, stream, pdl, a);
        launches++;
    }
    if (ev) cudaEventRecord(ev[2], stream);
    // the single-design trace re-traces its own flagged rays; what reaches the queue there
    // (the setup's guard bands, a warp's flags past kWarpFlags) is usually little, and a
    // grid of one block per SM is resident beside the trace, ready when it completes
    launch_k(a.mode == CPD_TRACE_FP64 ? retrace_exact_kernel : retrace_kernel,
             (unsigned)(num_sms * (a.spans ? 1 : 8)), 32, 0, stream, pdl, a);
    launches++;
    }
    if (ev) cudaEventRecord(ev[3], stream);
    if (a.total_tiles) {
        const uint64_t wpb = (uint64_t)kEntropyThreads / 32u;
        if (a.total_tiles <= (uint64_t)num_sms * wpb) {
            // few tiles: one block per tile
            const size_t smem = 2u * sizeof(unsigned long long) * (a.max_B ? a.max_B : (uint32_t)CPD_MAX_BINS);
            int per_sm = 0;
            auto k = a.p_out ? entropy_block_kernel<true> : entropy_block_kernel<false>;
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kEntropyThreads, smem);
            if (per_sm < 1) per_sm = 1;
            uint64_t grid = a.total_tiles;
            if (grid > (uint64_t)num_sms * per_sm) grid = (uint64_t)num_sms * per_sm;
            launch_k(k, (unsigned)grid, kEntropyThreads, smem, stream, pdl, a);
        } else {
            // one warp per tile, as many blocks as are resident at once
            int per_sm = 0;
            auto k = a.p_out ? entropy_warp_kernel<true> : entropy_warp_kernel<false>;
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kEntropyThreads, 0);
            if (per_sm < 1) per_sm = 1;
            uint64_t grid = (a.total_tiles + wpb - 1) / wpb;
            if (grid > (uint64_t)num_sms * per_sm) grid = (uint64_t)num_sms * per_sm;
            launch_k(k, (unsigned)grid, kEntropyThreads, 0, stream, pdl, a);
        }
        launches++;
    }
    if (a.njobs > 1 || !a.total_tiles) {
        launch_k(finalize_kernel, (a.njobs + 3u) / 4u, 128, 0, stream, pdl, a);
        launches++;
    }
    if (ev) cudaEventRecord(ev[4], stream);
    return launches;
}

cudaError_t configure_kernels()
{
    const int bytes = (int)adapt_smem_bytes(kMaxAdaptWarps, CPD_MAX_BINS);
    cudaError_t e = cudaFuncSetAttribute(adaptive_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(adaptive1_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)adapt1_smem_bytes(CPD_MAX_BINS));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(adaptive_exact_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    return e;
}

const void *trace_spans_kernel_fn() { return reinterpret_cast<const void *>(trace_spans_kernel); }

uint64_t trace_resident_warps(int num_sms, uint32_t warps_per_cta)
{
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, trace_kernel, (int)warps_per_cta * 32, 0);
    if (per_sm < 1) per_sm = 1;
    return (uint64_t)num_sms * (uint64_t)per_sm * warps_per_cta;
}

void launch_build_records(const cpd_spectrometer_params *p, uint32_t n, double acceptance, cpd_design *out,
                          int32_t *status, cudaStream_t stream)
{
    if (!n) return;
    build_records_kernel<<<(n + 31) / 32, 32, 0, stream>>>(p, n, acceptance, out, status);
}

void launch_trace_pairs(const DevDesign *d, const double *lam_u, const double *z64, uint32_t n, uint32_t mode,
                        uint32_t *bins, double *ts, uint8_t *flags, cudaStream_t stream)
{
    if (!n) return;
    trace_pairs_kernel<<<(n + 127) / 128, 128, 0, stream>>>(d, lam_u, z64, n, mode, bins, ts, flags);
}

void launch_tp_adaptive(const DevDesign *d, uint32_t B, const double *lambdas, uint32_t n, const double *z64,
                        uint32_t max_m, double *out, uint32_t *rays_out, cudaStream_t stream)
{
    if (!n) return;
    tp_adaptive_kernel<<<n, kTpRays, 3 * sizeof(double) * B, stream>>>(d, lambdas, z64, max_m, out, rays_out);
}

void launch_mufu_peak(float *out, uint32_t iters, int blocks, int threads, cudaStream_t stream)
{
    mufu_peak_kernel<<<blocks, threads, 0, stream>>>(out, iters);
}

size_t loop_slab_bytes(uint32_t max_rows, uint32_t max_cells, uint32_t max_B, uint32_t qcap)
{
    return slab_layout(max_rows, max_cells, max_B, qcap).bytes;
}

void launch_loop(const LoopArgs &a, uint32_t grid, cudaStream_t stream)
{
    loop_kernel<<<grid, kLoopThreads, 2 * sizeof(unsigned long long) * a.max_B, stream>>>(a);
}

int loop_ctas_per_sm()
{
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, loop_kernel, kLoopThreads,
                                                  2 * sizeof(unsigned long long) * CPD_MAX_BINS);
    return per_sm < 1 ? 1 : per_sm;
}

void launch_fma_peak(float *out, uint32_t iters, int blocks, int threads, cudaStream_t stream)
{
    fma_peak_kernel<<<blocks, threads, 0, stream>>>(out, iters);
}

}  // namespace cpd
