// cpd_kernels.cu -- the GB300 kernels of the fitness path.
//
// A pass over a set of designs runs four kernels on one stream:
//   setup    one thread per (design, wavelength): exact f64 flat-face chain ->
//            LamParams; guard-band rays of the y interval go to the re-trace queue
//   trace    persistent warps over work items (design, 32-wavelength block, ray
//            chunk); lane = wavelength; FP32 exit face + detector per ray; hits
//            accumulate per lane as run-length fixed-point sums (rays are sorted by
//            start height, so consecutive rays mostly share a bin) flushed with one
//            64-bit atomic per run; guard-band rays go to the queue
//   retrace  exact f64 trace of every queued ray (bit-identical to the reference's
//            f64 CPU trace)
//   entropy  per (design, row tile): p = sum/R, p log2 p, per-bin sums of p and p^2,
//            all in FP64 with fixed-point accumulation (order independent); the last
//            tile of each design runs the fused finalize (MI, SEM convergence).
#include <cuda_runtime.h>

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

__global__ void __launch_bounds__(32) setup_kernel(const LaunchArgs a)
{
    const uint64_t row = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (row >= a.total_rows) return;
    const uint32_t d = find_job<F_ROW>(a.jobs, a.njobs, row);
    const DesignJob &J = a.jobs[d];
    const uint32_t k = (uint32_t)(row - J.row_off);
    const DevDesign &D = a.designs[d];
    const double lambda = x::wavelength(D, a.lam_u[J.lam_off + k]);
    LamParams P;
    lambda_setup(D, lambda, a.z64 + J.ray_off, J.Rz, P, a.yguard_rel, a.lx + row);
    if (a.mode == CPD_TRACE_FP64 || (P.all_exact && a.mode == CPD_TRACE_HYBRID)) {
        for (uint32_t j = P.band_lo; j < P.band_hi; j++) push_ray(a, d, k, j);
        P.core_lo = P.core_hi = 0;
    } else if (P.all_exact) {
        // FP32-only study mode without a reference ray: these rays are counted as lost
        P.core_lo = P.core_hi = 0;
    } else {
        for (uint32_t j = P.band_lo; j < P.core_lo; j++) push_ray(a, d, k, j);
        for (uint32_t j = P.core_hi; j < P.band_hi; j++) push_ray(a, d, k, j);
    }
    a.lp[row] = P;
}

__global__ void __launch_bounds__(256, 3) trace_kernel(const LaunchArgs a)
{
    const uint32_t lane = threadIdx.x & 31u;
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
        const uint32_t k = blk * 32u + lane;
        const FastConst C = a.designs[d].fc;
        LamParams P;
        uint32_t lo = 0, hi = 0;
        if (k < J.W) {
            P = a.lp[J.row_off + k];
            const uint32_t j0 = chunk * a.ray_tile;
            const uint32_t j1 = min(j0 + a.ray_tile, J.Rz);
            lo = max(j0, P.core_lo);
            hi = min(j1, P.core_hi);
        }
        const float2 *__restrict__ zt = reinterpret_cast<const float2 *>(a.z32) + J.ray_off;
        unsigned long long *hrow = a.hist + J.hist_off + (uint64_t)k * J.B;
        uint32_t cur = 0xffffffffu;
        unsigned long long sum = 0ull;
        uint32_t nhit = 0;
        const Guards g = a.guards;
        for (uint32_t j = lo; j < hi; ++j) {
            const float2 z = __ldg(zt + j);
            uint32_t bin = 0;
            float t = 0.f;
            const int r = fast_ray(C, P, g, z.x, z.y, bin, t);
            if (r == RAY_HIT) {
                if (bin != cur) {
                    if (sum) atomicAdd(hrow + cur, sum);
                    cur = bin;
                    sum = 0ull;
                }
                sum += t_fixed(t);
                nhit++;
            } else if (r == RAY_FLAG) {
                push_ray(a, d, k, j);
            }
        }
        if (sum) atomicAdd(hrow + cur, sum);
        nhit = __reduce_add_sync(0xffffffffu, nhit);
        const uint32_t nfast = __reduce_add_sync(0xffffffffu, hi > lo ? hi - lo : 0u);
        if (lane == 0 && nhit) atomicAdd(&a.acc[d].hits, (unsigned long long)nhit);
        if (lane == 0 && nfast) atomicAdd(&a.acc[d].fast, (unsigned long long)nfast);
    }
}

__global__ void __launch_bounds__(32) retrace_kernel(const LaunchArgs a)
{
    const unsigned long long qn = a.ctl->queue_count;
    const uint64_t n = qn < a.qcap ? qn : a.qcap;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const QEntry e = a.queue[i];
        const DevDesign &D = a.designs[e.design];
        const DesignJob &J = a.jobs[e.design];
        const double y = x::beam_y(D, a.z64[J.ray_off + e.j]);
        uint32_t bin = 0;
        double t = 0.0;
        if (x::trace_lam(D, a.lx[J.row_off + e.k], y, bin, t) == 0) {
            atomicAdd(a.hist + J.hist_off + (uint64_t)e.k * J.B + bin, (unsigned long long)t_fixed64(t));
            atomicAdd(&a.acc[e.design].hits, 1ull);
        }
        atomicAdd(&a.acc[e.design].retraced, 1ull);
    }
}

__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

constexpr int kEntropyThreads = 256;

// Fused per-design finalize, run by the block that finished the design's last tile.
__device__ void finalize(const LaunchArgs &a, uint32_t d, const DesignJob &J)
{
    __shared__ double red[kEntropyThreads];
    __shared__ double red_sem[kEntropyThreads];
    __shared__ int red_conv[kEntropyThreads];
    const uint32_t tid = threadIdx.x;
    const unsigned long long rows = __ldcg(&a.acc[d].rows) + J.W;
    const double n = (double)rows;
    const double e2 = 5e-3 * 5e-3;
    double hdet = 0.0, msem = 0.0;
    int conv = 1;
    const double p_unit = kTScaleInv / (double)J.R;  // p per count unit
    for (uint32_t b = tid; b < J.B; b += blockDim.x) {
        const double s1 = (double)__ldcg(&a.S1[J.acc_off + b]) * p_unit;  // sum over rows of p
        const double s2 = (double)__ldcg(&a.S2[J.acc_off + b]) * kPScaleInv;
        const double pbar = s1 / n;
        if (pbar > 0.0) hdet += pbar * log2(pbar);
        // Welford M2 of the per-wavelength p(d|lambda) (welford.rs:26-57)
        double m2 = s2 - s1 * s1 / n;
        if (m2 < 0.0) m2 = 0.0;
        const double thr = e2 * (n * (n - 1.0));
        conv &= (m2 < thr) ? 1 : 0;
        const double sem = n > 1.0 ? sqrt(m2 / (n - 1.0) / n) : INFINITY;
        msem = fmax(msem, sem);
    }
    red[tid] = hdet;
    red_sem[tid] = msem;
    red_conv[tid] = conv;
    __syncthreads();
    for (uint32_t s = blockDim.x >> 1; s > 0; s >>= 1) {
        if (tid < s) {
            red[tid] += red[tid + s];
            red_sem[tid] = fmax(red_sem[tid], red_sem[tid + s]);
            red_conv[tid] &= red_conv[tid + s];
        }
        __syncthreads();
    }
    if (tid == 0) {
        const double H = (double)__ldcg(&a.acc[d].H) * kHScaleInv;
        const double h_cond = -H / n;
        DesignOut o;
        o.h_cond = h_cond;
        o.h_det = red[0];
        o.info = h_cond - red[0];
        o.max_sem = red_sem[0];
        o.hits = __ldcg(&a.acc[d].hits);
        o.retraced = __ldcg(&a.acc[d].retraced);
        o.rows = rows;
        o.fast = __ldcg(&a.acc[d].fast);
        o.converged = red_conv[0];
        o.pad = 0;
        a.out[d] = o;
        a.acc[d].rows = rows;
    }
}

// Thread -> (bin, row group) map of an entropy tile: for B <= 256 each thread owns one
// bin and every (256/B)-th row of the tile; for wider detectors each thread owns the
// bins tid, tid+256, ... of every row. Per-thread partial sums are therefore fixed by
// B alone, whatever else shares the launch.
__global__ void __launch_bounds__(kEntropyThreads) entropy_kernel(const LaunchArgs a)
{
    extern __shared__ unsigned long long sm[];  // S1[B], S2[B] of this tile
    __shared__ unsigned long long hsum;
    __shared__ int last;
    __shared__ float tab[4 * ff::kLogTable];
    const uint32_t tid = threadIdx.x;
    // A pass whose re-trace queue overflowed is re-run by the host: leave every
    // accumulator untouched.
    if (a.ctl->overflow || a.ctl->queue_count > a.qcap) return;
    for (uint32_t i = tid; i < 4u * ff::kLogTable; i += blockDim.x) tab[i] = a.logtab[i];
    __syncthreads();
    for (uint64_t tile = blockIdx.x; tile < a.total_tiles; tile += gridDim.x) {
        const uint32_t d = find_job<F_TILE>(a.jobs, a.njobs, tile);
        const DesignJob J = a.jobs[d];
        const uint32_t tl = (uint32_t)(tile - J.tile_off);
        const uint32_t r0 = tl * J.tile_rows;
        const uint32_t r1 = min(r0 + J.tile_rows, J.W);
        const uint32_t B = J.B;
        for (uint32_t b = tid; b < 2 * B; b += blockDim.x) sm[b] = 0ull;
        if (tid == 0) hsum = 0ull;
        __syncthreads();
        const double p_unit = kTScaleInv / (double)J.R;
        const ff::F2 unit{J.unit_hi, J.unit_lo}, lu{J.lu_hi, J.lu_lo};
        unsigned long long *base = a.hist + J.hist_off;
        const uint32_t groups = B <= (uint32_t)kEntropyThreads ? (uint32_t)kEntropyThreads / B : 1u;
        const uint32_t grp = tid / (B <= (uint32_t)kEntropyThreads ? B : (uint32_t)kEntropyThreads);
        const uint32_t bin0 = B <= (uint32_t)kEntropyThreads ? tid % B : tid;
        ff::F2 h{0.f, 0.f};
        if (grp < groups) {
            for (uint32_t b = bin0; b < B; b += kEntropyThreads) {
                unsigned long long c1 = 0ull;
                ff::F2 q2{0.f, 0.f};
                for (uint32_t row = r0 + grp; row < r1; row += groups) {
                    unsigned long long *cell = base + (uint64_t)row * B + b;
                    const unsigned long long c = *cell;
                    if (c) {
                        *cell = 0ull;  // leaves the histogram zeroed for the next pass
                        // p = c unit and p log2 p in float-float (FP32 pipe)
                        const ff::F2 p = ff::mul(ff::from_u64(c), unit);
                        const ff::F2 lp = ff::add(ff::log2_u64(c, tab), lu);
                        h = ff::add(h, ff::mul(p, lp));
                        q2 = ff::add(q2, ff::mul(p, p));
                        c1 += c;
                    }
                    if (a.p_out) a.p_out[(uint64_t)row * B + b] = (double)c * p_unit;
                }
                if (c1) {
                    atomicAdd(&sm[b], c1);
                    atomicAdd(&sm[B + b], __double2ull_rn(((double)q2.hi + (double)q2.lo) * kPScale));
                }
            }
        }
        unsigned long long hl = __double2ull_rn(-((double)h.hi + (double)h.lo) * kHScale);
        hl = warp_sum_u64(hl);
        if ((tid & 31u) == 0 && hl) atomicAdd(&hsum, hl);
        __syncthreads();
        for (uint32_t b = tid; b < B; b += blockDim.x) {
            if (sm[b]) atomicAdd(&a.S1[J.acc_off + b], sm[b]);
            if (sm[B + b]) atomicAdd(&a.S2[J.acc_off + b], sm[B + b]);
        }
        if (tid == 0 && hsum) atomicAdd(&a.acc[d].H, hsum);
        __threadfence();
        __syncthreads();
        if (tid == 0) last = (atomicAdd(&a.tiles_done[d], 1u) == J.ntiles - 1u) ? 1 : 0;
        __syncthreads();
        if (last) {
            __threadfence();
            finalize(a, d, J);
        }
        __syncthreads();
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
    const double lambda = x::wavelength(D, lam_u[i]);
    const double z = z64[i];
    uint32_t bin = D.B;
    double t = 0.0;
    uint8_t fl = 0;
    if (isfinite(z)) {
        bool exact = mode == CPD_TRACE_FP64;
        if (!exact) {
            LamParams P;
            const double yg = mode == CPD_TRACE_FP32 ? 0.0 : kYGuardRel;
            lambda_setup(D, lambda, &z, 1u, P, yg);
            if (P.core_lo == 0 && P.core_hi == 1 && P.all_exact) {
                // the ray is its own reference and it has no usable exit/detector geometry
                exact = mode == CPD_TRACE_HYBRID;
            } else if (P.core_lo == 0 && P.core_hi == 1) {
                const Guards g = mode == CPD_TRACE_FP32 ? no_guards() : default_guards();
                float zh, zl;
                split_f32(z, zh, zl);
                uint32_t b = 0;
                float tf = 0.f;
                const int r = fast_ray(D.fc, P, g, zh, zl, b, tf);
                if (r == RAY_HIT) {
                    bin = b;
                    t = tf;
                } else if (r == RAY_FLAG) {
                    exact = true;
                }
            } else if (P.band_lo == 0 && P.band_hi == 1) {
                exact = true;  // in a y-interval guard band
            }
        }
        if (exact) {
            fl = mode == CPD_TRACE_FP64 ? 0 : 1;
            uint32_t b = 0;
            double te = 0.0;
            if (x::trace(D, lambda, x::beam_y(D, z), b, te) == 0) {
                bin = b;
                t = te;
            }
        }
    }
    bins[i] = bin;
    ts[i] = t;
    if (flags) flags[i] = fl;
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

}  // namespace

int launch_pass(const LaunchArgs &a, int num_sms, uint32_t warps_per_cta, cudaStream_t stream, cudaEvent_t *ev)
{
    int launches = 0;
    if (ev) cudaEventRecord(ev[0], stream);
    if (a.total_rows) {
        // one warp per block: f64-pipe bound, so spreading rows over every SM matters
        const uint32_t blocks = (uint32_t)((a.total_rows + 31) / 32);
        setup_kernel<<<blocks, 32, 0, stream>>>(a);
        launches++;
    }
    if (ev) cudaEventRecord(ev[1], stream);
    if (a.mode != CPD_TRACE_FP64 && a.total_items) {
        int per_sm = 0;
        const int threads = (int)warps_per_cta * 32;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, trace_kernel, threads, 0);
        if (per_sm < 1) per_sm = 1;
        uint64_t grid = (uint64_t)num_sms * per_sm;
        const uint64_t need = (a.total_items + warps_per_cta - 1) / warps_per_cta;
        if (grid > need) grid = need;
        trace_kernel<<<(unsigned)grid, threads, 0, stream>>>(a);
        launches++;
    }
    if (ev) cudaEventRecord(ev[2], stream);
    retrace_kernel<<<(unsigned)(num_sms * 8), 32, 0, stream>>>(a);
    launches++;
    if (ev) cudaEventRecord(ev[3], stream);
    if (a.total_tiles) {
        uint32_t maxB = 0;
        // the entropy kernel sizes its shared per-bin sums for the widest detector
        maxB = CPD_MAX_BINS;
        uint64_t grid = (uint64_t)num_sms * 8;
        if (grid > a.total_tiles) grid = a.total_tiles;
        entropy_kernel<<<(unsigned)grid, kEntropyThreads, 2 * maxB * sizeof(unsigned long long), stream>>>(a);
        launches++;
    }
    if (ev) cudaEventRecord(ev[4], stream);
    return launches;
}

void launch_trace_pairs(const DevDesign *d, const double *lam_u, const double *z64, uint32_t n, uint32_t mode,
                        uint32_t *bins, double *ts, uint8_t *flags, cudaStream_t stream)
{
    if (!n) return;
    trace_pairs_kernel<<<(n + 127) / 128, 128, 0, stream>>>(d, lam_u, z64, n, mode, bins, ts, flags);
}

void launch_fma_peak(float *out, uint32_t iters, int blocks, int threads, cudaStream_t stream)
{
    fma_peak_kernel<<<blocks, threads, 0, stream>>>(out, iters);
}

}  // namespace cpd
