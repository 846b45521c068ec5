// cpd_runtime.cu -- the GPU side of the C ABI: context, pooled buffers, ray-table
// cache, pass planning and CUDA-graph replay of the per-pass launch sequence.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "cpd_gpu.cuh"
#include "cpd_host.h"

namespace cpd {
namespace {

struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t bytes)
    {
        if (bytes <= cap) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        size_t want = std::max<size_t>(bytes, 256);
        want = want + want / 4;
        cudaError_t e = cudaMalloc(&p, want);
        if (e == cudaSuccess) cap = want;
        return e;
    }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
    template <class T>
    T *as() const
    {
        return reinterpret_cast<T *>(p);
    }
};

struct HostBuf {
    void *p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t bytes)
    {
        if (bytes <= cap) return cudaSuccess;
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
        size_t want = std::max<size_t>(bytes, 256);
        want = want + want / 4;
        cudaError_t e = cudaMallocHost(&p, want);
        if (e == cudaSuccess) cap = want;
        return e;
    }
    void release()
    {
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
    }
    template <class T>
    T *as() const
    {
        return reinterpret_cast<T *>(p);
    }
};

struct RayKey {
    uint64_t seed_bits;
    uint32_t R;
    bool operator<(const RayKey &o) const { return seed_bits != o.seed_bits ? seed_bits < o.seed_bits : R < o.R; }
};

struct RayTable {
    std::vector<double> z64;
    std::vector<float> z32;
};

}  // namespace
}  // namespace cpd

using namespace cpd;

struct cpd_context {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::mutex mu;
    // device buffers
    DevBuf designs, jobs, lam_u, z64, z32, lp, lx, hist, S1, S2, acc, tiles, out, ctl, queue, pout;
    DevBuf pair_lam, pair_z, pair_bins, pair_ts, pair_flags, peak, logtab;
    // pinned staging
    HostBuf h_designs, h_jobs, h_lam, h_z64, h_z32, h_out, h_ctl, h_pout, h_pairs;
    bool hist_dirty = true;
    uint32_t ray_tile = 32;
    uint32_t warps_per_cta = 8;
    uint32_t qcap = 1u << 18;
    double last_ms = 0.0;
    uint32_t last_launches = 0;
    uint64_t last_h2d = 0, last_d2h = 0;
    bool profiling = false;
    cudaEvent_t kev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    double kernel_ms[4] = {0, 0, 0, 0};
    // ray-table cache (host side), keyed by (seed, R)
    std::map<RayKey, RayTable> ray_cache;
    // graph cache: one executable graph per pass signature
    std::vector<uint8_t> graph_key;
    cudaGraphExec_t graph_exec = nullptr;
    int graph_launches = 0;
    bool use_graphs = true;
};

namespace {

#define CPD_TRY(expr)                         \
    do {                                      \
        cudaError_t _e = (expr);              \
        if (_e != cudaSuccess) return CPD_CUDA_ERROR; \
    } while (0)

const RayTable &ray_table_cached(cpd_context *ctx, double seed, uint32_t R)
{
    uint64_t bits;
    std::memcpy(&bits, &seed, 8);
    RayKey key{bits, R};
    auto it = ctx->ray_cache.find(key);
    if (it != ctx->ray_cache.end()) return it->second;
    if (ctx->ray_cache.size() > 64) ctx->ray_cache.clear();
    std::vector<double> u(R);
    seed_points(seed, 1, R, u.data());
    RayTable t;
    ray_table(u.data(), R, t.z64, t.z32);
    return ctx->ray_cache.emplace(key, std::move(t)).first->second;
}

// One design's sampling inputs for a pass.
struct PassDesign {
    const DevDesign *dev;      // host copy
    uint32_t W, R;
    const double *lam_u;       // W wavelength u-points (host)
    const RayTable *rays;
};

struct PassResult {
    std::vector<DesignOut> outs;
    bool overflow = false;
};

uint32_t tile_rows_for(uint32_t B) { return std::max<uint32_t>(1u, 1024u / B); }

// Plans and runs one pass over `ds`. Accumulators (S1, S2, acc) are zeroed when
// `fresh`; they persist otherwise (the seeds of one call).
int run_pass(cpd_context *ctx, const std::vector<PassDesign> &ds, uint32_t mode, bool fresh, double *p_out_host,
             PassResult &res)
{
    const uint32_t n = (uint32_t)ds.size();
    std::vector<DesignJob> jobs(n);
    uint64_t rows = 0, hist = 0, lam = 0, ray = 0, accc = 0, items = 0, tiles = 0;
    for (uint32_t i = 0; i < n; i++) {
        const PassDesign &p = ds[i];
        DesignJob &J = jobs[i];
        std::memset(&J, 0, sizeof(J));
        J.W = p.W;
        J.R = p.R;
        J.Rz = (uint32_t)p.rays->z64.size();
        J.B = p.dev->B;
        J.row_off = rows;
        J.hist_off = hist;
        J.lam_off = lam;
        J.ray_off = ray;
        J.acc_off = accc;
        J.item_off = items;
        J.tile_off = tiles;
        J.nchunk = std::max<uint32_t>(1u, (J.Rz + ctx->ray_tile - 1) / ctx->ray_tile);
        J.tile_rows = tile_rows_for(J.B);
        J.ntiles = (J.W + J.tile_rows - 1) / J.tile_rows;
        ff::split(kTScaleInv / (double)J.R, J.unit_hi, J.unit_lo);
        ff::split(-31.0 - std::log2((double)J.R), J.lu_hi, J.lu_lo);
        rows += J.W;
        hist += (uint64_t)J.W * J.B;
        lam += J.W;
        ray += J.Rz;
        accc += J.B;
        items += (uint64_t)((J.W + 31) / 32) * J.nchunk;
        tiles += J.ntiles;
    }
    // staging
    CPD_TRY(ctx->h_designs.ensure(sizeof(DevDesign) * n));
    CPD_TRY(ctx->h_jobs.ensure(sizeof(DesignJob) * n));
    CPD_TRY(ctx->h_lam.ensure(sizeof(double) * std::max<uint64_t>(lam, 1)));
    CPD_TRY(ctx->h_z64.ensure(sizeof(double) * std::max<uint64_t>(ray, 1)));
    CPD_TRY(ctx->h_z32.ensure(2 * sizeof(float) * std::max<uint64_t>(ray, 1)));
    CPD_TRY(ctx->h_out.ensure(sizeof(DesignOut) * n));
    CPD_TRY(ctx->h_ctl.ensure(sizeof(Control)));
    for (uint32_t i = 0; i < n; i++) {
        ctx->h_designs.as<DevDesign>()[i] = *ds[i].dev;
        ctx->h_jobs.as<DesignJob>()[i] = jobs[i];
        std::memcpy(ctx->h_lam.as<double>() + jobs[i].lam_off, ds[i].lam_u, sizeof(double) * ds[i].W);
        std::memcpy(ctx->h_z64.as<double>() + jobs[i].ray_off, ds[i].rays->z64.data(), sizeof(double) * jobs[i].Rz);
        std::memcpy(ctx->h_z32.as<float>() + 2 * jobs[i].ray_off, ds[i].rays->z32.data(),
                    2 * sizeof(float) * jobs[i].Rz);
    }
    // device buffers
    const size_t hist_bytes = sizeof(unsigned long long) * std::max<uint64_t>(hist, 1);
    size_t old_hist = ctx->hist.cap;
    CPD_TRY(ctx->designs.ensure(sizeof(DevDesign) * n));
    CPD_TRY(ctx->jobs.ensure(sizeof(DesignJob) * n));
    CPD_TRY(ctx->lam_u.ensure(sizeof(double) * std::max<uint64_t>(lam, 1)));
    CPD_TRY(ctx->z64.ensure(sizeof(double) * std::max<uint64_t>(ray, 1)));
    CPD_TRY(ctx->z32.ensure(2 * sizeof(float) * std::max<uint64_t>(ray, 1)));
    CPD_TRY(ctx->lp.ensure(sizeof(LamParams) * std::max<uint64_t>(rows, 1)));
    CPD_TRY(ctx->lx.ensure(sizeof(ExactLam) * std::max<uint64_t>(rows, 1)));
    CPD_TRY(ctx->hist.ensure(hist_bytes));
    if (ctx->hist.cap != old_hist) ctx->hist_dirty = true;
    CPD_TRY(ctx->S1.ensure(sizeof(unsigned long long) * std::max<uint64_t>(accc, 1)));
    CPD_TRY(ctx->S2.ensure(sizeof(unsigned long long) * std::max<uint64_t>(accc, 1)));
    CPD_TRY(ctx->acc.ensure(sizeof(DesignAcc) * n));
    CPD_TRY(ctx->tiles.ensure(sizeof(unsigned int) * n));
    CPD_TRY(ctx->out.ensure(sizeof(DesignOut) * n));
    CPD_TRY(ctx->ctl.ensure(sizeof(Control)));
    CPD_TRY(ctx->queue.ensure(sizeof(QEntry) * ctx->qcap));
    if (p_out_host) CPD_TRY(ctx->pout.ensure(hist_bytes));

    cudaStream_t s = ctx->stream;
    if (ctx->hist_dirty) {
        CPD_TRY(cudaMemsetAsync(ctx->hist.p, 0, ctx->hist.cap, s));
        ctx->hist_dirty = false;
    }
    CPD_TRY(cudaMemcpyAsync(ctx->designs.p, ctx->h_designs.p, sizeof(DevDesign) * n, cudaMemcpyHostToDevice, s));
    CPD_TRY(cudaMemcpyAsync(ctx->jobs.p, ctx->h_jobs.p, sizeof(DesignJob) * n, cudaMemcpyHostToDevice, s));
    CPD_TRY(cudaMemcpyAsync(ctx->lam_u.p, ctx->h_lam.p, sizeof(double) * lam, cudaMemcpyHostToDevice, s));
    CPD_TRY(cudaMemcpyAsync(ctx->z64.p, ctx->h_z64.p, sizeof(double) * ray, cudaMemcpyHostToDevice, s));
    CPD_TRY(cudaMemcpyAsync(ctx->z32.p, ctx->h_z32.p, 2 * sizeof(float) * ray, cudaMemcpyHostToDevice, s));
    ctx->last_h2d += sizeof(DevDesign) * n + sizeof(DesignJob) * n + sizeof(double) * lam +
                     (sizeof(double) + 2 * sizeof(float)) * ray;
    ctx->last_d2h += sizeof(DesignOut) * n + sizeof(Control) + (p_out_host ? sizeof(double) * hist : 0);
    if (fresh) {
        CPD_TRY(cudaMemsetAsync(ctx->S1.p, 0, sizeof(unsigned long long) * accc, s));
        CPD_TRY(cudaMemsetAsync(ctx->S2.p, 0, sizeof(unsigned long long) * accc, s));
        CPD_TRY(cudaMemsetAsync(ctx->acc.p, 0, sizeof(DesignAcc) * n, s));
    }

    LaunchArgs a;
    std::memset(&a, 0, sizeof(a));
    a.designs = ctx->designs.as<DevDesign>();
    a.jobs = ctx->jobs.as<DesignJob>();
    a.njobs = n;
    a.total_rows = rows;
    a.total_items = items;
    a.total_tiles = tiles;
    a.lam_u = ctx->lam_u.as<double>();
    a.z64 = ctx->z64.as<double>();
    a.z32 = ctx->z32.as<float>();
    a.lp = ctx->lp.as<LamParams>();
    a.lx = ctx->lx.as<ExactLam>();
    a.hist = ctx->hist.as<unsigned long long>();
    a.S1 = ctx->S1.as<unsigned long long>();
    a.S2 = ctx->S2.as<unsigned long long>();
    a.acc = ctx->acc.as<DesignAcc>();
    a.tiles_done = ctx->tiles.as<unsigned int>();
    a.out = ctx->out.as<DesignOut>();
    a.ctl = ctx->ctl.as<Control>();
    a.queue = ctx->queue.as<QEntry>();
    a.qcap = ctx->qcap;
    a.ray_tile = ctx->ray_tile;
    a.mode = mode;
    if (mode == CPD_TRACE_FP32) {
        a.guards = Guards{0.f, 0.f, 0.f, 0.f};
        a.yguard_rel = 0.0;
    } else {
        a.guards = default_guards();
        a.yguard_rel = kYGuardRel;
    }
    a.p_out = p_out_host ? ctx->pout.as<double>() : nullptr;
    a.logtab = ctx->logtab.as<float>();

    // The device work of a pass, captured once per signature and replayed.
    std::vector<uint8_t> key(sizeof(a) + 3 * sizeof(uint32_t));
    std::memcpy(key.data(), &a, sizeof(a));
    uint32_t extra[3] = {n, ctx->warps_per_cta, (uint32_t)ctx->num_sms};
    std::memcpy(key.data() + sizeof(a), extra, sizeof(extra));
    auto record = [&](cudaStream_t st) -> int {
        int l = 0;
        cudaMemsetAsync(ctx->ctl.p, 0, sizeof(Control), st);
        cudaMemsetAsync(ctx->tiles.p, 0, sizeof(unsigned int) * n, st);
        l = launch_pass(a, ctx->num_sms, ctx->warps_per_cta, st, ctx->profiling ? ctx->kev : nullptr);
        cudaMemcpyAsync(ctx->h_out.p, ctx->out.p, sizeof(DesignOut) * n, cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(ctx->h_ctl.p, ctx->ctl.p, sizeof(Control), cudaMemcpyDeviceToHost, st);
        return l;
    };
    CPD_TRY(cudaEventRecord(ctx->ev0, s));
    int launches = 0;
    if (ctx->use_graphs && !ctx->profiling) {
        if (!ctx->graph_exec || key != ctx->graph_key) {
            if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
            ctx->graph_exec = nullptr;
            cudaGraph_t g = nullptr;
            CPD_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
            ctx->graph_launches = record(s);
            CPD_TRY(cudaStreamEndCapture(s, &g));
            cudaError_t e = cudaGraphInstantiate(&ctx->graph_exec, g, 0);
            cudaGraphDestroy(g);
            CPD_TRY(e);
            ctx->graph_key = key;
        }
        CPD_TRY(cudaGraphLaunch(ctx->graph_exec, s));
        launches = ctx->graph_launches;
    } else {
        launches = record(s);
        CPD_TRY(cudaGetLastError());
    }
    CPD_TRY(cudaEventRecord(ctx->ev1, s));
    if (p_out_host)
        CPD_TRY(cudaMemcpyAsync(p_out_host, ctx->pout.p, sizeof(double) * hist, cudaMemcpyDeviceToHost, s));
    CPD_TRY(cudaStreamSynchronize(s));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    ctx->last_ms = ms;
    ctx->last_launches = (uint32_t)launches;
    if (ctx->profiling)
        for (int i = 0; i < 4; i++) {
            float km = 0.f;
            cudaEventElapsedTime(&km, ctx->kev[i], ctx->kev[i + 1]);
            ctx->kernel_ms[i] = km;
        }
    const Control *c = ctx->h_ctl.as<Control>();
    res.overflow = c->overflow != 0 || c->queue_count > ctx->qcap;
    if (res.overflow) ctx->hist_dirty = true;
    res.outs.assign(ctx->h_out.as<DesignOut>(), ctx->h_out.as<DesignOut>() + n);
    return CPD_OK;
}

void fill_fitness(const cpd_design &d, const DesignOut &o, uint64_t rays, cpd_fitness &f, bool need_conv)
{
    std::memset(&f, 0, sizeof(f));
    f.size = d.size;
    f.deviation = d.deviation;
    f.info = o.info;
    f.h_cond = o.h_cond;
    f.h_det = o.h_det;
    f.max_sem = o.max_sem;
    f.rays = rays;
    f.hits = o.hits;
    f.retraced = o.retraced;
    f.fast_rays = o.fast;
    f.wavelengths = (uint32_t)o.rows;
    f.status = (need_conv && !o.converged) ? CPD_NOT_CONVERGED : CPD_OK;
}

bool valid_design(const cpd_design *d)
{
    return d && d->nglass >= 1 && d->nglass <= CPD_MAX_GLASS && d->bin_count >= 1 && d->bin_count <= CPD_MAX_BINS;
}

// Runs one pass, growing the re-trace queue and re-running the pass if it overflowed.
// A pass that overflowed leaves the persistent accumulators untouched (the entropy
// kernel skips such a pass), so the re-run is exact.
int run_pass_checked(cpd_context *ctx, const std::vector<PassDesign> &ds, uint32_t mode, bool fresh,
                     double *p_out, PassResult &res)
{
    for (int attempt = 0; attempt < 6; attempt++) {
        int e = run_pass(ctx, ds, mode, fresh, p_out, res);
        if (e) {
            ctx->hist_dirty = true;
            return e;
        }
        if (!res.overflow) return CPD_OK;
        ctx->qcap *= 4;
    }
    return CPD_NO_CAPACITY;
}

}  // namespace

extern "C" {

int cpd_context_create(int device, cpd_context **out)
{
    if (!out) return CPD_INVALID_ARGUMENT;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return CPD_CUDA_ERROR;
    cpd_context *ctx = new cpd_context();
    ctx->device = device;
    if (cudaSetDevice(device) != cudaSuccess) {
        delete ctx;
        return CPD_CUDA_ERROR;
    }
    cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&ctx->ev0) != cudaSuccess || cudaEventCreate(&ctx->ev1) != cudaSuccess) {
        delete ctx;
        return CPD_CUDA_ERROR;
    }
    for (int i = 0; i < 5; i++)
        if (cudaEventCreate(&ctx->kev[i]) != cudaSuccess) {
            delete ctx;
            return CPD_CUDA_ERROR;
        }
    {
        std::vector<float> tab(4 * ff::kLogTable);
        ff::make_log_table(tab.data());
        if (ctx->logtab.ensure(sizeof(float) * tab.size()) != cudaSuccess ||
            cudaMemcpy(ctx->logtab.p, tab.data(), sizeof(float) * tab.size(), cudaMemcpyHostToDevice) !=
                cudaSuccess) {
            delete ctx;
            return CPD_CUDA_ERROR;
        }
    }
    *out = ctx;
    return CPD_OK;
}

void cpd_context_destroy(cpd_context *ctx)
{
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
    for (DevBuf *b : {&ctx->designs, &ctx->jobs, &ctx->lam_u, &ctx->z64, &ctx->z32, &ctx->lp, &ctx->lx, &ctx->hist, &ctx->S1,
                      &ctx->S2, &ctx->acc, &ctx->tiles, &ctx->out, &ctx->ctl, &ctx->queue, &ctx->pout,
                      &ctx->pair_lam, &ctx->pair_z, &ctx->pair_bins, &ctx->pair_ts, &ctx->pair_flags, &ctx->peak,
                      &ctx->logtab})
        b->release();
    for (HostBuf *b : {&ctx->h_designs, &ctx->h_jobs, &ctx->h_lam, &ctx->h_z64, &ctx->h_z32, &ctx->h_out, &ctx->h_ctl,
                       &ctx->h_pout, &ctx->h_pairs})
        b->release();
    cudaEventDestroy(ctx->ev0);
    cudaEventDestroy(ctx->ev1);
    for (int i = 0; i < 5; i++) cudaEventDestroy(ctx->kev[i]);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
}

int cpd_set_launch_shape(cpd_context *ctx, uint32_t ray_tile, uint32_t warps_per_cta)
{
    if (!ctx) return CPD_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (ray_tile) ctx->ray_tile = std::min<uint32_t>(ray_tile, CPD_MAX_RAYS);
    if (warps_per_cta) {
        if (warps_per_cta > 8) return CPD_INVALID_ARGUMENT;
        ctx->warps_per_cta = warps_per_cta;
    }
    return CPD_OK;
}

int cpd_get_launch_shape(cpd_context *ctx, uint32_t *ray_tile, uint32_t *warps_per_cta)
{
    if (!ctx) return CPD_INVALID_ARGUMENT;
    if (ray_tile) *ray_tile = ctx->ray_tile;
    if (warps_per_cta) *warps_per_cta = ctx->warps_per_cta;
    return CPD_OK;
}

int cpd_last_timing(cpd_context *ctx, double *kernel_ms, uint32_t *launches)
{
    if (!ctx) return CPD_INVALID_ARGUMENT;
    if (kernel_ms) *kernel_ms = ctx->last_ms;
    if (launches) *launches = ctx->last_launches;
    return CPD_OK;
}

int cpd_set_profiling(cpd_context *ctx, int on)
{
    if (!ctx) return CPD_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->profiling = on != 0;
    return CPD_OK;
}

int cpd_last_transfer_bytes(cpd_context *ctx, uint64_t *h2d, uint64_t *d2h)
{
    if (!ctx) return CPD_INVALID_ARGUMENT;
    if (h2d) *h2d = ctx->last_h2d;
    if (d2h) *d2h = ctx->last_d2h;
    return CPD_OK;
}

int cpd_last_kernel_times(cpd_context *ctx, double ms[4])
{
    if (!ctx || !ms) return CPD_INVALID_ARGUMENT;
    for (int i = 0; i < 4; i++) ms[i] = ctx->kernel_ms[i];
    return CPD_OK;
}

int cpd_fitness_gpu_points(cpd_context *ctx, const cpd_design *d, const double *lam_u, uint32_t W,
                           const double *ray_u, uint32_t R, uint32_t trace_mode, cpd_fitness *out, double *p_out)
{
    if (!ctx || !valid_design(d) || !lam_u || !ray_u || !out) return CPD_INVALID_ARGUMENT;
    if (W == 0 || W > CPD_MAX_WAVELENGTHS || R == 0 || R > CPD_MAX_RAYS || trace_mode > CPD_TRACE_FP64)
        return CPD_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (cudaSetDevice(ctx->device) != cudaSuccess) return CPD_CUDA_ERROR;
    ctx->last_h2d = ctx->last_d2h = 0;
    DevDesign D;
    design_to_dev(*d, D);
    RayTable rt;
    ray_table(ray_u, R, rt.z64, rt.z32);
    std::vector<PassDesign> ds{PassDesign{&D, W, R, lam_u, &rt}};
    PassResult res;
    int e = run_pass_checked(ctx, ds, trace_mode, true, p_out, res);
    if (e) return e;
    fill_fitness(*d, res.outs[0], (uint64_t)W * R, *out, false);
    return CPD_OK;
}

int cpd_fitness_gpu(cpd_context *ctx, const cpd_design *d, const double *seeds, uint32_t nseeds, uint32_t max_n,
                    uint32_t nwarp, uint32_t max_eval, cpd_fitness *out)
{
    if (!ctx || !valid_design(d) || !seeds || !out || nseeds == 0) return CPD_INVALID_ARGUMENT;
    if (max_n == 0 || max_eval == 0 || max_eval > CPD_MAX_RAYS) return CPD_INVALID_ARGUMENT;
    if ((uint64_t)max_n * nseeds > CPD_MAX_WAVELENGTHS) return CPD_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (cudaSetDevice(ctx->device) != cudaSuccess) return CPD_CUDA_ERROR;
    ctx->last_h2d = ctx->last_d2h = 0;
    if (nwarp >= 1 && nwarp <= 8) ctx->warps_per_cta = nwarp;
    DevDesign D;
    design_to_dev(*d, D);
    std::vector<double> lam(max_n);
    PassResult res;
    uint64_t rays = 0;
    for (uint32_t s = 0; s < nseeds; s++) {
        seed_points(seeds[s], 0, max_n, lam.data());
        const RayTable &rt = ray_table_cached(ctx, seeds[s], max_eval);
        std::vector<PassDesign> ds{PassDesign{&D, max_n, max_eval, lam.data(), &rt}};
        int e = run_pass_checked(ctx, ds, CPD_TRACE_HYBRID, s == 0, nullptr, res);
        if (e) return e;
        rays += (uint64_t)max_n * max_eval;
        if (res.outs[0].converged) break;
    }
    fill_fitness(*d, res.outs[0], rays, *out, true);
    return out->status;
}

int cpd_fitness_gpu_batch(cpd_context *ctx, const cpd_design *designs, const cpd_batch_item *items, uint32_t n,
                          uint32_t trace_mode, cpd_fitness *outs)
{
    if (!ctx || !designs || !items || !outs || n == 0 || trace_mode > CPD_TRACE_FP64) return CPD_INVALID_ARGUMENT;
    for (uint32_t i = 0; i < n; i++) {
        if (!valid_design(&designs[i])) return CPD_INVALID_ARGUMENT;
        if (items[i].max_n == 0 || items[i].max_n > CPD_MAX_WAVELENGTHS || items[i].max_eval == 0 ||
            items[i].max_eval > CPD_MAX_RAYS)
            return CPD_INVALID_ARGUMENT;
    }
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (cudaSetDevice(ctx->device) != cudaSuccess) return CPD_CUDA_ERROR;
    ctx->last_h2d = ctx->last_d2h = 0;
    std::vector<DevDesign> devs(n);
    std::vector<std::vector<double>> lams(n);
    std::vector<PassDesign> ds(n);
    for (uint32_t i = 0; i < n; i++) {
        design_to_dev(designs[i], devs[i]);
        lams[i].resize(items[i].max_n);
        seed_points(items[i].seed, 0, items[i].max_n, lams[i].data());
    }
    for (uint32_t i = 0; i < n; i++) {
        const RayTable &rt = ray_table_cached(ctx, items[i].seed, items[i].max_eval);
        ds[i] = PassDesign{&devs[i], items[i].max_n, items[i].max_eval, lams[i].data(), &rt};
    }
    PassResult res;
    int e = run_pass_checked(ctx, ds, trace_mode, true, nullptr, res);
    if (e) return e;
    for (uint32_t i = 0; i < n; i++)
        fill_fitness(designs[i], res.outs[i], (uint64_t)items[i].max_n * items[i].max_eval, outs[i], true);
    return CPD_OK;
}

int cpd_transmission_probability(cpd_context *ctx, const cpd_design *d, const double *wavelengths, uint32_t n,
                                 uint32_t max_m, double *out)
{
    if (!ctx || !valid_design(d) || !wavelengths || !out || n == 0 || n > CPD_MAX_WAVELENGTHS || max_m == 0 ||
        max_m > CPD_MAX_RAYS)
        return CPD_INVALID_ARGUMENT;
    // explicit wavelengths: bounds (0, 1) make wmin + (wmax - wmin)*u == u exactly
    cpd_design dd = *d;
    dd.wavelength_bounds[0] = 0.0;
    dd.wavelength_bounds[1] = 1.0;
    std::vector<double> ray_u(max_m);
    double st = 0.5;  // the reference CPU ray points (fitness.rs:19)
    for (uint32_t j = 0; j < max_m; j++) {
        st = st + kAlpha;
        st = st - std::trunc(st);
        ray_u[j] = st;
    }
    cpd_fitness f;
    return cpd_fitness_gpu_points(ctx, &dd, wavelengths, n, ray_u.data(), max_m, CPD_TRACE_HYBRID, &f, out);
}

int cpd_trace_rays(cpd_context *ctx, const cpd_design *d, const double *lam_u, const double *ray_u, uint32_t n,
                   uint32_t trace_mode, uint32_t *bins, double *ts, uint8_t *flags)
{
    if (!ctx || !valid_design(d) || !lam_u || !ray_u || !bins || !ts || trace_mode > CPD_TRACE_FP64)
        return CPD_INVALID_ARGUMENT;
    if (n == 0) return CPD_OK;
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (cudaSetDevice(ctx->device) != cudaSuccess) return CPD_CUDA_ERROR;
    ctx->last_h2d = ctx->last_d2h = 0;
    DevDesign D;
    design_to_dev(*d, D);
    std::vector<double> z(n);
    for (uint32_t i = 0; i < n; i++) z[i] = norminv(ray_u[i]);
    cudaStream_t s = ctx->stream;
    CPD_TRY(ctx->designs.ensure(sizeof(DevDesign)));
    CPD_TRY(ctx->pair_lam.ensure(sizeof(double) * n));
    CPD_TRY(ctx->pair_z.ensure(sizeof(double) * n));
    CPD_TRY(ctx->pair_bins.ensure(sizeof(uint32_t) * n));
    CPD_TRY(ctx->pair_ts.ensure(sizeof(double) * n));
    CPD_TRY(ctx->pair_flags.ensure(n));
    CPD_TRY(cudaMemcpyAsync(ctx->designs.p, &D, sizeof(DevDesign), cudaMemcpyHostToDevice, s));
    CPD_TRY(cudaMemcpyAsync(ctx->pair_lam.p, lam_u, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    CPD_TRY(cudaMemcpyAsync(ctx->pair_z.p, z.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s));
    CPD_TRY(cudaEventRecord(ctx->ev0, s));
    launch_trace_pairs(ctx->designs.as<DevDesign>(), ctx->pair_lam.as<double>(), ctx->pair_z.as<double>(), n,
                       trace_mode, ctx->pair_bins.as<uint32_t>(), ctx->pair_ts.as<double>(),
                       ctx->pair_flags.as<uint8_t>(), s);
    CPD_TRY(cudaGetLastError());
    CPD_TRY(cudaEventRecord(ctx->ev1, s));
    CPD_TRY(cudaMemcpyAsync(bins, ctx->pair_bins.p, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, s));
    CPD_TRY(cudaMemcpyAsync(ts, ctx->pair_ts.p, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    if (flags) CPD_TRY(cudaMemcpyAsync(flags, ctx->pair_flags.p, n, cudaMemcpyDeviceToHost, s));
    CPD_TRY(cudaStreamSynchronize(s));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    ctx->last_ms = ms;
    ctx->last_launches = 1;
    return CPD_OK;
}

int cpd_measure_fp32_peak(cpd_context *ctx, uint32_t iters, double *tflops)
{
    if (!ctx || !tflops || iters == 0) return CPD_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (cudaSetDevice(ctx->device) != cudaSuccess) return CPD_CUDA_ERROR;
    ctx->last_h2d = ctx->last_d2h = 0;
    const int threads = 256;
    const int blocks = ctx->num_sms * 8;
    CPD_TRY(ctx->peak.ensure(sizeof(float) * blocks));
    cudaStream_t s = ctx->stream;
    launch_fma_peak(ctx->peak.as<float>(), 16, blocks, threads, s);  // warm-up
    CPD_TRY(cudaEventRecord(ctx->ev0, s));
    launch_fma_peak(ctx->peak.as<float>(), iters, blocks, threads, s);
    CPD_TRY(cudaEventRecord(ctx->ev1, s));
    CPD_TRY(cudaStreamSynchronize(s));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    const double flops = 2.0 * 8.0 * 16.0 * (double)iters * threads * (double)blocks;
    *tflops = flops / (ms * 1e-3) / 1e12;
    ctx->last_ms = ms;
    ctx->last_launches = 2;
    return CPD_OK;
}

}  // extern "C"
