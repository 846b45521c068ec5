// cpd_runtime.cu -- the GPU side of the C ABI: contexts, per-pass slots (stream,
// pooled device buffers, pinned staging, captured CUDA graph), the ray-table cache,
// the synchronous entry points and the continuous-batching server.
#include <cuda_runtime.h>

#include <algorithm>
#include <iterator>
#include <array>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
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
    void *dev = nullptr;  // the device's address of a mapped buffer
    size_t cap = 0;
    // mapped: the GPU reads and writes the buffer in place (over NVLink-C2C on this
    // machine), so a kernel can deliver results without a copy
    cudaError_t ensure(size_t bytes, bool mapped = false)
    {
        if (bytes <= cap) return cudaSuccess;
        if (p) cudaFreeHost(p);
        p = dev = nullptr;
        cap = 0;
        size_t want = std::max<size_t>(bytes, 256);
        want = want + want / 4;
        cudaError_t e = cudaHostAlloc(&p, want, mapped ? cudaHostAllocMapped : cudaHostAllocDefault);
        if (e == cudaSuccess && mapped) e = cudaHostGetDevicePointer(&dev, p, 0);
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

// The sampling flags a trace mode may carry.
constexpr uint32_t kSamplingBits = CPD_SAMPLING_ADAPTIVE | CPD_SAMPLING_EXACT;
// Most rows of a pass whose trace takes equal shares of span slots: every warp scans the
// blocks' spans (32 per step) to find its share.
constexpr uint64_t kBalancedMaxRows = 16384;

// The kernel node of `fn` in a captured graph (nullptr if none).
cudaGraphNode_t find_kernel_node(cudaGraph_t g, const void *fn)
{
    size_t n = 0;
    if (cudaGraphGetNodes(g, nullptr, &n) != cudaSuccess || n == 0) return nullptr;
    std::vector<cudaGraphNode_t> nodes(n);
    if (cudaGraphGetNodes(g, nodes.data(), &n) != cudaSuccess) return nullptr;
    for (cudaGraphNode_t nd : nodes) {
        cudaGraphNodeType t;
        if (cudaGraphNodeGetType(nd, &t) != cudaSuccess || t != cudaGraphNodeTypeKernel) continue;
        cudaKernelNodeParams kp{};
        if (cudaGraphKernelNodeGetParams(nd, &kp) == cudaSuccess && kp.func == fn) return nd;
    }
    return nullptr;
}

// Everything one pass needs on the device, plus its staging and its captured graph.
// A context owns one slot (the synchronous calls); a server owns several, so that
// passes overlap on the device.
struct PassSlot {
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, done = nullptr;
    cudaEvent_t kev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    // inputs (tables, designs, jobs) in one arena, uploaded with one copy; results
    // (DesignOut[n] then HostStatus) written by the kernels into mapped host memory;
    // `in` ends with the device-side Control words
    DevBuf in, lp, lx, hist, S1, S2, acc, queue, pout;
    HostBuf h_in, h_outs;
    size_t ctl_off = 0;
    bool hist_dirty = true;
    uint32_t qcap = 1u << 18;
    // Captured passes, most recently used first: a caller that alternates between a few
    // launch signatures (designs of different detector sizes, say) replays each one's
    // graph instead of capturing anew. The key holds every pointer and size the graph
    // bakes in, plus buf_gen, which changes whenever a buffer of the slot is reallocated.
    struct CachedGraph {
        std::vector<uint8_t> key;
        cudaGraphExec_t exec;
        int launches;
        // a single-design pass: the captured graph (kept: its node handle addresses the
        // exec's node), the trace node, and the launch arguments it holds, whose design
        // constants (fc, fl) change from call to call while the key stays the same
        cudaGraph_t graph = nullptr;
        cudaGraphNode_t trace_node = nullptr;
        LaunchArgs args{};
    };
    std::vector<CachedGraph> graphs;
    static constexpr size_t kGraphCache = 8;
    uint64_t buf_gen = 0;
    // The wavelength-point and ray tables (the arena after the designs and jobs) of the
    // last pass, when they came from the context's caches: identity of each table in
    // upload order, and references that keep those tables (and so their addresses)
    // alive. A pass with the same key leaves them in place and uploads the designs and
    // jobs only.
    std::vector<const void *> tables_key;
    std::vector<std::shared_ptr<const void>> tables_refs;
    // the pass in flight / last finished
    uint32_t n = 0;
    uint64_t hist_cells = 0;
    double *p_out_host = nullptr;
    bool profiled = false;
    int launches = 0;
    double last_ms = 0.0;
    uint64_t h2d = 0, d2h = 0;
    double kernel_ms[4] = {0, 0, 0, 0};

    cudaError_t create()
    {
        cudaError_t e = cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreate(&ev0);
        if (e == cudaSuccess) e = cudaEventCreate(&ev1);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&done, cudaEventDisableTiming);
        for (int i = 0; i < 5 && e == cudaSuccess; i++) e = cudaEventCreate(&kev[i]);
        return e;
    }
    void destroy()
    {
        if (stream) cudaStreamSynchronize(stream);
        for (CachedGraph &c : graphs) {
            cudaGraphExecDestroy(c.exec);
            if (c.graph) cudaGraphDestroy(c.graph);
        }
        graphs.clear();
        for (DevBuf *b : {&in, &lp, &lx, &hist, &S1, &S2, &acc, &queue, &pout}) b->release();
        for (HostBuf *b : {&h_in, &h_outs}) b->release();
        for (cudaEvent_t *ev : {&ev0, &ev1, &done, &kev[0], &kev[1], &kev[2], &kev[3], &kev[4]})
            if (*ev) cudaEventDestroy(*ev), *ev = nullptr;
        if (stream) cudaStreamDestroy(stream);
        stream = nullptr;
    }
};

}  // namespace
}  // namespace cpd

using namespace cpd;

struct cpd_context {
    int device = 0;
    int num_sms = 0;
    std::mutex mu;        // serialises the synchronous entry points (main slot)
    std::mutex cache_mu;  // ray-table cache
    PassSlot main;
    DevBuf pair_design, pair_lam, pair_z, pair_bins, pair_ts, pair_flags, peak, logtab;
    DevBuf bld_params, bld_out, bld_status;  // cpd_design_build_device
    // cpd_transmission_probability: the design, the wavelengths, the ray table of the
    // reference's ray points (kept while max_m stays the same), the results
    DevBuf tp_design, tp_lam, tp_z, tp_out, tp_rays;
    uint32_t tp_m = 0;
    uint32_t ray_tile = 32;
    uint32_t warps_per_cta = 8;
    bool profiling = false;
    bool use_graphs = true;
    bool autotune = false;
    std::map<RayKey, RayTablePtr> ray_cache;
    std::map<RayKey, std::shared_ptr<const std::vector<double>>> lam_cache;  // wavelength u-points per (seed, W)
    // launch shape picked by the autotuner per class of batch
    std::map<std::array<uint64_t, 5>, std::pair<uint32_t, uint32_t>> tune_cache;
};

namespace {

#define CPD_TRY(expr)                                 \
    do {                                              \
        cudaError_t _e = (expr);                      \
        if (_e != cudaSuccess) return CPD_CUDA_ERROR; \
    } while (0)

RayTablePtr ray_table_cached(cpd_context *ctx, double seed, uint32_t R)
{
    uint64_t bits;
    std::memcpy(&bits, &seed, 8);
    RayKey key{bits, R};
    {
        std::lock_guard<std::mutex> lk(ctx->cache_mu);
        auto it = ctx->ray_cache.find(key);
        if (it != ctx->ray_cache.end()) return it->second;
    }
    std::vector<double> u(R);
    seed_points(seed, 1, R, u.data());
    auto t = std::make_shared<RayTable>();
    ray_table(u.data(), R, t->z64, t->z32, &t->rank);
    std::lock_guard<std::mutex> lk(ctx->cache_mu);
    if (ctx->ray_cache.size() > 256) ctx->ray_cache.clear();
    return ctx->ray_cache.emplace(key, t).first->second;
}

// The wavelength u-points of the GPU seed policy, u_i = fract(fma(i, 1/phi, seed)),
// cached per seed like the ray tables (an optimizer reuses its seeds). The points of W
// wavelengths are the first W of any longer table of the same seed, so one table of
// max(1024, W rounded up to a power of two) points serves every W up to its length:
// the designs of a batch with mixed W share a few tables.
LamPtr lam_points_cached(cpd_context *ctx, double seed, uint32_t W)
{
    uint64_t bits;
    std::memcpy(&bits, &seed, 8);
    uint32_t L = 1024;
    while (L < W) L <<= 1;
    W = L;
    RayKey key{bits, W};
    {
        std::lock_guard<std::mutex> lk(ctx->cache_mu);
        auto it = ctx->lam_cache.find(key);
        if (it != ctx->lam_cache.end()) return it->second;
    }
    auto v = std::make_shared<std::vector<double>>(W);
    seed_points(seed, 0, W, v->data());
    std::lock_guard<std::mutex> lk(ctx->cache_mu);
    if (ctx->lam_cache.size() > 256) ctx->lam_cache.clear();
    return ctx->lam_cache.emplace(key, v).first->second;
}

// One design's sampling inputs for a pass. lam_keep / rays_keep: set when lam_u / rays are
// immutable tables of the context's caches (their device copies may then stay resident).
struct PassDesign {
    const DevDesign *dev;      // host copy
    uint32_t W, R;
    const double *lam_u;       // W wavelength u-points (host), the first W of lam_len
    const RayTable *rays;
    std::shared_ptr<const void> lam_keep = nullptr, rays_keep = nullptr;
    uint32_t lam_len = 0;      // length of the lam_u table (0: W)
    // set instead of dev: the design is built on the device from this record (detector
    // positioned first when acceptance > 0; the same acceptance for every design of a pass)
    const cpd_spectrometer_params *params = nullptr;
    double acceptance = 0.0;
};

struct PassResult {
    std::vector<DesignOut> outs;
    bool overflow = false;
};

uint32_t tile_rows_for(uint32_t B, uint32_t n)
{
    return std::max<uint32_t>(1u, (n > 1 ? kTileCellsBatch : kTileCells) / B);
}

// Device bytes one design occupies in a pass (histogram, per-row tables, ray tables):
// the admission unit of the server.
uint64_t design_bytes(uint32_t W, uint32_t R, uint32_t B)
{
    return (uint64_t)W * (8ull * B + sizeof(LamParams) + sizeof(LamDF) + 8) + 16ull * R + 16ull * B +
           sizeof(DevDesign) + sizeof(DesignJob) + sizeof(DesignAcc) + sizeof(DesignOut);
}

// Plans, stages and issues one pass on slot `s` (asynchronously; `s.done` is recorded
// at the end). Accumulators are zeroed when `fresh`; they persist otherwise (the seeds
// of one call).
int pass_issue(cpd_context *ctx, PassSlot &S, const std::vector<PassDesign> &ds, uint32_t mode, bool fresh,
               double *p_out_host, bool use_graph, bool profile)
{
    const uint32_t n = (uint32_t)ds.size();
    const bool adaptive = (mode & CPD_SAMPLING_ADAPTIVE) != 0u;
    const bool all_exact = adaptive && (mode & CPD_SAMPLING_EXACT) != 0u;
    const bool on_device = n > 0 && ds[0].params != nullptr;  // every design of the pass, or none
    mode &= ~kSamplingBits;
    std::vector<DesignJob> jobs(n);
    std::vector<uint8_t> owns_rays(n, 1);  // designs that share a ray table share its copy
    std::vector<uint8_t> owns_lam(n, 1);   // likewise for wavelength-point tables
    std::map<const RayTable *, std::pair<uint64_t, uint64_t>> ray_offs;
    std::map<std::pair<const double *, uint32_t>, uint64_t> lam_offs;
    // identity of the tables in upload order (null entries: not from a cache)
    std::vector<const void *> tables_key;
    bool cacheable = true;
    uint64_t rows = 0, hist = 0, lam = 0, ray = 0, rnk = 0, accc = 0, items = 0, tiles = 0;
    uint32_t max_B = 0;
    for (uint32_t i = 0; i < n; i++) {
        const PassDesign &p = ds[i];
        DesignJob &J = jobs[i];
        std::memset(&J, 0, sizeof(J));
        J.W = p.W;
        J.R = p.R;
        J.Rz = (uint32_t)p.rays->z64.size();
        J.B = on_device ? p.params->bin_count : p.dev->B;
        J.row_off = rows;
        J.hist_off = hist;
        const uint32_t lam_len = std::max(p.lam_len, p.W);
        auto lo = lam_offs.emplace(std::make_pair(p.lam_u, lam_len), lam);
        J.lam_off = lo.first->second;
        owns_lam[i] = lo.second;
        if (owns_lam[i]) {
            lam += lam_len;
            tables_key.push_back(p.lam_u);
            cacheable = cacheable && p.lam_keep;
        }
        auto ro = ray_offs.emplace(p.rays, std::make_pair(ray, rnk));
        J.ray_off = ro.first->second.first;
        J.rank_off = ro.first->second.second;
        owns_rays[i] = ro.second;
        if (owns_rays[i]) {
            tables_key.push_back(p.rays);
            cacheable = cacheable && p.rays_keep;
        }
        max_B = std::max(max_B, J.B);
        J.acc_off = accc;
        J.item_off = items;
        J.tile_off = tiles;
        J.nchunk = std::max<uint32_t>(1u, (J.Rz + ctx->ray_tile - 1) / ctx->ray_tile);
        J.tile_rows = tile_rows_for(J.B, n);
        J.ntiles = (J.W + J.tile_rows - 1) / J.tile_rows;
        ff::split(kTScaleInv / (double)J.R, J.unit_hi, J.unit_lo);
        ff::split(-31.0 - std::log2((double)J.R), J.lu_hi, J.lu_lo);
        J.pscale = kTScaleInv / (double)J.R;
        rows += J.W;
        hist += (uint64_t)J.W * J.B;
        if (owns_rays[i]) {
            ray += (J.Rz + 1u) & ~1u;  // even: every table starts 16-byte aligned
            if (adaptive) rnk += J.R;
        }
        accc += J.B;
        items += (uint64_t)((J.W + 31) / 32) * J.nchunk;
        tiles += J.ntiles;
    }
    // one input arena: wavelength points | z64 | z32 | ranks | designs | jobs (256-byte
    // sections; the ranks only under adaptive sampling). The tables come first, so their
    // offsets depend on the tables alone and a pass that finds them resident uploads the
    // tail from the designs on.
    auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
    const size_t o_lam = 0;
    const size_t o_z64 = o_lam + al(sizeof(double) * lam);
    const size_t o_z32 = o_z64 + al(sizeof(double) * ray);
    const size_t o_rank = o_z32 + al(2 * sizeof(float) * ray);
    const size_t o_des = o_rank + al(sizeof(uint32_t) * rnk);
    const size_t o_job = o_des + al(sizeof(DevDesign) * n);
    const size_t o_par = o_job + al(sizeof(DesignJob) * n);  // parameter records (device builds)
    // the pass's Control words close the arena: uploaded as zeros with the inputs (one copy
    // node instead of a copy and a memset ahead of the first kernel)
    const size_t o_ctl = o_par + (on_device ? al(sizeof(cpd_spectrometer_params) * n) : 0);
    const size_t in_bytes = o_ctl + sizeof(Control);
    const size_t ctl_off = al(sizeof(DesignOut) * n);
    const size_t out_bytes = ctl_off + sizeof(HostStatus);
    CPD_TRY(S.h_in.ensure(in_bytes));
    CPD_TRY(S.h_outs.ensure(out_bytes, true));
    const void *in_before = S.in.p;
    CPD_TRY(S.in.ensure(in_bytes));
    // the tables already on the device from the previous pass of this slot
    tables_key.push_back(adaptive ? &kSamplingBits : nullptr);  // the rank section
    tables_key.push_back(S.in.p);
    const bool resident = cacheable && S.in.p == in_before && tables_key == S.tables_key;
    // a device build writes the design records itself: they are not uploaded
    const size_t up_off = resident ? (on_device ? o_job : o_des) : 0, up_bytes = in_bytes - up_off;
    char *hin = S.h_in.as<char>();
    std::memset(hin + o_ctl, 0, sizeof(Control));
    for (uint32_t i = 0; i < n; i++) {
        if (on_device) reinterpret_cast<cpd_spectrometer_params *>(hin + o_par)[i] = *ds[i].params;
        else reinterpret_cast<DevDesign *>(hin + o_des)[i] = *ds[i].dev;
        reinterpret_cast<DesignJob *>(hin + o_job)[i] = jobs[i];
        if (resident) continue;
        if (owns_lam[i])
            std::memcpy(reinterpret_cast<double *>(hin + o_lam) + jobs[i].lam_off, ds[i].lam_u,
                        sizeof(double) * std::max(ds[i].lam_len, ds[i].W));
        if (!owns_rays[i]) continue;
        std::memcpy(reinterpret_cast<double *>(hin + o_z64) + jobs[i].ray_off, ds[i].rays->z64.data(),
                    sizeof(double) * jobs[i].Rz);
        std::memcpy(reinterpret_cast<float *>(hin + o_z32) + 2 * jobs[i].ray_off, ds[i].rays->z32.data(),
                    2 * sizeof(float) * jobs[i].Rz);
        if (adaptive)
            std::memcpy(reinterpret_cast<uint32_t *>(hin + o_rank) + jobs[i].rank_off, ds[i].rays->rank.data(),
                        sizeof(uint32_t) * jobs[i].R);
    }
    if (cacheable) {
        S.tables_key = tables_key;
        S.tables_refs.clear();
        for (const PassDesign &p : ds) {
            S.tables_refs.push_back(p.lam_keep);
            S.tables_refs.push_back(p.rays_keep);
        }
    } else {
        S.tables_key.clear();
        S.tables_refs.clear();
    }
    // device buffers (a reallocation retires the captured graphs that hold the old addresses)
    const void *bufs_before[] = {S.lp.p, S.lx.p, S.hist.p, S.S1.p, S.S2.p, S.acc.p, S.queue.p, S.h_in.p, S.h_outs.p, in_before};
    const size_t hist_bytes = sizeof(unsigned long long) * std::max<uint64_t>(hist, 1);
    const size_t old_hist = S.hist.cap;
    // the LamParams, then (single-design passes) one span per 32-row block
    CPD_TRY(S.lp.ensure(sizeof(LamParams) * std::max<uint64_t>(rows, 1) + sizeof(uint2) * ((rows + 31) / 32)));
    CPD_TRY(S.lx.ensure(sizeof(LamDF) * std::max<uint64_t>(rows, 1)));
    CPD_TRY(S.hist.ensure(hist_bytes));
    if (S.hist.cap != old_hist) S.hist_dirty = true;
    CPD_TRY(S.S1.ensure(sizeof(unsigned long long) * std::max<uint64_t>(accc, 1)));
    CPD_TRY(S.S2.ensure(sizeof(unsigned long long) * std::max<uint64_t>(accc, 1)));
    CPD_TRY(S.acc.ensure(sizeof(DesignAcc) * n));
    CPD_TRY(S.queue.ensure(sizeof(QEntry) * S.qcap));
    if (p_out_host) CPD_TRY(S.pout.ensure(hist_bytes));
    S.ctl_off = ctl_off;
    {
        const void *after[] = {S.lp.p, S.lx.p, S.hist.p, S.S1.p, S.S2.p, S.acc.p, S.queue.p, S.h_in.p, S.h_outs.p, S.in.p};
        if (!std::equal(std::begin(after), std::end(after), std::begin(bufs_before))) S.buf_gen++;
    }

    cudaStream_t s = S.stream;
    if (S.hist_dirty) {
        CPD_TRY(cudaMemsetAsync(S.hist.p, 0, S.hist.cap, s));
        S.hist_dirty = false;
    }
    S.h2d += up_bytes;
    S.d2h += out_bytes + (p_out_host ? sizeof(double) * hist : 0);
    char *din = S.in.as<char>();

    LaunchArgs a;
    std::memset(&a, 0, sizeof(a));
    a.designs = reinterpret_cast<const DevDesign *>(din + o_des);
    a.jobs = reinterpret_cast<const DesignJob *>(din + o_job);
    a.njobs = n;
    a.total_rows = rows;
    a.total_items = items;
    a.total_tiles = tiles;
    a.lam_u = reinterpret_cast<const double *>(din + o_lam);
    a.z64 = reinterpret_cast<const double *>(din + o_z64);
    a.z32 = reinterpret_cast<const float *>(din + o_z32);
    a.rank = adaptive ? reinterpret_cast<const uint32_t *>(din + o_rank) : nullptr;
    a.adaptive = adaptive ? (all_exact ? 2u : 1u) : 0u;
    a.max_B = max_B;
    a.lp = S.lp.as<LamParams>();
    a.lx = S.lx.as<LamDF>();
    a.hist = S.hist.as<unsigned long long>();
    a.S1 = S.S1.as<unsigned long long>();
    a.S2 = S.S2.as<unsigned long long>();
    a.acc = S.acc.as<DesignAcc>();
    a.out = reinterpret_cast<DesignOut *>(S.h_outs.dev);
    a.status = reinterpret_cast<HostStatus *>(reinterpret_cast<char *>(S.h_outs.dev) + ctl_off);
    a.ctl = reinterpret_cast<Control *>(din + o_ctl);
    a.clear_acc = fresh ? 1u : 0u;
    a.acc_cells = accc;
    a.queue = S.queue.as<QEntry>();
    a.qcap = S.qcap;
    a.ray_tile = ctx->ray_tile;
    for (uint32_t i = 0; i < n; i++)
        if (jobs[i].Rz <= kStageRays && jobs[i].Rz > a.stage_cap) a.stage_cap = jobs[i].Rz;
    a.mode = mode;
    if (mode == CPD_TRACE_FP32) {
        a.guards = no_guards();
        a.yguard_rel = 0.0;
    } else {
        a.guards = default_guards();
        a.yguard_rel = kYGuardRel;
    }
    // One host-built design with a fixed ray count: the trace splits its rays into equal
    // shares per warp (no work-item counter, no tail of unequal items) and reads the
    // design's constants as kernel parameters. The bound on rows x rays keeps each warp's
    // share arithmetic in range.
    if (n == 1 && !on_device && !adaptive && mode != CPD_TRACE_FP64 &&
        rows <= kBalancedMaxRows && rows * (uint64_t)jobs[0].Rz <= (1ull << 31)) {
        a.spans = reinterpret_cast<uint2 *>(S.lp.as<LamParams>() + rows);
        a.fc = ds[0].dev->fc;
        a.fl = fast_limits(a.fc, a.guards);
        a.one = jobs[0];
    }
    a.p_out = p_out_host ? S.pout.as<double>() : nullptr;
    a.logtab = ctx->logtab.as<float>();
    if (on_device) {
        a.params = reinterpret_cast<const cpd_spectrometer_params *>(din + o_par);
        a.build_acceptance = ds[0].acceptance;
    }

    // The device work of a pass, captured once per signature and replayed.
    // The whole pass -- input upload, accumulator clears, kernels, read-back, and the two
    // timing events around the kernels -- is one graph, captured once per signature.
    // The design constants of a single-design pass are not part of the key: the cached
    // graph's trace node gets them per call.
    std::vector<uint8_t> key(sizeof(a) + 8 * sizeof(uint64_t));
    {
        LaunchArgs ka = a;
        std::memset(&ka.fc, 0, sizeof(ka.fc));
        std::memset(&ka.fl, 0, sizeof(ka.fl));
        std::memcpy(key.data(), &ka, sizeof(ka));
    }
    const uint64_t extra[8] = {n, ctx->warps_per_cta, (uint64_t)ctx->num_sms, (in_bytes << 1) | (resident ? 1u : 0u),
                               out_bytes, fresh ? accc + 1 : 0, S.buf_gen, (uint64_t)(uintptr_t)S.h_in.p};
    std::memcpy(key.data() + sizeof(a), extra, sizeof(extra));
    auto record = [&](cudaStream_t st, bool capturing) -> int {
        const unsigned evf = capturing ? cudaEventRecordExternal : cudaEventRecordDefault;
        // the per-design accumulators are cleared by the setup kernel (clear_acc), the
        // Control words arrive zeroed with the inputs, and the results are written into
        // mapped host memory: one copy ahead of the kernels
        cudaMemcpyAsync(S.in.as<char>() + up_off, S.h_in.as<char>() + up_off, up_bytes, cudaMemcpyHostToDevice, st);
        // External: under stream capture these become event-record nodes of the graph
        cudaEventRecordWithFlags(S.ev0, st, evf);
        const int l = launch_pass(a, ctx->num_sms, ctx->warps_per_cta, st, profile ? S.kev : nullptr, true);
        cudaEventRecordWithFlags(S.ev1, st, evf);
        return l;
    };
    if (use_graph && !profile) {
        auto hit = std::find_if(S.graphs.begin(), S.graphs.end(),
                                [&](const PassSlot::CachedGraph &c) { return c.key == key; });
        if (hit == S.graphs.end()) {
            cudaGraph_t g = nullptr;
            CPD_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
            const int launches = record(s, true);
            CPD_TRY(cudaStreamEndCapture(s, &g));
            cudaGraphExec_t exec = nullptr;
            const cudaError_t e = cudaGraphInstantiate(&exec, g, 0);
            if (e != cudaSuccess) cudaGraphDestroy(g);
            CPD_TRY(e);
            PassSlot::CachedGraph c{key, exec, launches};
            c.args = a;
            if (a.spans) {
                c.graph = g;
                c.trace_node = find_kernel_node(g, trace_spans_kernel_fn());
                if (!c.trace_node) {
                    cudaGraphExecDestroy(exec);
                    cudaGraphDestroy(g);
                    return CPD_CUDA_ERROR;
                }
            } else {
                cudaGraphDestroy(g);
            }
            if (S.graphs.size() >= PassSlot::kGraphCache) {
                cudaGraphExecDestroy(S.graphs.back().exec);
                if (S.graphs.back().graph) cudaGraphDestroy(S.graphs.back().graph);
                S.graphs.pop_back();
            }
            S.graphs.insert(S.graphs.begin(), c);
        } else if (hit != S.graphs.begin()) {
            std::rotate(S.graphs.begin(), hit, hit + 1);  // most recently used first
        }
        PassSlot::CachedGraph &cg = S.graphs.front();
        if (cg.trace_node && (std::memcmp(&cg.args.fc, &a.fc, sizeof(a.fc)) != 0 ||
                              std::memcmp(&cg.args.fl, &a.fl, sizeof(a.fl)) != 0)) {
            cudaKernelNodeParams kp{};
            CPD_TRY(cudaGraphKernelNodeGetParams(cg.trace_node, &kp));
            void *args[] = {&a};
            kp.kernelParams = args;
            kp.extra = nullptr;
            CPD_TRY(cudaGraphExecKernelNodeSetParams(cg.exec, cg.trace_node, &kp));
            cg.args = a;
        }
        CPD_TRY(cudaGraphLaunch(cg.exec, s));
        S.launches = cg.launches;
    } else {
        S.launches = record(s, false);
        CPD_TRY(cudaGetLastError());
    }
    if (p_out_host)
        CPD_TRY(cudaMemcpyAsync(p_out_host, S.pout.p, sizeof(double) * hist, cudaMemcpyDeviceToHost, s));
    CPD_TRY(cudaEventRecord(S.done, s));
    S.n = n;
    S.hist_cells = hist;
    S.p_out_host = p_out_host;
    S.profiled = profile;
    return CPD_OK;
}

// Collects the results of the pass issued on `S` (its `done` event has completed).
int pass_finish(PassSlot &S, PassResult &res)
{
    CPD_TRY(cudaEventSynchronize(S.done));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, S.ev0, S.ev1);
    S.last_ms = ms;
    if (S.profiled)
        for (int i = 0; i < 4; i++) {
            float km = 0.f;
            cudaEventElapsedTime(&km, S.kev[i], S.kev[i + 1]);
            S.kernel_ms[i] = km;
        }
    const HostStatus *c = reinterpret_cast<const HostStatus *>(S.h_outs.as<char>() + S.ctl_off);
    res.overflow = c->overflow != 0 || c->queue_count > S.qcap;
    if (res.overflow) S.hist_dirty = true;
    res.outs.assign(S.h_outs.as<DesignOut>(), S.h_outs.as<DesignOut>() + S.n);
    return CPD_OK;
}

// rays: the fixed-N estimator's ray count; under adaptive sampling the rays actually
// consumed (counted on the device) replace it.
void fill_fitness(const DesignOut &o, uint64_t rays, cpd_fitness &f, bool need_conv, bool adaptive = false)
{
    std::memset(&f, 0, sizeof(f));
    f.size = o.size;  // from the design record (built on the host or on the device)
    f.deviation = o.deviation;
    f.info = o.info;
    f.h_cond = o.h_cond;
    f.h_det = o.h_det;
    f.max_sem = o.max_sem;
    f.rays = adaptive ? o.fast : rays;
    f.hits = o.hits;
    f.retraced = o.retraced;
    f.fast_rays = adaptive ? o.fast - std::min(o.fast, o.retraced) : o.fast;
    f.wavelengths = (uint32_t)o.rows;
    f.status = o.status ? o.status : (need_conv && !o.converged) ? CPD_NOT_CONVERGED : CPD_OK;
}

bool valid_design(const cpd_design *d)
{
    return d && d->nglass >= 1 && d->nglass <= CPD_MAX_GLASS && d->bin_count >= 1 && d->bin_count <= CPD_MAX_BINS;
}

// A CPD_TRACE_* value, optionally with CPD_SAMPLING_ADAPTIVE (hybrid trace only) and
// then CPD_SAMPLING_EXACT.
bool valid_mode(uint32_t m)
{
    const uint32_t t = m & ~kSamplingBits, smp = m & kSamplingBits;
    if (t > CPD_TRACE_FP64) return false;
    return smp == 0u || (t == CPD_TRACE_HYBRID && (smp & CPD_SAMPLING_ADAPTIVE));
}

bool is_adaptive(uint32_t m) { return (m & CPD_SAMPLING_ADAPTIVE) != 0u; }

// What the pass needs of a parameter record before the device builds it (the build
// checks the rest and reports failures per design).
bool valid_params(const cpd_spectrometer_params &p)
{
    return p.nglass >= 1 && p.nglass <= CPD_MAX_GLASS && p.bin_count >= 1 && p.bin_count <= CPD_MAX_BINS;
}

bool valid_item(const cpd_batch_item &it)
{
    return it.max_n >= 1 && it.max_n <= CPD_MAX_WAVELENGTHS && it.max_eval >= 1 && it.max_eval <= CPD_MAX_RAYS;
}

// Runs one pass on `S` to completion, growing the re-trace queue and re-running the
// pass if it overflowed. A pass that overflowed leaves the persistent accumulators
// untouched (the entropy kernel skips such a pass), so the re-run is exact.
int run_pass_checked(cpd_context *ctx, PassSlot &S, const std::vector<PassDesign> &ds, uint32_t mode, bool fresh,
                     double *p_out, PassResult &res, bool use_graph)
{
    for (int attempt = 0; attempt < 6; attempt++) {
        int e = pass_issue(ctx, S, ds, mode, fresh, p_out, use_graph, ctx->profiling);
        if (!e) e = pass_finish(S, res);
        if (e) {
            S.hist_dirty = true;
            return e;
        }
        if (!res.overflow) return CPD_OK;
        S.qcap *= 4;
    }
    return CPD_NO_CAPACITY;
}

// The class of a batch for the launch-shape cache: trace mode and the binary orders of
// magnitude of its design count, wavelength rows, rays and widest detector.
std::array<uint64_t, 5> tune_class(const std::vector<PassDesign> &ds, uint32_t mode)
{
    uint64_t rows = 0, rays = 0, maxB = 0;
    for (const PassDesign &p : ds) {
        rows += p.W;
        rays += (uint64_t)p.W * p.R;
        maxB = std::max<uint64_t>(maxB, p.params ? p.params->bin_count : p.dev->B);
    }
    auto lg = [](uint64_t v) {
        uint64_t b = 0;
        while ((1ull << b) < v && b < 63) b++;
        return b;
    };
    return {mode, lg(ds.size()), lg(rows), lg(rays), lg(maxB)};
}

// The autotuner: times every (ray tile, warps per CTA) candidate on the batch itself
// (captured graph, two timed passes after one warm-up each, minimum device time) and
// keeps the fastest. Results do not depend on the launch shape (integer accumulation),
// so any candidate is safe to pick.
int tune_pass(cpd_context *ctx, const std::vector<PassDesign> &ds, uint32_t mode, double *best_ms)
{
    static const uint32_t kTiles[] = {4, 8, 16, 32, 64, 128, 256};
    static const uint32_t kWarps[] = {2, 4, 8};
    const uint32_t rt0 = ctx->ray_tile, w0 = ctx->warps_per_cta;
    double best = 1e300;
    uint32_t brt = rt0, bw = w0;
    PassResult res;
    // Besides the powers of two: tiles that make the work items a whole number of rounds
    // of the resident warps (2..6 items per warp), so that the last round is not a tail.
    std::vector<std::pair<uint32_t, uint32_t>> cands;
    for (uint32_t w : kWarps) {
        for (uint32_t rt : kTiles) cands.push_back({rt, w});
        uint64_t blocks = 0, rays = 0;
        for (const PassDesign &p : ds) {
            blocks += (p.W + 31) / 32;
            rays += (uint64_t)((p.W + 31) / 32) * p.rays->z64.size();
        }
        const uint64_t warps = trace_resident_warps(ctx->num_sms, w);
        for (uint64_t k = 2; k <= 6 && blocks; k++) {
            const uint64_t per = (rays + k * warps - 1) / (k * warps);  // rays per item
            if (per >= 2 && per <= 4096) cands.push_back({(uint32_t)per, w});
        }
    }
    for (const auto &cw : cands) {
        const uint32_t rt = cw.first, w = cw.second;
        {
            ctx->ray_tile = rt;
            ctx->warps_per_cta = w;
            double m = 1e300;
            for (int k = 0; k < 3; k++) {
                const int e = run_pass_checked(ctx, ctx->main, ds, mode, true, nullptr, res, ctx->use_graphs);
                if (e) {
                    ctx->ray_tile = rt0;
                    ctx->warps_per_cta = w0;
                    return e;
                }
                if (k) m = std::min(m, ctx->main.last_ms);
            }
            if (m < best) {
                best = m;
                brt = rt;
                bw = w;
            }
        }
    }
    ctx->ray_tile = brt;
    ctx->warps_per_cta = bw;
    ctx->tune_cache[tune_class(ds, mode)] = {brt, bw};
    if (best_ms) *best_ms = best;
    return CPD_OK;
}

// Builds the pass inputs of a batch (host copies kept alive by the caller's vectors).
void batch_inputs(cpd_context *ctx, const cpd_design *designs, const cpd_batch_item *items, uint32_t n,
                  std::vector<DevDesign> &devs, std::vector<LamPtr> &lams, std::vector<RayTablePtr> &rts,
                  std::vector<PassDesign> &ds)
{
    devs.resize(n);
    lams.resize(n);
    rts.resize(n);
    ds.resize(n);
    for (uint32_t i = 0; i < n; i++) {
        design_to_dev(designs[i], devs[i]);
        lams[i] = lam_points_cached(ctx, items[i].seed, items[i].max_n);
        rts[i] = ray_table_cached(ctx, items[i].seed, items[i].max_eval);
        ds[i] = PassDesign{&devs[i], items[i].max_n, items[i].max_eval, lams[i]->data(), rts[i].get(), lams[i], rts[i],
                           (uint32_t)lams[i]->size()};
    }
}

}  // namespace

namespace cpd {
int context_device(const cpd_context *ctx) { return ctx->device; }
int context_sms(const cpd_context *ctx) { return ctx->num_sms; }
const float *context_logtab(const cpd_context *ctx) { return ctx->logtab.as<float>(); }
RayTablePtr context_ray_table(cpd_context *ctx, double seed, uint32_t R) { return ray_table_cached(ctx, seed, R); }
LamPtr context_lam_points(cpd_context *ctx, double seed, uint32_t W) { return lam_points_cached(ctx, seed, W); }
void fitness_from_out(const DesignOut &o, uint64_t rays, cpd_fitness &f) { fill_fitness(o, rays, f, true, false); }
}  // namespace cpd

// ------------------------------------------------------------------ the server

namespace {
struct SrvRequest {
    std::vector<cpd_design> designs;
    std::vector<cpd_spectrometer_params> params;  // instead of designs: built on the device
    double acceptance = 0.0;
    std::vector<cpd_batch_item> items;
    std::vector<cpd_fitness> outs;
    uint32_t remaining = 0;
    uint32_t mode = 0;
    int status = CPD_OK;
    bool done = false;
    std::chrono::steady_clock::time_point t_submit, t_done;
};
struct SrvWork {
    uint64_t req;
    uint32_t idx;
    uint64_t bytes;
};
}  // namespace

struct cpd_server {
    cpd_context *ctx = nullptr;
    std::vector<std::unique_ptr<PassSlot>> slots;
    std::vector<std::vector<SrvWork>> slot_work;
    std::vector<bool> busy;
    uint64_t budget = 0, in_use = 0;
    uint32_t max_designs_per_pass = 256;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<SrvWork> pending;
    std::map<uint64_t, SrvRequest> reqs;
    uint64_t next_id = 1;
    std::thread worker;
    bool stop = false;
    uint64_t designs_done = 0, passes = 0, max_in_flight = 0;
};

namespace {

// Completes the pass on slot i (called by the worker without the lock held for the
// device wait; the lock is taken to publish results).
void srv_complete(cpd_server *sv, size_t i)
{
    PassSlot &S = *sv->slots[i];
    PassResult res;
    int e = pass_finish(S, res);
    std::lock_guard<std::mutex> lk(sv->mu);
    auto &work = sv->slot_work[i];
    if (!e && res.overflow) e = CPD_NO_CAPACITY;  // re-queued below with a larger queue
    if (e == CPD_NO_CAPACITY && S.qcap < (1u << 26)) {
        // grow the re-trace queue and run the same designs again
        S.qcap *= 4;
        for (auto it = work.rbegin(); it != work.rend(); ++it) {
            sv->in_use -= it->bytes;
            sv->pending.push_front(*it);
        }
        e = CPD_OK;
        work.clear();
    }
    for (size_t k = 0; k < work.size(); k++) {
        auto rit = sv->reqs.find(work[k].req);
        if (rit == sv->reqs.end()) continue;
        SrvRequest &r = rit->second;
        if (e) r.status = e;
        else fill_fitness(res.outs[k], (uint64_t)r.items[work[k].idx].max_n * r.items[work[k].idx].max_eval,
                          r.outs[work[k].idx], true, is_adaptive(r.mode));
        if (--r.remaining == 0) {
            r.done = true;
            r.t_done = std::chrono::steady_clock::now();
        }
        sv->designs_done++;
    }
    for (auto &w : work) sv->in_use -= w.bytes;
    work.clear();
    sv->busy[i] = false;
    sv->passes++;
    sv->cv_done.notify_all();
}

void srv_loop(cpd_server *sv)
{
    cudaSetDevice(sv->ctx->device);
    for (;;) {
        bool progressed = false;
        // completions
        for (size_t i = 0; i < sv->slots.size(); i++) {
            bool b;
            {
                std::lock_guard<std::mutex> lk(sv->mu);
                b = sv->busy[i];
            }
            if (b && cudaEventQuery(sv->slots[i]->done) != cudaErrorNotReady) {
                srv_complete(sv, i);
                progressed = true;
            }
        }
        // admissions: each free slot takes the oldest pending designs of one trace mode
        // while they fit the device-memory budget
        for (size_t i = 0; i < sv->slots.size(); i++) {
            std::vector<SrvWork> take;
            std::vector<DevDesign> devs;
            std::vector<LamPtr> lams;
            std::vector<RayTablePtr> rays;
            uint32_t mode = 0;
            {
                std::lock_guard<std::mutex> lk(sv->mu);
                if (sv->busy[i] || sv->pending.empty()) continue;
                bool others = false;
                for (size_t j = 0; j < sv->slots.size(); j++) others |= sv->busy[j];
                const SrvRequest &r0 = sv->reqs[sv->pending.front().req];
                mode = r0.mode;
                const bool dev0 = !r0.params.empty();
                const double acc0 = r0.acceptance;
                while (!sv->pending.empty() && take.size() < sv->max_designs_per_pass) {
                    const SrvWork &w = sv->pending.front();
                    // a pass holds designs of one trace mode and one kind (built on the host,
                    // or on the device with one acceptance)
                    const SrvRequest &rw = sv->reqs[w.req];
                    if (rw.mode != mode || rw.params.empty() != !dev0 || rw.acceptance != acc0) break;
                    if (sv->in_use + w.bytes > sv->budget && (others || !take.empty())) break;
                    sv->in_use += w.bytes;
                    take.push_back(w);
                    sv->pending.pop_front();
                }
                if (take.empty()) continue;
                sv->busy[i] = true;
                sv->slot_work[i] = take;
                uint64_t nb = 0;
                for (size_t j = 0; j < sv->slots.size(); j++) nb += sv->busy[j];
                sv->max_in_flight = std::max<uint64_t>(sv->max_in_flight, nb);
            }
            // host preparation and issue without the lock (the slot belongs to the worker)
            std::vector<PassDesign> ds(take.size());
            devs.resize(take.size());
            lams.resize(take.size());
            rays.resize(take.size());
            for (size_t k = 0; k < take.size(); k++) {
                const SrvRequest *r;
                {
                    std::lock_guard<std::mutex> lk(sv->mu);
                    r = &sv->reqs[take[k].req];
                }
                const cpd_batch_item &it = r->items[take[k].idx];
                if (r->params.empty()) design_to_dev(r->designs[take[k].idx], devs[k]);
                lams[k] = lam_points_cached(sv->ctx, it.seed, it.max_n);
                rays[k] = ray_table_cached(sv->ctx, it.seed, it.max_eval);
                ds[k] = PassDesign{&devs[k], it.max_n, it.max_eval, lams[k]->data(), rays[k].get(), lams[k], rays[k],
                                   (uint32_t)lams[k]->size()};
                if (!r->params.empty()) {
                    ds[k].dev = nullptr;
                    ds[k].params = &r->params[take[k].idx];
                    ds[k].acceptance = r->acceptance;
                }
            }
            int e = pass_issue(sv->ctx, *sv->slots[i], ds, mode, true, nullptr, false, false);
            if (e) {
                std::lock_guard<std::mutex> lk(sv->mu);
                sv->slots[i]->hist_dirty = true;
                for (auto &w : take) {
                    SrvRequest &r = sv->reqs[w.req];
                    r.status = e;
                    if (--r.remaining == 0) {
                        r.done = true;
                        r.t_done = std::chrono::steady_clock::now();
                    }
                    sv->in_use -= w.bytes;
                }
                sv->busy[i] = false;
                sv->slot_work[i].clear();
                sv->cv_done.notify_all();
            }
            progressed = true;
        }
        {
            std::unique_lock<std::mutex> lk(sv->mu);
            bool any_busy = false;
            for (bool b : sv->busy) any_busy |= b;
            if (sv->stop && !any_busy && sv->pending.empty()) return;
            if (!progressed) {
                if (any_busy) {
                    lk.unlock();
                    std::this_thread::sleep_for(std::chrono::microseconds(20));
                } else {
                    sv->cv_work.wait_for(lk, std::chrono::milliseconds(50));
                }
            }
        }
    }
}

}  // namespace

// ------------------------------------------------------------------ C ABI

extern "C" {

int cpd_context_create(int device, cpd_context **out)
{
    if (!out) return CPD_INVALID_ARGUMENT;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return CPD_CUDA_ERROR;
    if (cudaSetDevice(device) != cudaSuccess) return CPD_CUDA_ERROR;
    cpd_context *ctx = new cpd_context();
    ctx->device = device;
    cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
    std::vector<float> tab(4 * ff::kLogTable);
    ff::make_log_table(tab.data());
    if (configure_kernels() != cudaSuccess || ctx->main.create() != cudaSuccess || ctx->logtab.ensure(sizeof(float) * tab.size()) != cudaSuccess ||
        cudaMemcpy(ctx->logtab.p, tab.data(), sizeof(float) * tab.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
        ctx->main.destroy();
        ctx->logtab.release();
        delete ctx;
        return CPD_CUDA_ERROR;
    }
    *out = ctx;
    return CPD_OK;
}

void cpd_context_destroy(cpd_context *ctx)
{
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    ctx->main.destroy();
    for (DevBuf *b : {&ctx->tp_design, &ctx->tp_lam, &ctx->tp_z, &ctx->tp_out, &ctx->tp_rays})
        b->release();
    for (DevBuf *b : {&ctx->bld_params, &ctx->bld_out, &ctx->bld_status, &ctx->pair_design, &ctx->pair_lam,
                      &ctx->pair_z, &ctx->pair_bins, &ctx->pair_ts,
                      &ctx->pair_flags, &ctx->peak, &ctx->logtab})
        b->release();
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
    if (kernel_ms) *kernel_ms = ctx->main.last_ms;
    if (launches) *launches = (uint32_t)ctx->main.launches;
    return CPD_OK;
}

int cpd_set_profiling(cpd_context *ctx, int on)
{
    if (!ctx) return CPD_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->profiling = on != 0;
    return CPD_OK;
}

int cpd_last_kernel_times(cpd_context *ctx, double ms[4])
{
    if (!ctx || !ms) return CPD_INVALID_ARGUMENT;
    for (int i = 0; i < 4; i++) ms[i] = ctx->main.kernel_ms[i];
    return CPD_OK;
}

int cpd_last_transfer_bytes(cpd_context *ctx, uint64_t *h2d, uint64_t *d2h)
{
    if (!ctx) return CPD_INVALID_ARGUMENT;
    if (h2d) *h2d = ctx->main.h2d;
    if (d2h) *d2h = ctx->main.d2h;
    return CPD_OK;
}

#define CPD_SYNC_ENTRY(ctx)                                                 \
    std::lock_guard<std::mutex> lk((ctx)->mu);                              \
    if (cudaSetDevice((ctx)->device) != cudaSuccess) return CPD_CUDA_ERROR; \
    (ctx)->main.h2d = (ctx)->main.d2h = 0

int cpd_fitness_gpu_points(cpd_context *ctx, const cpd_design *d, const double *lam_u, uint32_t W,
                           const double *ray_u, uint32_t R, uint32_t trace_mode, cpd_fitness *out, double *p_out)
{
    if (!ctx || !valid_design(d) || !lam_u || !ray_u || !out) return CPD_INVALID_ARGUMENT;
    if (W == 0 || W > CPD_MAX_WAVELENGTHS || R == 0 || R > CPD_MAX_RAYS || !valid_mode(trace_mode))
        return CPD_INVALID_ARGUMENT;
    CPD_SYNC_ENTRY(ctx);
    DevDesign D;
    design_to_dev(*d, D);
    RayTable rt;
    ray_table(ray_u, R, rt.z64, rt.z32, &rt.rank);
    std::vector<PassDesign> ds{PassDesign{&D, W, R, lam_u, &rt}};
    PassResult res;
    int e = run_pass_checked(ctx, ctx->main, ds, trace_mode, true, p_out, res, ctx->use_graphs);
    if (e) return e;
    fill_fitness(res.outs[0], (uint64_t)W * R, *out, false, is_adaptive(trace_mode));
    return CPD_OK;
}

int cpd_fitness_gpu(cpd_context *ctx, const cpd_design *d, const double *seeds, uint32_t nseeds, uint32_t max_n,
                    uint32_t nwarp, uint32_t max_eval, cpd_fitness *out)
{
    return cpd_fitness_gpu_ex(ctx, d, seeds, nseeds, max_n, nwarp, max_eval, 0u, out);
}

int cpd_fitness_gpu_ex(cpd_context *ctx, const cpd_design *d, const double *seeds, uint32_t nseeds, uint32_t max_n,
                       uint32_t nwarp, uint32_t max_eval, uint32_t sampling, cpd_fitness *out)
{
    if (!ctx || !valid_design(d) || !seeds || !out || nseeds == 0) return CPD_INVALID_ARGUMENT;
    if (max_n == 0 || max_eval == 0 || max_eval > CPD_MAX_RAYS) return CPD_INVALID_ARGUMENT;
    if ((uint64_t)max_n * nseeds > CPD_MAX_WAVELENGTHS) return CPD_INVALID_ARGUMENT;
    const uint32_t mode = CPD_TRACE_HYBRID | sampling;
    if ((sampling & ~kSamplingBits) || !valid_mode(mode)) return CPD_INVALID_ARGUMENT;
    CPD_SYNC_ENTRY(ctx);
    // the adaptive kernels have no launch shape to tune
    const bool tune = ctx->autotune && !ctx->profiling && !is_adaptive(mode);
    if (!tune && nwarp >= 1 && nwarp <= 8) ctx->warps_per_cta = nwarp;
    DevDesign D;
    design_to_dev(*d, D);
    PassResult res;
    uint64_t rays = 0;
    for (uint32_t s = 0; s < nseeds; s++) {
        const auto lam = lam_points_cached(ctx, seeds[s], max_n);
        RayTablePtr rt = ray_table_cached(ctx, seeds[s], max_eval);
        std::vector<PassDesign> ds{
            PassDesign{&D, max_n, max_eval, lam->data(), rt.get(), lam, rt, (uint32_t)lam->size()}};
        if (tune && s == 0) {
            // the autotuner replaces the reference's nwarp hint
            auto it = ctx->tune_cache.find(tune_class(ds, mode));
            if (it != ctx->tune_cache.end()) {
                ctx->ray_tile = it->second.first;
                ctx->warps_per_cta = it->second.second;
            } else {
                const int te = tune_pass(ctx, ds, mode, nullptr);
                if (te) return te;
            }
        }
        int e = run_pass_checked(ctx, ctx->main, ds, mode, s == 0, nullptr, res, ctx->use_graphs);
        if (e) return e;
        rays += (uint64_t)max_n * max_eval;
        if (res.outs[0].converged) break;
    }
    fill_fitness(res.outs[0], rays, *out, true, is_adaptive(mode));
    return out->status;
}

int cpd_fitness_gpu_batch(cpd_context *ctx, const cpd_design *designs, const cpd_batch_item *items, uint32_t n,
                          uint32_t trace_mode, cpd_fitness *outs)
{
    if (!ctx || !designs || !items || !outs || n == 0 || !valid_mode(trace_mode)) return CPD_INVALID_ARGUMENT;
    for (uint32_t i = 0; i < n; i++)
        if (!valid_design(&designs[i]) || !valid_item(items[i])) return CPD_INVALID_ARGUMENT;
    CPD_SYNC_ENTRY(ctx);
    std::vector<DevDesign> devs;
    std::vector<LamPtr> lams;
    std::vector<RayTablePtr> rts;
    std::vector<PassDesign> ds;
    batch_inputs(ctx, designs, items, n, devs, lams, rts, ds);
    if (ctx->autotune && !ctx->profiling && !is_adaptive(trace_mode)) {
        auto it = ctx->tune_cache.find(tune_class(ds, trace_mode));
        if (it != ctx->tune_cache.end()) {
            ctx->ray_tile = it->second.first;
            ctx->warps_per_cta = it->second.second;
        } else {
            const int te = tune_pass(ctx, ds, trace_mode, nullptr);
            if (te) return te;
        }
    }
    PassResult res;
    int e = run_pass_checked(ctx, ctx->main, ds, trace_mode, true, nullptr, res, ctx->use_graphs);
    if (e) return e;
    for (uint32_t i = 0; i < n; i++)
        fill_fitness(res.outs[i], (uint64_t)items[i].max_n * items[i].max_eval, outs[i], true,
                     is_adaptive(trace_mode));
    return CPD_OK;
}

int cpd_fitness_gpu_batch_params(cpd_context *ctx, const cpd_spectrometer_params *params,
                                 const cpd_batch_item *items, uint32_t n, double acceptance, uint32_t trace_mode,
                                 cpd_fitness *outs)
{
    if (!ctx || !params || !items || !outs || n == 0 || !valid_mode(trace_mode)) return CPD_INVALID_ARGUMENT;
    if (acceptance != 0.0 && !(acceptance > 0.0 && acceptance <= 1.0)) return CPD_INVALID_ARGUMENT;
    for (uint32_t i = 0; i < n; i++)
        if (!valid_params(params[i]) || !valid_item(items[i])) return CPD_INVALID_ARGUMENT;
    CPD_SYNC_ENTRY(ctx);
    std::vector<LamPtr> lams(n);
    std::vector<RayTablePtr> rts(n);
    std::vector<PassDesign> ds(n);
    for (uint32_t i = 0; i < n; i++) {
        lams[i] = lam_points_cached(ctx, items[i].seed, items[i].max_n);
        rts[i] = ray_table_cached(ctx, items[i].seed, items[i].max_eval);
        ds[i] = PassDesign{nullptr, items[i].max_n, items[i].max_eval, lams[i]->data(), rts[i].get(), lams[i], rts[i],
                           (uint32_t)lams[i]->size(), &params[i], acceptance};
    }
    if (ctx->autotune && !ctx->profiling && !is_adaptive(trace_mode)) {
        auto it = ctx->tune_cache.find(tune_class(ds, trace_mode));
        if (it != ctx->tune_cache.end()) {
            ctx->ray_tile = it->second.first;
            ctx->warps_per_cta = it->second.second;
        } else {
            const int te = tune_pass(ctx, ds, trace_mode, nullptr);
            if (te) return te;
        }
    }
    PassResult res;
    int e = run_pass_checked(ctx, ctx->main, ds, trace_mode, true, nullptr, res, ctx->use_graphs);
    if (e) return e;
    for (uint32_t i = 0; i < n; i++)
        fill_fitness(res.outs[i], (uint64_t)items[i].max_n * items[i].max_eval, outs[i], true,
                     is_adaptive(trace_mode));
    return CPD_OK;
}

int cpd_design_build_device(cpd_context *ctx, const cpd_spectrometer_params *params, uint32_t n, double acceptance,
                            cpd_design *out, int32_t *status)
{
    if (!ctx || ((!params || !out || !status) && n)) return CPD_INVALID_ARGUMENT;
    if (acceptance != 0.0 && !(acceptance > 0.0 && acceptance <= 1.0)) return CPD_INVALID_ARGUMENT;
    if (n == 0) return CPD_OK;
    CPD_SYNC_ENTRY(ctx);
    cudaStream_t s = ctx->main.stream;
    CPD_TRY(ctx->bld_params.ensure(sizeof(cpd_spectrometer_params) * n));
    CPD_TRY(ctx->bld_out.ensure(sizeof(cpd_design) * n));
    CPD_TRY(ctx->bld_status.ensure(sizeof(int32_t) * n));
    CPD_TRY(cudaMemcpyAsync(ctx->bld_params.p, params, sizeof(cpd_spectrometer_params) * n, cudaMemcpyHostToDevice, s));
    launch_build_records(ctx->bld_params.as<cpd_spectrometer_params>(), n, acceptance, ctx->bld_out.as<cpd_design>(),
                         ctx->bld_status.as<int32_t>(), s);
    CPD_TRY(cudaGetLastError());
    CPD_TRY(cudaMemcpyAsync(out, ctx->bld_out.p, sizeof(cpd_design) * n, cudaMemcpyDeviceToHost, s));
    CPD_TRY(cudaMemcpyAsync(status, ctx->bld_status.p, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, s));
    CPD_TRY(cudaStreamSynchronize(s));
    ctx->main.h2d += sizeof(cpd_spectrometer_params) * n;
    ctx->main.d2h += (sizeof(cpd_design) + sizeof(int32_t)) * n;
    return CPD_OK;
}

int cpd_autotune_batch(cpd_context *ctx, const cpd_design *designs, const cpd_batch_item *items, uint32_t n,
                       uint32_t trace_mode, uint32_t *ray_tile, uint32_t *warps_per_cta, double *best_ms)
{
    if (!ctx || !designs || !items || n == 0 || trace_mode > CPD_TRACE_FP64) return CPD_INVALID_ARGUMENT;  // fixed-N only
    for (uint32_t i = 0; i < n; i++)
        if (!valid_design(&designs[i]) || !valid_item(items[i])) return CPD_INVALID_ARGUMENT;
    CPD_SYNC_ENTRY(ctx);
    std::vector<DevDesign> devs;
    std::vector<LamPtr> lams;
    std::vector<RayTablePtr> rts;
    std::vector<PassDesign> ds;
    batch_inputs(ctx, designs, items, n, devs, lams, rts, ds);
    const int e = tune_pass(ctx, ds, trace_mode, best_ms);
    if (e) return e;
    if (ray_tile) *ray_tile = ctx->ray_tile;
    if (warps_per_cta) *warps_per_cta = ctx->warps_per_cta;
    return CPD_OK;
}

int cpd_set_autotune(cpd_context *ctx, int on)
{
    if (!ctx) return CPD_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->autotune = on != 0;
    return CPD_OK;
}

int cpd_transmission_probability(cpd_context *ctx, const cpd_design *d, const double *wavelengths, uint32_t n,
                                 uint32_t max_m, double *out)
{
    return cpd_transmission_probability_ex(ctx, d, wavelengths, n, max_m, 0u, out, nullptr);
}

int cpd_transmission_probability_ex(cpd_context *ctx, const cpd_design *d, const double *wavelengths, uint32_t n,
                                    uint32_t max_m, uint32_t flags, double *out, uint32_t *rays_out)
{
    if (!ctx || !valid_design(d) || !wavelengths || !out || n == 0 || n > CPD_MAX_WAVELENGTHS || max_m == 0 ||
        max_m > CPD_MAX_RAYS || (flags & ~(uint32_t)CPD_TP_FIXED_N))
        return CPD_INVALID_ARGUMENT;
    // the reference CPU ray points (fitness.rs:19): the incremental R1 sequence from 0.5
    auto ref_points = [](uint32_t m, double *u) {
        double st = 0.5;
        for (uint32_t j = 0; j < m; j++) {
            st = st + kAlpha;
            st = st - std::trunc(st);
            u[j] = st;
        }
    };
    if (flags & CPD_TP_FIXED_N) {
        // explicit wavelengths: bounds (0, 1) make wmin + (wmax - wmin)*u == u exactly
        cpd_design dd = *d;
        dd.wavelength_bounds[0] = 0.0;
        dd.wavelength_bounds[1] = 1.0;
        std::vector<double> ray_u(max_m);
        ref_points(max_m, ray_u.data());
        cpd_fitness f;
        const int e = cpd_fitness_gpu_points(ctx, &dd, wavelengths, n, ray_u.data(), max_m, CPD_TRACE_HYBRID, &f, out);
        if (!e && rays_out)
            for (uint32_t i = 0; i < n; i++) rays_out[i] = max_m;
        return e;
    }
    CPD_SYNC_ENTRY(ctx);
    PassSlot &S = ctx->main;
    cudaStream_t s = S.stream;
    DevDesign D;
    design_to_dev(*d, D);
    if (ctx->tp_m != max_m) {
        std::vector<double> z(max_m);
        ref_points(max_m, z.data());
        for (uint32_t j = 0; j < max_m; j++) z[j] = norminv(z[j]);
        CPD_TRY(ctx->tp_z.ensure(sizeof(double) * max_m));
        CPD_TRY(cudaMemcpyAsync(ctx->tp_z.p, z.data(), sizeof(double) * max_m, cudaMemcpyHostToDevice, s));
        ctx->tp_m = max_m;
        S.h2d += sizeof(double) * max_m;
    }
    const size_t out_bytes = sizeof(double) * (size_t)n * D.B;
    CPD_TRY(ctx->tp_design.ensure(sizeof(DevDesign)));
    CPD_TRY(ctx->tp_lam.ensure(sizeof(double) * n));
    CPD_TRY(ctx->tp_out.ensure(out_bytes));
    CPD_TRY(ctx->tp_rays.ensure(sizeof(uint32_t) * n));
    CPD_TRY(cudaMemcpyAsync(ctx->tp_design.p, &D, sizeof(DevDesign), cudaMemcpyHostToDevice, s));
    CPD_TRY(cudaMemcpyAsync(ctx->tp_lam.p, wavelengths, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    CPD_TRY(cudaEventRecord(S.ev0, s));
    launch_tp_adaptive(ctx->tp_design.as<DevDesign>(), D.B, ctx->tp_lam.as<double>(), n, ctx->tp_z.as<double>(),
                       max_m, ctx->tp_out.as<double>(), ctx->tp_rays.as<uint32_t>(), s);
    CPD_TRY(cudaGetLastError());
    CPD_TRY(cudaEventRecord(S.ev1, s));
    CPD_TRY(cudaMemcpyAsync(out, ctx->tp_out.p, out_bytes, cudaMemcpyDeviceToHost, s));
    if (rays_out)
        CPD_TRY(cudaMemcpyAsync(rays_out, ctx->tp_rays.p, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, s));
    CPD_TRY(cudaStreamSynchronize(s));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, S.ev0, S.ev1);
    S.last_ms = ms;
    S.launches = 1;
    S.h2d += sizeof(DevDesign) + sizeof(double) * n;
    S.d2h += out_bytes + (rays_out ? sizeof(uint32_t) * n : 0);
    return CPD_OK;
}

int cpd_trace_rays(cpd_context *ctx, const cpd_design *d, const double *lam_u, const double *ray_u, uint32_t n,
                   uint32_t trace_mode, uint32_t *bins, double *ts, uint8_t *flags)
{
    if (!ctx || !valid_design(d) || !lam_u || !ray_u || !bins || !ts || trace_mode > CPD_TRACE_FP64)
        return CPD_INVALID_ARGUMENT;
    if (n == 0) return CPD_OK;
    CPD_SYNC_ENTRY(ctx);
    PassSlot &S = ctx->main;
    DevDesign D;
    design_to_dev(*d, D);
    std::vector<double> z(n);
    for (uint32_t i = 0; i < n; i++) z[i] = norminv(ray_u[i]);
    cudaStream_t s = S.stream;
    CPD_TRY(ctx->pair_design.ensure(sizeof(DevDesign)));
    CPD_TRY(ctx->pair_lam.ensure(sizeof(double) * n));
    CPD_TRY(ctx->pair_z.ensure(sizeof(double) * n));
    CPD_TRY(ctx->pair_bins.ensure(sizeof(uint32_t) * n));
    CPD_TRY(ctx->pair_ts.ensure(sizeof(double) * n));
    CPD_TRY(ctx->pair_flags.ensure(n));
    CPD_TRY(cudaMemcpyAsync(ctx->pair_design.p, &D, sizeof(DevDesign), cudaMemcpyHostToDevice, s));
    CPD_TRY(cudaMemcpyAsync(ctx->pair_lam.p, lam_u, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    CPD_TRY(cudaMemcpyAsync(ctx->pair_z.p, z.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s));
    CPD_TRY(cudaEventRecord(S.ev0, s));
    launch_trace_pairs(ctx->pair_design.as<DevDesign>(), ctx->pair_lam.as<double>(), ctx->pair_z.as<double>(), n,
                       trace_mode, ctx->pair_bins.as<uint32_t>(), ctx->pair_ts.as<double>(),
                       ctx->pair_flags.as<uint8_t>(), s);
    CPD_TRY(cudaGetLastError());
    CPD_TRY(cudaEventRecord(S.ev1, s));
    CPD_TRY(cudaMemcpyAsync(bins, ctx->pair_bins.p, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, s));
    CPD_TRY(cudaMemcpyAsync(ts, ctx->pair_ts.p, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    if (flags) CPD_TRY(cudaMemcpyAsync(flags, ctx->pair_flags.p, n, cudaMemcpyDeviceToHost, s));
    CPD_TRY(cudaStreamSynchronize(s));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, S.ev0, S.ev1);
    S.last_ms = ms;
    S.launches = 1;
    return CPD_OK;
}

int cpd_measure_fp32_peak(cpd_context *ctx, uint32_t iters, double *tflops)
{
    if (!ctx || !tflops || iters == 0) return CPD_INVALID_ARGUMENT;
    CPD_SYNC_ENTRY(ctx);
    PassSlot &S = ctx->main;
    const int threads = 256;
    const int blocks = ctx->num_sms * 8;
    CPD_TRY(ctx->peak.ensure(sizeof(float) * blocks));
    cudaStream_t s = S.stream;
    launch_fma_peak(ctx->peak.as<float>(), 16, blocks, threads, s);  // warm-up
    CPD_TRY(cudaEventRecord(S.ev0, s));
    launch_fma_peak(ctx->peak.as<float>(), iters, blocks, threads, s);
    CPD_TRY(cudaEventRecord(S.ev1, s));
    CPD_TRY(cudaStreamSynchronize(s));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, S.ev0, S.ev1);
    const double flops = 2.0 * 8.0 * 16.0 * (double)iters * threads * (double)blocks;
    *tflops = flops / (ms * 1e-3) / 1e12;
    S.last_ms = ms;
    S.launches = 2;
    return CPD_OK;
}

int cpd_measure_sfu_peak(cpd_context *ctx, uint32_t iters, double *gops)
{
    if (!ctx || !gops || iters == 0) return CPD_INVALID_ARGUMENT;
    CPD_SYNC_ENTRY(ctx);
    PassSlot &S = ctx->main;
    const int threads = 256;
    const int blocks = ctx->num_sms * 8;
    CPD_TRY(ctx->peak.ensure(sizeof(float) * blocks));
    cudaStream_t s = S.stream;
    launch_mufu_peak(ctx->peak.as<float>(), 16, blocks, threads, s);  // warm-up
    CPD_TRY(cudaEventRecord(S.ev0, s));
    launch_mufu_peak(ctx->peak.as<float>(), iters, blocks, threads, s);
    CPD_TRY(cudaEventRecord(S.ev1, s));
    CPD_TRY(cudaStreamSynchronize(s));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, S.ev0, S.ev1);
    const double ops = 8.0 * 16.0 * (double)iters * threads * (double)blocks;
    *gops = ops / (ms * 1e-3) / 1e9;
    S.last_ms = ms;
    S.launches = 2;
    return CPD_OK;
}

// ------------------------------------------------------------------ server ABI

int cpd_server_create(cpd_context *ctx, uint64_t mem_budget_bytes, uint32_t slots, uint32_t max_designs_per_pass,
                      cpd_server **out)
{
    if (!ctx || !out || slots == 0 || slots > 8 || mem_budget_bytes == 0) return CPD_INVALID_ARGUMENT;
    *out = nullptr;
    if (cudaSetDevice(ctx->device) != cudaSuccess) return CPD_CUDA_ERROR;
    cpd_server *sv = new cpd_server();
    sv->ctx = ctx;
    sv->budget = mem_budget_bytes;
    if (max_designs_per_pass) sv->max_designs_per_pass = max_designs_per_pass;
    for (uint32_t i = 0; i < slots; i++) {
        sv->slots.emplace_back(new PassSlot());
        if (sv->slots.back()->create() != cudaSuccess) {
            for (auto &s : sv->slots) s->destroy();
            delete sv;
            return CPD_CUDA_ERROR;
        }
    }
    sv->slot_work.resize(slots);
    sv->busy.assign(slots, false);
    sv->worker = std::thread(srv_loop, sv);
    *out = sv;
    return CPD_OK;
}

int cpd_server_submit(cpd_server *sv, const cpd_design *designs, const cpd_batch_item *items, uint32_t n,
                      uint32_t trace_mode, uint64_t *request_id)
{
    if (!sv || !designs || !items || !request_id || n == 0 || !valid_mode(trace_mode)) return CPD_INVALID_ARGUMENT;
    for (uint32_t i = 0; i < n; i++)
        if (!valid_design(&designs[i]) || !valid_item(items[i])) return CPD_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(sv->mu);
    if (sv->stop) return CPD_INVALID_ARGUMENT;
    const uint64_t id = sv->next_id++;
    SrvRequest &r = sv->reqs[id];
    r.designs.assign(designs, designs + n);
    r.items.assign(items, items + n);
    r.outs.resize(n);
    r.remaining = n;
    r.mode = trace_mode;
    r.t_submit = std::chrono::steady_clock::now();
    for (uint32_t i = 0; i < n; i++)
        sv->pending.push_back(
            SrvWork{id, i, design_bytes(items[i].max_n, items[i].max_eval, designs[i].bin_count)});
    *request_id = id;
    sv->cv_work.notify_one();
    return CPD_OK;
}

int cpd_server_submit_params(cpd_server *sv, const cpd_spectrometer_params *params, const cpd_batch_item *items,
                             uint32_t n, double acceptance, uint32_t trace_mode, uint64_t *request_id)
{
    if (!sv || !params || !items || !request_id || n == 0 || !valid_mode(trace_mode)) return CPD_INVALID_ARGUMENT;
    if (acceptance != 0.0 && !(acceptance > 0.0 && acceptance <= 1.0)) return CPD_INVALID_ARGUMENT;
    for (uint32_t i = 0; i < n; i++)
        if (!valid_params(params[i]) || !valid_item(items[i])) return CPD_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(sv->mu);
    if (sv->stop) return CPD_INVALID_ARGUMENT;
    const uint64_t id = sv->next_id++;
    SrvRequest &r = sv->reqs[id];
    r.params.assign(params, params + n);
    r.acceptance = acceptance;
    r.items.assign(items, items + n);
    r.outs.resize(n);
    r.remaining = n;
    r.mode = trace_mode;
    r.t_submit = std::chrono::steady_clock::now();
    for (uint32_t i = 0; i < n; i++)
        sv->pending.push_back(
            SrvWork{id, i, design_bytes(items[i].max_n, items[i].max_eval, params[i].bin_count)});
    *request_id = id;
    sv->cv_work.notify_one();
    return CPD_OK;
}

int cpd_server_wait(cpd_server *sv, uint64_t request_id, cpd_fitness *outs, double timeout_ms, double *latency_ms)
{
    if (!sv || !outs) return CPD_INVALID_ARGUMENT;
    std::unique_lock<std::mutex> lk(sv->mu);
    auto it = sv->reqs.find(request_id);
    if (it == sv->reqs.end()) return CPD_INVALID_ARGUMENT;
    const auto deadline = std::chrono::steady_clock::now() +
                          std::chrono::microseconds((int64_t)(std::max(0.0, timeout_ms) * 1000.0));
    while (!it->second.done) {
        if (sv->cv_done.wait_until(lk, deadline) == std::cv_status::timeout && !it->second.done) return CPD_TIMEOUT;
        it = sv->reqs.find(request_id);
        if (it == sv->reqs.end()) return CPD_INVALID_ARGUMENT;
    }
    SrvRequest &r = it->second;
    std::memcpy(outs, r.outs.data(), sizeof(cpd_fitness) * r.outs.size());
    if (latency_ms) *latency_ms = std::chrono::duration<double, std::milli>(r.t_done - r.t_submit).count();
    const int status = r.status;
    sv->reqs.erase(it);
    return status;
}

int cpd_server_stats(cpd_server *sv, uint64_t *designs_done, uint64_t *passes, uint64_t *max_in_flight,
                     uint64_t *pending)
{
    if (!sv) return CPD_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(sv->mu);
    if (designs_done) *designs_done = sv->designs_done;
    if (passes) *passes = sv->passes;
    if (max_in_flight) *max_in_flight = sv->max_in_flight;
    if (pending) *pending = sv->pending.size();
    return CPD_OK;
}

void cpd_server_destroy(cpd_server *sv)
{
    if (!sv) return;
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        sv->stop = true;
        sv->cv_work.notify_all();
    }
    if (sv->worker.joinable()) sv->worker.join();
    cudaSetDevice(sv->ctx->device);
    for (auto &s : sv->slots) s->destroy();
    delete sv;
}

}  // extern "C"
