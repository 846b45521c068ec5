// cpd_loop.cu -- the device-resident serving loop: the host side.
//
// The device side is loop_kernel (cpd_kernels.cu): a persistent kernel whose CTAs each
// hold one histogram slab and take designs from a ring in mapped host memory, evaluating
// every design start to finish. The host's part here is to keep the ring fed:
//  * submit() queues a request's designs;
//  * a feeder thread copies the tables a design needs (its wavelength points and sorted
//    ray table) into a device table arena once per (seed, size), writes the design's ring
//    record, and publishes ring indices with a release store of `published`;
//  * CTAs claim published indices with a compare-and-swap on a device counter, evaluate,
//    and write each result into the entry's result slot, then its sequence word;
//  * the feeder reads the sequence words, completes requests, and frees ring slots.
// Admission is by histogram memory: the budget is split into slabs of max_cells cells,
// one per resident CTA, and a design is accepted when its W x B cells fit a slab.
// The kernel's only wait (for new work) ends after an idle limit or on the stop word; the
// feeder relaunches the kernel when work is published after every CTA has left.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include "cpd_gpu.cuh"
#include "cpd_host.h"

using namespace cpd;

namespace {

struct LoopReq {
    std::vector<cpd_design> designs;
    std::vector<cpd_batch_item> items;
    std::vector<cpd_fitness> outs;
    uint32_t remaining = 0;
    int status = CPD_OK;
    bool done = false;
    std::chrono::steady_clock::time_point t_submit, t_done;
};

struct Owner {
    uint64_t req = 0;
    uint32_t idx = 0;
    bool busy = false;
};

constexpr uint32_t kLoopQueue = 16384;  // flagged rays a slab queues (more: re-traced inline)

}  // namespace

struct cpd_loop {
    cpd_context *ctx = nullptr;
    int device = 0;
    cudaStream_t kstream = nullptr, cstream = nullptr;
    cudaEvent_t ev_exit = nullptr;
    bool launched = false;
    // mapped host memory (host and device addresses)
    LoopWork *ring = nullptr, *ring_d = nullptr;
    LoopDone *done = nullptr, *done_d = nullptr;
    LoopCtl *ctl = nullptr, *ctl_d = nullptr;
    // device memory
    LoopCounters *cnt = nullptr;
    unsigned char *slabs = nullptr;
    size_t slab_bytes = 0;
    double *lam_arena = nullptr, *z64_arena = nullptr;
    float *z32_arena = nullptr;
    uint64_t lam_cap = 0, ray_cap = 0, lam_used = 0, ray_used = 0;
    std::map<std::pair<uint64_t, uint32_t>, uint64_t> lam_off;  // (seed bits, table length) -> offset
    std::map<std::pair<uint64_t, uint32_t>, std::pair<uint64_t, uint32_t>> ray_off;  // (seed bits, R) -> (offset, Rz)
    uint32_t capacity = 0, grid = 0, max_rows = 0, max_cells = 0, max_B = 0, ray_tile = 64;
    unsigned long long idle_ns = 0;
    std::mutex mu;
    std::condition_variable cv_done, cv_work;
    std::deque<std::pair<uint64_t, uint32_t>> pending;  // (request, design index)
    std::vector<Owner> owner;                            // per ring slot
    uint64_t published = 0, oldest = 0;                  // [oldest, published): maybe in flight
    std::map<uint64_t, LoopReq> reqs;
    uint64_t next_id = 1;
    std::thread feeder;
    bool stop = false;
    int fault = CPD_OK;  // a CUDA error met by the feeder: every request fails with it
    uint64_t designs_done = 0, kernel_launches = 0, table_resets = 0, max_in_flight = 0;
};

namespace {

uint64_t seed_bits(double s)
{
    uint64_t b;
    std::memcpy(&b, &s, 8);
    return b;
}

// Device copies of a design's tables, from the context's caches. Returns CPD_NO_CAPACITY
// when the arena is full (the caller waits for the ring to drain and resets it).
int ensure_tables(cpd_loop *L, const cpd_batch_item &it, uint64_t &lam_o, uint64_t &ray_o, uint32_t &Rz)
{
    const LamPtr lam = context_lam_points(L->ctx, it.seed, it.max_n);
    const uint32_t llen = (uint32_t)lam->size();
    auto lk = L->lam_off.find({seed_bits(it.seed), llen});
    if (lk == L->lam_off.end()) {
        if (L->lam_used + llen > L->lam_cap) return CPD_NO_CAPACITY;
        if (cudaMemcpyAsync(L->lam_arena + L->lam_used, lam->data(), sizeof(double) * llen, cudaMemcpyHostToDevice,
                            L->cstream) != cudaSuccess)
            return CPD_CUDA_ERROR;
        lk = L->lam_off.emplace(std::make_pair(seed_bits(it.seed), llen), L->lam_used).first;
        L->lam_used += llen;
    }
    auto rk = L->ray_off.find({seed_bits(it.seed), it.max_eval});
    if (rk == L->ray_off.end()) {
        const RayTablePtr rt = context_ray_table(L->ctx, it.seed, it.max_eval);
        const uint32_t n = (uint32_t)rt->z64.size();
        const uint64_t span = (n + 1u) & ~1u;  // even: every table starts 16-byte aligned
        if (L->ray_used + span > L->ray_cap) return CPD_NO_CAPACITY;
        if (n && (cudaMemcpyAsync(L->z64_arena + L->ray_used, rt->z64.data(), sizeof(double) * n,
                                  cudaMemcpyHostToDevice, L->cstream) != cudaSuccess ||
                  cudaMemcpyAsync(L->z32_arena + 2 * L->ray_used, rt->z32.data(), 2 * sizeof(float) * n,
                                  cudaMemcpyHostToDevice, L->cstream) != cudaSuccess))
            return CPD_CUDA_ERROR;
        rk = L->ray_off.emplace(std::make_pair(seed_bits(it.seed), it.max_eval), std::make_pair(L->ray_used, n)).first;
        L->ray_used += span;
    }
    lam_o = lk->second;
    ray_o = rk->second.first;
    Rz = rk->second.second;
    return CPD_OK;
}

void fail_all(cpd_loop *L, int e)
{
    L->fault = e;
    for (auto &kv : L->reqs)
        if (!kv.second.done) {
            kv.second.status = e;
            kv.second.done = true;
            kv.second.t_done = std::chrono::steady_clock::now();
        }
    L->pending.clear();
    L->cv_done.notify_all();
}

void launch_loop_kernel(cpd_loop *L)
{
    LoopArgs a;
    std::memset(&a, 0, sizeof(a));
    a.ring = L->ring_d;
    a.done = L->done_d;
    a.ctl = L->ctl_d;
    a.cnt = L->cnt;
    a.capacity = L->capacity;
    a.max_cells = L->max_cells;
    a.max_rows = L->max_rows;
    a.max_B = L->max_B;
    a.qcap = kLoopQueue;
    a.slabs = L->slabs;
    a.slab_bytes = L->slab_bytes;
    a.lam = L->lam_arena;
    a.z64 = L->z64_arena;
    a.z32 = L->z32_arena;
    a.logtab = context_logtab(L->ctx);
    a.idle_ns = L->idle_ns;
    launch_loop(a, L->grid, L->kstream);
}

// The feeder thread (see the file comment). Holds L->mu except while it sleeps.
void loop_feeder(cpd_loop *L)
{
    cudaSetDevice(L->device);
    std::unique_lock<std::mutex> lk(L->mu);
    const uint32_t C = L->capacity;
    for (;;) {
        bool progressed = false;
        // completions (any order). CTAs claim in index order and hold at most `grid` entries
        // at a time, so every finished entry not yet read lies within a few grids of the
        // oldest unfinished one; the rest are read once `oldest` moves past them.
        const uint64_t scan_end = std::min<uint64_t>(L->published, L->oldest + 4ull * L->grid + 64ull);
        for (uint64_t i = L->oldest; i < scan_end; i++) {
            const uint32_t slot = (uint32_t)(i % C);
            Owner &o = L->owner[slot];
            if (!o.busy) continue;
            const unsigned long long seq = __atomic_load_n(&L->done[slot].seq, __ATOMIC_ACQUIRE);
            if (seq != i + 1ull) continue;
            auto it = L->reqs.find(o.req);
            if (it != L->reqs.end()) {
                LoopReq &r = it->second;
                const cpd_batch_item &bi = r.items[o.idx];
                fitness_from_out(L->done[slot].o, (uint64_t)bi.max_n * bi.max_eval, r.outs[o.idx]);
                if (--r.remaining == 0 && !r.done) {
                    r.done = true;
                    r.t_done = std::chrono::steady_clock::now();
                }
            }
            o.busy = false;
            L->designs_done++;
            progressed = true;
        }
        while (L->oldest < L->published && !L->owner[L->oldest % C].busy) L->oldest++;
        if (progressed) L->cv_done.notify_all();
        // publication
        if (!L->fault && !L->pending.empty()) {
            const uint64_t before = L->published;
            bool drained_reset = false;
            while (!L->pending.empty() && L->published - L->oldest < C) {
                const auto [rid, idx] = L->pending.front();
                auto rit = L->reqs.find(rid);
                if (rit == L->reqs.end()) {
                    L->pending.pop_front();
                    continue;
                }
                LoopReq &r = rit->second;
                const cpd_batch_item &it = r.items[idx];
                uint64_t lam_o = 0, ray_o = 0;
                uint32_t Rz = 0;
                int e = ensure_tables(L, it, lam_o, ray_o, Rz);
                if (e == CPD_NO_CAPACITY) {
                    // the table arena is full: reset it once the ring has drained
                    if (L->published == L->oldest && L->published == before && !drained_reset) {
                        L->lam_off.clear();
                        L->ray_off.clear();
                        L->lam_used = L->ray_used = 0;
                        L->table_resets++;
                        drained_reset = true;
                        continue;
                    }
                    break;
                }
                if (e) {
                    fail_all(L, e);
                    break;
                }
                const uint32_t slot = (uint32_t)(L->published % C);
                LoopWork &w = L->ring[slot];
                std::memset(&w, 0, sizeof(w));
                design_to_dev(r.designs[idx], w.d);
                DesignJob &J = w.j;
                J.W = it.max_n;
                J.R = it.max_eval;
                J.Rz = Rz;
                J.B = w.d.B;
                J.lam_off = lam_o;
                J.ray_off = ray_o;
                ff::split(kTScaleInv / (double)J.R, J.unit_hi, J.unit_lo);
                ff::split(-31.0 - std::log2((double)J.R), J.lu_hi, J.lu_lo);
                J.pscale = kTScaleInv / (double)J.R;
                w.mode = CPD_TRACE_HYBRID;
                w.ray_tile = L->ray_tile;
                L->owner[slot] = Owner{rid, idx, true};
                L->published++;
                L->pending.pop_front();
            }
            if (L->published != before) {
                // the tables reach the device before any index that uses them is published
                if (cudaStreamSynchronize(L->cstream) != cudaSuccess) {
                    fail_all(L, CPD_CUDA_ERROR);
                } else {
                    __atomic_store_n(&L->ctl->published, (unsigned long long)L->published, __ATOMIC_RELEASE);
                    progressed = true;
                }
            }
        }
        L->max_in_flight = std::max<uint64_t>(L->max_in_flight, L->published - L->oldest);
        // the kernel: launch it when work is published and every CTA has left
        if (!L->fault && L->published > L->oldest &&
            (!L->launched || cudaEventQuery(L->ev_exit) == cudaSuccess)) {
            LoopCounters c;
            if (cudaMemcpy(&c, L->cnt, sizeof(c), cudaMemcpyDeviceToHost) != cudaSuccess) {
                fail_all(L, CPD_CUDA_ERROR);
            } else if (c.claimed < L->published) {
                __atomic_store_n(&L->ctl->stop, 0u, __ATOMIC_RELEASE);
                launch_loop_kernel(L);
                if (cudaGetLastError() != cudaSuccess || cudaEventRecord(L->ev_exit, L->kstream) != cudaSuccess) {
                    fail_all(L, CPD_CUDA_ERROR);
                } else {
                    L->launched = true;
                    L->kernel_launches++;
                }
            }
        }
        if (L->stop && L->pending.empty() && L->oldest == L->published) break;
        if (!progressed) {
            if (L->published > L->oldest) {
                lk.unlock();
                std::this_thread::sleep_for(std::chrono::microseconds(10));
                lk.lock();
            } else {
                L->cv_work.wait_for(lk, std::chrono::milliseconds(20));
            }
        }
    }
    // drained: tell the CTAs to leave, and wait for them (bounded)
    __atomic_store_n(&L->ctl->stop, 1u, __ATOMIC_RELEASE);
    lk.unlock();
    if (L->launched) {
        const auto t_end = std::chrono::steady_clock::now() + std::chrono::seconds(30);
        while (cudaEventQuery(L->ev_exit) == cudaErrorNotReady && std::chrono::steady_clock::now() < t_end)
            std::this_thread::sleep_for(std::chrono::microseconds(200));
    }
}

bool loop_design_ok(const cpd_loop *L, const cpd_design &d, const cpd_batch_item &it)
{
    return it.max_n <= L->max_rows && (uint64_t)it.max_n * d.bin_count <= L->max_cells && d.bin_count <= L->max_B &&
           (uint64_t)it.max_eval + 2u <= L->ray_cap;
}

}  // namespace

extern "C" {

int cpd_loop_create(cpd_context *ctx, const cpd_loop_config *cfg, cpd_loop **out)
{
    if (!ctx || !out) return CPD_INVALID_ARGUMENT;
    *out = nullptr;
    cpd_loop_config c;
    std::memset(&c, 0, sizeof(c));
    if (cfg) c = *cfg;
    if (!c.hist_budget_bytes) c.hist_budget_bytes = 4ull << 30;
    if (!c.max_cells) c.max_cells = 1u << 20;
    if (!c.max_rows) c.max_rows = 8192;
    if (!c.ring_capacity) c.ring_capacity = 16384;
    if (!c.idle_ms) c.idle_ms = 200;
    if (!c.ray_tile) c.ray_tile = 64;
    if (c.max_rows > CPD_MAX_WAVELENGTHS || c.max_cells < c.max_rows || c.ring_capacity > (1u << 22))
        return CPD_INVALID_ARGUMENT;
    const int dev = context_device(ctx);
    if (cudaSetDevice(dev) != cudaSuccess) return CPD_CUDA_ERROR;
    cpd_loop *L = new cpd_loop();
    L->ctx = ctx;
    L->device = dev;
    L->capacity = c.ring_capacity;
    L->max_rows = c.max_rows;
    L->max_cells = c.max_cells;
    L->max_B = std::min<uint32_t>(CPD_MAX_BINS, c.max_cells);
    L->idle_ns = (unsigned long long)c.idle_ms * 1000000ull;
    L->ray_tile = std::min<uint32_t>(c.ray_tile, 4096);
    const int per_sm = c.ctas_per_sm ? (int)std::min<uint32_t>(c.ctas_per_sm, (uint32_t)loop_ctas_per_sm())
                                     : loop_ctas_per_sm();
    const uint64_t by_budget = c.hist_budget_bytes / (8ull * c.max_cells);
    L->grid = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)context_sms(ctx) * per_sm, by_budget));
    L->slab_bytes = loop_slab_bytes(L->max_rows, L->max_cells, L->max_B, kLoopQueue);
    L->lam_cap = 1ull << 22;  // wavelength points (32 MiB)
    L->ray_cap = 1ull << 24;  // sorted rays (z64 + z32: 256 MiB)
    L->owner.resize(L->capacity);
    auto fail = [&](int e) {
        if (L->ring) cudaFreeHost(L->ring);
        if (L->done) cudaFreeHost(L->done);
        if (L->ctl) cudaFreeHost(L->ctl);
        for (void *p : {(void *)L->cnt, (void *)L->slabs, (void *)L->lam_arena, (void *)L->z64_arena,
                        (void *)L->z32_arena})
            if (p) cudaFree(p);
        if (L->kstream) cudaStreamDestroy(L->kstream);
        if (L->cstream) cudaStreamDestroy(L->cstream);
        if (L->ev_exit) cudaEventDestroy(L->ev_exit);
        delete L;
        return e;
    };
    if (cudaHostAlloc((void **)&L->ring, sizeof(LoopWork) * L->capacity, cudaHostAllocMapped) != cudaSuccess ||
        cudaHostAlloc((void **)&L->done, sizeof(LoopDone) * L->capacity, cudaHostAllocMapped) != cudaSuccess ||
        cudaHostAlloc((void **)&L->ctl, sizeof(LoopCtl), cudaHostAllocMapped) != cudaSuccess ||
        cudaHostGetDevicePointer((void **)&L->ring_d, L->ring, 0) != cudaSuccess ||
        cudaHostGetDevicePointer((void **)&L->done_d, L->done, 0) != cudaSuccess ||
        cudaHostGetDevicePointer((void **)&L->ctl_d, L->ctl, 0) != cudaSuccess)
        return fail(CPD_CUDA_ERROR);
    std::memset(L->ring, 0, sizeof(LoopWork) * L->capacity);
    std::memset(L->done, 0, sizeof(LoopDone) * L->capacity);
    std::memset(L->ctl, 0, sizeof(LoopCtl));
    if (cudaMalloc((void **)&L->cnt, sizeof(LoopCounters)) != cudaSuccess ||
        cudaMalloc((void **)&L->slabs, L->slab_bytes * L->grid) != cudaSuccess ||
        cudaMalloc((void **)&L->lam_arena, sizeof(double) * L->lam_cap) != cudaSuccess ||
        cudaMalloc((void **)&L->z64_arena, sizeof(double) * L->ray_cap) != cudaSuccess ||
        cudaMalloc((void **)&L->z32_arena, 2 * sizeof(float) * L->ray_cap) != cudaSuccess ||
        cudaMemset(L->cnt, 0, sizeof(LoopCounters)) != cudaSuccess ||
        cudaMemset(L->slabs, 0, L->slab_bytes * L->grid) != cudaSuccess ||
        cudaStreamCreateWithFlags(&L->kstream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&L->cstream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&L->ev_exit, cudaEventDisableTiming) != cudaSuccess ||
        cudaDeviceSynchronize() != cudaSuccess)
        return fail(CPD_CUDA_ERROR);
    L->feeder = std::thread(loop_feeder, L);
    *out = L;
    return CPD_OK;
}

int cpd_loop_submit(cpd_loop *L, const cpd_design *designs, const cpd_batch_item *items, uint32_t n,
                    uint32_t trace_mode, uint64_t *request_id)
{
    if (!L || !designs || !items || !request_id || n == 0) return CPD_INVALID_ARGUMENT;
    if (trace_mode != CPD_TRACE_HYBRID) return CPD_INVALID_ARGUMENT;
    for (uint32_t i = 0; i < n; i++) {
        const cpd_design &d = designs[i];
        const cpd_batch_item &it = items[i];
        if (d.nglass < 1 || d.nglass > CPD_MAX_GLASS || d.bin_count < 1 || d.bin_count > CPD_MAX_BINS ||
            it.max_n < 1 || it.max_eval < 1 || it.max_eval > CPD_MAX_RAYS)
            return CPD_INVALID_ARGUMENT;
        if (!loop_design_ok(L, d, it)) return CPD_NO_CAPACITY;
    }
    std::lock_guard<std::mutex> lk(L->mu);
    if (L->stop) return CPD_INVALID_ARGUMENT;
    if (L->fault) return L->fault;
    const uint64_t id = L->next_id++;
    LoopReq &r = L->reqs[id];
    r.designs.assign(designs, designs + n);
    r.items.assign(items, items + n);
    r.outs.resize(n);
    r.remaining = n;
    r.t_submit = std::chrono::steady_clock::now();
    for (uint32_t i = 0; i < n; i++) L->pending.emplace_back(id, i);
    *request_id = id;
    L->cv_work.notify_one();
    return CPD_OK;
}

int cpd_loop_wait(cpd_loop *L, uint64_t request_id, cpd_fitness *outs, double timeout_ms, double *latency_ms)
{
    if (!L || !outs) return CPD_INVALID_ARGUMENT;
    std::unique_lock<std::mutex> lk(L->mu);
    auto it = L->reqs.find(request_id);
    if (it == L->reqs.end()) return CPD_INVALID_ARGUMENT;
    const auto deadline =
        std::chrono::steady_clock::now() + std::chrono::microseconds((int64_t)(std::max(0.0, timeout_ms) * 1000.0));
    while (!it->second.done) {
        if (L->cv_done.wait_until(lk, deadline) == std::cv_status::timeout && !it->second.done) return CPD_TIMEOUT;
        it = L->reqs.find(request_id);
        if (it == L->reqs.end()) return CPD_INVALID_ARGUMENT;
    }
    LoopReq &r = it->second;
    std::memcpy(outs, r.outs.data(), sizeof(cpd_fitness) * r.outs.size());
    if (latency_ms) *latency_ms = std::chrono::duration<double, std::milli>(r.t_done - r.t_submit).count();
    const int status = r.status;
    L->reqs.erase(it);
    return status;
}

int cpd_loop_stats(cpd_loop *L, cpd_loop_report *out)
{
    if (!L || !out) return CPD_INVALID_ARGUMENT;
    std::memset(out, 0, sizeof(*out));
    LoopCounters c;
    std::memset(&c, 0, sizeof(c));
    {
        std::lock_guard<std::mutex> lk(L->mu);
        out->designs_done = L->designs_done;
        out->kernel_launches = L->kernel_launches;
        out->max_designs_in_flight = L->max_in_flight;
        out->pending_designs = L->pending.size();
        out->table_resets = L->table_resets;
        out->ctas = L->grid;
        out->slab_bytes = L->slab_bytes;
    }
    // the device counters, read on the copy stream while the kernel may run
    cudaSetDevice(L->device);
    if (cudaMemcpyAsync(&c, L->cnt, sizeof(c), cudaMemcpyDeviceToHost, L->cstream) != cudaSuccess ||
        cudaStreamSynchronize(L->cstream) != cudaSuccess)
        return CPD_CUDA_ERROR;
    out->device_designs = c.designs;
    out->idle_exits = c.idle_exits;
    out->stop_exits = c.stop_exits;
    out->inline_retraced = c.inline_retraced;
    return CPD_OK;
}

void cpd_loop_destroy(cpd_loop *L)
{
    if (!L) return;
    {
        std::lock_guard<std::mutex> lk(L->mu);
        L->stop = true;
        L->cv_work.notify_all();
    }
    if (L->feeder.joinable()) L->feeder.join();
    cudaSetDevice(L->device);
    cudaStreamSynchronize(L->kstream);
    cudaStreamSynchronize(L->cstream);
    cudaFreeHost(L->ring);
    cudaFreeHost(L->done);
    cudaFreeHost(L->ctl);
    for (void *p : {(void *)L->cnt, (void *)L->slabs, (void *)L->lam_arena, (void *)L->z64_arena, (void *)L->z32_arena})
        cudaFree(p);
    cudaStreamDestroy(L->kstream);
    cudaStreamDestroy(L->cstream);
    cudaEventDestroy(L->ev_exit);
    delete L;
}

}  // extern "C"
