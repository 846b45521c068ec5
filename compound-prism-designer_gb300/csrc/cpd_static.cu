// cpd_static.cu -- a fitness entry point that allocates no device memory.
//
// Some callers cannot allocate device memory themselves. Examples:
// * a host application that owns the GPU's memory budget and forbids plug-in libraries
//   from calling cudaMalloc;
// * a latency-critical loop that must not take the device-wide synchronisation a
//   cudaMalloc/cudaFree can imply.
// cpd_fitness_gpu_points_static serves them. It runs the same kernels as
// cpd_fitness_gpu_points, with every intermediate buffer carved out of one file-scope
// device array of fixed size (limits below). The caller passes host inputs and outputs
// only, and no context is needed. Every call resolves the array's address in the
// current context (cudaGetSymbolAddress) and uploads the log2 table with its inputs, so a
// call made after a cudaDeviceReset, or from another driver context on the same GPU, finds
// a valid array with the table in it. Calls share the array, which keeps the last call's
// contents; each call clears what must start at zero. Calls that overlapped on the GPU
// would race on it, so calls from threads of one process are serialised per device; the
// work runs on the legacy default stream, and the call returns when it is done.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>

#include "cpd_gpu.cuh"
#include "cpd_host.h"

namespace cpd {
namespace {

// Limits of one call (the scratch array is sized for them).
constexpr uint32_t kStaticMaxW = 1024;    // wavelengths
constexpr uint32_t kStaticMaxR = 4096;    // rays per wavelength
constexpr uint32_t kStaticMaxB = 128;     // detector bins
constexpr uint32_t kStaticQueue = 32768;  // guard-band rays re-traced in one call

constexpr size_t al256(size_t x) { return (x + 255) & ~size_t(255); }
constexpr size_t kOffDesign = 0;
constexpr size_t kOffJob = kOffDesign + al256(sizeof(DevDesign));
constexpr size_t kOffCtl = kOffJob + al256(sizeof(DesignJob));
constexpr size_t kOffAcc = kOffCtl + al256(sizeof(Control));
constexpr size_t kOffOut = kOffAcc + al256(sizeof(DesignAcc));
constexpr size_t kOffS1 = kOffOut + al256(sizeof(DesignOut));
constexpr size_t kOffS2 = kOffS1 + al256(8 * kStaticMaxB);
constexpr size_t kOffLog = kOffS2 + al256(8 * kStaticMaxB);
constexpr size_t kOffLam = kOffLog + al256(sizeof(float) * 4 * ff::kLogTable);
constexpr size_t kOffZ64 = kOffLam + al256(8 * kStaticMaxW);
constexpr size_t kOffZ32 = kOffZ64 + al256(8 * kStaticMaxR);
constexpr size_t kOffLp = kOffZ32 + al256(8 * kStaticMaxR);
constexpr size_t kOffLx = kOffLp + al256(sizeof(LamParams) * kStaticMaxW);
constexpr size_t kOffHist = kOffLx + al256(sizeof(LamDF) * kStaticMaxW);
constexpr size_t kOffPout = kOffHist + al256(8 * (size_t)kStaticMaxW * kStaticMaxB);
constexpr size_t kOffQueue = kOffPout + al256(8 * (size_t)kStaticMaxW * kStaticMaxB);
constexpr size_t kScratchBytes = kOffQueue + al256(sizeof(QEntry) * kStaticQueue);  // about 3 MiB

// The scratch array. Every GPU that loads this library holds one copy until exit.
// In host code `g_scratch` is only a handle for cudaGetSymbolAddress, never a device
// address: the kernels receive the address that call returns.
static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

// One upload per call: design | job | log2 table | wavelength points | z64 | z32, at the
// offsets they have in the array (kOffDesign .. kOffLog, then kOffLam .. kOffZ32 as one
// contiguous span).
constexpr size_t kUpHead = kOffLog + sizeof(float) * 4 * ff::kLogTable;  // design, job, table
constexpr size_t kUpTail = kOffLp - kOffLam;                             // lam, z64, z32

// Host-side state of one device: the call lock and fixed staging storage (file-scope, no
// allocation; used only under `call`).
struct DeviceState {
    std::mutex call;  // one call at a time per device within this process
    int sms = 0;
    double z64[kStaticMaxR];
    alignas(256) unsigned char head[kUpHead];
    alignas(256) unsigned char tail[kUpTail];
};
constexpr int kMaxDevices = 16;
DeviceState g_dev[kMaxDevices];

// The scratch array's device address in the current context. Resolved on every call (a
// host-side lookup): after a cudaDeviceReset the module is loaded again, and another
// driver context on the same GPU has its own copy of the array.
int static_base(int dev, DeviceState &st, unsigned char *&base)
{
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_scratch) != cudaSuccess || !p) return CPD_CUDA_ERROR;
    if (st.sms == 0 && cudaDeviceGetAttribute(&st.sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return CPD_CUDA_ERROR;
    base = static_cast<unsigned char *>(p);
    return CPD_OK;
}

}  // namespace
}  // namespace cpd

using namespace cpd;

extern "C" int cpd_fitness_gpu_points_static(const cpd_design *d, const double *lam_u, uint32_t W,
                                             const double *ray_u, uint32_t R, uint32_t trace_mode,
                                             cpd_fitness *out, double *p_out)
{
    if (!d || !lam_u || !ray_u || !out || W == 0 || R == 0 || trace_mode > CPD_TRACE_FP64) return CPD_INVALID_ARGUMENT;
    if (d->nglass < 1 || d->nglass > CPD_MAX_GLASS || d->bin_count < 1) return CPD_INVALID_ARGUMENT;
    if (W > kStaticMaxW || R > kStaticMaxR || d->bin_count > kStaticMaxB) return CPD_NO_CAPACITY;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return CPD_CUDA_ERROR;
    if (dev < 0 || dev >= kMaxDevices) return CPD_INVALID_ARGUMENT;
    DeviceState &st = g_dev[dev];
    std::lock_guard<std::mutex> lk(st.call);
    unsigned char *b = nullptr;
    int e = static_base(dev, st, b);
    if (e) return e;

    // host-side tables in the device's fixed staging storage (no allocation)
    double *z64 = reinterpret_cast<double *>(st.tail + (kOffZ64 - kOffLam));
    float *z32 = reinterpret_cast<float *>(st.tail + (kOffZ32 - kOffLam));
    uint32_t Rz = 0;
    for (uint32_t j = 0; j < R; j++) {
        const double z = norminv(ray_u[j]);
        if (std::isfinite(z)) st.z64[Rz++] = z;
    }
    std::sort(st.z64, st.z64 + Rz);
    for (uint32_t j = 0; j < Rz; j++) {
        z64[j] = st.z64[j];
        z32[2 * j] = (float)z64[j];
        z32[2 * j + 1] = (float)(z64[j] - (double)z32[2 * j]);
    }
    std::memcpy(st.tail, lam_u, 8 * (size_t)W);
    DevDesign &D = *reinterpret_cast<DevDesign *>(st.head + kOffDesign);
    design_to_dev(*d, D);
    DesignJob &J = *reinterpret_cast<DesignJob *>(st.head + kOffJob);
    std::memset(&J, 0, sizeof(J));
    const uint32_t ray_tile = 32;
    J.W = W;
    J.R = R;
    J.Rz = Rz;
    J.B = D.B;
    J.nchunk = std::max<uint32_t>(1u, (Rz + ray_tile - 1) / ray_tile);
    J.tile_rows = std::max<uint32_t>(1u, kTileCells / J.B);
    J.ntiles = (W + J.tile_rows - 1) / J.tile_rows;
    ff::split(kTScaleInv / (double)R, J.unit_hi, J.unit_lo);
    ff::split(-31.0 - std::log2((double)R), J.lu_hi, J.lu_lo);
    J.pscale = kTScaleInv / (double)R;
    ff::make_log_table(reinterpret_cast<float *>(st.head + kOffLog));

    // The array keeps the previous call's contents: everything that must start at zero is
    // cleared. The control words, accumulators and results lie between the job and the log2
    // table, so the head upload carries their zeros; the histogram is cleared on the device.
    std::memset(st.head + kOffCtl, 0, kOffLog - kOffCtl);
    const size_t cells = (size_t)W * D.B;
    const size_t tail_bytes = (kOffZ32 - kOffLam) + 8 * (size_t)Rz;
    if (cudaMemcpy(b, st.head, kUpHead, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(b + kOffLam, st.tail, tail_bytes, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(b + kOffHist, 0, 8 * cells) != cudaSuccess)
        return CPD_CUDA_ERROR;

    LaunchArgs a;
    std::memset(&a, 0, sizeof(a));
    a.designs = reinterpret_cast<const DevDesign *>(b + kOffDesign);
    a.jobs = reinterpret_cast<const DesignJob *>(b + kOffJob);
    a.njobs = 1;
    a.total_rows = W;
    a.total_items = (uint64_t)((W + 31) / 32) * J.nchunk;
    a.total_tiles = J.ntiles;
    a.lam_u = reinterpret_cast<const double *>(b + kOffLam);
    a.z64 = reinterpret_cast<const double *>(b + kOffZ64);
    a.z32 = reinterpret_cast<const float *>(b + kOffZ32);
    a.lp = reinterpret_cast<LamParams *>(b + kOffLp);
    a.lx = reinterpret_cast<LamDF *>(b + kOffLx);
    a.hist = reinterpret_cast<unsigned long long *>(b + kOffHist);
    a.S1 = reinterpret_cast<unsigned long long *>(b + kOffS1);
    a.S2 = reinterpret_cast<unsigned long long *>(b + kOffS2);
    a.acc = reinterpret_cast<DesignAcc *>(b + kOffAcc);
    a.out = reinterpret_cast<DesignOut *>(b + kOffOut);
    a.ctl = reinterpret_cast<Control *>(b + kOffCtl);
    a.queue = reinterpret_cast<QEntry *>(b + kOffQueue);
    a.qcap = kStaticQueue;
    a.ray_tile = ray_tile;
    a.stage_cap = Rz <= kStageRays ? Rz : 0u;
    a.mode = trace_mode;
    a.max_B = J.B;
    if (trace_mode == CPD_TRACE_FP32) {
        a.guards = no_guards();
        a.yguard_rel = 0.0;
    } else {
        a.guards = default_guards();
        a.yguard_rel = kYGuardRel;
    }
    a.p_out = p_out ? reinterpret_cast<double *>(b + kOffPout) : nullptr;
    a.logtab = reinterpret_cast<const float *>(b + kOffLog);
    launch_pass(a, st.sms, 8, 0);
    if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(0) != cudaSuccess) return CPD_CUDA_ERROR;

    Control ctl;
    DesignOut o;
    if (cudaMemcpy(&ctl, b + kOffCtl, sizeof(ctl), cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(&o, b + kOffOut, sizeof(o), cudaMemcpyDeviceToHost) != cudaSuccess)
        return CPD_CUDA_ERROR;
    if (ctl.overflow || ctl.queue_count > kStaticQueue) return CPD_NO_CAPACITY;
    if (p_out && cudaMemcpy(p_out, b + kOffPout, 8 * cells, cudaMemcpyDeviceToHost) != cudaSuccess)
        return CPD_CUDA_ERROR;
    std::memset(out, 0, sizeof(*out));
    out->size = d->size;
    out->deviation = d->deviation;
    out->info = o.info;
    out->h_cond = o.h_cond;
    out->h_det = o.h_det;
    out->max_sem = o.max_sem;
    out->rays = (uint64_t)W * R;
    out->hits = o.hits;
    out->retraced = o.retraced;
    out->fast_rays = o.fast;
    out->wavelengths = (uint32_t)o.rows;
    out->status = CPD_OK;
    return CPD_OK;
}
