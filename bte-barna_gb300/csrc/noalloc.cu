// noalloc.cu - bte_rta_run_noalloc: the production grid particle loop with
// no device allocation during the call.
//
// Who needs it: callers that cannot call cudaMalloc when they run the loop --
// a host framework that owns every device allocation through its own pool
// and forbids others, or a loop that must not reach the driver's allocator
// (whose calls can synchronise the device and take unbounded time).  They
// hand in a device buffer for the tallies and get the counters back in host
// memory.  The call synchronises the context's stream before it returns.
//
// The kernel's scratch (work counter, event counters, error word and the
// time grid) lives in one file-scope device array of fixed size instead of
// per-context allocations; every GPU that loads this library holds it until
// the process exits.  Limits and rules:
//   * at most BTE_NOALLOC_MAX_BINS time bins per run;
//   * the context must already hold the tables for these parameters: load
//     the mode table and geometry and run bte_rta_run once with the same T0
//     and source (and, for the initial source, the same N and seed);
//   * every call shares the one array: the call clears the counters, error
//     word and work counter and rewrites the time grid, so results never
//     depend on an earlier call, but calls that overlap on the GPU (on
//     several streams or threads at once) race and must be serialised;
//   * the first call on a device looks up the array's device address with
//     cudaGetSymbolAddress (set-up, once per device); every call
//     synchronises its stream, so none can be recorded in a stream
//     capture.  The address is kept for the life of the
//     process and never looked up again, so a process that calls
//     cudaDeviceReset must not use this entry point on that device after it.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/btegpu.h"
#include "kernels.h"

namespace bte {
bte_status prepared_grid_run(bte_ctx* c, const bte_rta_params* p, PreparedRun* r, std::string* why);
void set_ctx_error(bte_ctx* c, const std::string& m);
}  // namespace bte

namespace {

constexpr int kHeaderBytes = 256;  // counters (8 x u64), error word (4 x int), work counter
constexpr size_t kScratchBytes = kHeaderBytes + sizeof(double) * (2 * BTE_NOALLOC_MAX_BINS + 1);

// The scratch of every allocation-free call.  Host code must not use the
// symbol as an address; it asks the runtime for the device address below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
unsigned char* g_scratch_addr[kMaxDevices] = {nullptr};

// Device address of the scratch on `device` (which must be current); looked
// up once per device, on the first call there, and kept.
bool scratch_address(int device, unsigned char** out, std::string* why) {
    if (device < 0 || device >= kMaxDevices) {
        *why = "device ordinal beyond the allocation-free path's table";
        return false;
    }
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[device]) {
        void* ptr = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || !ptr) {
            *why = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e);
            return false;
        }
        g_scratch_addr[device] = static_cast<unsigned char*>(ptr);
    }
    *out = g_scratch_addr[device];
    return true;
}

// The time grid of src/RTA_MC2D.cpp:2118-2124 (LinSpaced: i * step, the
// last point exactly maxtime) and its ntime - 1 bin widths after it, written
// into the scratch.
__device__ __forceinline__ double noalloc_point(int i, int ntime, double maxtime, double step) {
    return (i == ntime - 1) ? maxtime : 0.0 + double(i) * step;
}
__global__ void noalloc_time_grid(double* grid, int ntime, double maxtime, double step) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < ntime) grid[i] = noalloc_point(i, ntime, maxtime, step);
    if (i + 1 < ntime)
        grid[ntime + i] = noalloc_point(i + 1, ntime, maxtime, step) - noalloc_point(i, ntime, maxtime, step);
}

bte_status fail(bte_ctx* c, bte_status s, const std::string& m) {
    bte::set_ctx_error(c, m);
    return s;
}

}  // namespace

extern "C" bte_status bte_rta_run_noalloc(bte_ctx* ctx, const bte_rta_params* params,
                                          double* d_tally, bte_rta_result* out) {
    if (!ctx || !params || !d_tally || !out) return BTE_ERR_INPUT;
    std::string why;
    bte::PreparedRun r;
    const bte_status st = bte::prepared_grid_run(ctx, params, &r, &why);
    if (st != BTE_OK) return fail(ctx, st, why);
    if (r.nbins > BTE_NOALLOC_MAX_BINS) {
        char m[160];
        std::snprintf(m, sizeof m, "%d time bins exceed the allocation-free limit of %d",
                      r.nbins, BTE_NOALLOC_MAX_BINS);
        return fail(ctx, BTE_ERR_INPUT, m);
    }
    if (cudaSetDevice(r.device) != cudaSuccess) return fail(ctx, BTE_ERR_CUDA, "cudaSetDevice failed");
    unsigned char* base = nullptr;
    if (!scratch_address(r.device, &base, &why)) return fail(ctx, BTE_ERR_CUDA, why);
    auto* counters = reinterpret_cast<unsigned long long*>(base);
    auto* err = reinterpret_cast<int*>(base + 64);
    auto* work = reinterpret_cast<unsigned long long*>(base + 128);
    auto* grid = reinterpret_cast<double*>(base + kHeaderBytes);
    cudaStream_t s = r.stream;
    const size_t tally_bytes = size_t(3) * size_t(r.nboxes) * size_t(r.nbins) * sizeof(double);
    // everything that must start at zero is cleared on every call
    if (cudaMemsetAsync(base, 0, kHeaderBytes, s) != cudaSuccess ||
        cudaMemsetAsync(d_tally, 0, tally_bytes, s) != cudaSuccess)
        return fail(ctx, BTE_ERR_CUDA, "cudaMemsetAsync failed (is d_tally a device pointer?)");
    noalloc_time_grid<<<(r.ntime + 255) / 256, 256, 0, s>>>(grid, r.ntime, r.maxtime, r.step);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(ctx, BTE_ERR_CUDA, std::string("time grid launch: ") + cudaGetErrorString(e));
    r.T.timegrid = grid;
    if (cudaEventRecord(r.ev0, s) != cudaSuccess) return fail(ctx, BTE_ERR_CUDA, "cudaEventRecord failed");
    if (!bte::launch_prod_grid(r.T, r.A, d_tally, counters, err, work, r.tune, r.nsm, s))
        return fail(ctx, BTE_ERR_INPUT, "tuning not supported by the grid kernel");
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(ctx, BTE_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
    if (cudaEventRecord(r.ev1, s) != cudaSuccess) return fail(ctx, BTE_ERR_CUDA, "cudaEventRecord failed");
    unsigned long long hc[8];
    int herr[4];
    if (cudaMemcpyAsync(hc, counters, sizeof hc, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaMemcpyAsync(herr, err, sizeof herr, cudaMemcpyDeviceToHost, s) != cudaSuccess)
        return fail(ctx, BTE_ERR_CUDA, "cudaMemcpyAsync failed");
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(ctx, BTE_ERR_CUDA, std::string("kernel: ") + cudaGetErrorString(e));
    float ms = 0.f;
    e = cudaEventElapsedTime(&ms, r.ev0, r.ev1);
    if (e != cudaSuccess) return fail(ctx, BTE_ERR_CUDA, std::string("cudaEventElapsedTime: ") + cudaGetErrorString(e));
    if (herr[0] != 0) {
        const long long pid = (long long)herr[1] | ((long long)herr[2] << 31);
        char m[160];
        std::snprintf(m, sizeof m, "particle %lld: device error %d", pid, herr[0]);
        return fail(ctx, bte_status(herr[0]), m);
    }
    out->nboxes = r.nboxes;
    out->nbins = r.nbins;
    out->Eeff = r.Eeff;
    out->energy_rate = r.energy;
    out->events = (int64_t)hc[0];
    out->wall_hits = (int64_t)hc[1];
    out->crossings = (int64_t)hc[2];
    out->absorbed = (int64_t)hc[3];
    out->specular_hits = (int64_t)hc[4];
    out->tally_updates = (int64_t)hc[7];
    out->translations = 0;
    out->kernel_ms = ms;
    return BTE_OK;
}
