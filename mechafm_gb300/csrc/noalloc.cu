// noalloc.cu — mafm_run_batch_noalloc: the batched FP32C relaxation for
// callers that must not have the library allocate device memory.
//
// Some callers cannot let a library call cudaMalloc or cudaFree: applications
// that hand all device memory to their own pool or caching allocator and cap
// it, pipelines that cannot afford the implicit device-wide synchronisation of
// cudaFree or the latency of a first-touch allocation in their steady state,
// and hosts that account for every byte on a shared GPU.  For them this entry
// point keeps the relax kernel's scratch (the persistent work-queue counters
// and the per-scan descriptors) in a fixed device array that is part of the
// loaded library, so a call allocates nothing.  The caller still provides the
// scans (created once, beforehand, with mafm_scan_create) and the output
// buffers in device memory.
//
// The array is shared by every call on a device and keeps the last call's
// contents; each call clears the counters it needs at zero before the launch.
// Two calls whose work overlaps on the GPU (different streams, no ordering
// between them) race on the array and corrupt each other's results: order
// such calls on one stream or with events.
#include <cstring>
#include <mutex>
#include <vector>

#include "mafm_internal.h"

namespace mafm {
namespace {

// Scratch layout: RunCounters at offset 0, the BatchScan list at offset 256.
constexpr size_t kCountersBytes = 256;
constexpr size_t kScratchBytes = kCountersBytes + (size_t)MAFM_NOALLOC_MAX_SCANS * sizeof(BatchScan);
static_assert(sizeof(RunCounters) <= kCountersBytes, "counters fit their slot");

// Held by every GPU that loads the library until the process exits.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// Device address of g_noalloc_scratch, looked up once per device.  In host
// code the symbol's name denotes a host-side stand-in, not a device address,
// so kernels get this address instead.
void* scratch_address(int device) {
    static std::mutex mu;
    static std::vector<void*> addr;
    std::lock_guard<std::mutex> lock(mu);
    if ((int)addr.size() <= device) addr.resize((size_t)device + 1, nullptr);
    if (!addr[device]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            fail(MAFM_E_CUDA, "cudaGetSymbolAddress of the scratch array failed: %s",
                 cudaGetErrorString(e));
        addr[device] = p;
    }
    return addr[device];
}

// Up to four descriptors per launch travel as a kernel parameter.
struct DescChunk {
    BatchScan b[4];
    int n;
};

__global__ void store_descriptors(BatchScan* dst, DescChunk c) {
    for (int i = 0; i < c.n; ++i) dst[i] = c.b[i];
}

// Device (or managed) memory of the given GPU: the kernel writes the points
// there directly, so an output on another GPU, or in host memory, is refused.
bool on_device(const void* p, int device) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (a.type == cudaMemoryTypeManaged) return true;
    return a.type == cudaMemoryTypeDevice && a.device == device;
}

}  // namespace
}  // namespace mafm

using namespace mafm;

extern "C" int mafm_run_batch_noalloc(mafm_scan* const* scans, int32_t n_scans,
                                      const mafm_run_opts* opts, mafm_point* const* outs,
                                      mafm_run_stats* stats, void* stream) {
    return guarded([&] {
        if (!scans || !outs || n_scans <= 0) fail(MAFM_E_INVALID, "empty batch");
        if (n_scans > MAFM_NOALLOC_MAX_SCANS)
            fail(MAFM_E_RANGE, "mafm_run_batch_noalloc takes at most %d scans per call, got %d",
                 MAFM_NOALLOC_MAX_SCANS, n_scans);
        if (opts && opts->precision != MAFM_FP32C)
            fail(MAFM_E_UNSUPPORTED, "mafm_run_batch_noalloc runs MAFM_FP32C only");
        if (opts && (opts->col_begin || opts->col_end))
            fail(MAFM_E_INVALID, "mafm_run_batch_noalloc relaxes whole scans");
        if (!scans[0]) fail(MAFM_E_INVALID, "null scan 0");
        const int device = scan_device(scans[0]);
        cuda_check(cudaSetDevice(device), "cudaSetDevice");
        long long total_cols = 0;
        int max_terms = 0;
        for (int i = 0; i < n_scans; ++i) {
            if (!scans[i] || !outs[i]) fail(MAFM_E_INVALID, "null scan or output %d", i);
            if (scan_device(scans[i]) != device) fail(MAFM_E_INVALID, "scans of one call must share a device");
            if (!on_device(outs[i], device))
                fail(MAFM_E_INVALID, "output %d is not device memory of GPU %d; this entry point "
                                     "copies nothing", i, device);
            if (!scan_fp32_ready(scans[i]))
                fail(MAFM_E_INVALID, "scan %d uses a rigid grid whose FP32 copy is not built yet: "
                                     "relax it once with mafm_run (MAFM_FP32C) first", i);
            total_cols += scan_columns(scans[i]);
            max_terms = max_terms > scan_direct_terms(scans[i]) ? max_terms : scan_direct_terms(scans[i]);
        }
        const Relax32Config cfg = relax32_config(total_cols, max_terms, opts, n_scans);
        cudaStream_t st = (cudaStream_t)stream;
        unsigned char* base = static_cast<unsigned char*>(scratch_address(device));
        RunCounters* ctr = reinterpret_cast<RunCounters*>(base);
        BatchScan* list = reinterpret_cast<BatchScan*>(base + kCountersBytes);
        long long tiles = 0;
        DescChunk chunk{};
        int at = 0;
        for (int i = 0; i < n_scans; ++i) {
            BatchScan b = scan_batch_entry(scans[i], outs[i]);
            b.tile_begin = tiles;
            tiles += ((long long)b.col_end + cfg.cols_per_tile - 1) / cfg.cols_per_tile;
            chunk.b[chunk.n++] = b;
            if (chunk.n == 4 || i == n_scans - 1) {
                store_descriptors<<<1, 1, 0, st>>>(list + at, chunk);
                at += chunk.n;
                chunk.n = 0;
            }
        }
        cuda_check(cudaGetLastError(), "store descriptors");
        cuda_check(cudaMemsetAsync(ctr, 0, sizeof(RunCounters), st), "clear counters");
        cuda_check(launch_relax32(list, n_scans, tiles, cfg, ctr, st), "relax32 launch");
        // The counters hold the device error word (watchdog, grid exit, staging
        // timeout): read them on every call, so that a failed relaxation is
        // reported whether or not the caller asked for statistics.
        RunCounters c{};
        cuda_check(cudaMemcpyAsync(&c, ctr, sizeof c, cudaMemcpyDeviceToHost, st), "read counters");
        cuda_check(cudaStreamSynchronize(st), "relax");
        if (stats) {
            std::memset(stats, 0, sizeof *stats);
            stats->total_steps = c.total_steps;
            stats->force_evals = c.force_evals;
            stats->pair_evals = c.pair_evals;
            stats->error_word = c.error_word;
        }
        check_run_errors(c);
    });
}
