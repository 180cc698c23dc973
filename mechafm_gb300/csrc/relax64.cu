// relax64.cu — the plain FP64 GPU path (precision MAFM_FP64).
//
// One thread per pixel column, columns handed out by a global atomic counter.
// Every floating-point expression keeps the reference's operation order and
// this translation unit is compiled with -fmad=false, so no a*b+c is fused:
// with LJ and Coulomb terms the results are bit-identical to the reference's
// x86-64 build (division and square root are correctly rounded in both; exp
// in the Morse term may differ in the last bit).
//
// Reference correspondence (src/):
//   vdW / Coulomb terms        interactions.cpp:15-51
//   tip–dummy terms            interactions.cpp:252-266, simulation.cpp:503-515
//   trilinear grid lookup      force_grid.cpp:88-275
//   integrators                integrators.cpp:8-111
//   FIRE / SD / convergence    minimiser.cpp:15-129
//   pixel column, z descent    simulation.cpp:93-122, system.cpp:28-51, 139-162
//   rigid grid build           simulation.cpp:420-501
#include "relax64_dev.cuh"

namespace mafm {
namespace {

// Stage the terms into shared memory when they fit.
__device__ const AtomRec64* stage64(const ScanParams& p, AtomRec64* sm, int cap) {
    if (p.n_terms_direct <= cap) {
        for (int i = threadIdx.x; i < p.n_terms_direct; i += blockDim.x) sm[i] = p.atoms64[i];
        __syncthreads();
        return sm;
    }
    return p.atoms64;
}

__global__ void __launch_bounds__(128) relax64_kernel(const ScanParams p, mafm_point* out,
                                                      RunCounters* ctr, int col_begin,
                                                      int col_end, int smem_cap) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const AtomRec64* atoms = stage64(p, reinterpret_cast<AtomRec64*>(smem_raw), smem_cap);
    Eval64 ev{p, atoms, p.n_terms_direct, p.ts_mode, 0u, 0ull};
    long long steps = 0;
    unsigned long long evals = 0;
    unsigned status_or = 0;
    for (;;) {
        const long long c = (long long)atomicAdd(&ctr->next_work, 1ull) + col_begin;
        if (c >= col_end) break;
        relax_column_t<double>(ev, p, c, out + (size_t)(c - col_begin) * p.nz, true, false, steps, evals,
                       status_or);
    }
    atomicAdd(&ctr->total_steps, (unsigned long long)steps);
    atomicAdd(&ctr->force_evals, evals);
    atomicAdd(&ctr->pair_evals, ev.pairs);
    if (status_or | ev.err) atomicOr(&ctr->error_word, status_or | ev.err);
}

// FP64 relaxation of listed columns (scan << 32 | column), one warp per
// column: the re-relaxation of the double-float kernel's near-tie columns
// (replace = true), or a plain FP64 run of chosen columns.  Persistent: each
// warp takes the next listed column and relaxes it from its top height with
// EvalWarp64, which forms every sum exactly as relax64_kernel does, so the
// column holds the plain FP64 kernel's bits.  A replacement corrects the step
// total by the difference; force and pair evaluations count every pass.
__global__ void __launch_bounds__(128) repair64_kernel(const BatchScan* __restrict__ scans,
                                                       const unsigned long long* __restrict__ list,
                                                       unsigned cap, long long n_fixed,
                                                       bool replace, bool list_out,
                                                       RunCounters* ctr) {
    extern __shared__ __align__(32) unsigned char rraw[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    Node64* buf = reinterpret_cast<Node64*>(rraw) + (size_t)warp * 2 * kWarpChunk;
    const unsigned long long count =
        n_fixed >= 0 ? (unsigned long long)n_fixed : (unsigned long long)ctr->n_tie;
    const unsigned long long listed = min(count, (unsigned long long)cap);
    long long steps = 0;
    unsigned long long evals = 0, pairs = 0;
    unsigned status_or = 0, err = 0;
    for (;;) {
        unsigned long long t = 0;
        if (lane == 0) t = atomicAdd(&ctr->repair_next, 1ull);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= listed) break;
        const unsigned long long e = list[t];
        const BatchScan& B = scans[(int)(e >> 32)];
        const long long c = (long long)(unsigned)(e & 0xffffffffull);
        const ScanParams& p = B.p;
        EvalWarp64 ev{p, p.atoms64, p.n_terms_direct, p.ts_mode, lane, buf, B.n_pairs_per_eval, 0u, 0ull};
        mafm_point* o = B.out + (size_t)(list_out ? (long long)t : c - B.col_begin) * p.nz;
        relax_column_t<double>(ev, p, c, o, lane == 0, replace, steps,
                       evals, status_or);
        pairs += ev.pairs;
        err |= ev.err;
        __syncwarp();
    }
    if (lane == 0) {
        atomicAdd(&ctr->total_steps, (unsigned long long)steps);
        atomicAdd(&ctr->force_evals, evals);
        atomicAdd(&ctr->pair_evals, pairs);
        if (status_or | err) atomicOr(&ctr->error_word, status_or | err);
    }
}

__global__ void sample64_kernel(const ScanParams p, int what, const double* pts, long long n,
                                double* out, RunCounters* ctr) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Eval64 ev{p, p.atoms64, p.n_terms_direct, p.ts_mode, 0u, 0ull};
    V3 tip = {pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]};
    V3 F = {0, 0, 0};
    double E = 0;
    int outside = 0;
    if (what == 1) {
        if (p.es.g64) interp64(p.es, tip, F, E, outside, ev.err);
    } else {
        ev.ts(tip, F, E, outside);
    }
    out[4 * i] = F.x; out[4 * i + 1] = F.y; out[4 * i + 2] = F.z; out[4 * i + 3] = E;
    if (ev.err) atomicOr(&ctr->error_word, ev.err);
}

// Simulation::buildTipGridInteractions: one thread per node, the tip-surface
// terms (and the external field) evaluated with the tip on the node.
__global__ void __launch_bounds__(128) grid_build64_kernel(const ScanParams p, const GridView g,
                                                           Node64* out, int smem_cap,
                                                           RunCounters* ctr) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const AtomRec64* atoms = stage64(p, reinterpret_cast<AtomRec64*>(smem_raw), smem_cap);
    Eval64 ev{p, atoms, p.n_terms_direct, p.es.g64 ? 1 : 0, 0u, 0ull};
    const long long total = (long long)g.n[0] * g.n[1] * g.n[2];
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(idx % g.n[2]);
        const long long ij = idx / g.n[2];
        const int j = (int)(ij % g.n[1]), i = (int)(ij / g.n[1]);
        double x, y;
        dummy_xy_t<double>(p, p.tip_pbc != 0, i * g.basis[0] + g.origin[0],
                           j * g.basis[4] + g.origin[1], x, y);
        V3 tip = {x, y, k * g.basis[8] + g.origin[2]};
        V3 F;
        double E;
        int outside = 0;
        ev.ts(tip, F, E, outside);
        out[idx] = Node64{F.x, F.y, F.z, E};
    }
    if (ev.err) atomicOr(&ctr->error_word, ev.err);
}

int smem_cap64(int bytes_limit) { return bytes_limit / (int)sizeof(AtomRec64); }

}  // namespace

static size_t smem_bytes64(const ScanParams& p, int& cap) {
    const int limit = 96 * 1024;
    cap = smem_cap64(limit);
    const int n = p.n_terms_direct;
    return n <= cap ? (size_t)n * sizeof(AtomRec64) : 0;
}

cudaError_t launch_relax64(const ScanParams& p, mafm_point* out, RunCounters* ctr, int col_begin,
                           int col_end, cudaStream_t s) {
    int cap;
    size_t sm = smem_bytes64(p, cap);
    cudaError_t e = cudaFuncSetAttribute(relax64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         96 * 1024);
    if (e != cudaSuccess) return e;
    const long long cols = (long long)col_end - col_begin;
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, relax64_kernel, 128, sm);
    if (per_sm <= 0) per_sm = 1;
    long long blocks = (long long)sm_count() * per_sm;
    const long long need = (cols + 127) / 128;
    if (blocks > need) blocks = need;
    if (blocks < 1) blocks = 1;
    relax64_kernel<<<(unsigned)blocks, 128, sm, s>>>(p, out, ctr, col_begin, col_end, cap);
    return cudaGetLastError();
}

cudaError_t launch_repair64(const BatchScan* scans, const unsigned long long* list, unsigned cap,
                            long long n_fixed, bool replace, bool list_out, RunCounters* ctr,
                            cudaStream_t s) {
    constexpr int kThreads = 128;
    const size_t smem = (size_t)(kThreads / 32) * 2 * kWarpChunk * sizeof(Node64);
    unsigned blocks = (unsigned)sm_count();
    if (n_fixed >= 0) {
        const long long need = (std::min<long long>(n_fixed, cap) + kThreads / 32 - 1) / (kThreads / 32);
        blocks = (unsigned)std::max(1ll, std::min<long long>(need, 8ll * sm_count()));
    }
    repair64_kernel<<<blocks, kThreads, smem, s>>>(scans, list, cap, n_fixed, replace, list_out, ctr);
    return cudaGetLastError();
}

cudaError_t launch_sample64(const ScanParams& p, int what, const double* pts, int64_t n,
                            double* out, RunCounters* ctr, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    sample64_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(p, what, pts, n, out, ctr);
    return cudaGetLastError();
}

cudaError_t launch_grid_build64(const ScanParams& p, const GridView& g, Node64* out,
                                RunCounters* ctr, cudaStream_t s) {
    int cap;
    size_t sm = smem_bytes64(p, cap);
    cudaError_t e = cudaFuncSetAttribute(grid_build64_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024);
    if (e != cudaSuccess) return e;
    const long long total = (long long)g.n[0] * g.n[1] * g.n[2];
    long long blocks = (total + 127) / 128;
    const long long cap_blocks = (long long)sm_count() * 16;
    if (blocks > cap_blocks) blocks = cap_blocks;
    if (blocks < 1) blocks = 1;
    grid_build64_kernel<<<(unsigned)blocks, 128, sm, s>>>(p, g, out, cap, ctr);
    return cudaGetLastError();
}

}  // namespace mafm
