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
#include "mafm_internal.h"
#include "relax_tpl.cuh"

namespace mafm {
namespace {

using V3 = V3T<double>;

// LJInteraction::eval / MorseInteraction::eval; r = tip - (atom + shift).
__device__ __forceinline__ void vdw64(int kind, double p0, double p1, double p2, V3 r, V3& f,
                                      double& e) {
    if (kind == MAFM_PAIR_LJ) {
        double r_sqr = r.x * r.x + r.y * r.y + r.z * r.z;
        double r6 = r_sqr * r_sqr * r_sqr;
        double term_a = p1 / (r6 * r6);
        double term_b = p0 / r6;
        e = term_a - term_b;
        double s = (12 * term_a - 6 * term_b) / r_sqr;
        f.x = s * r.x; f.y = s * r.y; f.z = s * r.z;
    } else {
        double rl = len3(r);
        double d = exp(-p1 * (rl - p2));
        e = p0 * (d * d - 2 * d + 1);
        double f_abs = 2 * p0 * p1 * (d * d - d);
        double s = f_abs / rl;
        f.x = s * r.x; f.y = s * r.y; f.z = s * r.z;
    }
}

// CoulombInteraction::eval
__device__ __forceinline__ void coul64(double qq, V3 r, V3& f, double& e) {
    double rl = len3(r);
    e = qq / rl;
    double s = qq / (rl * rl * rl);
    f.x = s * r.x; f.y = s * r.y; f.z = s * r.z;
}

// ForceGrid::getGridPointIndex + pbcGridPoint.  A corner outside a
// non-periodic grid is an error in the reference; here it sets ERR_GRID_INDEX
// and is clamped so that no read leaves the grid.
__device__ __forceinline__ long long grid_index64(const GridView& g, int x, int y, int z,
                                                  unsigned& err) {
    if (x < 0 || y < 0 || z < 0 || x >= g.n[0] || y >= g.n[1] || z >= g.n[2]) {
        if (g.periodic) {
            int n;
            if (x < 0 || x >= g.n[0]) { n = (int)floor((double)x / g.n[0]); x -= n * g.n[0]; }
            if (y < 0 || y >= g.n[1]) { n = (int)floor((double)y / g.n[1]); y -= n * g.n[1]; }
            if (z < 0 || z >= g.n[2]) { n = (int)floor((double)z / g.n[2]); z -= n * g.n[2]; }
        } else {
            err |= ERR_GRID_INDEX;
            x = min(max(x, 0), g.n[0] - 1);
            y = min(max(y, 0), g.n[1] - 1);
            z = min(max(z, 0), g.n[2] - 1);
        }
    }
    return ((long long)x * g.n[1] + y) * g.n[2] + z;
}

// ForceGrid::interpolate
__device__ void interp64(const GridView& g, V3 pos, V3& f, double& e, int& outside,
                         unsigned& err) {
    V3 q = {pos.x - g.origin[0], pos.y - g.origin[1], pos.z - g.origin[2]};
    V3 pb;
    if (g.orthogonal) {
        pb.x = q.x / g.basis[0]; pb.y = q.y / g.basis[4]; pb.z = q.z / g.basis[8];
    } else {
        pb.x = g.inv[0] * q.x + g.inv[1] * q.y + g.inv[2] * q.z;
        pb.y = g.inv[3] * q.x + g.inv[4] * q.y + g.inv[5] * q.z;
        pb.z = g.inv[6] * q.x + g.inv[7] * q.y + g.inv[8] * q.z;
    }
    int gp[3] = {(int)floor(pb.x), (int)floor(pb.y), (int)floor(pb.z)};
    if (!g.periodic) {
        for (int a = 0; a < 3; ++a) {
            if (gp[a] < 0) { gp[a] = 0; outside = 1; }
            else if (gp[a] >= g.n[a]) { gp[a] = g.n[a] - 1; outside = 1; }
        }
    }
    Node64 s[8];
#pragma unroll
    for (int c = 0; c < 8; ++c)
        s[c] = g.g64[grid_index64(g, gp[0] + (c >> 2), gp[1] + ((c >> 1) & 1), gp[2] + (c & 1), err)];
    const double dx = pb.x - gp[0], dy = pb.y - gp[1], dz = pb.z - gp[2];
    double out[4];
#pragma unroll
    for (int m = 0; m < 4; ++m) {
        auto comp = [m](const Node64& n) { return m == 0 ? n.x : m == 1 ? n.y : m == 2 ? n.z : n.w; };
        double v00 = comp(s[0]) * (1 - dx) + comp(s[4]) * dx;
        double v01 = comp(s[1]) * (1 - dx) + comp(s[5]) * dx;
        double v10 = comp(s[2]) * (1 - dx) + comp(s[6]) * dx;
        double v11 = comp(s[3]) * (1 - dx) + comp(s[7]) * dx;
        double v0 = v00 * (1 - dy) + v10 * dy;
        double v1 = v01 * (1 - dy) + v11 * dy;
        out[m] = v0 * (1 - dz) + v1 * dz;
    }
    f.x = out[0]; f.y = out[1]; f.z = out[2]; e = out[3];
}

// The tip–dummy van der Waals (+ Coulomb) term and the XY spring, added to
// the tip–surface force and energy in Eval64::all's order
// (simulation.cpp:503-515, interactions.cpp:252-266).
__device__ __forceinline__ void add_tip_dummy(const ScanParams& p, V3 tip, V3 dum, V3& F,
                                              double& E) {
    V3 f;
    double e;
    V3 r = {dum.x - tip.x, dum.y - tip.y, dum.z - tip.z};
    vdw64(p.td_kind, p.td_p[0], p.td_p[1], p.td_p[2], r, f, e);
    F.x -= f.x; F.y -= f.y; F.z -= f.z; E += e;
    if (p.td_coul) {
        coul64(p.td_qq, r, f, e);
        F.x -= f.x; F.y -= f.y; F.z -= f.z; E += e;
    }
    double rx = dum.x - tip.x, ry = dum.y - tip.y;
    double rr = sqrt(rx * rx + ry * ry);
    double dr = rr - p.harm_r0;
    double eh = p.harm_k * dr * dr;
    double fx = 0, fy = 0;
    if (rr > 1e-10) {
        double s = -2 * p.harm_k * dr / rr;
        fx = s * rx; fy = s * ry;
    }
    F.x -= fx; F.y -= fy; F.z -= 0.0;
    E += eh;
}

struct Eval64 {
    const ScanParams& p;
    const AtomRec64* atoms;   // shared or global copy of the terms
    int n;                    // terms in the sum
    int mode;                 // ts_mode
    unsigned err;
    unsigned long long pairs;

    // Tip–surface terms: System::evalTipSurfaceForces (system.cpp:41-51).
    __device__ void ts(V3 tip, V3& F, double& E, int& outside) {
        V3 f;
        double e;
        F.x = F.y = F.z = 0;
        E = 0;
        if (mode == 2) {
            interp64(p.grid, tip, f, e, outside, err);
            F.x += f.x; F.y += f.y; F.z += f.z; E += e;
            return;
        }
        for (int i = 0; i < n; ++i) {
            const AtomRec64 t = atoms[i];
            V3 r = {tip.x - t.x, tip.y - t.y, tip.z - t.z};
            vdw64(t.kind, t.p0, t.p1, t.p2, r, f, e);
            F.x += f.x; F.y += f.y; F.z += f.z; E += e;
            if (t.coul) {
                coul64(t.qq, r, f, e);
                F.x += f.x; F.y += f.y; F.z += f.z; E += e;
                ++pairs;
            }
        }
        pairs += n;
        if (mode == 1) {
            int unused = 0;
            interp64(p.es, tip, f, e, unused, err);
            F.x += f.x; F.y += f.y; F.z += f.z; E += e;
        }
    }

    // All interactions of the relaxation (integrators.cpp evaluate them all).
    __device__ void all(V3 tip, V3 dum, V3& F, double& E, int& outside) {
        ts(tip, F, E, outside);
        add_tip_dummy(p, tip, dum, F, E);
    }

    // The FP64 path makes the reference's decisions itself: nothing to watch.
    __device__ void watch_conv(const ScanParams&, V3, double) {}
    __device__ void watch_p(double, double, double) {}
    __device__ int column_status() const { return 0; }
};

// Terms per chunk of the warp-cooperative evaluation (two per lane).
constexpr int kWarpChunk = 64;

// The same sums as Eval64, evaluated by a whole warp for one column: lane l
// computes terms l, l + 32, ... of a chunk into the warp's shared buffer, then
// lanes 0-3 add component x, y, z, E of every term in the reference's order
// (vdW part, then Coulomb part, term by term), so each sum is formed by the
// same sequence of FP64 additions as in Eval64 and the results are
// bit-identical.  A term without Coulomb contributes an exact +0, which
// leaves a sum that starts at +0 unchanged.  Every lane ends with the sums,
// and every lane runs the (warp-uniform) minimiser on them.
struct EvalWarp64 {
    const ScanParams& p;
    const AtomRec64* atoms;
    int n;
    int mode;                 // ts_mode
    int lane;
    Node64* buf;              // 2 * kWarpChunk records {x, y, z, E} of this warp
    unsigned err;
    unsigned long long pairs; // counted on lane 0

    __device__ void ts(V3 tip, V3& F, double& E, int& outside) {
        if (mode == 2) {
            // the rigid grid: one lookup, the same on every lane (Eval64::ts)
            V3 f;
            double e;
            interp64(p.grid, tip, f, e, outside, err);
            F.x = 0.0 + f.x; F.y = 0.0 + f.y; F.z = 0.0 + f.z;
            E = 0.0 + e;
            return;
        }
        double acc = 0.0;   // lane m < 4: component m of {Fx, Fy, Fz, E}
        for (int base = 0; base < n; base += kWarpChunk) {
            const int cnt = min(kWarpChunk, n - base);
            for (int j = lane; j < cnt; j += 32) {
                const AtomRec64 t = atoms[base + j];
                V3 r = {tip.x - t.x, tip.y - t.y, tip.z - t.z};
                V3 f;
                double e;
                vdw64(t.kind, t.p0, t.p1, t.p2, r, f, e);
                buf[2 * j] = Node64{f.x, f.y, f.z, e};
                if (t.coul) {
                    coul64(t.qq, r, f, e);
                    buf[2 * j + 1] = Node64{f.x, f.y, f.z, e};
                } else {
                    buf[2 * j + 1] = Node64{0.0, 0.0, 0.0, 0.0};
                }
            }
            __syncwarp();
            if (lane < 4) {
                const double* b = reinterpret_cast<const double*>(buf) + lane;
                for (int j = 0; j < 2 * cnt; ++j) acc += b[4 * j];
            }
            __syncwarp();
        }
        if (lane == 0) {
            unsigned long long c = 0;
            for (int i = 0; i < n; ++i) c += atoms[i].coul ? 1ull : 0ull;
            pairs += (unsigned long long)n + c;
        }
        if (mode == 1) {
            V3 f;
            double e;
            int unused = 0;
            interp64(p.es, tip, f, e, unused, err);
            if (lane < 4) acc += lane == 0 ? f.x : lane == 1 ? f.y : lane == 2 ? f.z : e;
        }
        F.x = __shfl_sync(0xffffffffu, acc, 0);
        F.y = __shfl_sync(0xffffffffu, acc, 1);
        F.z = __shfl_sync(0xffffffffu, acc, 2);
        E = __shfl_sync(0xffffffffu, acc, 3);
    }

    __device__ void all(V3 tip, V3 dum, V3& F, double& E, int& outside) {
        ts(tip, F, E, outside);
        add_tip_dummy(p, tip, dum, F, E);
    }

    __device__ void watch_conv(const ScanParams&, V3, double) {}
    __device__ void watch_p(double, double, double) {}
    __device__ int column_status() const { return 0; }
};

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
        EvalWarp64 ev{p, p.atoms64, p.n_terms_direct, p.ts_mode, lane, buf, 0u, 0ull};
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
