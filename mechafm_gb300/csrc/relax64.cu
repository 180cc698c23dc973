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

namespace mafm {
namespace {

struct V3 {
    double x, y, z;
};

__device__ __forceinline__ double len3(V3 v) { return sqrt(v.x * v.x + v.y * v.y + v.z * v.z); }

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
};

__device__ __forceinline__ bool converged64(const ScanParams& p, V3 F, double ediff) {
    if (p.minterm == MAFM_TERM_E) return fabs(ediff) < p.etol;
    if (p.minterm == MAFM_TERM_F) return len3(F) < p.ftol;
    return fabs(ediff) < p.etol && len3(F) < p.ftol;
}

struct State64 {
    V3 tip, vel, dum;
    double energy;
    int outside;
};

// FIREMinimisation, minimiser.cpp:67-129 (only the tip is free).
__device__ int fire64(Eval64& ev, const ScanParams& p, State64& s, unsigned long long& evals) {
    const int n_min = 5;
    const double f_inc = 1.1, f_dec = 0.5, f_a = 0.99, a_start = 0.1;
    const double dt_max = 10 * p.dt;
    double alpha = a_start, dt = p.dt;
    int n_non_neg = 0;
    int n_tot = 1;
    for (; n_tot < p.maxsteps; ++n_tot) {
        const double prev = s.energy;
        V3 F, pp = s.tip, v = s.vel;
        double E;
        if (p.integrator == MAFM_INT_EULER) {
            ev.all(pp, s.dum, F, E, s.outside);
            evals += 1;
            s.tip.x = pp.x + dt * v.x; s.tip.y = pp.y + dt * v.y; s.tip.z = pp.z + dt * v.z;
            s.vel.x = v.x + dt * F.x / 1.0; s.vel.y = v.y + dt * F.y / 1.0; s.vel.z = v.z + dt * F.z / 1.0;
        } else if (p.integrator == MAFM_INT_MIDPOINT) {
            V3 f1, f2;
            double e1, e2;
            ev.all(pp, s.dum, f1, e1, s.outside);
            V3 p2 = {pp.x + dt / 2 * v.x, pp.y + dt / 2 * v.y, pp.z + dt / 2 * v.z};
            V3 v2 = {v.x + dt / 2 * f1.x / 1.0, v.y + dt / 2 * f1.y / 1.0, v.z + dt / 2 * f1.z / 1.0};
            ev.all(p2, s.dum, f2, e2, s.outside);
            evals += 2;
            s.tip.x = pp.x + dt * v2.x; s.tip.y = pp.y + dt * v2.y; s.tip.z = pp.z + dt * v2.z;
            s.vel.x = v.x + dt * f2.x / 1.0; s.vel.y = v.y + dt * f2.y / 1.0; s.vel.z = v.z + dt * f2.z / 1.0;
            F = f2;
            E = e2;
        } else {
            V3 f1, f2, f3, f4;
            double e1, e2, e3, e4;
            ev.all(pp, s.dum, f1, e1, s.outside);
            V3 p2 = {pp.x + dt / 2 * v.x, pp.y + dt / 2 * v.y, pp.z + dt / 2 * v.z};
            V3 v2 = {v.x + dt / 2 * f1.x / 1.0, v.y + dt / 2 * f1.y / 1.0, v.z + dt / 2 * f1.z / 1.0};
            ev.all(p2, s.dum, f2, e2, s.outside);
            V3 p3 = {pp.x + dt / 2 * v2.x, pp.y + dt / 2 * v2.y, pp.z + dt / 2 * v2.z};
            V3 v3 = {v.x + dt / 2 * f2.x / 1.0, v.y + dt / 2 * f2.y / 1.0, v.z + dt / 2 * f2.z / 1.0};
            ev.all(p3, s.dum, f3, e3, s.outside);
            V3 p4 = {pp.x + dt * v3.x, pp.y + dt * v3.y, pp.z + dt * v3.z};
            V3 v4 = {v.x + dt * f3.x / 1.0, v.y + dt * f3.y / 1.0, v.z + dt * f3.z / 1.0};
            ev.all(p4, s.dum, f4, e4, s.outside);
            evals += 4;
            s.tip.x = pp.x + dt / 6 * (v.x + 2 * v2.x + 2 * v3.x + v4.x);
            s.tip.y = pp.y + dt / 6 * (v.y + 2 * v2.y + 2 * v3.y + v4.y);
            s.tip.z = pp.z + dt / 6 * (v.z + 2 * v2.z + 2 * v3.z + v4.z);
            s.vel.x = v.x + dt / 6 * (f1.x + 2 * f2.x + 2 * f3.x + f4.x) / 1.0;
            s.vel.y = v.y + dt / 6 * (f1.y + 2 * f2.y + 2 * f3.y + f4.y) / 1.0;
            s.vel.z = v.z + dt / 6 * (f1.z + 2 * f2.z + 2 * f3.z + f4.z) / 1.0;
            F.x = (f1.x + 2 * f2.x + 2 * f3.x + f4.x) / 6;
            F.y = (f1.y + 2 * f2.y + 2 * f3.y + f4.y) / 6;
            F.z = (f1.z + 2 * f2.z + 2 * f3.z + f4.z) / 6;
            E = (e1 + 2 * e2 + 2 * e3 + e4) / 6;
        }
        s.energy = E;
        if (converged64(p, F, E - prev)) break;
        const V3 w = s.vel;
        const double pw = w.x * F.x + w.y * F.y + w.z * F.z;
        const double fl = len3(F);
        V3 fh = {0, 0, 0};
        if (fl > 1e-10) { fh.x = F.x / fl; fh.y = F.y / fl; fh.z = F.z / fl; }
        const double vl = len3(w);
        s.vel.x = (1 - alpha) * w.x + alpha * fh.x * vl;
        s.vel.y = (1 - alpha) * w.y + alpha * fh.y * vl;
        s.vel.z = (1 - alpha) * w.z + alpha * fh.z * vl;
        if (pw < 0) {
            s.vel.x = s.vel.y = s.vel.z = 0;
            n_non_neg = 0;
            dt *= f_dec;
            alpha = a_start;
        } else {
            if (n_non_neg > n_min) {
                const double g = dt * f_inc;
                dt = dt_max < g ? dt_max : g;   // std::min(g, dt_max)
                alpha *= f_a;
            }
            n_non_neg++;
        }
    }
    return n_tot;
}

// SDMinimisation, minimiser.cpp:39-65.
__device__ int sd64(Eval64& ev, const ScanParams& p, State64& s, unsigned long long& evals) {
    int n = 1;
    for (; n < p.maxsteps; ++n) {
        const double prev = s.energy;
        V3 F;
        double E;
        ev.all(s.tip, s.dum, F, E, s.outside);
        evals += 1;
        s.energy = E;
        if (converged64(p, F, E - prev)) break;
        s.tip.x += p.dt * F.x; s.tip.y += p.dt * F.y; s.tip.z += p.dt * F.z;
    }
    return n;
}

// System::setDummyXY (system.cpp:139-162)
__device__ __forceinline__ void dummy_xy64(const ScanParams& p, bool wrap, double x, double y,
                                           double& ox, double& oy) {
    if (wrap) {
        const double* ci = p.cell_inv;
        const double* c = p.cell;
        V3 t = {x - p.offset[0], y - p.offset[1], 0 - p.offset[2]};
        V3 cn = {ci[0] * t.x + ci[1] * t.y + ci[2] * t.z, ci[3] * t.x + ci[4] * t.y + ci[5] * t.z,
                 ci[6] * t.x + ci[7] * t.y + ci[8] * t.z};
        cn.x -= floor(cn.x);
        cn.y -= floor(cn.y);
        ox = (c[0] * cn.x + c[1] * cn.y + c[2] * cn.z) + p.offset[0];
        oy = (c[3] * cn.x + c[4] * cn.y + c[5] * cn.z) + p.offset[1];
    } else {
        ox = x;
        oy = y;
    }
}

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
    unsigned long long steps = 0, evals = 0;
    unsigned status_or = 0;
    const bool wrap = p.tip_pbc && p.ts_mode != 2;
    for (;;) {
        const long long c = (long long)atomicAdd(&ctr->next_work, 1ull) + col_begin;
        if (c >= col_end) break;
        const int i = (int)(c / p.ny), j = (int)(c % p.ny);
        State64 s;
        s.vel = {0, 0, 0};
        s.energy = 0;
        double x, y;
        dummy_xy64(p, wrap, i * p.dx, j * p.dy, x, y);
        s.dum = {x, y, p.zhigh};
        s.tip = {x, y, p.zhigh - p.tip_dummy_d};
        mafm_point* o = out + (size_t)(c - col_begin) * p.nz;
        for (int k = 0; k < p.nz; ++k) {
            s.outside = 0;
            const int n = p.minimiser == MAFM_MIN_SD ? sd64(ev, p, s, evals) : fire64(ev, p, s, evals);
            V3 F;
            double E;
            ev.ts(s.tip, F, E, s.outside);
            evals += 1;
            int st = (n >= p.maxsteps ? MAFM_PT_MAXSTEPS : 0) | (s.outside ? MAFM_PT_OUTSIDE : 0);
            if (!isfinite(F.x) || !isfinite(F.y) || !isfinite(F.z) || !isfinite(E)) st |= MAFM_PT_NONFINITE;
            mafm_point r;
            r.tip[0] = s.tip.x; r.tip[1] = s.tip.y; r.tip[2] = s.tip.z;
            r.force[0] = F.x; r.force[1] = F.y; r.force[2] = F.z;
            r.energy = E;
            r.steps = n;
            r.status = st;
            o[k] = r;
            status_or |= (unsigned)st;
            steps += (unsigned long long)n;
            s.dum.z -= p.dz;
            s.tip.z -= p.dz;
        }
    }
    atomicAdd(&ctr->total_steps, steps);
    atomicAdd(&ctr->force_evals, evals);
    atomicAdd(&ctr->pair_evals, ev.pairs);
    if (status_or | ev.err) atomicOr(&ctr->error_word, status_or | ev.err);
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
        dummy_xy64(p, p.tip_pbc != 0, i * g.basis[0] + g.origin[0], j * g.basis[4] + g.origin[1], x, y);
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
