// relaxdf.cu — the double-float relaxation (precision MAFM_DF).
//
// Every quantity of the relaxation is a dfloat (dfloat.cuh): the tip–atom
// terms, their sums, the tip–dummy terms, positions, velocities, the FIRE
// time step and mixing factor, energies.  The minimiser and the integrators
// are the FP64 kernel's own code (relax_tpl.cuh) instantiated for dfloat, so
// the relaxation takes the same steps as FP64 unless one of FIRE's discrete
// decisions — the convergence test, the sign of P = v.F — falls within the
// double-float error (about 1e-13 of the largest term) of its threshold.
// The evaluator records such near-ties with a margin far above that error
// (TieMargins); relax_column_t then marks the column's points
// MAFM_PT_NEAR_TIE and the kernel lists the column for the FP64
// re-relaxation (repair64_kernel), which replaces it with the plain FP64
// kernel's bits.
//
// Why not FP32 with a near-tie repair: with FP32 pair terms (about 1e-6 of a
// term) FIRE's decisions come within FP32 error of their thresholds in
// nearly every pixel column of a scan, and the FP32 trajectory itself drifts
// from FP64's by about 1e-7 A, so no decision margin separates the columns
// that follow FP64 from those that do not.
//
// One thread relaxes one pixel column (columns from a global queue, in the
// scan's expected-cost order); its terms are read through the read-only
// cache, every lane of a warp reading the same record (broadcast).
//
// Reference correspondence (src/): LJ / Morse / Coulomb interactions.cpp:15-51,
// tip–dummy terms interactions.cpp:252-266 and simulation.cpp:503-515,
// external field lookup force_grid.cpp:88-275, minimiser and column as in
// relax_tpl.cuh.
#include <algorithm>
#include <cstdlib>

#include "mafm_df.h"
#include "relax_tpl.cuh"

namespace mafm {
namespace {

using D = dfloat;
using V3D = V3T<dfloat>;

// Sum of many double-floats: the high parts through two_sum, every rounding
// error and low part into one FP32 word (a few ulps of the high part after
// hundreds of terms, far below the double-float error of a term).
struct LazySum {
    float h = 0.0f, l = 0.0f;
    __device__ __forceinline__ void add(D x) {
        const D s = dfl_two_sum(h, x.h);
        h = s.h;
        l = __fadd_rn(l, __fadd_rn(s.l, x.l));
    }
    __device__ __forceinline__ D value() const { return dfl_fast_two_sum(h, l); }
};

// One tip–atom term for the separation d = tip - atom: LJ (interactions.cpp:
// 15-27) or Morse (:29-40), plus Coulomb (:42-51) when coul.  1/r comes from
// a double-float rsqrt; f is the force on the tip.
__device__ __forceinline__ void pair_df(int kind, D p0, D p1, D p2, bool coul, D qq, V3D d,
                                        V3D& f, D& e) {
    const D r2 = d.x * d.x + d.y * d.y + d.z * d.z;
    const D ir = dfl_rsqrt(r2);
    const D ir2 = ir * ir;
    D s;
    if (kind == MAFM_PAIR_LJ) {
        const D ir6 = ir2 * ir2 * ir2;
        const D a = p1 * (ir6 * ir6);   // es12 / r^12
        const D b = p0 * ir6;           // es6 / r^6
        e = a - b;
        s = (a * 12.0f - b * 6.0f) * ir2;
    } else {
        const D r = r2 * ir;
        const D q = dfl_exp(-(p1 * (r - p2)));
        const D q2 = q * q;
        e = p0 * ((q2 - q * 2.0f) + D(1.0f, 0.0f));
        s = ((p0 * p1) * 2.0f) * (q2 - q) * ir;
    }
    if (coul) {
        const D ec = qq * ir;
        e = e + ec;
        s = s + ec * ir2;
    }
    f.x = s * d.x;
    f.y = s * d.y;
    f.z = s * d.z;
}

__device__ __forceinline__ AtomRecDF load_term(const AtomRecDF* t) {
    const float4* q = reinterpret_cast<const float4*>(t);
    const float4 a = __ldg(q), b = __ldg(q + 1), c = __ldg(q + 2), g = __ldg(q + 3);
    AtomRecDF r;
    r.x = D(a.x, a.y); r.y = D(a.z, a.w); r.z = D(b.x, b.y); r.qq = D(b.z, b.w);
    r.p0 = D(c.x, c.y); r.p1 = D(c.z, c.w); r.p2 = D(g.x, g.y);
    r.kind = __float_as_int(g.z);
    r.coul = __float_as_int(g.w);
    return r;
}

// ForceGrid::interpolate (force_grid.cpp:88-155) on the double-float copy of
// a periodic grid (the external field).
__device__ void interp_df(const GridViewDF& g, V3D pos, V3D& f, D& e) {
    const V3D q = {pos.x - g.origin[0], pos.y - g.origin[1], pos.z - g.origin[2]};
    V3D pb;
    if (g.orthogonal) {
        pb.x = q.x / g.basis[0];
        pb.y = q.y / g.basis[4];
        pb.z = q.z / g.basis[8];
    } else {
        pb.x = g.inv[0] * q.x + g.inv[1] * q.y + g.inv[2] * q.z;
        pb.y = g.inv[3] * q.x + g.inv[4] * q.y + g.inv[5] * q.z;
        pb.z = g.inv[6] * q.x + g.inv[7] * q.y + g.inv[8] * q.z;
    }
    const D fl[3] = {dfl_floor(pb.x), dfl_floor(pb.y), dfl_floor(pb.z)};
    int gp[3];
    for (int a = 0; a < 3; ++a) gp[a] = (int)fl[a].h + (int)fl[a].l;
    int lo[3], hi[3];
    for (int a = 0; a < 3; ++a) {
        int x0 = gp[a] % g.n[a];
        if (x0 < 0) x0 += g.n[a];
        lo[a] = x0;
        hi[a] = x0 + 1 == g.n[a] ? 0 : x0 + 1;
    }
    const D dx = pb.x - fl[0], dy = pb.y - fl[1], dz = pb.z - fl[2];
    const D one(1.0f, 0.0f);
    const long long n12 = (long long)g.n[1] * g.n[2];
    NodeDF s[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        const int x = (c >> 2) ? hi[0] : lo[0];
        const int y = ((c >> 1) & 1) ? hi[1] : lo[1];
        const int z = (c & 1) ? hi[2] : lo[2];
        const float4* p = reinterpret_cast<const float4*>(g.g + (long long)x * n12 +
                                                          (long long)y * g.n[2] + z);
        const float4 u = __ldg(p), v = __ldg(p + 1);
        s[c].x = D(u.x, u.y); s[c].y = D(u.z, u.w); s[c].z = D(v.x, v.y); s[c].w = D(v.z, v.w);
    }
    D out[4];
#pragma unroll
    for (int m = 0; m < 4; ++m) {
        auto comp = [m](const NodeDF& n) { return m == 0 ? n.x : m == 1 ? n.y : m == 2 ? n.z : n.w; };
        const D v00 = comp(s[0]) * (one - dx) + comp(s[4]) * dx;
        const D v01 = comp(s[1]) * (one - dx) + comp(s[5]) * dx;
        const D v10 = comp(s[2]) * (one - dx) + comp(s[6]) * dx;
        const D v11 = comp(s[3]) * (one - dx) + comp(s[7]) * dx;
        const D v0 = v00 * (one - dy) + v10 * dy;
        const D v1 = v01 * (one - dy) + v11 * dy;
        out[m] = v0 * (one - dz) + v1 * dz;
    }
    f = {out[0], out[1], out[2]};
    e = out[3];
}

struct EvalDF {
    const ScanParamsDF& p;
    unsigned err;
    unsigned long long pairs;
    int tie;   // a decision of this column was a near-tie

    // System::evalTipSurfaceForces (system.cpp:41-51)
    __device__ void ts(V3D tip, V3D& F, D& E, int& outside) {
        (void)outside;
        LazySum fx, fy, fz, ee;
        const int n = p.n_terms;
        for (int i = 0; i < n; ++i) {
            const AtomRecDF t = load_term(p.atoms + i);
            const V3D d = {tip.x - t.x, tip.y - t.y, tip.z - t.z};
            V3D f;
            D e;
            pair_df(t.kind, t.p0, t.p1, t.p2, t.coul != 0, t.qq, d, f, e);
            fx.add(f.x);
            fy.add(f.y);
            fz.add(f.z);
            ee.add(e);
            pairs += 1ull + (t.coul ? 1ull : 0ull);
        }
        if (p.ts_mode == 1) {
            V3D f;
            D e;
            interp_df(p.es, tip, f, e);
            fx.add(f.x);
            fy.add(f.y);
            fz.add(f.z);
            ee.add(e);
        }
        F = {fx.value(), fy.value(), fz.value()};
        E = ee.value();
    }

    // the tip–dummy terms in Eval64::all's order (simulation.cpp:503-515,
    // interactions.cpp:252-266)
    __device__ void all(V3D tip, V3D dum, V3D& F, D& E, int& outside) {
        ts(tip, F, E, outside);
        const V3D r = {dum.x - tip.x, dum.y - tip.y, dum.z - tip.z};
        V3D f;
        D e;
        pair_df(p.td_kind, p.td_p[0], p.td_p[1], p.td_p[2], p.td_coul != 0, p.td_qq, r, f, e);
        F.x = F.x - f.x; F.y = F.y - f.y; F.z = F.z - f.z;
        E = E + e;
        const D rr = dfl_sqrt(r.x * r.x + r.y * r.y);
        const D dr = rr - p.harm_r0;
        E = E + p.harm_k * dr * dr;
        if (rr > D(1e-10)) {
            const D s = -(p.harm_k * 2.0f) * dr / rr;
            F.x = F.x - s * r.x;
            F.y = F.y - s * r.y;
        }
    }

    // checkConvergence (minimiser.cpp:15-37): a test within its margin of the
    // tolerance is a near-tie (FP64 could decide either way)
    __device__ void watch_conv(const ScanParamsDF& q, V3D F, D ediff) {
        const D ea = dfl_fabs(ediff) - q.etol;
        const D fa = len3(F) - q.ftol;
        const bool e_tie = dfl_fabs(ea) < q.tie.conv_e, f_tie = dfl_fabs(fa) < q.tie.conv_f;
        bool near;
        if (q.minterm == MAFM_TERM_E) near = e_tie;
        else if (q.minterm == MAFM_TERM_F) near = f_tie;
        else near = (e_tie && !(fa > q.tie.conv_f)) || (f_tie && !(ea > q.tie.conv_e));
        tie |= near;
    }

    // the sign of P = v.F (minimiser.cpp:107-124)
    __device__ void watch_p(D pw, D vl, D fl) {
        tie |= dfl_fabs(pw) < vl * (p.tie.p_f + p.tie.p_v * fl);
    }

    __device__ int column_status() const { return tie ? MAFM_PT_NEAR_TIE : 0; }
};

__device__ __forceinline__ unsigned long long df_global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__global__ void __launch_bounds__(128) relaxdf_kernel(const BatchDF* __restrict__ scans,
                                                      int n_scans, long long n_cols,
                                                      RunCounters* ctr,
                                                      unsigned long long* __restrict__ repair_list,
                                                      unsigned repair_cap,
                                                      unsigned long long watchdog_ns) {
    long long steps = 0;
    unsigned long long evals = 0, pairs = 0;
    unsigned status_or = 0, err = 0;
    const unsigned long long t0 = df_global_ns();
    for (;;) {
        const long long g = (long long)atomicAdd(&ctr->next_work, 1ull);
        if (g >= n_cols) break;
        int lo = 0, hi = n_scans - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (scans[mid].col_first <= g) lo = mid;
            else hi = mid - 1;
        }
        const BatchDF& B = scans[lo];
        const long long a = g - B.col_first;
        const long long c = B.order ? (long long)__ldg(B.order + a) : B.col_begin + a;
        EvalDF ev{B.p, 0u, 0ull, 0};
        relax_column_t<dfloat>(ev, B.p, c, B.out + (size_t)(c - B.col_begin) * B.p.nz, true, false,
                               steps, evals, status_or);
        pairs += ev.pairs;
        err |= ev.err;
        if (ev.tie && repair_list) {
            const unsigned slot = atomicAdd(&ctr->n_tie, 1u);
            if (slot < repair_cap) repair_list[slot] = ((unsigned long long)lo << 32) | (unsigned)c;
        }
        // time limit, checked between columns
        if (df_global_ns() - t0 > watchdog_ns) {
            err |= ERR_WATCHDOG;
            break;
        }
    }
    atomicAdd(&ctr->total_steps, (unsigned long long)steps);
    atomicAdd(&ctr->force_evals, evals);
    atomicAdd(&ctr->pair_evals, pairs);
    if (status_or | err) atomicOr(&ctr->error_word, status_or | err);
}

__global__ void nodes_to_df_kernel(const Node64* in, NodeDF* out, long long n) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const Node64 v = in[i];
        out[i] = NodeDF{D(v.x), D(v.y), D(v.z), D(v.w)};
    }
}

}  // namespace

AtomRecDF term_df(const AtomRec64& r) {
    AtomRecDF t;
    t.x = D(r.x); t.y = D(r.y); t.z = D(r.z); t.qq = D(r.qq);
    t.p0 = D(r.p0); t.p1 = D(r.p1); t.p2 = D(r.p2);
    t.kind = r.kind;
    t.coul = r.coul;
    return t;
}

ScanParamsDF params_df(const ScanParams& p, const AtomRecDF* atoms, const NodeDF* es_nodes) {
    ScanParamsDF q{};
    q.n_terms = p.n_terms_direct;
    q.ts_mode = p.ts_mode;
    q.atoms = atoms;
    q.es.g = es_nodes;
    for (int a = 0; a < 3; ++a) {
        q.es.n[a] = p.es.n[a];
        q.es.origin[a] = D(p.es.origin[a]);
        q.offset[a] = D(p.offset[a]);
        q.td_p[a] = D(p.td_p[a]);
    }
    q.es.periodic = p.es.periodic;
    q.es.orthogonal = p.es.orthogonal;
    for (int k = 0; k < 9; ++k) {
        q.es.basis[k] = D(p.es.basis[k]);
        q.es.inv[k] = D(p.es.inv[k]);
        q.cell[k] = D(p.cell[k]);
        q.cell_inv[k] = D(p.cell_inv[k]);
    }
    q.td_kind = p.td_kind;
    q.td_coul = p.td_coul;
    q.td_qq = D(p.td_qq);
    q.harm_k = D(p.harm_k);
    q.harm_r0 = D(p.harm_r0);
    q.tip_dummy_d = D(p.tip_dummy_d);
    q.nx = p.nx; q.ny = p.ny; q.nz = p.nz;
    q.tip_pbc = p.tip_pbc;
    q.dx = D(p.dx); q.dy = D(p.dy); q.dz = D(p.dz); q.zhigh = D(p.zhigh);
    q.minimiser = p.minimiser;
    q.integrator = p.integrator;
    q.minterm = p.minterm;
    q.maxsteps = p.maxsteps;
    q.etol = D(p.etol);
    q.ftol = D(p.ftol);
    q.dt = D(p.dt);
    // Near-tie margins: 1e-8 of the tolerances, 1e-10 of |F| for the sign of
    // P; the double-float error of a force is about 1e-13 of the largest term.
    // MAFM_DF_TIE_SCALE multiplies them (a diagnostic: a huge scale sends
    // every column to the FP64 re-relaxation).
    double k = 1.0;
    if (const char* e = std::getenv("MAFM_DF_TIE_SCALE")) {
        const double v = std::atof(e);
        if (v > 0.0 && v <= 1.0e30) k = v;
    }
    q.tie.conv_e = D(k * 1.0e-8 * p.etol);
    q.tie.conv_f = D(k * 1.0e-8 * p.ftol);
    q.tie.p_f = D(k * 1.0e-8 * p.ftol);
    q.tie.p_v = D(k * 1.0e-10);
    return q;
}

cudaError_t launch_relaxdf(const BatchDF* scans, int n_scans, long long n_cols, RunCounters* ctr,
                           unsigned long long* repair_list, unsigned repair_cap,
                           unsigned long long watchdog_ns, cudaStream_t s) {
    if (n_cols <= 0) return cudaSuccess;
    constexpr int kThreads = 128;
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, relaxdf_kernel, kThreads, 0);
    if (e != cudaSuccess) return e;
    if (per_sm <= 0) per_sm = 1;
    long long blocks = (long long)sm_count() * per_sm;
    const long long need = (n_cols + kThreads - 1) / kThreads;
    blocks = std::max(1ll, std::min(blocks, need));
    relaxdf_kernel<<<(unsigned)blocks, kThreads, 0, s>>>(scans, n_scans, n_cols, ctr, repair_list,
                                                         repair_list ? repair_cap : 0u, watchdog_ns);
    return cudaGetLastError();
}

cudaError_t launch_nodes_to_df(const Node64* in, NodeDF* out, long long n, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    long long blocks = std::min((n + 255) / 256, (long long)sm_count() * 32);
    nodes_to_df_kernel<<<(unsigned)blocks, 256, 0, s>>>(in, out, n);
    return cudaGetLastError();
}

}  // namespace mafm
