// relaxdf.cu — the double-float relaxation (precision MAFM_DF).
//
// Every quantity of the relaxation is a dfloat (dfloat.cuh): the tip–atom
// terms, their sums, the tip–dummy terms, positions, velocities, the FIRE
// time step and mixing factor, energies.  The minimiser's and integrators'
// operations are those of the FP64 kernel (fire_t / sd_t, relax_tpl.cuh),
// stage by stage, so the relaxation takes the same steps as FP64 unless one
// of FIRE's discrete decisions — the convergence test, the sign of P = v.F —
// falls within the double-float error (about 1e-13 of the largest term) of
// its threshold.  Such near-ties are recorded with a margin far above that
// error (TieMargins): the column's later points carry MAFM_PT_NEAR_TIE and
// the column goes on the list of the FP64 re-relaxation (repair64_kernel),
// which replaces it with the plain FP64 kernel's bits.
//
// Why not FP32 with a near-tie repair: with FP32 pair terms (about 1e-6 of a
// term) FIRE's decisions come within FP32 error of their thresholds in
// nearly every pixel column of a scan, and the FP32 trajectory itself drifts
// from FP64's by about 1e-7 A, so no decision margin separates the columns
// that follow FP64 from those that do not.
//
// Every lane relaxes one pixel column at a time (columns from a global
// queue, in each scan's expected-cost order) in a slot machine: one force
// evaluation per lane per iteration, then the lane's own minimiser stage, so
// a warp's lanes stay busy whatever their columns' step counts (one thread
// running a whole column kept only 13 of 32 lanes active on average).  The
// terms are read through the read-only cache, every lane of a warp reading
// the same record (broadcast).
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

// System::evalTipSurfaceForces (system.cpp:41-51): the tip–surface force and
// energy at tip.  The loop over terms is the same for every lane of a scan.
__device__ __forceinline__ void ts_df(const ScanParamsDF& p, V3D tip, V3D& F, D& E,
                                      unsigned long long& pairs) {
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

// The tip–dummy terms and the XY spring, added in Eval64::all's order
// (simulation.cpp:503-515, interactions.cpp:252-266).
__device__ __forceinline__ void tip_dummy_df(const ScanParamsDF& p, V3D tip, V3D dum, V3D& F,
                                             D& E) {
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

enum : int { DF_EVAL0 = 0, DF_EVAL1 = 1, DF_EVAL2 = 2, DF_EVAL3 = 3, DF_OUT = 4 };

// One lane's column: the state fire_t / sd_t keep in locals, held across
// slots.  u is the midpoint v2 / the RK4 v_k; vs, fs, es the RK4 sums.
struct LaneDF {
    int col, scan, k, n, nnn, phase, tie;
    V3D tip, vel, dum, ex, u, vs, fs;
    D energy, es, alpha, dt;
};

__device__ __forceinline__ unsigned long long df_global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// The double-float relaxation as a slot machine: every lane of a warp holds
// one pixel column, and each loop iteration performs one force evaluation
// for every lane that has one (the costly, uniform part), then advances each
// lane's minimiser by that evaluation: the integrator's stages (euler 1,
// midpoint 2, rk4 4 evaluations per step), the convergence test and FIRE's
// mixing and time-step control, exactly in the order of fire_t / sd_t
// (relax_tpl.cuh), and the output evaluation of each height.  A lane whose
// column is done takes the next one from the global queue, so lanes never
// wait for the slowest column of their warp.
__global__ void __launch_bounds__(128) relaxdf_kernel(const BatchDF* __restrict__ scans,
                                                      int n_scans, long long n_cols,
                                                      RunCounters* ctr,
                                                      unsigned long long* __restrict__ repair_list,
                                                      unsigned repair_cap,
                                                      unsigned long long watchdog_ns) {
    constexpr unsigned kFull = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    unsigned long long steps = 0, evals = 0, pairs = 0;
    unsigned status_or = 0, err = 0;
    const unsigned long long t0 = df_global_ns();
    unsigned ticks = 0;

    LaneDF s;
    s.col = -1;
    s.scan = 0;
    s.tie = 0;
    bool done = false;
    const BatchDF* B = scans;

    auto start_level = [&]() {
        s.alpha = D(0.1);
        s.dt = B->p.dt;
        s.nnn = 0;
        s.n = 1;
        s.phase = s.n >= B->p.maxsteps ? DF_OUT : DF_EVAL0;
        s.ex = s.tip;
    };

    for (;;) {
        // lanes without a column take the next queue entries (one atomic per warp)
        const unsigned idle = __ballot_sync(kFull, s.col < 0 && !done);
        if (idle) {
            unsigned long long base = 0;
            if (lane == 0) base = atomicAdd(&ctr->next_work, (unsigned long long)__popc(idle));
            base = __shfl_sync(kFull, base, 0);
            if (s.col < 0 && !done) {
                const long long g = (long long)base + __popc(idle & ((1u << lane) - 1u));
                if (g >= n_cols) {
                    done = true;
                } else {
                    int lo = 0, hi = n_scans - 1;
                    while (lo < hi) {
                        const int mid = (lo + hi + 1) >> 1;
                        if (scans[mid].col_first <= g) lo = mid;
                        else hi = mid - 1;
                    }
                    s.scan = lo;
                    B = scans + lo;
                    const long long a = g - B->col_first;
                    s.col = B->order ? __ldg(B->order + a) : B->col_begin + (int)a;
                    // a new column (Simulation::run, simulation.cpp:93-99)
                    const ScanParamsDF& P = B->p;
                    const bool wrap = P.tip_pbc && P.ts_mode != 2;
                    const int i = s.col / P.ny, j = s.col % P.ny;
                    D x, y;
                    dummy_xy_t(P, wrap, D(i) * P.dx, D(j) * P.dy, x, y);
                    s.dum = {x, y, P.zhigh};
                    s.tip = {x, y, P.zhigh - P.tip_dummy_d};
                    s.vel = {D(0), D(0), D(0)};
                    s.energy = D(0);
                    s.k = 0;
                    s.tie = 0;
                    start_level();
                }
            }
        }
        if (__all_sync(kFull, done)) break;
        if ((++ticks & 255u) == 0 && __any_sync(kFull, df_global_ns() - t0 > watchdog_ns)) {
            err |= ERR_WATCHDOG;
            break;
        }
        if (s.col < 0) continue;

        // ---- one evaluation per lane ----
        const ScanParamsDF& P = B->p;
        V3D F;
        D E;
        ts_df(P, s.ex, F, E, pairs);
        evals += 1;
        if (s.phase == DF_OUT) {
            // System::getOutput (system.cpp:28-51)
            int st = (s.n >= P.maxsteps ? MAFM_PT_MAXSTEPS : 0) | (s.tie ? MAFM_PT_NEAR_TIE : 0);
            if (!dfl_isfinite(F.x) || !dfl_isfinite(F.y) || !dfl_isfinite(F.z) || !dfl_isfinite(E))
                st |= MAFM_PT_NONFINITE;
            mafm_point r;
            r.tip[0] = to_double(s.tip.x); r.tip[1] = to_double(s.tip.y); r.tip[2] = to_double(s.tip.z);
            r.force[0] = to_double(F.x); r.force[1] = to_double(F.y); r.force[2] = to_double(F.z);
            r.energy = to_double(E);
            r.steps = s.n;
            r.status = st;
            B->out[(size_t)(s.col - B->col_begin) * P.nz + s.k] = r;
            steps += (unsigned long long)s.n;
            status_or |= (unsigned)st;
            // System::lowerTip (system.hpp:51-54)
            s.dum.z = s.dum.z - P.dz;
            s.tip.z = s.tip.z - P.dz;
            if (++s.k < P.nz) {
                start_level();
            } else {
                if (s.tie && repair_list) {
                    const unsigned slot = atomicAdd(&ctr->n_tie, 1u);
                    if (slot < repair_cap)
                        repair_list[slot] = ((unsigned long long)s.scan << 32) | (unsigned)s.col;
                }
                s.col = -1;
            }
            continue;
        }
        tip_dummy_df(P, s.ex, s.dum, F, E);

        // ---- the integrator stage this evaluation belongs to (integrators.cpp:8-111) ----
        bool step_done = false;
        V3D SF = F;
        D SE = E;
        const D dt = s.dt;
        if (P.minimiser == MAFM_MIN_SD) {
            step_done = true;
        } else if (P.integrator == MAFM_INT_EULER) {
            const V3D pp = s.tip, v = s.vel;
            s.tip = {pp.x + dt * v.x, pp.y + dt * v.y, pp.z + dt * v.z};
            s.vel = {v.x + dt * F.x, v.y + dt * F.y, v.z + dt * F.z};
            step_done = true;
        } else if (P.integrator == MAFM_INT_MIDPOINT) {
            const D h = dt / D(2);
            if (s.phase == DF_EVAL0) {
                const V3D pp = s.tip, v = s.vel;
                s.ex = {pp.x + h * v.x, pp.y + h * v.y, pp.z + h * v.z};
                s.u = {v.x + h * F.x, v.y + h * F.y, v.z + h * F.z};
                s.phase = DF_EVAL1;
            } else {
                const V3D pp = s.tip, v = s.vel;
                s.tip = {pp.x + dt * s.u.x, pp.y + dt * s.u.y, pp.z + dt * s.u.z};
                s.vel = {v.x + dt * F.x, v.y + dt * F.y, v.z + dt * F.z};
                step_done = true;
            }
        } else {   // RK4
            const D h = dt / D(2);
            const V3D pp = s.tip, v = s.vel;
            if (s.phase == DF_EVAL0) {
                s.fs = F; s.es = E; s.vs = v;
                s.ex = {pp.x + h * v.x, pp.y + h * v.y, pp.z + h * v.z};
                s.u = {v.x + h * F.x, v.y + h * F.y, v.z + h * F.z};
                s.phase = DF_EVAL1;
            } else if (s.phase == DF_EVAL1 || s.phase == DF_EVAL2) {
                const D two(2);
                s.fs = {s.fs.x + two * F.x, s.fs.y + two * F.y, s.fs.z + two * F.z};
                s.es = s.es + two * E;
                s.vs = {s.vs.x + two * s.u.x, s.vs.y + two * s.u.y, s.vs.z + two * s.u.z};
                const D w = s.phase == DF_EVAL1 ? h : dt;
                s.ex = {pp.x + w * s.u.x, pp.y + w * s.u.y, pp.z + w * s.u.z};
                s.u = {v.x + w * F.x, v.y + w * F.y, v.z + w * F.z};
                s.phase = s.phase + 1;
            } else {
                s.fs = {s.fs.x + F.x, s.fs.y + F.y, s.fs.z + F.z};
                s.es = s.es + E;
                s.vs = {s.vs.x + s.u.x, s.vs.y + s.u.y, s.vs.z + s.u.z};
                const D s6 = dt / D(6);
                s.tip = {pp.x + s6 * s.vs.x, pp.y + s6 * s.vs.y, pp.z + s6 * s.vs.z};
                s.vel = {v.x + s6 * s.fs.x, v.y + s6 * s.fs.y, v.z + s6 * s.fs.z};
                SF = {s.fs.x / D(6), s.fs.y / D(6), s.fs.z / D(6)};
                SE = s.es / D(6);
                step_done = true;
            }
        }
        if (!step_done) continue;

        // ---- end of a minimiser step: FIREMinimisation / SDMinimisation
        //      (minimiser.cpp:39-129) ----
        const D prev = s.energy;
        s.energy = SE;
        const D ediff = SE - prev;
        const D fl = len3(SF);
        bool conv;
        {
            // checkConvergence (minimiser.cpp:15-37), and its near-ties
            const bool e_ok = dfl_fabs(ediff) < P.etol, f_ok = fl < P.ftol;
            conv = P.minterm == MAFM_TERM_E ? e_ok : P.minterm == MAFM_TERM_F ? f_ok : (e_ok && f_ok);
            const D ea = dfl_fabs(ediff) - P.etol, fa = fl - P.ftol;
            const bool e_tie = dfl_fabs(ea) < P.tie.conv_e, f_tie = dfl_fabs(fa) < P.tie.conv_f;
            bool near;
            if (P.minterm == MAFM_TERM_E) near = e_tie;
            else if (P.minterm == MAFM_TERM_F) near = f_tie;
            else near = (e_tie && !(fa > P.tie.conv_f)) || (f_tie && !(ea > P.tie.conv_e));
            s.tie |= near;
        }
        if (conv) {
            s.phase = DF_OUT;
            s.ex = s.tip;
            continue;
        }
        if (P.minimiser == MAFM_MIN_SD) {
            s.tip = {s.tip.x + P.dt * SF.x, s.tip.y + P.dt * SF.y, s.tip.z + P.dt * SF.z};
        } else {
            const V3D w = s.vel;
            const D pw = w.x * SF.x + w.y * SF.y + w.z * SF.z;
            V3D fh = {D(0), D(0), D(0)};
            if (fl > D(1e-10)) fh = {SF.x / fl, SF.y / fl, SF.z / fl};
            const D vl = len3(w);
            s.tie |= dfl_fabs(pw) < vl * (P.tie.p_f + P.tie.p_v * fl);
            const D one_a = D(1) - s.alpha;
            s.vel = {one_a * w.x + s.alpha * fh.x * vl, one_a * w.y + s.alpha * fh.y * vl,
                     one_a * w.z + s.alpha * fh.z * vl};
            if (pw < D(0)) {
                s.vel = {D(0), D(0), D(0)};
                s.nnn = 0;
                s.dt = s.dt * D(0.5);
                s.alpha = D(0.1);
            } else {
                if (s.nnn > 5) {
                    const D g = s.dt * D(1.1);
                    const D dt_max = D(10) * P.dt;
                    s.dt = dt_max < g ? dt_max : g;
                    s.alpha = s.alpha * D(0.99);
                }
                s.nnn++;
            }
        }
        s.n++;
        s.phase = s.n >= P.maxsteps ? DF_OUT : DF_EVAL0;
        s.ex = s.tip;
    }
    for (int off = 16; off > 0; off >>= 1) {
        steps += __shfl_xor_sync(kFull, steps, off);
        evals += __shfl_xor_sync(kFull, evals, off);
        pairs += __shfl_xor_sync(kFull, pairs, off);
        status_or |= __shfl_xor_sync(kFull, status_or, off);
        err |= __shfl_xor_sync(kFull, err, off);
    }
    if (lane == 0) {
        atomicAdd(&ctr->total_steps, steps);
        atomicAdd(&ctr->force_evals, evals);
        atomicAdd(&ctr->pair_evals, pairs);
        if (status_or | err) atomicOr(&ctr->error_word, status_or | err);
    }
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
