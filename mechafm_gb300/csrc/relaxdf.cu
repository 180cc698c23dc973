// relaxdf.cu — the double-float relaxation (precision MAFM_DF).
//
// Every quantity of the relaxation is a dfloat (dfloat.cuh): the tip–atom
// terms, their sums, the tip–dummy terms, positions, velocities, the FIRE
// time step and mixing factor, energies.  The minimiser's and integrators'
// operations are those of the FP64 kernel (fire_t / sd_t, relax_tpl.cuh),
// stage by stage, so the relaxation takes the same steps as FP64 unless one
// of FIRE's discrete decisions — the convergence test, the sign of P = v.F —
// falls within the double-float error (about 1e-13 of the largest term) of
// its threshold.  Such near-ties are recognised with a margin far above that
// error (TieMargins): the column is given up at its first one, goes on the
// list of the FP64 re-relaxation, and is relaxed again from its top height by
// one warp in FP64 with the plain FP64 kernel's bits (its points from that
// height on carry MAFM_PT_NEAR_TIE, all of them MAFM_PT_FP64) — inside this
// kernel by warps that have run out of columns, the rest by repair64_kernel
// after it.
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
#include "relax64_dev.cuh"
#include "relax_tpl.cuh"

namespace mafm {
namespace {

using D = dfloat;
using V3D = V3T<dfloat>;

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

using D2 = dfloat2;

// Sum of many double-floats, two at a time: the high parts through two_sum,
// every rounding error and low part into one FP32 word per element (a few
// ulps of the high part after hundreds of terms, far below the double-float
// error of a term).
struct LazySum2 {
    float2 h = {0.0f, 0.0f}, l = {0.0f, 0.0f};
    __device__ __forceinline__ void add(D2 x) {
        const D2 s = dfl2_two_sum(h, x.h);
        h = s.h;
        l = p_add(l, p_add(s.l, x.l));
    }
    // both elements' sums, added
    __device__ __forceinline__ D value() const {
        const D a = dfl_two_sum(h.x, l.x), b = dfl_two_sum(h.y, l.y);
        return a + b;
    }
};

__device__ __forceinline__ float2 f2(float4 v, int hi) {
    return hi ? make_float2(v.z, v.w) : make_float2(v.x, v.y);
}

// x^2: the square of the high part exactly (product and FMA residue), the
// cross term 2 h l into the low part (l^2 is below 2^-46 of the square).
__device__ __forceinline__ D2 sq_u(D2 x) {
    const float2 p = p_mul(x.h, x.h);
    return {p, p_fma(p_add(x.h, x.h), x.l, p_fma(x.h, x.h, p_neg(p)))};
}

// 1 / sqrt(a) as dfl2_rsqrt, for an operand that need not be normalised
__device__ __forceinline__ D2 rsqrt_u(D2 a) {
    const float2 y = make_float2(dfl_rsqrt_approx(a.h.x), dfl_rsqrt_approx(a.h.y));
    const D2 t = dfl2_mulf_u(dfl2_mulf_u(a, y), y);
    const float2 e = p_sub(p_sub(p_bcast(1.0f), t.h), t.l);
    return dfl2_fast_two_sum(y, p_mul(p_mul(y, e), p_bcast(0.5f)));
}

// The two terms of a TermPairDF record (element .x the first, .y the second).
struct PairDF2 {
    D2 x, y, z, qq, p0, p1, p2;
    int coul;
};

template <int KIND>
__device__ __forceinline__ PairDF2 load_pair(const TermPairDF* rec) {
    const float4* q = reinterpret_cast<const float4*>(rec);
    const float4 a = __ldg(q), b = __ldg(q + 1), c = __ldg(q + 2), g = __ldg(q + 3);
    const float4 h = __ldg(q + 4), m = __ldg(q + 5);
    PairDF2 t;
    t.x = {f2(a, 0), f2(a, 1)};
    t.y = {f2(b, 0), f2(b, 1)};
    t.z = {f2(c, 0), f2(c, 1)};
    t.qq = {f2(g, 0), f2(g, 1)};
    t.p0 = {f2(h, 0), f2(h, 1)};
    t.p1 = {f2(m, 0), f2(m, 1)};
    if (KIND == MAFM_PAIR_MORSE) {
        const float4 n = __ldg(q + 6);
        t.p2 = {f2(n, 0), f2(n, 1)};
    } else {
        t.p2 = {p_bcast(0.0f), p_bcast(0.0f)};
    }
    t.coul = __float_as_int(__ldg(reinterpret_cast<const float*>(q + 7)));
    return t;
}

// LJ (interactions.cpp:15-27) or Morse (:29-40), plus Coulomb (:42-51) when
// the record has one, for the separation d = tip - atom with r2 = |d|^2; the
// force on the tip and the energy go into the lazy sums.  1/r comes from a
// double-float rsqrt.
template <int KIND>
__device__ __forceinline__ void pair_df2_at(const PairDF2& t, D2 dx, D2 dy, D2 dz, D2 r2, LazySum2& fx,
                                            LazySum2& fy, LazySum2& fz, LazySum2& ee) {
    const D2 ir = rsqrt_u(r2);
    const D2 ir2 = dfl2_mul_u(ir, ir);
    D2 e, s;
    if (KIND == MAFM_PAIR_LJ) {
        // A = es12 / r^6, u = A - es6: E = u / r^6 = es12 / r^12 - es6 / r^6 and
        // (12 es12 / r^12 - 6 es6 / r^6) / r^2 = 6 (A + u) / r^6 / r^2; the
        // Coulomb term's qq / r^3 = (qq / r) / r^2 joins before the last / r^2
        const D2 ir6 = dfl2_norm(dfl2_mul_u(dfl2_mul_u(ir2, ir2), ir2));
        const D2 A = dfl2_mul_u(t.p1, ir6);
        const D2 u = dfl2_sub_u(A, t.p0);
        e = dfl2_mul_u(ir6, u);
        D2 sr = dfl2_mulf_u(dfl2_mul_u(dfl2_add_u(A, u), ir6), p_bcast(6.0f));
        if (t.coul) {
            const D2 ec = dfl2_mul_u(t.qq, ir);
            e = dfl2_add_u(e, ec);
            sr = dfl2_add_u(sr, ec);
        }
        s = dfl2_mul_u(sr, ir2);
    } else {
        const D2 r = dfl2_mul_u(r2, ir);
        const D2 qe = dfl2_exp(-dfl2_mul_u(t.p1, dfl2_sub_u(r, t.p2)));
        const D2 qe2 = dfl2_mul_u(qe, qe);
        // De (q^2 - 2 q + 1), 2 De a (q^2 - q) / r
        e = dfl2_mul_u(t.p0, dfl2_add_u(dfl2_sub_u(qe2, dfl2_mulf_u(qe, p_bcast(2.0f))),
                                        D2{p_bcast(1.0f), p_bcast(0.0f)}));
        s = dfl2_mul_u(dfl2_mul_u(dfl2_mulf_u(dfl2_mul_u(t.p0, t.p1), p_bcast(2.0f)),
                                  dfl2_sub_u(qe2, qe)), ir);
    }
    if (KIND == MAFM_PAIR_MORSE && t.coul) {
        const D2 ec = dfl2_mul_u(t.qq, ir);
        e = dfl2_add_u(e, ec);
        s = dfl2_add_u(s, dfl2_mul_u(ec, ir2));
    }
    fx.add(dfl2_mul_u(s, dx));
    fy.add(dfl2_mul_u(s, dy));
    fz.add(dfl2_mul_u(s, dz));
    ee.add(e);
}

// The two terms of a record at the tip (tx, ty, tz).
template <int KIND>
__device__ __forceinline__ void pair_df2(const TermPairDF* rec, D2 tx, D2 ty, D2 tz, LazySum2& fx,
                                         LazySum2& fy, LazySum2& fz, LazySum2& ee) {
    const PairDF2 t = load_pair<KIND>(rec);
    const D2 dx = dfl2_sub_u(tx, t.x), dy = dfl2_sub_u(ty, t.y), dz = dfl2_sub_u(tz, t.z);
    const D2 r2 = dfl2_add_u(dfl2_add_u(sq_u(dx), sq_u(dy)), sq_u(dz));
    pair_df2_at<KIND>(t, dx, dy, dz, r2, fx, fy, fz, ee);
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

// The sum of v over a group of G lanes (G a power of two, the group aligned
// in the warp), added in the same order on every lane of the group, so all
// of them hold the same bits.
template <int G>
__device__ __forceinline__ D group_sum(D v, int sub, unsigned gmask) {
#pragma unroll
    for (int m = 1; m < G; m <<= 1) {
        const D o(__shfl_xor_sync(gmask, v.h, m), __shfl_xor_sync(gmask, v.l, m));
        v = (sub & m) ? o + v : v + o;
    }
    return v;
}

// ForceGrid::interpolate (force_grid.cpp:88-275) on the double-float rigid
// grid, with interp64's handling of its border: a base node outside the grid
// is clamped and marks the point MAFM_PT_OUTSIDE (the reference's warning), a
// corner outside sets ERR_GRID_INDEX (the reference stops) and is clamped so
// that no read leaves the grid.
__device__ void interp_df_grid(const GridViewDF& g, V3D pos, V3D& f, D& e, int& outside,
                               unsigned& err) {
    const V3D q = {pos.x - g.origin[0], pos.y - g.origin[1], pos.z - g.origin[2]};
    const V3D pb = {q.x / g.basis[0], q.y / g.basis[4], q.z / g.basis[8]};
    const D fl[3] = {dfl_floor(pb.x), dfl_floor(pb.y), dfl_floor(pb.z)};
    int gp[3];
    for (int a = 0; a < 3; ++a) {
        gp[a] = (int)fl[a].h + (int)fl[a].l;
        if (gp[a] < 0) { gp[a] = 0; outside = 1; }
        else if (gp[a] >= g.n[a]) { gp[a] = g.n[a] - 1; outside = 1; }
    }
    int lo[3], hi[3];
    for (int a = 0; a < 3; ++a) {
        lo[a] = gp[a];
        hi[a] = gp[a] + 1;
        if (hi[a] >= g.n[a]) {
            err |= ERR_GRID_INDEX;
            hi[a] = g.n[a] - 1;
        }
    }
    const D dx = pb.x - D(gp[0]), dy = pb.y - D(gp[1]), dz = pb.z - D(gp[2]);
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
// energy at tip, by the G lanes of a group (lane sub of the group takes the
// term pairs sub, sub + G, ...; the external field on lane 0).  The loop over
// terms is the same for every group of a scan.
template <int G>
__device__ __forceinline__ void ts_df(const ScanParamsDF& p, V3D tip, int sub, unsigned gmask,
                                      V3D& F, D& E, int& outside, unsigned& err) {
    if (p.ts_mode == 2) {
        // the rigid grid alone; every lane of the group looks it up
        interp_df_grid(p.grid, tip, F, E, outside, err);
        return;
    }
    LazySum2 fx, fy, fz, ee;
    const D2 tx = dfl2(tip.x), ty = dfl2(tip.y), tz = dfl2(tip.z);
    const int n_lj = p.n_lj_pairs, n_all = p.n_lj_pairs + p.n_morse_pairs;
    for (int i = sub; i < n_lj; i += G)
        pair_df2<MAFM_PAIR_LJ>(p.pairs + i, tx, ty, tz, fx, fy, fz, ee);
    for (int i = n_lj + sub; i < n_all; i += G)
        pair_df2<MAFM_PAIR_MORSE>(p.pairs + i, tx, ty, tz, fx, fy, fz, ee);
    if (p.ts_mode == 1 && sub == 0) {
        V3D f;
        D e;
        interp_df(p.es, tip, f, e);
        fx.add(D2{make_float2(f.x.h, 0.0f), make_float2(f.x.l, 0.0f)});
        fy.add(D2{make_float2(f.y.h, 0.0f), make_float2(f.y.l, 0.0f)});
        fz.add(D2{make_float2(f.z.h, 0.0f), make_float2(f.z.l, 0.0f)});
        ee.add(D2{make_float2(e.h, 0.0f), make_float2(e.l, 0.0f)});
    }
    F = {group_sum<G>(fx.value(), sub, gmask), group_sum<G>(fy.value(), sub, gmask),
         group_sum<G>(fz.value(), sub, gmask)};
    E = group_sum<G>(ee.value(), sub, gmask);
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
    int col, scan, k, n, nnn, phase, tie, outside;
    V3D tip, vel, dum, ex, u, vs, fs;
    D energy, es, alpha, dt;
};

// An unwritten entry of the near-tie list (the host fills the list with it
// before each launch); real entries are scan << 32 | column.
constexpr unsigned long long kNoEntry = ~0ull;

// Claim the next near-tie list slot that a producer has already reserved
// (never past the count pushed so far, nor past the list); kNoEntry when
// there is none now.  Each failed compare-and-swap means another warp took a
// slot, so the loop ends; its bound is a safeguard.
__device__ unsigned long long claim_repair(RunCounters* ctr, unsigned cap) {
    unsigned long long cur = *reinterpret_cast<volatile unsigned long long*>(&ctr->repair_next);
    for (int i = 0; i < (1 << 20); ++i) {
        const unsigned n = min(*reinterpret_cast<volatile unsigned*>(&ctr->n_tie), cap);
        if (cur >= n) return kNoEntry;
        const unsigned long long prev = atomicCAS(&ctr->repair_next, cur, cur + 1);
        if (prev == cur) return cur;
        cur = prev;
    }
    return kNoEntry;
}

// The entry of a claimed slot: its producer reserved the slot and writes it
// right after, so the wait is short; it is bounded all the same (about half
// a second), after which ERR_REPAIR_WAIT is set and kNoEntry returned.
__device__ unsigned long long wait_entry(const unsigned long long* slot, unsigned& err) {
    for (int i = 0; i < (1 << 22); ++i) {
        const unsigned long long v = *reinterpret_cast<const volatile unsigned long long*>(slot);
        if (v != kNoEntry) return v;
        __nanosleep(100);
    }
    err |= ERR_REPAIR_WAIT;
    return kNoEntry;
}

__device__ __forceinline__ unsigned long long df_global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// The double-float relaxation as a slot machine: every group of G lanes of a
// warp holds one pixel column, and each loop iteration performs one force
// evaluation for every group that has one (the costly, uniform part; the
// group's lanes split the terms), then advances each group's minimiser by
// that evaluation: the integrator's stages (euler 1, midpoint 2, rk4 4
// evaluations per step), the convergence test and FIRE's mixing and time-step
// control, exactly in the order of fire_t / sd_t (relax_tpl.cuh), and the
// output evaluation of each height.  Every lane of a group holds the same
// state (the group sums are formed in one order on all of them) and runs the
// same minimiser code; lane 0 of the group writes.  A group whose column is
// done takes the next one from the global queue, so groups never wait for
// the slowest column of their warp.  G > 1 shortens each column's
// evaluations, which pays when a scan's longest columns, not the total work,
// set the launch's duration.
//
// Near-ties: at its first near-tie decision a column is given up.  Its
// unwritten heights get placeholder records (no steps, MAFM_PT_NEAR_TIE),
// and after a fence the column goes on repair_list.  A warp whose groups
// find the queue empty then re-relaxes listed columns in FP64, one warp per
// column (EvalWarp64 and relax_column_t<double>, the bits of repair64_kernel
// and relax64_kernel), while other warps still relax their last columns;
// repair64_kernel, launched after this kernel, takes the entries left.
template <int G>
__global__ void __launch_bounds__(128) relaxdf_kernel(const BatchDF* __restrict__ scans,
                                                      const BatchScan* __restrict__ scans64,
                                                      int n_scans, long long n_cols,
                                                      RunCounters* ctr,
                                                      unsigned long long* __restrict__ repair_list,
                                                      unsigned repair_cap,
                                                      unsigned long long watchdog_ns) {
    extern __shared__ __align__(32) unsigned char df_smem[];
    constexpr unsigned kFull = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int sub = lane & (G - 1);
    const int leader = lane & ~(G - 1);
    const unsigned gmask = G == 32 ? kFull : ((1u << G) - 1u) << leader;
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

    // the column's first near-tie: placeholders for its unwritten heights, a
    // fence (the re-relaxation's records must land after these), then the
    // list; the group drops the column
    auto give_up = [&]() {
        const ScanParamsDF& P = B->p;
        if (sub == 0) {
            mafm_point* o = B->out + (size_t)(s.col - B->col_begin) * P.nz;
            mafm_point r{};
            r.status = MAFM_PT_NEAR_TIE;
            for (int kk = s.k; kk < P.nz; ++kk) o[kk] = r;
            __threadfence();
            const unsigned slot = atomicAdd(&ctr->n_tie, 1u);
            if (slot < repair_cap)
                repair_list[slot] = ((unsigned long long)s.scan << 32) | (unsigned)s.col;
        }
        s.col = -1;
    };

    auto start_level = [&]() {
        s.outside = 0;
        s.alpha = D(0.1);
        s.dt = B->p.dt;
        s.nnn = 0;
        s.n = 1;
        s.phase = s.n >= B->p.maxsteps ? DF_OUT : DF_EVAL0;
        s.ex = s.tip;
    };

    for (;;) {
        // groups without a column take the next queue entries (one atomic per
        // warp; a group is counted by its first lane)
        const unsigned idle = __ballot_sync(kFull, sub == 0 && s.col < 0 && !done);
        if (idle) {
            unsigned long long base = 0;
            if (lane == 0) base = atomicAdd(&ctr->next_work, (unsigned long long)__popc(idle));
            base = __shfl_sync(kFull, base, 0);
            if (s.col < 0 && !done) {
                const long long g = (long long)base + __popc(idle & ((1u << leader) - 1u));
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
        ts_df<G>(P, s.ex, sub, gmask, F, E, s.outside, err);
        if (sub == 0) {
            evals += 1;
            pairs += (unsigned long long)B->n_pairs_per_eval;
        }
        if (s.phase == DF_OUT) {
            // System::getOutput (system.cpp:28-51)
            int st = (s.n >= P.maxsteps ? MAFM_PT_MAXSTEPS : 0) | (s.tie ? MAFM_PT_NEAR_TIE : 0) |
                     (s.outside ? MAFM_PT_OUTSIDE : 0);
            if (!dfl_isfinite(F.x) || !dfl_isfinite(F.y) || !dfl_isfinite(F.z) || !dfl_isfinite(E))
                st |= MAFM_PT_NONFINITE;
            mafm_point r;
            r.tip[0] = to_double(s.tip.x); r.tip[1] = to_double(s.tip.y); r.tip[2] = to_double(s.tip.z);
            r.force[0] = to_double(F.x); r.force[1] = to_double(F.y); r.force[2] = to_double(F.z);
            r.energy = to_double(E);
            r.steps = s.n;
            r.status = st;
            if (sub == 0) {
                B->out[(size_t)(s.col - B->col_begin) * P.nz + s.k] = r;
                steps += (unsigned long long)s.n;
                status_or |= (unsigned)st;
            }
            // System::lowerTip (system.hpp:51-54)
            s.dum.z = s.dum.z - P.dz;
            s.tip.z = s.tip.z - P.dz;
            if (++s.k < P.nz) {
                start_level();
            } else {
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
            const D h(__fmul_rn(dt.h, 0.5f), __fmul_rn(dt.l, 0.5f));   // dt / 2, exactly
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
            const D h(__fmul_rn(dt.h, 0.5f), __fmul_rn(dt.l, 0.5f));   // dt / 2, exactly
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
                const D sixth = D(1.0 / 6.0);
                s.tip = {pp.x + s6 * s.vs.x, pp.y + s6 * s.vs.y, pp.z + s6 * s.vs.z};
                s.vel = {v.x + s6 * s.fs.x, v.y + s6 * s.fs.y, v.z + s6 * s.fs.z};
                SF = {s.fs.x * sixth, s.fs.y * sixth, s.fs.z * sixth};
                SE = s.es * sixth;
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
        if (s.tie && repair_list) {
            give_up();
            continue;
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
            if (fl > D(1e-10)) {
                const D ifl = dfl_rcp(fl);
                fh = {SF.x * ifl, SF.y * ifl, SF.z * ifl};
            }
            const D vl = len3(w);
            s.tie |= dfl_fabs(pw) < vl * (P.tie.p_f + P.tie.p_v * fl);
            if (s.tie && repair_list) {
                give_up();
                continue;
            }
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

    // ---- the warp's columns are done: FP64 re-relaxation of listed columns ----
    if (repair_list && !(err & ERR_WATCHDOG)) {
        Node64* buf = reinterpret_cast<Node64*>(df_smem) + (size_t)(threadIdx.x >> 5) * 2 * kWarpChunk;
        long long rsteps = 0;
        unsigned long long revals = 0, rpairs = 0;
        unsigned rstatus = 0;
        for (;;) {
            unsigned long long slot = kNoEntry;
            if (lane == 0) slot = claim_repair(ctr, repair_cap);
            slot = __shfl_sync(kFull, slot, 0);
            if (slot == kNoEntry) break;
            unsigned long long e = kNoEntry;
            if (lane == 0) e = wait_entry(repair_list + slot, err);
            e = __shfl_sync(kFull, e, 0);
            if (e == kNoEntry) break;
            const BatchScan& R = scans64[(int)(e >> 32)];
            const long long c = (long long)(unsigned)(e & 0xffffffffull);
            EvalWarp64 ev{R.p, R.p.atoms64, R.p.n_terms_direct, R.p.ts_mode, lane, buf,
                          R.n_pairs_per_eval, 0u, 0ull};
            relax_column_t<double>(ev, R.p, c, R.out + (size_t)(c - R.col_begin) * R.p.nz, lane == 0,
                                   true, rsteps, revals, rstatus);
            rpairs += ev.pairs;
            err |= ev.err;
            __syncwarp();
        }
        if (lane == 0) {
            steps += (unsigned long long)rsteps;   // modular: a replacement subtracts
            evals += revals;
            pairs += rpairs;
            status_or |= rstatus;
        }
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

// Simulation::buildTipGridInteractions (simulation.cpp:420-501) in
// double-float.  One thread per strip of NB consecutive nodes of a grid
// column (z fastest, so a warp's strips share x and y and read the same term
// records): the tip on each node (the node's x and y wrapped into the cell
// under tip_pbc, as temp_system does, :462-464), every tip–surface term of p
// (ts_mode 1: with the external field).  The x and y separations of a record
// and their squares are formed once for the strip.
template <int NB>
__global__ void __launch_bounds__(128) grid_builddf_kernel(const ScanParamsDF p, NodeDF* out,
                                                           unsigned* err_word) {
    const GridViewDF& g = p.grid;
    const int nzs = (g.n[2] + NB - 1) / NB;
    const long long total = (long long)g.n[0] * g.n[1] * nzs;
    const int n_lj = p.n_lj_pairs, n_all = p.n_lj_pairs + p.n_morse_pairs;
    unsigned err = 0;
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const int k0 = (int)(idx % nzs) * NB;
        const long long ij = idx / nzs;
        const int j = (int)(ij % g.n[1]), i = (int)(ij / g.n[1]);
        D x, y;
        dummy_xy_t(p, p.tip_pbc != 0, D(i) * g.basis[0] + g.origin[0], D(j) * g.basis[4] + g.origin[1],
                   x, y);
        const D2 tx = dfl2(x), ty = dfl2(y);
        D2 tz[NB];
#pragma unroll
        for (int m = 0; m < NB; ++m) tz[m] = dfl2(D(k0 + m) * g.basis[8] + g.origin[2]);
        LazySum2 fx[NB], fy[NB], fz[NB], ee[NB];
#pragma unroll 1
        for (int r = 0; r < n_all; ++r) {
            const bool lj = r < n_lj;
            const PairDF2 t = lj ? load_pair<MAFM_PAIR_LJ>(p.pairs + r) : load_pair<MAFM_PAIR_MORSE>(p.pairs + r);
            const D2 dx = dfl2_sub_u(tx, t.x), dy = dfl2_sub_u(ty, t.y);
            const D2 dxy2 = dfl2_add_u(sq_u(dx), sq_u(dy));
#pragma unroll
            for (int m = 0; m < NB; ++m) {
                const D2 dz = dfl2_sub_u(tz[m], t.z);
                const D2 r2 = dfl2_add_u(dxy2, sq_u(dz));
                if (lj) pair_df2_at<MAFM_PAIR_LJ>(t, dx, dy, dz, r2, fx[m], fy[m], fz[m], ee[m]);
                else pair_df2_at<MAFM_PAIR_MORSE>(t, dx, dy, dz, r2, fx[m], fy[m], fz[m], ee[m]);
            }
        }
#pragma unroll
        for (int m = 0; m < NB; ++m) {
            if (k0 + m >= g.n[2]) break;
            V3D F = {fx[m].value(), fy[m].value(), fz[m].value()};
            D E = ee[m].value();
            if (p.ts_mode == 1) {
                V3D f;
                D e;
                interp_df(p.es, V3D{x, y, D(k0 + m) * g.basis[8] + g.origin[2]}, f, e);
                F = {F.x + f.x, F.y + f.y, F.z + f.z};
                E = E + e;
            }
            out[ij * g.n[2] + k0 + m] = NodeDF{F.x, F.y, F.z, E};
        }
    }
    if (err) atomicOr(err_word, err);
}

// Each double-float node as FP64: h + l (exact, both parts fit 53 bits).
__global__ void nodes_df_to_64_kernel(const NodeDF* in, Node64* out, long long n) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const NodeDF v = in[i];
        out[i] = Node64{to_double(v.x), to_double(v.y), to_double(v.z), to_double(v.w)};
    }
}

}  // namespace

std::vector<TermPairDF> term_pairs_df(const std::vector<AtomRec64>& terms, int& n_lj_pairs,
                                      int& n_morse_pairs) {
    auto split = [](double v, float2& hi, float2& lo, int e) {
        const float h = (float)v, l = (float)(v - (double)h);
        (e ? hi.y : hi.x) = h;
        (e ? lo.y : lo.x) = l;
    };
    std::vector<TermPairDF> out;
    auto add_run = [&](int kind) {
        std::vector<const AtomRec64*> run;
        for (const AtomRec64& r : terms)
            if (r.kind == kind) run.push_back(&r);
        for (size_t i = 0; i < run.size(); i += 2) {
            TermPairDF q{};
            for (int e = 0; e < 2; ++e) {
                // the second element of an odd run's last record: zero
                // parameters and charge at the first element's position
                const AtomRec64& r = *run[i + e < run.size() ? i + e : i];
                const bool real = i + e < run.size();
                split(r.x, q.xh, q.xl, e);
                split(r.y, q.yh, q.yl, e);
                split(r.z, q.zh, q.zl, e);
                split(real && r.coul ? r.qq : 0.0, q.qqh, q.qql, e);
                split(real ? r.p0 : 0.0, q.p0h, q.p0l, e);
                split(real ? r.p1 : 0.0, q.p1h, q.p1l, e);
                split(real ? r.p2 : 0.0, q.p2h, q.p2l, e);
                if (real && r.coul) q.coul = 1;
            }
            out.push_back(q);
        }
        return (int)((run.size() + 1) / 2);
    };
    n_lj_pairs = add_run(MAFM_PAIR_LJ);
    n_morse_pairs = add_run(MAFM_PAIR_MORSE);
    return out;
}

static GridViewDF grid_view_df(const GridView& g, const NodeDF* nodes) {
    GridViewDF q{};
    q.g = nodes;
    for (int a = 0; a < 3; ++a) {
        q.n[a] = g.n[a];
        q.origin[a] = D(g.origin[a]);
    }
    q.periodic = g.periodic;
    q.orthogonal = g.orthogonal;
    for (int k = 0; k < 9; ++k) {
        q.basis[k] = D(g.basis[k]);
        q.inv[k] = D(g.inv[k]);
    }
    return q;
}

ScanParamsDF params_df(const ScanParams& p, const TermPairDF* pairs, int n_lj_pairs,
                       int n_morse_pairs, const NodeDF* es_nodes, const NodeDF* grid_nodes) {
    ScanParamsDF q{};
    q.n_lj_pairs = n_lj_pairs;
    q.n_morse_pairs = n_morse_pairs;
    q.pairs = pairs;
    q.ts_mode = p.ts_mode;
    q.es = grid_view_df(p.es, es_nodes);
    q.grid = grid_view_df(p.grid, grid_nodes);
    for (int a = 0; a < 3; ++a) {
        q.offset[a] = D(p.offset[a]);
        q.td_p[a] = D(p.td_p[a]);
    }
    for (int k = 0; k < 9; ++k) {
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

// Shared memory of a block: the FP64 re-relaxation's per-warp buffers.
constexpr size_t kDfSmem = (size_t)(128 / 32) * 2 * kWarpChunk * sizeof(Node64);

// Default: one lane per column while the columns fill the resident lanes;
// fewer columns share out their terms, G = the largest power of two up to 8
// with G x columns <= 1.25 x the resident lanes.  Measured (MAFM_DF_LANES
// overrides), G = 1 / 2 / 4 / 8: 401 x 401 cluster (160,801 columns, 58,368
// resident lanes) 768 / 823 / 935 / 1627 ms; 128 x 128 cluster (16,384
// columns) 183 / 162 / 142 / 182 ms; 101 x 101 graphene (10,201 columns)
// 147 / 129 / 111 / 158 ms.
int df_lanes_per_column(long long n_cols, int requested) {
    if (requested == 1 || requested == 2 || requested == 4 || requested == 8) return requested;
    if (const char* e = std::getenv("MAFM_DF_LANES")) {
        const int v = std::atoi(e);
        if (v == 1 || v == 2 || v == 4 || v == 8) return v;
    }
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, relaxdf_kernel<1>, 128, kDfSmem) != cudaSuccess ||
        per_sm <= 0)
        per_sm = 1;
    const long long lanes = (long long)sm_count() * per_sm * 128;
    int g = 1;
    while (g < 8 && n_cols > 0 && 4 * (2 * g * n_cols) <= 5 * lanes) g *= 2;
    return g;
}

template <int G>
static cudaError_t launch_relaxdf_g(const BatchDF* scans, const BatchScan* scans64, int n_scans,
                                   long long n_cols, RunCounters* ctr,
                                   unsigned long long* repair_list, unsigned repair_cap,
                                   unsigned long long watchdog_ns, cudaStream_t s) {
    constexpr int kThreads = 128;
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, relaxdf_kernel<G>, kThreads,
                                                                  kDfSmem);
    if (e != cudaSuccess) return e;
    if (per_sm <= 0) per_sm = 1;
    long long blocks = (long long)sm_count() * per_sm;
    const long long need = (n_cols * G + kThreads - 1) / kThreads;
    blocks = std::max(1ll, std::min(blocks, need));
    relaxdf_kernel<G><<<(unsigned)blocks, kThreads, kDfSmem, s>>>(
        scans, scans64, n_scans, n_cols, ctr, repair_list, repair_list ? repair_cap : 0u, watchdog_ns);
    return cudaGetLastError();
}

cudaError_t launch_relaxdf(const BatchDF* scans, const BatchScan* scans64, int n_scans, long long n_cols,
                           RunCounters* ctr, unsigned long long* repair_list, unsigned repair_cap,
                           unsigned long long watchdog_ns, int lanes_per_column, cudaStream_t s) {
    if (n_cols <= 0) return cudaSuccess;
    if (repair_list) {
        // an unwritten entry reads as kNoEntry (all bits set)
        const cudaError_t e = cudaMemsetAsync(repair_list, 0xFF, (size_t)repair_cap * sizeof(*repair_list), s);
        if (e != cudaSuccess) return e;
    }
    switch (df_lanes_per_column(n_cols, lanes_per_column)) {
        case 2: return launch_relaxdf_g<2>(scans, scans64, n_scans, n_cols, ctr, repair_list, repair_cap, watchdog_ns, s);
        case 4: return launch_relaxdf_g<4>(scans, scans64, n_scans, n_cols, ctr, repair_list, repair_cap, watchdog_ns, s);
        case 8: return launch_relaxdf_g<8>(scans, scans64, n_scans, n_cols, ctr, repair_list, repair_cap, watchdog_ns, s);
        default: return launch_relaxdf_g<1>(scans, scans64, n_scans, n_cols, ctr, repair_list, repair_cap, watchdog_ns, s);
    }
}

cudaError_t launch_nodes_to_df(const Node64* in, NodeDF* out, long long n, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    long long blocks = std::min((n + 255) / 256, (long long)sm_count() * 32);
    nodes_to_df_kernel<<<(unsigned)blocks, 256, 0, s>>>(in, out, n);
    return cudaGetLastError();
}

cudaError_t launch_grid_builddf(const ScanParamsDF& p, NodeDF* out, Node64* out64, unsigned* err_word,
                                cudaStream_t s) {
    const long long n = (long long)p.grid.n[0] * p.grid.n[1] * p.grid.n[2];
    if (n <= 0) return cudaSuccess;
    ScanParamsDF q = p;
    q.grid.g = out;
    constexpr int kNB = 4;
    const long long strips = (long long)p.grid.n[0] * p.grid.n[1] * ((p.grid.n[2] + kNB - 1) / kNB);
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, grid_builddf_kernel<kNB>, 128, 0);
    if (e != cudaSuccess) return e;
    if (per_sm <= 0) per_sm = 1;
    const long long blocks = std::max(1ll, std::min((strips + 127) / 128, (long long)sm_count() * per_sm * 8));
    grid_builddf_kernel<kNB><<<(unsigned)blocks, 128, 0, s>>>(q, out, err_word);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const long long b64 = std::min((n + 255) / 256, (long long)sm_count() * 32);
    nodes_df_to_64_kernel<<<(unsigned)b64, 256, 0, s>>>(out, out64, n);
    return cudaGetLastError();
}

}  // namespace mafm
