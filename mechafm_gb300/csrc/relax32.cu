// relax32.cu — the FP32-compensated GPU path (precision MAFM_FP32C).
//
// Persistent, multi-scan relaxation kernel.  Work is a list of tiles of pixel
// columns, possibly from many scans (a batch); each warp takes one tile at a
// time with an atomic counter, and G lanes share one column (G = 1..32, a
// launch parameter from the autotuner or the default rule in scan.cu).  The warp's current scan's
// tip–atom terms are staged into the warp's slice of shared memory with a
// bulk copy (cp.async.bulk + mbarrier); every lane of a group sums its share
// of the terms, then the group combines its sums with xor shuffles.
//
// The main loop runs in "slots": one force evaluation per group per slot,
// then a per-group state machine advances FIRE/SD and the integrator
// (euler 1, midpoint 2, rk4 4 evaluations per step).  The evaluation that
// produces a point's output (System::getOutput, system.cpp:28-51) is one more
// slot, so lanes never wait on a divergent extra pair loop.
//
// Precision: pair terms in FP32, two per packed f32x2 instruction in the relax
// loop (1/r from rsqrt.approx, LJ's 1/r^2 its square, exp from __expf); the
// scalar paths (tip–dummy term, sampling) take 1/r^2 from rcp.approx refined
// by one Newton step.  Tip positions, the energy behind the e/ef convergence
// test and the spring energy are double-floats (hi + lo FP32), so that
// tip–atom separations keep ~1e-7 relative accuracy without FP64 arithmetic
// in the slot path; sums are compensated (Kahan) over chunks of 8 terms in
// the relax loop and 64 in the grid build, and groups combine them with
// two-sums.
//
// Reference correspondence (src/): as relax64.cu — interactions.cpp:15-51,
// 244-266; force_grid.cpp:88-275; integrators.cpp:8-111; minimiser.cpp:15-129;
// simulation.cpp:93-122, 420-501; system.cpp:28-51, 139-162.
#include <cstdint>

#include "mafm_internal.h"

namespace mafm {
namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kChunk = 8;                 // terms summed plainly before a compensated add
// Records (term pairs) per compensated add in the grid build: a node sums
// thousands of terms (18,432 on the periodic slab), most of them small; 64
// terms per plain FP32 sum keep the grid's accuracy (tip within 1e-3 A on the
// same fraction of points as 8 terms per sum) and take the compensation from
// a quarter of the FMA-pipe work to a few percent (slab build 1504 -> 1326 ms).
constexpr int kBuildChunkUnits = 32;
constexpr long long kWaitLimit = 1ll << 24;  // bounded mbarrier wait (iterations)

enum : int { PH_EVAL0 = 0, PH_EVAL1 = 1, PH_EVAL2 = 2, PH_EVAL3 = 3, PH_OUT = 4 };

// ---------------------------------------------------------------- helpers ----

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

struct DF {   // double-float value hi + lo
    float hi, lo;
};

__device__ __forceinline__ DF df_split(double x) {
    const float h = (float)x;
    return DF{h, (float)(x - (double)h)};
}

__device__ __forceinline__ double df_val(DF a) { return (double)a.hi + (double)a.lo; }

// a + b for a small float b
__device__ __forceinline__ DF df_add(DF a, float b) {
    float s, e;
    two_sum(a.hi, b, s, e);
    e += a.lo;
    const float h = s + e;
    return DF{h, e - (h - s)};
}

__device__ __forceinline__ float rcp_nr(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    const float e = fmaf(-x, r, 1.0f);
    return fmaf(r, e, r);
}

__device__ __forceinline__ float rsqrt_fast(float x) {
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// Compensated accumulator of {Fx, Fy, Fz, E}.
struct Acc {
    float s[4], c[4];
    __device__ __forceinline__ void zero() {
#pragma unroll
        for (int m = 0; m < 4; ++m) s[m] = c[m] = 0.f;
    }
    // Kahan step: c carries the negated low part lost so far.
    __device__ __forceinline__ void add(const float v[4]) {
#pragma unroll
        for (int m = 0; m < 4; ++m) {
            const float y = v[m] - c[m];
            const float t = s[m] + y;
            c[m] = (t - s[m]) - y;
            s[m] = t;
        }
    }
    // value = s - c
    __device__ __forceinline__ float val(int m) const { return s[m] - c[m]; }
    // Combine across the G lanes of a group; every lane ends with the same sums
    // (two-sum and + are commutative, so partners compute identical values).
    template <int G>
    __device__ __forceinline__ void group_reduce() {
#pragma unroll
        for (int off = G / 2; off > 0; off >>= 1) {
#pragma unroll
            for (int m = 0; m < 4; ++m) {
                const float so = __shfl_xor_sync(kFull, s[m], off);
                const float co = __shfl_xor_sync(kFull, c[m], off);
                float t, e;
                two_sum(s[m], so, t, e);
                s[m] = t;
                c[m] = (c[m] + co) - e;
            }
        }
    }
};

// One tip–atom term: LJ or Morse (interactions.cpp:15-40) plus Coulomb
// (:42-51, qq = 0 when absent).  d = tip - atom.
__device__ __forceinline__ void pair32(const AtomRec32& t, float dx, float dy, float dz,
                                       bool coul, float v[4]) {
    const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    float fs, e;
    if (__float_as_int(t.b.w) == MAFM_PAIR_LJ) {
        const float ir2 = rcp_nr(r2);
        const float ir6 = ir2 * ir2 * ir2;
        const float t6 = t.b.x * ir6;
        const float t12 = t.b.y * ir6 * ir6;
        e = t12 - t6;
        fs = fmaf(12.f, t12, -6.f * t6) * ir2;
    } else {
        const float ir = rsqrt_fast(r2);
        const float r = r2 * ir;
        const float d = __expf(-t.b.y * (r - t.b.z));
        const float dm1 = d - 1.f;
        e = t.b.x * dm1 * dm1;
        fs = 2.f * t.b.x * t.b.y * d * dm1 * ir;
    }
    if (coul) {
        const float ir = rsqrt_fast(r2);
        const float ec = t.a.w * ir;
        fs = fmaf(ec * ir, ir, fs);
        e += ec;
    }
    v[0] = fmaf(fs, dx, v[0]);
    v[1] = fmaf(fs, dy, v[1]);
    v[2] = fmaf(fs, dz, v[2]);
    v[3] += e;
}

// ---- packed (f32x2) tip–atom terms: two terms per instruction -------------

__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

// Tip position broadcast to both components.  Separations use the high
// word of the double-float position only: the atoms are FP32-rounded, so the
// low word (< half an FP32 ulp of the position) adds nothing to the accuracy
// of a separation; it still carries the position update between steps.
struct Tip2 {
    float2 hx, hy, hz;
};

// Sums of one chunk: negated forces and the energy, per component.
struct Sum2 {
    float2 gx, gy, gz, e;
};

// Two terms of a TermPair32 at one tip position, given the separation
// d = tip - atom and dx^2 + dy^2: LJ (interactions.cpp:15-27) or Morse
// (:29-40), plus Coulomb (:42-51) when `coul`.  1/r comes from rsqrt.approx
// and LJ's 1/r^2 is its square, which Coulomb reuses (qq/r^3 = (qq/r)/r^2).
// Accumulates -F and E into s.
template <bool kMorse, bool kDeriveLJ>
__device__ __forceinline__ void unit32_at(const TermPair32& t, float2 dx, float2 dy, float2 dxy2,
                                          float2 dz, bool coul, Sum2& s) {
    const float4 zq = t.zq, pa = t.pa, pb = t.pb;
    const float2 r2 = fma2(dz, dz, dxy2);
    const float2 ir = make_float2(rsqrt_fast(r2.x), rsqrt_fast(r2.y));
    float2 nfs, e;
    if (!kMorse) {
        const float2 ir2 = mul2(ir, ir);
        const float2 ir6 = mul2(mul2(ir2, ir2), ir2);
        if (kDeriveLJ) {
            // A = es12 r^-6, t = A - es6: E = r^-6 t, -F/d = -6 r^-8 (A + t);
            // the record's fourth float4 is not read (one shared load fewer
            // per record for two multiplies: the relax loop is limited by
            // shared loads as much as by the FMA pipe)
            const float2 A = mul2(make_float2(pa.z, pa.w), ir6);
            const float2 tt = add2(A, make_float2(pa.x, pa.y));
            e = mul2(ir6, tt);
            nfs = mul2(mul2(ir6, ir2), mul2(add2(A, tt), f2(-6.f)));
        } else {
            // E = r^-6 (es12 r^-6 - es6), -F/d = r^-8 (6 es6 - 12 es12 r^-6)
            e = mul2(ir6, fma2(make_float2(pa.z, pa.w), ir6, make_float2(pa.x, pa.y)));
            nfs = mul2(mul2(ir6, ir2), fma2(make_float2(pb.x, pb.y), ir6, make_float2(pb.z, pb.w)));
        }
        if (coul) {
            const float2 nec = mul2(make_float2(zq.z, zq.w), ir);          // -qq/r
            nfs = fma2(nec, ir2, nfs);
            e = fma2(nec, f2(-1.f), e);
        }
    } else {
        const float2 r = mul2(r2, ir);
        const float2 arg = mul2(make_float2(pa.z, pa.w), add2(r, make_float2(pb.x, pb.y)));
        const float2 d = make_float2(__expf(arg.x), __expf(arg.y));
        const float2 dm1 = add2(d, f2(-1.f));
        e = mul2(mul2(make_float2(pa.x, pa.y), dm1), dm1);
        nfs = mul2(mul2(mul2(make_float2(pb.z, pb.w), d), dm1), ir);
        if (coul) {
            const float2 nec = mul2(make_float2(zq.z, zq.w), ir);
            nfs = fma2(mul2(nec, ir), ir, nfs);
            e = fma2(nec, f2(-1.f), e);
        }
    }
    s.gx = fma2(nfs, dx, s.gx);
    s.gy = fma2(nfs, dy, s.gy);
    s.gz = fma2(nfs, dz, s.gz);
    s.e = add2(s.e, e);
}

// Two terms of a TermPair32 at the tip position p.
template <bool kMorse>
__device__ __forceinline__ void unit32(const TermPair32& t, const Tip2& p, bool coul, Sum2& s) {
    const float4 xy = t.xy, zq = t.zq;
    const float2 dx = add2(p.hx, make_float2(xy.x, xy.y));   // tip - atom
    const float2 dy = add2(p.hy, make_float2(xy.z, xy.w));
    const float2 dz = add2(p.hz, make_float2(zq.x, zq.y));
    unit32_at<kMorse, true>(t, dx, dy, fma2(dy, dy, mul2(dx, dx)), dz, coul, s);
}

// Units [begin, end) of one kind: lane lg of the group takes begin + lg,
// begin + lg + G, ...; kChunk / 2 units (kChunk terms) are summed plainly
// before one compensated add.  Full chunks run without bounds tests.
template <int G, bool kMorse, bool kCoul>
__device__ __forceinline__ void sum_units(const TermPair32* units, int begin, int end, int lg,
                                          const Tip2& tp, Acc& acc) {
    constexpr bool coul = kCoul;
    constexpr int kUnits = kChunk / 2;
    int u0 = begin + lg;
    for (; u0 + (kUnits - 1) * G < end; u0 += G * kUnits) {
        Sum2 sm;
        sm.gx = sm.gy = sm.gz = sm.e = f2(0.f);
#pragma unroll
        for (int c = 0; c < kUnits; ++c) unit32<kMorse>(units[u0 + c * G], tp, coul, sm);
        const float v[4] = {-(sm.gx.x + sm.gx.y), -(sm.gy.x + sm.gy.y), -(sm.gz.x + sm.gz.y),
                            sm.e.x + sm.e.y};
        acc.add(v);
    }
    if (u0 < end) {
        Sum2 sm;
        sm.gx = sm.gy = sm.gz = sm.e = f2(0.f);
#pragma unroll
        for (int c = 0; c < kUnits - 1; ++c)
            if (u0 + c * G < end) unit32<kMorse>(units[u0 + c * G], tp, coul, sm);
        const float v[4] = {-(sm.gx.x + sm.gx.y), -(sm.gy.x + sm.gy.y), -(sm.gz.x + sm.gz.y),
                            sm.e.x + sm.e.y};
        acc.add(v);
    }
}

// Units [begin, end) of one kind for NB tip positions that share x and y (a
// strip of NB nodes of one grid column): the x and y separations and
// dx^2 + dy^2 are computed once per record for all NB positions.
// One record for the NB positions of a strip.
template <bool kMorse, bool kCoul, int NB>
__device__ __forceinline__ void unit32_strip(const TermPair32& t, float2 hx, float2 hy,
                                             const float2 (&hz)[NB], Sum2 (&sm)[NB]) {
    const float4 xy = t.xy, zq = t.zq;
    const float2 dx = add2(hx, make_float2(xy.x, xy.y));
    const float2 dy = add2(hy, make_float2(xy.z, xy.w));
    const float2 dxy2 = fma2(dy, dy, mul2(dx, dx));
    const float2 naz = make_float2(zq.x, zq.y);
#pragma unroll
    for (int n = 0; n < NB; ++n)
        unit32_at<kMorse, false>(t, dx, dy, dxy2, add2(hz[n], naz), kCoul, sm[n]);
}

template <int NB>
__device__ __forceinline__ void add_strip(const Sum2 (&sm)[NB], Acc (&acc)[NB]) {
#pragma unroll
    for (int n = 0; n < NB; ++n) {
        const float v[4] = {-(sm[n].gx.x + sm[n].gx.y), -(sm[n].gy.x + sm[n].gy.y),
                            -(sm[n].gz.x + sm[n].gz.y), sm[n].e.x + sm[n].e.y};
        acc[n].add(v);
    }
}

// Coulomb on or off is a compile-time choice.  kU records (2 kU terms) are
// summed plainly per compensated add, four at a time; full chunks run
// without bounds tests and the last, partial chunk with them.
template <bool kMorse, bool kCoul, int NB, int kU>
__device__ __forceinline__ void sum_units_strip(const TermPair32* units, int begin, int end,
                                                float2 hx, float2 hy, const float2 (&hz)[NB],
                                                Acc (&acc)[NB]) {
    static_assert(kU % 4 == 0, "records per chunk: a multiple of 4");
    int u0 = begin;
    for (; u0 + kU <= end; u0 += kU) {
        Sum2 sm[NB];
#pragma unroll
        for (int n = 0; n < NB; ++n) sm[n].gx = sm[n].gy = sm[n].gz = sm[n].e = f2(0.f);
#pragma unroll 1
        for (int h = 0; h < kU; h += 4) {
#pragma unroll
            for (int c = 0; c < 4; ++c) unit32_strip<kMorse, kCoul, NB>(units[u0 + h + c], hx, hy, hz, sm);
        }
        add_strip<NB>(sm, acc);
    }
    if (u0 < end) {
        Sum2 sm[NB];
#pragma unroll
        for (int n = 0; n < NB; ++n) sm[n].gx = sm[n].gy = sm[n].gz = sm[n].e = f2(0.f);
#pragma unroll 1
        for (; u0 + 4 <= end; u0 += 4) {
#pragma unroll
            for (int c = 0; c < 4; ++c) unit32_strip<kMorse, kCoul, NB>(units[u0 + c], hx, hy, hz, sm);
        }
#pragma unroll
        for (int c = 0; c < 3; ++c)
            if (u0 + c < end) unit32_strip<kMorse, kCoul, NB>(units[u0 + c], hx, hy, hz, sm);
        add_strip<NB>(sm, acc);
    }
}

// FP32 view of a trilinear grid (ForceGrid, force_grid.hpp:15-51), converted
// from the FP64 GridView once per scan: reciprocal steps (orthogonal) or the
// inverse basis, and the origin split into hi + lo floats.
struct Lookup32 {
    const float4* g;
    int n[3];
    int periodic, orthogonal;
    float inv[9];
    float org_hi[3], org_lo[3];
};

__device__ Lookup32 make_lookup(const GridView& g) {
    Lookup32 L;
    L.g = g.g32;
    for (int a = 0; a < 3; ++a) {
        L.n[a] = g.n[a];
        const DF o = df_split(g.origin[a]);
        L.org_hi[a] = o.hi;
        L.org_lo[a] = o.lo;
    }
    L.periodic = g.periodic;
    L.orthogonal = g.orthogonal;
    for (int k = 0; k < 9; ++k) L.inv[k] = 0.f;
    if (g.orthogonal) {
        L.inv[0] = (float)(1.0 / g.basis[0]);
        L.inv[4] = (float)(1.0 / g.basis[4]);
        L.inv[8] = (float)(1.0 / g.basis[8]);
    } else {
        for (int k = 0; k < 9; ++k) L.inv[k] = (float)g.inv[k];
    }
    return L;
}

// Trilinear lookup (ForceGrid::interpolate) at a double-float position; adds
// {Fx,Fy,Fz,E} into v.  Sets outside when clamped at the border, and
// ERR_GRID_INDEX when a corner of a non-periodic grid falls outside (the
// corner is then clamped, so no read leaves the grid).
__device__ void interp32(const Lookup32& L, DF px, DF py, DF pz, float v[4], int& outside,
                         unsigned& err) {
    const float qx = (px.hi - L.org_hi[0]) + (px.lo - L.org_lo[0]);
    const float qy = (py.hi - L.org_hi[1]) + (py.lo - L.org_lo[1]);
    const float qz = (pz.hi - L.org_hi[2]) + (pz.lo - L.org_lo[2]);
    float pb[3];
    if (L.orthogonal) {
        pb[0] = qx * L.inv[0];
        pb[1] = qy * L.inv[4];
        pb[2] = qz * L.inv[8];
    } else {
        pb[0] = L.inv[0] * qx + L.inv[1] * qy + L.inv[2] * qz;
        pb[1] = L.inv[3] * qx + L.inv[4] * qy + L.inv[5] * qz;
        pb[2] = L.inv[6] * qx + L.inv[7] * qy + L.inv[8] * qz;
    }
    int gp[3];
    float d[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        gp[a] = (int)floorf(pb[a]);
        if (!L.periodic) {
            if (gp[a] < 0) { gp[a] = 0; outside = 1; }
            else if (gp[a] >= L.n[a]) { gp[a] = L.n[a] - 1; outside = 1; }
        }
        d[a] = pb[a] - (float)gp[a];
    }
    int lo[3], hi[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        int x0 = gp[a], x1 = gp[a] + 1;
        if (L.periodic) {
            x0 %= L.n[a]; if (x0 < 0) x0 += L.n[a];
            x1 %= L.n[a]; if (x1 < 0) x1 += L.n[a];
        } else if (x1 >= L.n[a]) {
            err |= ERR_GRID_INDEX;
            x1 = L.n[a] - 1;
        }
        lo[a] = x0;
        hi[a] = x1;
    }
    const long long n12 = (long long)L.n[1] * L.n[2];
    float4 s[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        const int x = (c >> 2) ? hi[0] : lo[0];
        const int y = ((c >> 1) & 1) ? hi[1] : lo[1];
        const int z = (c & 1) ? hi[2] : lo[2];
        s[c] = __ldg(L.g + (long long)x * n12 + (long long)y * L.n[2] + z);
    }
    const float dx = d[0], dy = d[1], dz = d[2];
    auto lerp3 = [&](float a0, float a1, float a2, float a3, float a4, float a5, float a6, float a7) {
        const float v00 = a0 * (1 - dx) + a4 * dx, v01 = a1 * (1 - dx) + a5 * dx;
        const float v10 = a2 * (1 - dx) + a6 * dx, v11 = a3 * (1 - dx) + a7 * dx;
        const float v0 = v00 * (1 - dy) + v10 * dy, v1 = v01 * (1 - dy) + v11 * dy;
        return v0 * (1 - dz) + v1 * dz;
    };
    v[0] += lerp3(s[0].x, s[1].x, s[2].x, s[3].x, s[4].x, s[5].x, s[6].x, s[7].x);
    v[1] += lerp3(s[0].y, s[1].y, s[2].y, s[3].y, s[4].y, s[5].y, s[6].y, s[7].y);
    v[2] += lerp3(s[0].z, s[1].z, s[2].z, s[3].z, s[4].z, s[5].z, s[6].z, s[7].z);
    v[3] += lerp3(s[0].w, s[1].w, s[2].w, s[3].w, s[4].w, s[5].w, s[6].w, s[7].w);
}

// System::setDummyXY (system.cpp:139-162) in FP64.
__device__ __forceinline__ void dummy_xy(const ScanParams& p, bool wrap, double x, double y,
                                         double& ox, double& oy) {
    if (wrap) {
        const double* ci = p.cell_inv;
        const double* c = p.cell;
        const double tx = x - p.offset[0], ty = y - p.offset[1], tz = 0 - p.offset[2];
        double cx = ci[0] * tx + ci[1] * ty + ci[2] * tz;
        double cy = ci[3] * tx + ci[4] * ty + ci[5] * tz;
        const double cz = ci[6] * tx + ci[7] * ty + ci[8] * tz;
        cx -= floor(cx);
        cy -= floor(cy);
        ox = (c[0] * cx + c[1] * cy + c[2] * cz) + p.offset[0];
        oy = (c[3] * cx + c[4] * cy + c[5] * cz) + p.offset[1];
    } else {
        ox = x;
        oy = y;
    }
}

// The scan's scalars in FP32, converted once per scan switch: the relax
// loop then runs without FP64 instructions (the FP64 pipe of GB300 is 1/64
// of the FP32 rate).
struct WarpParams {
    Lookup32 grid, es;
    float dt0, dt_max, etol, ftol;
    float td_p0, td_p1, td_p2, td_qq;
    float harm_k, harm_r0;
    DF dz;
    int maxsteps, minimiser, integrator, minterm;
    int ts_mode, td_kind, td_coul, nz;
    int ny, col_begin, pad0, pad1;
};

__device__ void make_warp_params(const BatchScan& B, WarpParams& w) {
    const ScanParams& P = B.p;
    w.grid = make_lookup(P.grid);
    w.es = make_lookup(P.es);
    w.dt0 = (float)P.dt;
    w.dt_max = (float)(10 * P.dt);
    w.etol = (float)P.etol;
    w.ftol = (float)P.ftol;
    w.td_p0 = (float)P.td_p[0];
    w.td_p1 = (float)P.td_p[1];
    w.td_p2 = (float)P.td_p[2];
    w.td_qq = (float)P.td_qq;
    w.harm_k = (float)P.harm_k;
    w.harm_r0 = (float)P.harm_r0;
    w.dz = df_split(P.dz);
    w.maxsteps = P.maxsteps;
    w.minimiser = P.minimiser;
    w.integrator = P.integrator;
    w.minterm = P.minterm;
    w.ts_mode = P.ts_mode;
    w.td_kind = P.td_kind;
    w.td_coul = P.td_coul;
    w.nz = P.nz;
    w.ny = P.ny;
    w.col_begin = B.col_begin;
    w.pad0 = w.pad1 = 0;
}

// vdW (+ Coulomb) term of the dummy–tip pair in FP32; r = dummy - tip.
__device__ __forceinline__ void td_vdw32(const WarpParams& w, float rx, float ry, float rz,
                                         float f[3], float& e) {
    const float r2 = rx * rx + ry * ry + rz * rz;
    float fs;
    if (w.td_kind == MAFM_PAIR_LJ) {
        const float ir2 = rcp_nr(r2);
        const float ir6 = ir2 * ir2 * ir2;
        const float t6 = w.td_p0 * ir6;
        const float t12 = w.td_p1 * ir6 * ir6;
        e = t12 - t6;
        fs = fmaf(12.f, t12, -6.f * t6) * ir2;
    } else {
        const float ir = rsqrt_fast(r2);
        const float r = r2 * ir;
        const float d = __expf(-w.td_p1 * (r - w.td_p2));
        const float dm1 = d - 1.f;
        e = w.td_p0 * dm1 * dm1;
        fs = 2.f * w.td_p0 * w.td_p1 * d * dm1 * ir;
    }
    if (w.td_coul) {
        const float ir = rsqrt_fast(r2);
        const float ec = w.td_qq * ir;
        fs = fmaf(ec * ir, ir, fs);
        e += ec;
    }
    f[0] = fs * rx;
    f[1] = fs * ry;
    f[2] = fs * rz;
}

// double-float helpers
__device__ __forceinline__ DF df_norm(float s, float c) {
    const float h = s + c;
    return DF{h, c - (h - s)};
}

__device__ __forceinline__ DF df_add2(DF a, DF b) {
    float s, e;
    two_sum(a.hi, b.hi, s, e);
    e += a.lo + b.lo;
    return df_norm(s, e);
}

__device__ __forceinline__ DF df_scale(DF a, float k) {   // exact for k a power of two
    return DF{a.hi * k, a.lo * k};
}

__device__ __forceinline__ DF df_div6(DF a) {
    const float q = a.hi / 6.f;
    const float r = fmaf(-q, 6.f, a.hi);   // exact remainder
    return df_norm(q, (r + a.lo) / 6.f);
}


__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// ---------------------------------------------------------------- staging ----

struct WarpHdr {
    unsigned long long mbar;
    int assign[32];
    int pad[2];
    WarpParams wp;
};
static_assert(sizeof(WarpHdr) % 16 == 0, "warp header keeps the atom slice 16-byte aligned");

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t mbar, uint32_t phase) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(mbar), "r"(phase)
        : "memory");
    return ok != 0;
}

// Bulk-copy `bytes` (multiple of 16) of terms into the warp's slice; all lanes
// wait on the warp's mbarrier with a bounded spin.  Returns false on timeout.
__device__ bool stage_terms(WarpHdr* hdr, void* dst, const void* src, uint32_t bytes,
                            uint32_t& phase, int lane) {
    const uint32_t mbar = smem_addr(&hdr->mbar);
    __syncwarp();
    if (lane == 0) {
        // Order this warp's earlier generic reads of the slice before the async writes.
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar),
                     "r"(bytes)
                     : "memory");
        uint64_t gsrc;
        asm("cvta.to.global.u64 %0, %1;" : "=l"(gsrc) : "l"(src));
        const uint32_t d0 = smem_addr(dst);
        constexpr uint32_t kPiece = 32768;
        for (uint32_t off = 0; off < bytes; off += kPiece) {
            const uint32_t len = bytes - off < kPiece ? bytes - off : kPiece;
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                    d0 + off),
                "l"(gsrc + off), "r"(len), "r"(mbar)
                : "memory");
        }
    }
    long long it = 0;
    bool ok = true;
    while (!mbar_try_wait(mbar, phase)) {
        if (++it > kWaitLimit) {
            ok = false;
            break;
        }
    }
    if (!ok) {
        // Give the copy a second bounded chance to land before the warp leaves.
        for (long long k = 0; k < kWaitLimit && !mbar_try_wait(mbar, phase); ++k) {
        }
    }
    phase ^= 1u;
    __syncwarp();
    return ok;
}

// ------------------------------------------------------------ the kernel ----

struct GroupState {
    int col;          // column (scan-relative), -1 idle, -2 no more work
    int k;            // z level
    int phase;
    int n_tot;        // FIRE / SD step counter
    int nnn;          // FIRE steps since the last P<0
    int outside;
    float fdt, alpha;
    DF px, py, pz;    // tip
    DF ex, ey, ez;    // evaluation position of this slot
    float vx, vy, vz;
    float ux, uy, uz; // midpoint v2 / rk4 v_k
    float sx, sy, sz; // rk4 sum of velocities
    float gx, gy, gz; // rk4 sum of forces
    DF esum;          // rk4 sum of energies
    DF e_last;        // System::energies_[1] of the last step
    DF dxy[2];        // dummy x, y
    DF dzd;           // dummy z
};

template <int G>
__global__ void __launch_bounds__(256) relax32_kernel(const BatchScan* __restrict__ scans,
                                                      int n_scans, long long n_tiles,
                                                      int cols_per_tile, int smem_terms,
                                                      unsigned long long watchdog_ns,
                                                      RunCounters* ctr) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int grp = lane / G, lg = lane % G;
    constexpr int kGroups = 32 / G;
    const size_t slice = sizeof(WarpHdr) + (size_t)smem_terms * sizeof(AtomRec32);
    WarpHdr* hdr = reinterpret_cast<WarpHdr*>(smem_raw + (size_t)warp * slice);
    AtomRec32* sm_terms = reinterpret_cast<AtomRec32*>(hdr + 1);
    const WarpParams& W = hdr->wp;

    if (lane == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&hdr->mbar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncwarp();
    uint32_t phase = 0;

    // warp-uniform state
    int cur = -1;                 // current scan
    int t_next = 0, t_end = 0;    // column cursor of the current tile
    long long pending = -1;       // next tile, of another scan
    bool exhausted = false;
    const BatchScan* S = nullptr;
    const TermPair32* units = nullptr;
    int n_units = 0, n_units_lj = 0;
    bool coul = false;
    int pairs_per_eval = 0;
    mafm_point* out = nullptr;

    unsigned err = 0;
    unsigned long long my_steps = 0, my_evals = 0, my_pairs = 0;
    unsigned status_or = 0;

    GroupState g;
    g.col = -1;
    g.ex = g.ey = g.ez = DF{0.f, 0.f};

    auto scan_of_tile = [&](long long t) {
        int lo = 0, hi = n_scans - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (scans[mid].tile_begin <= t) lo = mid;
            else hi = mid - 1;
        }
        return lo;
    };

    auto start_level = [&]() {
        g.fdt = W.dt0;
        g.alpha = 0.1f;
        g.nnn = 0;
        g.n_tot = 1;
        g.outside = 0;
        g.phase = W.maxsteps <= 1 ? PH_OUT : PH_EVAL0;
        g.ex = g.px; g.ey = g.py; g.ez = g.pz;
    };

    auto start_column = [&](const ScanParams& P, int c) {
        g.col = c;
        g.k = 0;
        const int i = c / P.ny, j = c % P.ny;
        double x, y;
        dummy_xy(P, P.tip_pbc && P.ts_mode != 2, i * P.dx, j * P.dy, x, y);
        g.dxy[0] = df_split(x);
        g.dxy[1] = df_split(y);
        g.dzd = df_split(P.zhigh);
        g.px = g.dxy[0];
        g.py = g.dxy[1];
        g.pz = df_split(P.zhigh - P.tip_dummy_d);
        g.vx = g.vy = g.vz = 0.f;
        g.e_last = DF{0.f, 0.f};
        start_level();
    };

    // Watchdog: a warp that runs longer than watchdog_ns stops with ERR_WATCHDOG
    // instead of holding the GPU (checked every 256 slots and scheduling rounds).
    const unsigned long long t_start = global_ns();
    unsigned ticks = 0;
    auto expired = [&]() -> bool {
        if ((++ticks & 255u) != 0) return false;
        const bool late = global_ns() - t_start > watchdog_ns;
        return __any_sync(kFull, late) != 0;
    };

    bool alive = true;
    while (alive) {
        // ---------------- scheduling (warp-collective) ----------------
        for (;;) {
            if (expired()) {
                err |= ERR_WATCHDOG;
                alive = false;
                break;
            }
            const unsigned need = __ballot_sync(kFull, lg == 0 && g.col == -1);
            if (need) {
                if (lane == 0) {
                    for (int gi = 0; gi < kGroups; ++gi) {
                        if (!(need & (1u << (gi * G)))) continue;
                        int a = -1;
                        for (;;) {
                            if (t_next < t_end) { a = t_next++; break; }
                            if (pending >= 0) { a = -1; break; }
                            if (exhausted) { a = -2; break; }
                            const long long t = (long long)atomicAdd(&ctr->next_work, 1ull);
                            if (t >= n_tiles) { exhausted = true; continue; }
                            const int s = scan_of_tile(t);
                            if (s == cur) {
                                const BatchScan& B = scans[s];
                                t_next = B.col_begin + (int)(t - B.tile_begin) * cols_per_tile;
                                t_end = min(B.col_end, t_next + cols_per_tile);
                                continue;
                            }
                            pending = t;
                        }
                        hdr->assign[gi] = a;
                    }
                }
                __syncwarp();
                t_next = __shfl_sync(kFull, t_next, 0);
                t_end = __shfl_sync(kFull, t_end, 0);
                pending = __shfl_sync(kFull, pending, 0);
                exhausted = __shfl_sync(kFull, (int)exhausted, 0) != 0;
                if (g.col == -1) {
                    const int a = hdr->assign[grp];
                    if (a >= 0) start_column(S->p, S->order ? __ldg(S->order + a) : a);
                    else if (a == -2) g.col = -2;
                }
                __syncwarp();
            }
            if (__any_sync(kFull, g.col >= 0)) break;
            if (pending >= 0) {
                // Every group is idle: switch the warp to the pending tile's scan.
                const int s = scan_of_tile(pending);
                cur = s;
                S = scans + s;
                const BatchScan& B = *S;
                t_next = B.col_begin + (int)(pending - B.tile_begin) * cols_per_tile;
                t_end = min(B.col_end, t_next + cols_per_tile);
                pending = -1;
                // rigid-grid scans evaluate no direct terms
                n_units = B.p.n_terms_direct > 0 ? B.p.n_units : 0;
                n_units_lj = B.p.n_terms_direct > 0 ? B.p.n_units_lj : 0;
                coul = B.has_coulomb != 0;
                pairs_per_eval = B.n_pairs_per_eval;
                out = B.out;
                __syncwarp();
                if (lane == 0) make_warp_params(B, hdr->wp);
                __syncwarp();
                if (n_units > 0 && 2 * n_units <= smem_terms) {
                    if (!stage_terms(hdr, sm_terms, B.p.units32,
                                     (uint32_t)n_units * (uint32_t)sizeof(TermPair32), phase, lane)) {
                        err |= ERR_STAGE_TIMEOUT;
                        alive = false;
                        break;
                    }
                    units = reinterpret_cast<const TermPair32*>(sm_terms);
                } else {
                    units = B.p.units32;
                }
                if (g.col == -2) g.col = -1;   // groups that found nothing may retry
                continue;
            }
            if (exhausted) {
                alive = false;
                break;
            }
        }
        if (!alive) break;

        const bool working = g.col >= 0;

        // ---------------- one force evaluation per group ----------------
        Acc acc;
        acc.zero();
        {
            Tip2 tp;
            tp.hx = f2(g.ex.hi);
            tp.hy = f2(g.ey.hi);
            tp.hz = f2(g.ez.hi);
            if (coul) {
                sum_units<G, false, true>(units, 0, n_units_lj, lg, tp, acc);
                sum_units<G, true, true>(units, n_units_lj, n_units, lg, tp, acc);
            } else {
                sum_units<G, false, false>(units, 0, n_units_lj, lg, tp, acc);
                sum_units<G, true, false>(units, n_units_lj, n_units, lg, tp, acc);
            }
        }
        if (G > 1) acc.template group_reduce<G>();

        if (working) {
            const int mode = W.ts_mode;
            if (mode != 0) {
                float v[4] = {0.f, 0.f, 0.f, 0.f};
                if (mode == 1) {
                    int unused = 0;
                    interp32(W.es, g.ex, g.ey, g.ez, v, unused, err);
                } else {
                    interp32(W.grid, g.ex, g.ey, g.ez, v, g.outside, err);
                }
                acc.add(v);
            }
            my_evals += (lg == 0);
            my_pairs += (lg == 0) ? (unsigned long long)pairs_per_eval : 0ull;

            if (g.phase == PH_OUT) {
                // Output record of this level (System::getOutput).
                const int n = g.n_tot;
                const int nz = W.nz;
                int st = (n >= W.maxsteps ? MAFM_PT_MAXSTEPS : 0) | (g.outside ? MAFM_PT_OUTSIDE : 0);
                if (lg == 0) {
                    const double Fx = (double)acc.s[0] - (double)acc.c[0];
                    const double Fy = (double)acc.s[1] - (double)acc.c[1];
                    const double Fz = (double)acc.s[2] - (double)acc.c[2];
                    const double Es = (double)acc.s[3] - (double)acc.c[3];
                    if (!isfinite(Fx) || !isfinite(Fy) || !isfinite(Fz) || !isfinite(Es))
                        st |= MAFM_PT_NONFINITE;
                    mafm_point r;
                    r.tip[0] = df_val(g.px);
                    r.tip[1] = df_val(g.py);
                    r.tip[2] = df_val(g.pz);
                    r.force[0] = Fx;
                    r.force[1] = Fy;
                    r.force[2] = Fz;
                    r.energy = Es;
                    r.steps = n;
                    r.status = st;
                    out[(size_t)(g.col - W.col_begin) * nz + g.k] = r;
                    my_steps += (unsigned long long)n;
                    status_or |= (unsigned)st;
                }
                // System::lowerTip (system.hpp:51-54)
                const DF mdz = DF{-W.dz.hi, -W.dz.lo};
                g.dzd = df_add2(g.dzd, mdz);
                g.pz = df_add2(g.pz, mdz);
                g.k++;
                if (g.k >= nz) g.col = -1;
                else start_level();
            } else {
                // Full evaluation: add the tip–dummy coupling (simulation.cpp:503-515).
                const float rx = (g.dxy[0].hi - g.ex.hi) + (g.dxy[0].lo - g.ex.lo);
                const float ry = (g.dxy[1].hi - g.ey.hi) + (g.dxy[1].lo - g.ey.lo);
                const float rz = (g.dzd.hi - g.ez.hi) + (g.dzd.lo - g.ez.lo);
                float ftd[3], etd;
                td_vdw32(W, rx, ry, rz, ftd, etd);
                // XY spring (interactions.cpp:252-266)
                const float rr2 = rx * rx + ry * ry;
                float eh, hx = 0.f, hy = 0.f;
                if (W.harm_r0 == 0.f) {
                    eh = W.harm_k * rr2;
                    if (rr2 > 1e-20f) { hx = -2.f * W.harm_k * rx; hy = -2.f * W.harm_k * ry; }
                } else {
                    const float rr = sqrtf(rr2);
                    const float dr = rr - W.harm_r0;
                    eh = W.harm_k * dr * dr;
                    if (rr > 1e-10f) {
                        const float sc = -2.f * W.harm_k * dr / rr;
                        hx = sc * rx;
                        hy = sc * ry;
                    }
                }
                float Fx, Fy, Fz;
                {
                    float t, e;
                    two_sum(acc.s[0], -ftd[0], t, e);
                    Fx = t + ((e - acc.c[0]) - hx);
                    two_sum(acc.s[1], -ftd[1], t, e);
                    Fy = t + ((e - acc.c[1]) - hy);
                    two_sum(acc.s[2], -ftd[2], t, e);
                    Fz = t + (e - acc.c[2]);
                }
                // total energy as a double-float: surface sum + dummy terms + spring
                DF E = df_norm(acc.s[3], -acc.c[3]);
                E = df_add(E, etd);
                E = df_add(E, eh);

                bool step_done = false;
                float SFx = Fx, SFy = Fy, SFz = Fz;
                DF SE = E;
                const float dt = g.fdt;
                const int integ = W.integrator;
                if (W.minimiser == MAFM_MIN_SD) {
                    step_done = true;
                } else if (integ == MAFM_INT_EULER) {
                    g.px = df_add(g.px, dt * g.vx);
                    g.py = df_add(g.py, dt * g.vy);
                    g.pz = df_add(g.pz, dt * g.vz);
                    g.vx = fmaf(dt, Fx, g.vx); g.vy = fmaf(dt, Fy, g.vy); g.vz = fmaf(dt, Fz, g.vz);
                    step_done = true;
                } else if (integ == MAFM_INT_MIDPOINT) {
                    if (g.phase == PH_EVAL0) {
                        const float h = 0.5f * dt;
                        g.ux = fmaf(h, Fx, g.vx); g.uy = fmaf(h, Fy, g.vy); g.uz = fmaf(h, Fz, g.vz);
                        g.ex = df_add(g.px, h * g.vx);
                        g.ey = df_add(g.py, h * g.vy);
                        g.ez = df_add(g.pz, h * g.vz);
                        g.phase = PH_EVAL1;
                    } else {
                        g.px = df_add(g.px, dt * g.ux);
                        g.py = df_add(g.py, dt * g.uy);
                        g.pz = df_add(g.pz, dt * g.uz);
                        g.vx = fmaf(dt, Fx, g.vx); g.vy = fmaf(dt, Fy, g.vy); g.vz = fmaf(dt, Fz, g.vz);
                        step_done = true;
                    }
                } else {   // RK4
                    const float h = 0.5f * dt;
                    if (g.phase == PH_EVAL0) {
                        g.gx = Fx; g.gy = Fy; g.gz = Fz; g.esum = E;
                        g.sx = g.vx; g.sy = g.vy; g.sz = g.vz;
                        g.ex = df_add(g.px, h * g.vx); g.ey = df_add(g.py, h * g.vy); g.ez = df_add(g.pz, h * g.vz);
                        g.ux = fmaf(h, Fx, g.vx); g.uy = fmaf(h, Fy, g.vy); g.uz = fmaf(h, Fz, g.vz);
                        g.phase = PH_EVAL1;
                    } else if (g.phase == PH_EVAL1) {
                        g.gx = fmaf(2.f, Fx, g.gx); g.gy = fmaf(2.f, Fy, g.gy); g.gz = fmaf(2.f, Fz, g.gz);
                        g.esum = df_add2(g.esum, df_scale(E, 2.f));
                        g.sx = fmaf(2.f, g.ux, g.sx); g.sy = fmaf(2.f, g.uy, g.sy); g.sz = fmaf(2.f, g.uz, g.sz);
                        g.ex = df_add(g.px, h * g.ux); g.ey = df_add(g.py, h * g.uy); g.ez = df_add(g.pz, h * g.uz);
                        g.ux = fmaf(h, Fx, g.vx); g.uy = fmaf(h, Fy, g.vy); g.uz = fmaf(h, Fz, g.vz);
                        g.phase = PH_EVAL2;
                    } else if (g.phase == PH_EVAL2) {
                        g.gx = fmaf(2.f, Fx, g.gx); g.gy = fmaf(2.f, Fy, g.gy); g.gz = fmaf(2.f, Fz, g.gz);
                        g.esum = df_add2(g.esum, df_scale(E, 2.f));
                        g.sx = fmaf(2.f, g.ux, g.sx); g.sy = fmaf(2.f, g.uy, g.sy); g.sz = fmaf(2.f, g.uz, g.sz);
                        g.ex = df_add(g.px, dt * g.ux); g.ey = df_add(g.py, dt * g.uy); g.ez = df_add(g.pz, dt * g.uz);
                        g.ux = fmaf(dt, Fx, g.vx); g.uy = fmaf(dt, Fy, g.vy); g.uz = fmaf(dt, Fz, g.vz);
                        g.phase = PH_EVAL3;
                    } else {
                        g.gx += Fx; g.gy += Fy; g.gz += Fz;
                        g.esum = df_add2(g.esum, E);
                        g.sx += g.ux; g.sy += g.uy; g.sz += g.uz;
                        const float s6 = dt / 6.f;
                        g.px = df_add(g.px, s6 * g.sx);
                        g.py = df_add(g.py, s6 * g.sy);
                        g.pz = df_add(g.pz, s6 * g.sz);
                        g.vx = fmaf(s6, g.gx, g.vx); g.vy = fmaf(s6, g.gy, g.vy); g.vz = fmaf(s6, g.gz, g.vz);
                        SFx = g.gx / 6.f; SFy = g.gy / 6.f; SFz = g.gz / 6.f;
                        SE = df_div6(g.esum);
                        step_done = true;
                    }
                }
                if (step_done) {
                    // checkConvergence (minimiser.cpp:15-37); the energy change is
                    // taken between double-float totals
                    const float ediff = (SE.hi - g.e_last.hi) + (SE.lo - g.e_last.lo);
                    g.e_last = SE;
                    // |F| and 1/|F| from one rsqrt (no IEEE sqrt or divide in the slot)
                    const float f2s = SFx * SFx + SFy * SFy + SFz * SFz;
                    const float irf = rsqrt_fast(f2s);
                    const float fl = f2s > 1e-30f ? f2s * irf : 0.f;
                    bool conv;
                    if (W.minterm == MAFM_TERM_E) conv = fabsf(ediff) < W.etol;
                    else if (W.minterm == MAFM_TERM_F) conv = fl < W.ftol;
                    else conv = fabsf(ediff) < W.etol && fl < W.ftol;
                    if (conv) {
                        g.phase = PH_OUT;
                    } else {
                        if (W.minimiser == MAFM_MIN_SD) {
                            const float sdt = W.dt0;
                            g.px = df_add(g.px, sdt * SFx);
                            g.py = df_add(g.py, sdt * SFy);
                            g.pz = df_add(g.pz, sdt * SFz);
                        } else {
                            // FIRE velocity mixing and time-step control (minimiser.cpp:105-126)
                            const float wx = g.vx, wy = g.vy, wz = g.vz;
                            const float pw = wx * SFx + wy * SFy + wz * SFz;
                            float hx2 = 0.f, hy2 = 0.f, hz2 = 0.f;
                            if (fl > 1e-10f) {
                                hx2 = SFx * irf; hy2 = SFy * irf; hz2 = SFz * irf;
                            }
                            const float w2 = wx * wx + wy * wy + wz * wz;
                            const float vl = w2 > 1e-30f ? w2 * rsqrt_fast(w2) : 0.f;
                            const float a = g.alpha, b = 1.f - a;
                            g.vx = b * wx + a * hx2 * vl;
                            g.vy = b * wy + a * hy2 * vl;
                            g.vz = b * wz + a * hz2 * vl;
                            if (pw < 0.f) {
                                g.vx = g.vy = g.vz = 0.f;
                                g.nnn = 0;
                                g.fdt *= 0.5f;
                                g.alpha = 0.1f;
                            } else {
                                if (g.nnn > 5) {
                                    g.fdt = fminf(g.fdt * 1.1f, W.dt_max);
                                    g.alpha *= 0.99f;
                                }
                                g.nnn++;
                            }
                        }
                        g.n_tot++;
                        g.phase = g.n_tot >= W.maxsteps ? PH_OUT : PH_EVAL0;
                    }
                    g.ex = g.px; g.ey = g.py; g.ez = g.pz;
                }
            }
        }
        __syncwarp();
    }

    // per-warp totals
    for (int off = 16; off > 0; off >>= 1) {
        my_steps += __shfl_xor_sync(kFull, my_steps, off);
        my_evals += __shfl_xor_sync(kFull, my_evals, off);
        my_pairs += __shfl_xor_sync(kFull, my_pairs, off);
        status_or |= __shfl_xor_sync(kFull, status_or, off);
        err |= __shfl_xor_sync(kFull, err, off);
    }
    if (lane == 0) {
        atomicAdd(&ctr->total_steps, my_steps);
        atomicAdd(&ctr->force_evals, my_evals);
        atomicAdd(&ctr->pair_evals, my_pairs);
        if (status_or | err) atomicOr(&ctr->error_word, status_or | err);
    }
}

// ---------------------------------------------------------------- sample ----

__global__ void sample32_kernel(const ScanParams p, int what, const double* pts, long long n,
                                double* out, RunCounters* ctr) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    unsigned err = 0;
    const DF x = df_split(pts[3 * i]), y = df_split(pts[3 * i + 1]), z = df_split(pts[3 * i + 2]);
    Acc acc;
    acc.zero();
    int outside = 0;
    if (what == 1) {
        float v[4] = {0, 0, 0, 0};
        if (p.es.g32) interp32(make_lookup(p.es), x, y, z, v, outside, err);
        acc.add(v);
    } else {
        const bool coul = p.has_coulomb != 0;
        for (int j0 = 0; j0 < p.n_terms_direct; j0 += kChunk) {
            float v[4] = {0, 0, 0, 0};
            for (int j = j0; j < min(j0 + kChunk, p.n_terms_direct); ++j) {
                const AtomRec32 t = p.atoms32[j];
                pair32(t, (x.hi - t.a.x) + x.lo, (y.hi - t.a.y) + y.lo, (z.hi - t.a.z) + z.lo, coul, v);
            }
            acc.add(v);
        }
        float v[4] = {0, 0, 0, 0};
        if (p.ts_mode == 1) interp32(make_lookup(p.es), x, y, z, v, outside, err);
        else if (p.ts_mode == 2) interp32(make_lookup(p.grid), x, y, z, v, outside, err);
        acc.add(v);
    }
    for (int m = 0; m < 4; ++m) out[4 * i + m] = (double)acc.s[m] - (double)acc.c[m];
    if (err) atomicOr(&ctr->error_word, err);
}

// ------------------------------------------------------------ grid build ----
// Simulation::buildTipGridInteractions (simulation.cpp:420-501) in FP32:
// one thread per node, terms staged through shared memory in tiles shared by
// the whole block (all threads read the same term: broadcast).

constexpr int kBuildUnits = 1024;  // paired-term records per shared-memory tile (64 KB)
constexpr int kStrip = 4;          // grid nodes of one column per thread

__global__ void __launch_bounds__(256, 2) grid_build32_kernel(const ScanParams p, const GridView g,
                                                           float4* out, RunCounters* ctr) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    TermPair32* tile = reinterpret_cast<TermPair32*>(smem_raw);
    // one thread per strip of kStrip consecutive nodes of a grid column (z fastest)
    const int nzs = (g.n[2] + kStrip - 1) / kStrip;
    const long long total = (long long)g.n[0] * g.n[1] * nzs;
    const int n = p.n_terms_direct > 0 ? p.n_units : 0;
    const int n_lj = p.n_terms_direct > 0 ? p.n_units_lj : 0;
    const bool coul = p.has_coulomb != 0;
    unsigned err = 0;
    for (long long base = (long long)blockIdx.x * blockDim.x; base < total;
         base += (long long)gridDim.x * blockDim.x) {
        const long long sid = base + threadIdx.x;
        const bool valid = sid < total;
        DF tx{0, 0}, ty{0, 0}, tz[kStrip];
        long long ij = 0;
        int k0 = 0;
        for (int q = 0; q < kStrip; ++q) tz[q] = DF{0, 0};
        if (valid) {
            k0 = (int)(sid % nzs) * kStrip;
            ij = sid / nzs;
            const int j = (int)(ij % g.n[1]), i = (int)(ij / g.n[1]);
            double x, y;
            dummy_xy(p, p.tip_pbc != 0, i * g.basis[0] + g.origin[0], j * g.basis[4] + g.origin[1], x, y);
            tx = df_split(x);
            ty = df_split(y);
            for (int q = 0; q < kStrip; ++q) tz[q] = df_split((k0 + q) * g.basis[8] + g.origin[2]);
        }
        Acc acc[kStrip];
        float2 hz[kStrip];
#pragma unroll
        for (int q = 0; q < kStrip; ++q) {
            acc[q].zero();
            hz[q] = f2(tz[q].hi);
        }
        const float2 hx = f2(tx.hi), hy = f2(ty.hi);
        // the paired terms in shared tiles of kBuildUnits records, read by the
        // whole block (broadcast); LJ records, then Morse records
        for (int t0 = 0; t0 < n; t0 += kBuildUnits) {
            const int cnt = min(kBuildUnits, n - t0);
            __syncthreads();
            for (int q = threadIdx.x; q < cnt; q += blockDim.x) tile[q] = p.units32[t0 + q];
            __syncthreads();
            const int lj_end = min(max(n_lj - t0, 0), cnt);
            if (coul) {
                sum_units_strip<false, true, kStrip, kBuildChunkUnits>(tile, 0, lj_end, hx, hy, hz, acc);
                sum_units_strip<true, true, kStrip, kBuildChunkUnits>(tile, lj_end, cnt, hx, hy, hz, acc);
            } else {
                sum_units_strip<false, false, kStrip, kBuildChunkUnits>(tile, 0, lj_end, hx, hy, hz, acc);
                sum_units_strip<true, false, kStrip, kBuildChunkUnits>(tile, lj_end, cnt, hx, hy, hz, acc);
            }
        }
        if (valid) {
#pragma unroll
            for (int q = 0; q < kStrip; ++q) {
                if (k0 + q >= g.n[2]) break;
                if (p.es.g32) {
                    float v[4] = {0, 0, 0, 0};
                    int unused = 0;
                    interp32(make_lookup(p.es), tx, ty, tz[q], v, unused, err);
                    acc[q].add(v);
                }
                out[ij * g.n[2] + k0 + q] =
                    make_float4(acc[q].val(0), acc[q].val(1), acc[q].val(2), acc[q].val(3));
            }
        }
    }
    if (err) atomicOr(&ctr->error_word, err);
}

template <int G>
cudaError_t launch_g(const BatchScan* scans, int n_scans, long long n_tiles,
                     const Relax32Config& cfg, RunCounters* ctr, cudaStream_t s) {
    const size_t slice = sizeof(WarpHdr) + (size_t)cfg.smem_terms * sizeof(AtomRec32);
    const size_t smem = slice * (size_t)(cfg.block / 32);
    cudaError_t e = cudaFuncSetAttribute(relax32_kernel<G>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int blocks = cfg.blocks;
    if (blocks <= 0) {
        int per_sm = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, relax32_kernel<G>, cfg.block, smem);
        if (e != cudaSuccess) return e;
        if (per_sm <= 0) return cudaErrorInvalidConfiguration;
        blocks = sm_count() * per_sm;
    }
    // No more warps than tiles.
    const long long warps_needed = n_tiles;
    const long long max_blocks = (warps_needed + cfg.block / 32 - 1) / (cfg.block / 32);
    if (blocks > max_blocks) blocks = (int)max_blocks;
    if (blocks < 1) blocks = 1;
    relax32_kernel<G><<<blocks, cfg.block, smem, s>>>(scans, n_scans, n_tiles, cfg.cols_per_tile,
                                                      cfg.smem_terms, cfg.watchdog_ns, ctr);
    return cudaGetLastError();
}

}  // namespace

int sm_count() {
    static int count = 0;
    if (!count) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&count, cudaDevAttrMultiProcessorCount, dev);
        if (count <= 0) count = 1;
    }
    return count;
}

cudaError_t launch_relax32(const BatchScan* scans_dev, int n_scans, long long n_tiles,
                           const Relax32Config& cfg, RunCounters* ctr, cudaStream_t s) {
    if (cfg.block % 32 != 0 || cfg.block < 32 || cfg.block > 256) return cudaErrorInvalidValue;
    switch (cfg.lanes) {
        case 1: return launch_g<1>(scans_dev, n_scans, n_tiles, cfg, ctr, s);
        case 2: return launch_g<2>(scans_dev, n_scans, n_tiles, cfg, ctr, s);
        case 4: return launch_g<4>(scans_dev, n_scans, n_tiles, cfg, ctr, s);
        case 8: return launch_g<8>(scans_dev, n_scans, n_tiles, cfg, ctr, s);
        case 16: return launch_g<16>(scans_dev, n_scans, n_tiles, cfg, ctr, s);
        case 32: return launch_g<32>(scans_dev, n_scans, n_tiles, cfg, ctr, s);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_sample32(const ScanParams& p, int what, const double* pts, int64_t n,
                            double* out, RunCounters* ctr, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    sample32_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(p, what, pts, n, out, ctr);
    return cudaGetLastError();
}

cudaError_t launch_grid_build32(const ScanParams& p, const GridView& g, float4* out,
                                RunCounters* ctr, cudaStream_t s) {
    const size_t smem = (size_t)kBuildUnits * sizeof(TermPair32);
    cudaError_t e = cudaFuncSetAttribute(grid_build32_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const long long total = (long long)g.n[0] * g.n[1] * ((g.n[2] + kStrip - 1) / kStrip);
    long long blocks = (total + 255) / 256;
    const long long cap = (long long)sm_count() * 8;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    grid_build32_kernel<<<(unsigned)blocks, 256, smem, s>>>(p, g, out, ctr);
    return cudaGetLastError();
}

}  // namespace mafm
