// relax64_dev.cuh — the FP64 evaluators of the tip–surface forces, shared by
// the plain FP64 kernels (relax64.cu) and the double-float kernel's own FP64
// re-relaxation of near-tie columns (relaxdf.cu).  Both translation units are
// compiled with -fmad=false, so every expression below gives the same bits
// in both; with LJ and Coulomb terms they are the reference's bits (division
// and square root are correctly rounded in both; exp in the Morse term may
// differ in the last bit).
//
// Reference correspondence (src/):
//   vdW / Coulomb terms        interactions.cpp:15-51
//   tip–dummy terms            interactions.cpp:252-266, simulation.cpp:503-515
//   trilinear grid lookup      force_grid.cpp:88-275
#pragma once

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
    int pairs_per_eval;       // vdW + Coulomb terms of one evaluation
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
        if (lane == 0) pairs += (unsigned long long)pairs_per_eval;
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

}  // namespace
}  // namespace mafm
