// relax_tpl.cuh — one pixel column's z descent with FIRE / SD and the
// euler / midpoint / rk4 integrators, in the reference's operation order,
// for a scalar type T: double (the plain FP64 kernel, bit-identical to the
// reference) or dfloat (the double-float kernel of MAFM_DF).
//
// The parameter block P is ScanParams (T = double) or ScanParamsDF (T =
// dfloat): the same member names, reals of type T.  The evaluator Ev provides
//   ts(tip, F, E, outside)        tip–surface force and energy
//   all(tip, dummy, F, E, outside) plus the tip–dummy terms
//   watch_conv(p, F, ediff)       called with every convergence test
//   watch_p(pw, vl, fl)           called with every sign test of P = v.F
// (the last two record near-ties for MAFM_DF and are empty for FP64).
//
// Reference correspondence (src/): FIREMinimisation minimiser.cpp:67-129,
// SDMinimisation :39-65, checkConvergence :15-37; eulerStep / midpointStep /
// rk4Step integrators.cpp:8-111; the pixel column of Simulation::run
// simulation.cpp:93-122 with System::setDummyXY system.cpp:139-162,
// System::getOutput system.cpp:28-51 and System::lowerTip system.hpp:51-54.
#pragma once

#include "dfloat.cuh"
#include "mafm_internal.h"

namespace mafm {

template <class T>
struct V3T {
    T x, y, z;
};

template <class T>
struct StateT {
    V3T<T> tip, vel, dum;
    T energy;
    int outside;
};

// Scalar functions by overload (distinct names keep ::sqrt et al. visible
// for double inside this namespace).
__device__ __forceinline__ double t_sqrt(double x) { return sqrt(x); }
__device__ __forceinline__ dfloat t_sqrt(dfloat x) { return dfl_sqrt(x); }
__device__ __forceinline__ double t_fabs(double x) { return fabs(x); }
__device__ __forceinline__ dfloat t_fabs(dfloat x) { return dfl_fabs(x); }
__device__ __forceinline__ double t_floor(double x) { return floor(x); }
__device__ __forceinline__ dfloat t_floor(dfloat x) { return dfl_floor(x); }
__device__ __forceinline__ bool t_isfinite(double x) { return isfinite(x); }
__device__ __forceinline__ bool t_isfinite(dfloat x) { return dfl_isfinite(x); }
__device__ __forceinline__ double t_double(double x) { return x; }
__device__ __forceinline__ double t_double(dfloat x) { return to_double(x); }

template <class T>
__device__ __forceinline__ T len3(V3T<T> v) {
    return t_sqrt(v.x * v.x + v.y * v.y + v.z * v.z);
}

template <class T, class P>
__device__ __forceinline__ bool converged_t(const P& p, V3T<T> F, T ediff) {
    if (p.minterm == MAFM_TERM_E) return t_fabs(ediff) < p.etol;
    if (p.minterm == MAFM_TERM_F) return len3(F) < p.ftol;
    return t_fabs(ediff) < p.etol && len3(F) < p.ftol;
}

// FIREMinimisation, minimiser.cpp:67-129 (only the tip is free).  Division by
// the unit mass of the reference (x / 1.0) is exact and left out.
template <class T, class P, class Ev>
__device__ int fire_t(Ev& ev, const P& p, StateT<T>& s, unsigned long long& evals) {
    const int n_min = 5;
    const T f_inc = T(1.1), f_dec = T(0.5), f_a = T(0.99), a_start = T(0.1);
    const T dt_max = T(10) * p.dt;
    T alpha = a_start, dt = p.dt;
    int n_non_neg = 0;
    int n_tot = 1;
    for (; n_tot < p.maxsteps; ++n_tot) {
        const T prev = s.energy;
        V3T<T> F, pp = s.tip, v = s.vel;
        T E;
        if (p.integrator == MAFM_INT_EULER) {
            ev.all(pp, s.dum, F, E, s.outside);
            evals += 1;
            s.tip.x = pp.x + dt * v.x; s.tip.y = pp.y + dt * v.y; s.tip.z = pp.z + dt * v.z;
            s.vel.x = v.x + dt * F.x; s.vel.y = v.y + dt * F.y; s.vel.z = v.z + dt * F.z;
        } else if (p.integrator == MAFM_INT_MIDPOINT) {
            V3T<T> f1, f2;
            T e1, e2;
            ev.all(pp, s.dum, f1, e1, s.outside);
            const T h = dt / T(2);
            V3T<T> p2 = {pp.x + h * v.x, pp.y + h * v.y, pp.z + h * v.z};
            V3T<T> v2 = {v.x + h * f1.x, v.y + h * f1.y, v.z + h * f1.z};
            ev.all(p2, s.dum, f2, e2, s.outside);
            evals += 2;
            s.tip.x = pp.x + dt * v2.x; s.tip.y = pp.y + dt * v2.y; s.tip.z = pp.z + dt * v2.z;
            s.vel.x = v.x + dt * f2.x; s.vel.y = v.y + dt * f2.y; s.vel.z = v.z + dt * f2.z;
            F = f2;
            E = e2;
        } else {
            V3T<T> f1, f2, f3, f4;
            T e1, e2, e3, e4;
            const T h = dt / T(2);
            ev.all(pp, s.dum, f1, e1, s.outside);
            V3T<T> p2 = {pp.x + h * v.x, pp.y + h * v.y, pp.z + h * v.z};
            V3T<T> v2 = {v.x + h * f1.x, v.y + h * f1.y, v.z + h * f1.z};
            ev.all(p2, s.dum, f2, e2, s.outside);
            V3T<T> p3 = {pp.x + h * v2.x, pp.y + h * v2.y, pp.z + h * v2.z};
            V3T<T> v3 = {v.x + h * f2.x, v.y + h * f2.y, v.z + h * f2.z};
            ev.all(p3, s.dum, f3, e3, s.outside);
            V3T<T> p4 = {pp.x + dt * v3.x, pp.y + dt * v3.y, pp.z + dt * v3.z};
            V3T<T> v4 = {v.x + dt * f3.x, v.y + dt * f3.y, v.z + dt * f3.z};
            ev.all(p4, s.dum, f4, e4, s.outside);
            evals += 4;
            const T s6 = dt / T(6);
            s.tip.x = pp.x + s6 * (v.x + T(2) * v2.x + T(2) * v3.x + v4.x);
            s.tip.y = pp.y + s6 * (v.y + T(2) * v2.y + T(2) * v3.y + v4.y);
            s.tip.z = pp.z + s6 * (v.z + T(2) * v2.z + T(2) * v3.z + v4.z);
            s.vel.x = v.x + s6 * (f1.x + T(2) * f2.x + T(2) * f3.x + f4.x);
            s.vel.y = v.y + s6 * (f1.y + T(2) * f2.y + T(2) * f3.y + f4.y);
            s.vel.z = v.z + s6 * (f1.z + T(2) * f2.z + T(2) * f3.z + f4.z);
            F.x = (f1.x + T(2) * f2.x + T(2) * f3.x + f4.x) / T(6);
            F.y = (f1.y + T(2) * f2.y + T(2) * f3.y + f4.y) / T(6);
            F.z = (f1.z + T(2) * f2.z + T(2) * f3.z + f4.z) / T(6);
            E = (e1 + T(2) * e2 + T(2) * e3 + e4) / T(6);
        }
        s.energy = E;
        ev.watch_conv(p, F, E - prev);
        if (converged_t(p, F, E - prev)) break;
        const V3T<T> w = s.vel;
        const T pw = w.x * F.x + w.y * F.y + w.z * F.z;
        const T fl = len3(F);
        V3T<T> fh = {T(0), T(0), T(0)};
        if (fl > T(1e-10)) { fh.x = F.x / fl; fh.y = F.y / fl; fh.z = F.z / fl; }
        const T vl = len3(w);
        ev.watch_p(pw, vl, fl);
        s.vel.x = (T(1) - alpha) * w.x + alpha * fh.x * vl;
        s.vel.y = (T(1) - alpha) * w.y + alpha * fh.y * vl;
        s.vel.z = (T(1) - alpha) * w.z + alpha * fh.z * vl;
        if (pw < T(0)) {
            s.vel.x = s.vel.y = s.vel.z = T(0);
            n_non_neg = 0;
            dt = dt * f_dec;
            alpha = a_start;
        } else {
            if (n_non_neg > n_min) {
                const T g = dt * f_inc;
                dt = dt_max < g ? dt_max : g;   // std::min(g, dt_max)
                alpha = alpha * f_a;
            }
            n_non_neg++;
        }
    }
    return n_tot;
}

// SDMinimisation, minimiser.cpp:39-65.
template <class T, class P, class Ev>
__device__ int sd_t(Ev& ev, const P& p, StateT<T>& s, unsigned long long& evals) {
    int n = 1;
    for (; n < p.maxsteps; ++n) {
        const T prev = s.energy;
        V3T<T> F;
        T E;
        ev.all(s.tip, s.dum, F, E, s.outside);
        evals += 1;
        s.energy = E;
        ev.watch_conv(p, F, E - prev);
        if (converged_t(p, F, E - prev)) break;
        s.tip.x = s.tip.x + p.dt * F.x; s.tip.y = s.tip.y + p.dt * F.y; s.tip.z = s.tip.z + p.dt * F.z;
    }
    return n;
}

// System::setDummyXY (system.cpp:139-162)
template <class T, class P>
__device__ __forceinline__ void dummy_xy_t(const P& p, bool wrap, T x, T y, T& ox, T& oy) {
    if (wrap) {
        const T* ci = p.cell_inv;
        const T* c = p.cell;
        V3T<T> t = {x - p.offset[0], y - p.offset[1], T(0) - p.offset[2]};
        V3T<T> cn = {ci[0] * t.x + ci[1] * t.y + ci[2] * t.z, ci[3] * t.x + ci[4] * t.y + ci[5] * t.z,
                     ci[6] * t.x + ci[7] * t.y + ci[8] * t.z};
        cn.x = cn.x - t_floor(cn.x);
        cn.y = cn.y - t_floor(cn.y);
        ox = (c[0] * cn.x + c[1] * cn.y + c[2] * cn.z) + p.offset[0];
        oy = (c[3] * cn.x + c[4] * cn.y + c[5] * cn.z) + p.offset[1];
    } else {
        ox = x;
        oy = y;
    }
}

// One pixel column (i, j) = (c / ny, c % ny): the z descent of
// Simulation::run (simulation.cpp:93-122) with the minimiser and the output
// record of every height (System::getOutput, system.cpp:28-51).  Only the
// writer stores records.  For a re-relaxation (replace = true) the writer
// first reads the record it replaces: its steps leave the step total and its
// near-tie bit stays, next to MAFM_PT_FP64.  extra_status is ORed into every
// record (the evaluator's near-tie bit for MAFM_DF is added by the caller
// through Ev::column_status()).
template <class T, class P, class Ev>
__device__ void relax_column_t(Ev& ev, const P& p, long long c, mafm_point* o, bool writer,
                               bool replace, long long& steps, unsigned long long& evals,
                               unsigned& status_or) {
    const bool wrap = p.tip_pbc && p.ts_mode != 2;
    const int i = (int)(c / p.ny), j = (int)(c % p.ny);
    StateT<T> s;
    s.vel = {T(0), T(0), T(0)};
    s.energy = T(0);
    T x, y;
    dummy_xy_t(p, wrap, T(i) * p.dx, T(j) * p.dy, x, y);
    s.dum = {x, y, p.zhigh};
    s.tip = {x, y, p.zhigh - p.tip_dummy_d};
    for (int k = 0; k < p.nz; ++k) {
        s.outside = 0;
        const int n = p.minimiser == MAFM_MIN_SD ? sd_t(ev, p, s, evals) : fire_t(ev, p, s, evals);
        V3T<T> F;
        T E;
        ev.ts(s.tip, F, E, s.outside);
        evals += 1;
        int st = (n >= p.maxsteps ? MAFM_PT_MAXSTEPS : 0) | (s.outside ? MAFM_PT_OUTSIDE : 0) |
                 ev.column_status();
        if (!t_isfinite(F.x) || !t_isfinite(F.y) || !t_isfinite(F.z) || !t_isfinite(E))
            st |= MAFM_PT_NONFINITE;
        status_or |= (unsigned)st;
        if (writer) {
            if (replace) {
                // through L2: the record may have been written on another SM
                // (the double-float kernel's placeholders) just before
                const int old_steps = __ldcg(&o[k].steps), old_status = __ldcg(&o[k].status);
                steps -= old_steps;
                st |= (old_status & MAFM_PT_NEAR_TIE) | MAFM_PT_FP64;
            }
            mafm_point r;
            r.tip[0] = t_double(s.tip.x); r.tip[1] = t_double(s.tip.y); r.tip[2] = t_double(s.tip.z);
            r.force[0] = t_double(F.x); r.force[1] = t_double(F.y); r.force[2] = t_double(F.z);
            r.energy = t_double(E);
            r.steps = n;
            r.status = st;
            o[k] = r;
            steps += n;
        }
        s.dum.z = s.dum.z - p.dz;
        s.tip.z = s.tip.z - p.dz;
    }
}

}  // namespace mafm
