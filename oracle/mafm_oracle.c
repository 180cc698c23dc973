/*
 * mafm_oracle.c — ORACLE / TEST INFRASTRUCTURE.  Not part of the product.
 *
 * A plain-C, FP64, CPU restatement of the MechAFM scan path, used only as the
 * checker by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline and
 * reference legs.  The product (libmafm) never links or calls it.
 *
 * It follows the reference's algorithm and floating-point operation order so
 * that, compiled with -ffp-contract=off, it reproduces the reference's FP64
 * results.  It is pinned against the reference itself: tests/golden/ holds
 * outputs of the unmodified reference sources (built by oracle/Makefile `ref`,
 * driver oracle/ref_dump.cpp) and tests/test_oracle_golden.py checks this file
 * against them.
 *
 * Reference correspondence (SINGROUP/MechAFM, src/):
 *   pair terms          LJ interactions.cpp:15-27, Morse :29-40, Coulomb :42-51
 *   tip–dummy coupling  TipHarmonic interactions.cpp:252-266, simulation.cpp:503-515
 *   force grid lookup   ForceGrid::interpolate force_grid.cpp:88-155, :158-275
 *   external field      ElectrostaticPotentialInteraction ctor interactions.cpp:53-234,
 *                       fft.cpp:11-94 (the 3-D DFT here is computed directly from
 *                       its definition instead of kiss_fft's mixed-radix FFT)
 *   rigid grid build    Simulation::buildTipGridInteractions simulation.cpp:420-501
 *   integrators         integrators.cpp:8-111
 *   minimisers          checkConvergence / SD / FIRE minimiser.cpp:15-129
 *   scan loop           Simulation::run simulation.cpp:78-122, System::setDummyXY
 *                       system.cpp:139-162, getOutput system.cpp:28-51
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <omp.h>

#include "mafm.h"

#define PI 3.14159265358979323846
#define TOL 1e-10

static char g_err[512];
const char* oracle_last_error(void) { return g_err; }

typedef struct { double x, y, z; } v3;

typedef struct {
    double x, y, z, qq, p0, p1, p2;
    int kind, coul;
} Term;

typedef struct {
    int n[3];
    int periodic, orth;
    double b[3][3], inv[3][3], origin[3];
    double* fe; /* 4 per node: Fx Fy Fz E */
} Grid;

typedef struct {
    const mafm_scan_desc* d;
    Term* terms;
    int nt;
    int mode; /* 0 pairs, 1 pairs + external field, 2 rigid grid */
    Grid es, grid;
    double cell[3][3], cinv[3][3];
    int err;
} Ctx;

/* ---- 3x3 helpers, matrices.hpp:89-160 ---------------------------------- */
static double det3(double (*m)[3]) {
    double d = 0;
    d = m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]);
    d += m[0][1] * (m[1][2] * m[2][0] - m[1][0] * m[2][2]);
    d += m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
    return d;
}
static void inv3(double (*m)[3], double (*r)[3]) {
    double inv_det = 1 / det3(m);
    double a = m[0][0], b = m[0][1], c = m[0][2], d = m[1][0], e = m[1][1], f = m[1][2];
    double g = m[2][0], h = m[2][1], i = m[2][2];
    r[0][0] = inv_det * (e * i - f * h);
    r[0][1] = -inv_det * (b * i - c * h);
    r[0][2] = inv_det * (b * f - c * e);
    r[1][0] = -inv_det * (d * i - f * g);
    r[1][1] = inv_det * (a * i - c * g);
    r[1][2] = -inv_det * (a * f - c * d);
    r[2][0] = inv_det * (d * h - e * g);
    r[2][1] = -inv_det * (a * h - b * g);
    r[2][2] = inv_det * (a * e - b * d);
}
static v3 mulv(double (*m)[3], v3 v) {
    v3 r;
    r.x = m[0][0] * v.x + m[0][1] * v.y + m[0][2] * v.z;
    r.y = m[1][0] * v.x + m[1][1] * v.y + m[1][2] * v.z;
    r.z = m[2][0] * v.x + m[2][1] * v.y + m[2][2] * v.z;
    return r;
}
static int is_diag(double (*m)[3]) {
    double ds = 0, nd = 0;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            if (i == j) ds += fabs(m[i][i]);
            else nd += fabs(m[i][j]);
        }
    return nd < 1.0e-10 * ds;
}
static double len3(v3 v) { return sqrt(v.x * v.x + v.y * v.y + v.z * v.z); }

/* ---- pair terms --------------------------------------------------------- */
/* r = tip - (atom + shift); the image shift is already in the term position. */
/* LJInteraction::eval interactions.cpp:15-27, MorseInteraction::eval :29-40. */
static void term_vdw(const Term* t, v3 tip, v3* f, double* e) {
    v3 r = {tip.x - t->x, tip.y - t->y, tip.z - t->z};
    if (t->kind == MAFM_PAIR_LJ) { /* interactions.cpp:15-27 */
        double r_sqr = r.x * r.x + r.y * r.y + r.z * r.z;
        double r6 = r_sqr * r_sqr * r_sqr;
        double term_a = t->p1 / (r6 * r6);
        double term_b = t->p0 / r6;
        *e = term_a - term_b;
        double s = (12 * term_a - 6 * term_b) / r_sqr;
        f->x = s * r.x; f->y = s * r.y; f->z = s * r.z;
    } else { /* Morse, interactions.cpp:29-40 */
        double rl = len3(r);
        double d = exp(-t->p1 * (rl - t->p2));
        *e = t->p0 * (d * d - 2 * d + 1);
        double f_abs = 2 * t->p0 * t->p1 * (d * d - d);
        double s = f_abs / rl;
        f->x = s * r.x; f->y = s * r.y; f->z = s * r.z;
    }
}
static void term_coul(double qq, v3 r, v3* f, double* e) { /* interactions.cpp:42-51 */
    double rl = len3(r);
    *e = qq / rl;
    double s = qq / (rl * rl * rl);
    f->x = s * r.x; f->y = s * r.y; f->z = s * r.z;
}

/* ---- trilinear grid lookup, force_grid.cpp:88-275 ----------------------- */
/* ForceGrid::getGridPointIndex force_grid.cpp:223-249 with pbcGridPoint :252-275. */
static int grid_index(Ctx* c, const Grid* g, int x, int y, int z) {
    if (x < 0 || y < 0 || z < 0 || x >= g->n[0] || y >= g->n[1] || z >= g->n[2]) {
        if (g->periodic) {
            int n;
            if (x < 0 || x >= g->n[0]) { n = (int)floor((double)x / g->n[0]); x -= n * g->n[0]; }
            if (y < 0 || y >= g->n[1]) { n = (int)floor((double)y / g->n[1]); y -= n * g->n[1]; }
            if (z < 0 || z >= g->n[2]) { n = (int)floor((double)z / g->n[2]); z -= n * g->n[2]; }
        } else {
            c->err |= 2;
            x = x < 0 ? 0 : (x >= g->n[0] ? g->n[0] - 1 : x);
            y = y < 0 ? 0 : (y >= g->n[1] ? g->n[1] - 1 : y);
            z = z < 0 ? 0 : (z >= g->n[2] ? g->n[2] - 1 : z);
        }
    }
    return (x * g->n[1] + y) * g->n[2] + z;
}

/* ForceGrid::interpolate force_grid.cpp:88-155, getGridPoint :158-220. */
static void grid_interp(Ctx* c, const Grid* g, v3 pos, v3* f, double* e, int* outside) {
    int gp[3];
    v3 q = {pos.x - g->origin[0], pos.y - g->origin[1], pos.z - g->origin[2]};
    v3 pb;
    if (g->orth) {
        pb.x = q.x / g->b[0][0]; pb.y = q.y / g->b[1][1]; pb.z = q.z / g->b[2][2];
    } else {
        double inv[3][3];
        memcpy(inv, g->inv, sizeof inv);
        pb = mulv(inv, q);
    }
    gp[0] = (int)floor(pb.x); gp[1] = (int)floor(pb.y); gp[2] = (int)floor(pb.z);
    if (!g->periodic) {
        for (int a = 0; a < 3; ++a) {
            if (gp[a] < 0) { gp[a] = 0; *outside = 1; }
            else if (gp[a] >= g->n[a]) { gp[a] = g->n[a] - 1; *outside = 1; }
        }
    }
    const double* s[8];
    for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j)
            for (int k = 0; k < 2; ++k)
                s[i * 4 + j * 2 + k] = g->fe + 4 * (size_t)grid_index(c, g, gp[0] + i, gp[1] + j, gp[2] + k);
    double dx = pb.x - gp[0], dy = pb.y - gp[1], dz = pb.z - gp[2];
    double out[4];
    for (int m = 0; m < 4; ++m) {
        double v00 = s[0][m] * (1 - dx) + s[4][m] * dx;
        double v01 = s[1][m] * (1 - dx) + s[5][m] * dx;
        double v10 = s[2][m] * (1 - dx) + s[6][m] * dx;
        double v11 = s[3][m] * (1 - dx) + s[7][m] * dx;
        double v0 = v00 * (1 - dy) + v10 * dy;
        double v1 = v01 * (1 - dy) + v11 * dy;
        out[m] = v0 * (1 - dz) + v1 * dz;
    }
    f->x = out[0]; f->y = out[1]; f->z = out[2]; *e = out[3];
}

/* ---- force evaluations --------------------------------------------------- */
/* Tip–surface terms (the interactions with isTipSurface(), system.cpp:41-51). */
/* The tip-surface terms in the reference's interaction order
 * (buildTipSurfaceInteractions simulation.cpp:297-320; GridInteraction
 * interactions.cpp:244-250; ElectrostaticPotentialInteraction :236-242). */
static void eval_ts(Ctx* c, v3 tip, v3* F, double* E, int* outside) {
    v3 f = {0, 0, 0};
    double e = 0;
    F->x = F->y = F->z = 0;
    *E = 0;
    if (c->mode == 2) {
        grid_interp(c, &c->grid, tip, &f, &e, outside);
        F->x += f.x; F->y += f.y; F->z += f.z; *E += e;
        return;
    }
    for (int i = 0; i < c->nt; ++i) {
        const Term* t = &c->terms[i];
        term_vdw(t, tip, &f, &e);
        F->x += f.x; F->y += f.y; F->z += f.z; *E += e;
        if (t->coul) {
            v3 r = {tip.x - t->x, tip.y - t->y, tip.z - t->z};
            term_coul(t->qq, r, &f, &e);
            F->x += f.x; F->y += f.y; F->z += f.z; *E += e;
        }
    }
    if (c->mode == 1) {
        int dummy = 0;
        grid_interp(c, &c->es, tip, &f, &e, &dummy);
        F->x += f.x; F->y += f.y; F->z += f.z; *E += e;
    }
}

/* All interactions of the relaxation: tip–surface, then the tip–dummy vdW,
 * optional Coulomb and the XY spring (buildTipDummyInteractions order). */
static void eval_all(Ctx* c, v3 tip, v3 dum, v3* F, double* E, int* outside) {
    const mafm_scan_desc* d = c->d;
    eval_ts(c, tip, F, E, outside);
    Term td;
    td.x = tip.x; td.y = tip.y; td.z = tip.z;
    td.kind = d->dummy_pair.kind;
    td.p0 = d->dummy_pair.p[0]; td.p1 = d->dummy_pair.p[1]; td.p2 = d->dummy_pair.p[2];
    v3 f;
    double e;
    term_vdw(&td, dum, &f, &e); /* r = dummy - tip; the tip receives -f */
    F->x -= f.x; F->y -= f.y; F->z -= f.z; *E += e;
    if (d->tip_dummy_coulomb && d->dummy_charge != 0 && d->tip_charge != 0) {
        double qq = d->qbase * d->dummy_charge * d->tip_charge;
        v3 r = {dum.x - tip.x, dum.y - tip.y, dum.z - tip.z};
        term_coul(qq, r, &f, &e);
        F->x -= f.x; F->y -= f.y; F->z -= f.z; *E += e;
    }
    { /* TipHarmonicInteraction, interactions.cpp:252-266 */
        double rx = dum.x - tip.x, ry = dum.y - tip.y;
        double r = sqrt(rx * rx + ry * ry);
        double dr = r - d->harm_r0;
        double eh = d->harm_k * dr * dr;
        double fx = 0, fy = 0;
        if (r > TOL) {
            double s = -2 * d->harm_k * dr / r;
            fx = s * rx; fy = s * ry;
        }
        F->x -= fx; F->y -= fy; F->z -= 0.0;
        *E += eh;
    }
}

/* ---- minimisers ---------------------------------------------------------- */
/* checkConvergence minimiser.cpp:15-37. */
static int converged(const mafm_scan_desc* d, v3 F, double ediff) {
    switch (d->minterm) {
        case MAFM_TERM_E: return fabs(ediff) < d->etol;
        case MAFM_TERM_F: return len3(F) < d->ftol;
        default: return fabs(ediff) < d->etol && len3(F) < d->ftol;
    }
}

typedef struct {
    v3 tip, vel, dum;
    double energy; /* System::energies_[1], carried across z levels */
    int outside;
} State;

/* FIREMinimisation minimiser.cpp:67-129 with eulerStep / midpointStep /
 * rk4Step integrators.cpp:8-21 / 23-54 / 56-111. */
static int fire(Ctx* c, State* s) {
    const mafm_scan_desc* d = c->d;
    const int n_min = 5;
    const double f_inc = 1.1, f_dec = 0.5, f_a = 0.99, a_start = 0.1;
    const double dt_max = 10 * d->dt;
    double alpha = a_start, dt = d->dt;
    int n_non_neg = 0;
    int n_tot = 1;
    for (; n_tot < d->maxsteps; ++n_tot) {
        double prev = s->energy;
        v3 F;
        double E;
        v3 p = s->tip, v = s->vel;
        if (d->integrator == MAFM_INT_EULER) {
            eval_all(c, p, s->dum, &F, &E, &s->outside);
            s->tip.x = p.x + dt * v.x; s->tip.y = p.y + dt * v.y; s->tip.z = p.z + dt * v.z;
            s->vel.x = v.x + dt * F.x / 1.0; s->vel.y = v.y + dt * F.y / 1.0; s->vel.z = v.z + dt * F.z / 1.0;
        } else if (d->integrator == MAFM_INT_MIDPOINT) {
            v3 f1, f2;
            double e1, e2;
            eval_all(c, p, s->dum, &f1, &e1, &s->outside);
            v3 p2 = {p.x + dt / 2 * v.x, p.y + dt / 2 * v.y, p.z + dt / 2 * v.z};
            v3 v2 = {v.x + dt / 2 * f1.x / 1.0, v.y + dt / 2 * f1.y / 1.0, v.z + dt / 2 * f1.z / 1.0};
            eval_all(c, p2, s->dum, &f2, &e2, &s->outside);
            s->tip.x = p.x + dt * v2.x; s->tip.y = p.y + dt * v2.y; s->tip.z = p.z + dt * v2.z;
            s->vel.x = v.x + dt * f2.x / 1.0; s->vel.y = v.y + dt * f2.y / 1.0; s->vel.z = v.z + dt * f2.z / 1.0;
            F = f2;
            E = e2;
        } else {
            v3 f1, f2, f3, f4;
            double e1, e2, e3, e4;
            eval_all(c, p, s->dum, &f1, &e1, &s->outside);
            v3 p2 = {p.x + dt / 2 * v.x, p.y + dt / 2 * v.y, p.z + dt / 2 * v.z};
            v3 v2 = {v.x + dt / 2 * f1.x / 1.0, v.y + dt / 2 * f1.y / 1.0, v.z + dt / 2 * f1.z / 1.0};
            eval_all(c, p2, s->dum, &f2, &e2, &s->outside);
            v3 p3 = {p.x + dt / 2 * v2.x, p.y + dt / 2 * v2.y, p.z + dt / 2 * v2.z};
            v3 v3_ = {v.x + dt / 2 * f2.x / 1.0, v.y + dt / 2 * f2.y / 1.0, v.z + dt / 2 * f2.z / 1.0};
            eval_all(c, p3, s->dum, &f3, &e3, &s->outside);
            v3 p4 = {p.x + dt * v3_.x, p.y + dt * v3_.y, p.z + dt * v3_.z};
            v3 v4 = {v.x + dt * f3.x / 1.0, v.y + dt * f3.y / 1.0, v.z + dt * f3.z / 1.0};
            eval_all(c, p4, s->dum, &f4, &e4, &s->outside);
            s->tip.x = p.x + dt / 6 * (v.x + 2 * v2.x + 2 * v3_.x + v4.x);
            s->tip.y = p.y + dt / 6 * (v.y + 2 * v2.y + 2 * v3_.y + v4.y);
            s->tip.z = p.z + dt / 6 * (v.z + 2 * v2.z + 2 * v3_.z + v4.z);
            s->vel.x = v.x + dt / 6 * (f1.x + 2 * f2.x + 2 * f3.x + f4.x) / 1.0;
            s->vel.y = v.y + dt / 6 * (f1.y + 2 * f2.y + 2 * f3.y + f4.y) / 1.0;
            s->vel.z = v.z + dt / 6 * (f1.z + 2 * f2.z + 2 * f3.z + f4.z) / 1.0;
            F.x = (f1.x + 2 * f2.x + 2 * f3.x + f4.x) / 6;
            F.y = (f1.y + 2 * f2.y + 2 * f3.y + f4.y) / 6;
            F.z = (f1.z + 2 * f2.z + 2 * f3.z + f4.z) / 6;
            E = (e1 + 2 * e2 + 2 * e3 + e4) / 6;
        }
        s->energy = E;
        if (converged(d, F, E - prev)) break;
        /* Only the tip moves, so P = v_tip . F_tip (minimiser.cpp:107-113). */
        v3 w = s->vel;
        double pw = w.x * F.x + w.y * F.y + w.z * F.z;
        double fl = len3(F);
        v3 fh = {0, 0, 0};
        if (fl > 1e-10) { fh.x = F.x / fl; fh.y = F.y / fl; fh.z = F.z / fl; }
        double vl = len3(w);
        s->vel.x = (1 - alpha) * w.x + alpha * fh.x * vl;
        s->vel.y = (1 - alpha) * w.y + alpha * fh.y * vl;
        s->vel.z = (1 - alpha) * w.z + alpha * fh.z * vl;
        if (pw < 0) {
            s->vel.x = s->vel.y = s->vel.z = 0;
            n_non_neg = 0;
            dt *= f_dec;
            alpha = a_start;
        } else {
            if (n_non_neg > n_min) {
                double g = dt * f_inc;
                dt = dt_max < g ? dt_max : g; /* std::min(g, dt_max) */
                alpha *= f_a;
            }
            n_non_neg++;
        }
    }
    return n_tot;
}

/* SDMinimisation minimiser.cpp:39-65. */
static int steepest(Ctx* c, State* s) {
    const mafm_scan_desc* d = c->d;
    int n = 1;
    for (; n < d->maxsteps; ++n) {
        double prev = s->energy;
        v3 F;
        double E;
        eval_all(c, s->tip, s->dum, &F, &E, &s->outside);
        s->energy = E;
        if (converged(d, F, E - prev)) break;
        s->tip.x += d->dt * F.x; s->tip.y += d->dt * F.y; s->tip.z += d->dt * F.z;
    }
    return n;
}

/* System::setDummyXY (system.cpp:139-162) */
/* System::setDummyXY system.cpp:139-162 (PBC wrap relative to the offset). */
static void dummy_xy(Ctx* c, int wrap, double x, double y, double* ox, double* oy) {
    if (wrap) {
        const mafm_scan_desc* d = c->d;
        v3 t = {x - d->offset[0], y - d->offset[1], 0 - d->offset[2]};
        v3 cn = mulv(c->cinv, t);
        cn.x -= floor(cn.x);
        cn.y -= floor(cn.y);
        v3 p = mulv(c->cell, cn);
        *ox = p.x + d->offset[0];
        *oy = p.y + d->offset[1];
    } else {
        *ox = x;
        *oy = y;
    }
}

/* One pixel column: the loop body of Simulation::run (simulation.cpp:93-122). */
/* One pixel column of Simulation::run simulation.cpp:93-122: the z descent with
 * System::lowerTip (system.hpp:51-54) and getOutput (system.cpp:28-51). */
static void column(Ctx* c, int col, mafm_point* out) {
    const mafm_scan_desc* d = c->d;
    const int i = col / d->ny, j = col % d->ny;
    State s;
    memset(&s, 0, sizeof s);
    double x, y;
    dummy_xy(c, d->tip_pbc && !d->rigidgrid, i * d->dx, j * d->dy, &x, &y);
    s.dum.x = s.tip.x = x;
    s.dum.y = s.tip.y = y;
    s.dum.z = d->zhigh;
    s.tip.z = d->zhigh - d->tip_dummy_d;
    for (int k = 0; k < d->nz; ++k) {
        s.outside = 0;
        int n = d->minimiser == MAFM_MIN_SD ? steepest(c, &s) : fire(c, &s);
        mafm_point* p = out + k;
        v3 F;
        double E;
        eval_ts(c, s.tip, &F, &E, &s.outside);
        p->tip[0] = s.tip.x; p->tip[1] = s.tip.y; p->tip[2] = s.tip.z;
        p->force[0] = F.x; p->force[1] = F.y; p->force[2] = F.z;
        p->energy = E;
        p->steps = n;
        p->status = (n >= d->maxsteps ? MAFM_PT_MAXSTEPS : 0) | (s.outside ? MAFM_PT_OUTSIDE : 0);
        if (!isfinite(F.x) || !isfinite(F.y) || !isfinite(F.z) || !isfinite(E))
            p->status |= MAFM_PT_NONFINITE;
        s.dum.z -= d->dz;
        s.tip.z -= d->dz;
    }
}

/* ---- 3-D DFT (definition of kiss_fftnd's transform, no normalisation) ---- */
/* One axis of the unnormalised 3-D DFT that fft_data_grid / ffti_data_grid
 * (fft.cpp:11-94) compute with kiss_fftnd. */
static void dft_axis(double* re, double* im, const int n[3], int axis, int inverse) {
    const int L = n[axis];
    const size_t stride = axis == 0 ? (size_t)n[1] * n[2] : (axis == 1 ? (size_t)n[2] : 1);
    const size_t total = (size_t)n[0] * n[1] * n[2];
    double* cs = malloc(sizeof(double) * L);
    double* sn = malloc(sizeof(double) * L);
    for (int m = 0; m < L; ++m) {
        double a = 2 * PI * m / L;
        cs[m] = cos(a);
        sn[m] = inverse ? sin(a) : -sin(a);
    }
    const size_t nlines = total / L;
#pragma omp parallel
    {
        double* tr = malloc(sizeof(double) * L);
        double* ti = malloc(sizeof(double) * L);
#pragma omp for schedule(static)
        for (long long line = 0; line < (long long)nlines; ++line) {
            size_t base;
            if (axis == 0) base = (size_t)line;
            else if (axis == 1) base = ((size_t)line / n[2]) * (size_t)n[1] * n[2] + (size_t)line % n[2];
            else base = (size_t)line * n[2];
            for (int k = 0; k < L; ++k) {
                double sr = 0, si = 0;
                for (int m = 0; m < L; ++m) {
                    int w = (int)(((long long)k * m) % L);
                    double xr = re[base + m * stride], xi = im[base + m * stride];
                    sr += xr * cs[w] - xi * sn[w];
                    si += xr * sn[w] + xi * cs[w];
                }
                tr[k] = sr;
                ti[k] = si;
            }
            for (int k = 0; k < L; ++k) {
                re[base + k * stride] = tr[k];
                im[base + k * stride] = ti[k];
            }
        }
        free(tr);
        free(ti);
    }
    free(cs);
    free(sn);
}

static void dft3(double* re, double* im, const int n[3], int inverse) {
    for (int a = 0; a < 3; ++a) dft_axis(re, im, n, a, inverse);
}

/* ElectrostaticPotentialInteraction ctor, interactions.cpp:53-234. */
/* ElectrostaticPotentialInteraction ctor interactions.cpp:53-234 and the
 * potential set-up of Simulation::buildTipSurfaceInteractions simulation.cpp:322-417. */
static int build_es(Ctx* c) {
    const mafm_scan_desc* d = c->d;
    Grid* g = &c->es;
    for (int a = 0; a < 3; ++a) g->n[a] = d->epot_n[a];
    for (int r = 0; r < 3; ++r)
        for (int q = 0; q < 3; ++q) g->b[r][q] = d->epot_basis[3 * r + q];
    for (int a = 0; a < 3; ++a) g->origin[a] = d->epot_origin[a];
    g->periodic = 1;
    g->orth = is_diag(g->b);
    inv3(g->b, g->inv);
    const int* n = g->n;
    const size_t N = (size_t)n[0] * n[1] * n[2];
    double* rho = calloc(N, sizeof(double));
    const double w = 0.5; /* g_tip_gaussian_width, globals.hpp:17 */
    const double w2 = w * w;
    const double norm = 1.0 / pow(w * sqrt(2.0 * PI), 3);
    int nmin = n[0] < n[1] ? n[0] : n[1];
    nmin = nmin < n[2] ? nmin : n[2];
    int cut[3] = {nmin, nmin, nmin};
    for (int a = 0; a < 3; ++a) {
        for (int i = 0; i < nmin - 1; i++) {
            double vx = i * g->b[0][a], vy = i * g->b[1][a], vz = i * g->b[2][a];
            double sq = vx * vx + vy * vy + vz * vz;
            if (exp(-0.5 * sq / w2) < 1.0e-10) { cut[a] = i; break; }
        }
    }
    const double q = d->tip_charge;
    for (int ix = -cut[0]; ix <= cut[0]; ix++)
        for (int iy = -cut[1]; iy <= cut[1]; iy++)
            for (int iz = -cut[2]; iz < cut[2]; iz++) {
                v3 p;
                if (g->orth) {
                    p.x = 0 + ix * g->b[0][0]; p.y = 0 + iy * g->b[1][1]; p.z = 0 + iz * g->b[2][2];
                } else {
                    v3 gv = {ix, iy, iz};
                    v3 m = mulv(g->b, gv);
                    p.x = 0 + m.x; p.y = 0 + m.y; p.z = 0 + m.z;
                }
                double r2 = p.x * p.x + p.y * p.y + p.z * p.z;
                int x = ix, y = iy, z = iz, k;
                if (x < 0 || x >= n[0]) { k = (int)floor((double)x / n[0]); x -= k * n[0]; }
                if (y < 0 || y >= n[1]) { k = (int)floor((double)y / n[1]); y -= k * n[1]; }
                if (z < 0 || z >= n[2]) { k = (int)floor((double)z / n[2]); z -= k * n[2]; }
                rho[((size_t)x * n[1] + y) * n[2] + z] += q * norm * exp(-0.5 * r2 / w2);
            }
    double* vr = malloc(N * sizeof(double));
    double* vi = calloc(N, sizeof(double));
    double* rr = rho;
    double* ri = calloc(N, sizeof(double));
    memcpy(vr, d->epot, N * sizeof(double));
    dft3(vr, vi, n, 0);
    dft3(rr, ri, n, 0);
    const double vol = det3(g->b);
    for (size_t i = 0; i < N; ++i) { /* E(k) = V(k) * vol * rho(k) */
        double ar = vol * rr[i], ai = vol * ri[i];
        double er = vr[i] * ar - vi[i] * ai, ei = vr[i] * ai + vi[i] * ar;
        vr[i] = er;
        vi[i] = ei;
    }
    /* reciprocal basis (B diag(n))^-1^T, fft.cpp:41-47 */
    double bn[3][3], bi[3][3], kb[3][3];
    for (int r = 0; r < 3; ++r)
        for (int q2 = 0; q2 < 3; ++q2) bn[r][q2] = g->b[r][q2] * n[q2];
    inv3(bn, bi);
    for (int r = 0; r < 3; ++r)
        for (int q2 = 0; q2 < 3; ++q2) kb[r][q2] = bi[q2][r];
    g->fe = malloc(4 * N * sizeof(double));
    double* tr = malloc(N * sizeof(double));
    double* ti = malloc(N * sizeof(double));
    int status = 0;
    for (int comp = -1; comp < 3 && !status; ++comp) {
        if (comp < 0) {
            memcpy(tr, vr, N * sizeof(double));
            memcpy(ti, vi, N * sizeof(double));
        } else {
            for (int ix = 0; ix < n[0]; ix++) {
                double ka = ix * kb[comp][0];
                if (ix >= n[0] / 2) ka -= n[0] * kb[comp][0];
                for (int iy = 0; iy < n[1]; iy++) {
                    double kbv = iy * kb[comp][1];
                    if (iy >= n[1] / 2) kbv -= n[1] * kb[comp][1];
                    for (int iz = 0; iz < n[2]; iz++) {
                        double kc = iz * kb[comp][2];
                        if (iz >= n[2] / 2) kc -= n[2] * kb[comp][2];
                        size_t i = ((size_t)ix * n[1] + iy) * n[2] + iz;
                        double kk = ka + kbv + kc;
                        /* -2 pi i k E(k) */
                        tr[i] = 2 * PI * kk * vi[i];
                        ti[i] = -2 * PI * kk * vr[i];
                    }
                }
            }
        }
        dft3(tr, ti, n, 1);
        for (size_t i = 0; i < N; ++i) {
            if (ti[i] / N > 1.0e-8) { /* fft.cpp:79-83 */
                snprintf(g_err, sizeof g_err,
                         "Imaginary part of inverse FFT exceeded threshold 1.0e-8! Value: %e", ti[i]);
                status = MAFM_E_RANGE;
                break;
            }
            g->fe[4 * i + (comp < 0 ? 3 : comp)] = tr[i] / N;
        }
    }
    free(tr); free(ti); free(vr); free(vi); free(rr); free(ri);
    return status;
}

/* Simulation::buildTipGridInteractions, simulation.cpp:420-501. */
/* Simulation::buildTipGridInteractions simulation.cpp:420-501. */
static void build_grid(Ctx* c) {
    const mafm_scan_desc* d = c->d;
    Grid* g = &c->grid;
    double sp[3] = {d->dx / 2, d->dy / 2, d->dz / 2};
    int border[3];
    for (int a = 0; a < 3; ++a) border[a] = (int)ceil(1.5 / sp[a]);
    g->n[0] = (int)(floor(d->area[0] / sp[0]) + 2 * border[0] + 1);
    g->n[1] = (int)(floor(d->area[1] / sp[1]) + 2 * border[1] + 1);
    g->n[2] = (int)(floor((d->zhigh - d->zlow) / sp[2]) + 2 * border[2] + 1);
    g->origin[0] = -border[0] * sp[0];
    g->origin[1] = -border[1] * sp[1];
    g->origin[2] = d->zlow - d->tip_dummy_d - border[2] * sp[2];
    memset(g->b, 0, sizeof g->b);
    for (int a = 0; a < 3; ++a) g->b[a][a] = sp[a];
    g->orth = 1;
    g->periodic = 0;
    const size_t N = (size_t)g->n[0] * g->n[1] * g->n[2];
    g->fe = malloc(4 * N * sizeof(double));
    const int saved = c->mode;
    c->mode = d->use_external_potential ? 1 : 0;
#pragma omp parallel for schedule(dynamic, 1)
    for (int i = 0; i < g->n[0]; ++i) {
        for (int j = 0; j < g->n[1]; ++j) {
            double x, y;
            dummy_xy(c, d->tip_pbc, i * sp[0] + g->origin[0], j * sp[1] + g->origin[1], &x, &y);
            for (int k = 0; k < g->n[2]; ++k) {
                v3 tip = {x, y, k * sp[2] + g->origin[2]};
                v3 F;
                double E;
                int dummy = 0;
                eval_ts(c, tip, &F, &E, &dummy);
                double* o = g->fe + 4 * (((size_t)i * g->n[1] + j) * g->n[2] + k);
                o[0] = F.x; o[1] = F.y; o[2] = F.z; o[3] = E;
            }
        }
    }
    c->mode = saved;
}

/* The interactions of Simulation::buildInteractions simulation.cpp:201-216
 * (tip-surface :297-417, tip grid :420-501, tip-dummy :503-515). */
static int ctx_init(Ctx* c, const mafm_scan_desc* d) {
    memset(c, 0, sizeof *c);
    c->d = d;
    for (int r = 0; r < 3; ++r)
        for (int q = 0; q < 3; ++q) c->cell[r][q] = d->cell[3 * r + q];
    if (d->tip_pbc) inv3(c->cell, c->cinv);
    const int images = d->vdw_pbc ? 9 : 1;
    c->nt = d->n_atoms * images;
    c->terms = malloc(sizeof(Term) * (c->nt > 0 ? c->nt : 1));
    int t = 0;
    for (int ia = -1; ia <= 1; ++ia)
        for (int ib = -1; ib <= 1; ++ib) {
            if (!d->vdw_pbc && (ia != 0 || ib != 0)) continue;
            double sx = 0, sy = 0, sz = 0;
            if (d->vdw_pbc) { /* simulation.cpp:303-306 */
                sx = ia * c->cell[0][0] + ib * c->cell[0][1];
                sy = ia * c->cell[1][0] + ib * c->cell[1][1];
                sz = ia * c->cell[2][0] + ib * c->cell[2][1];
            }
            for (int a = 0; a < d->n_atoms; ++a) {
                Term* tm = &c->terms[t++];
                const mafm_pair* p = &d->tip_pair[d->type[a]];
                tm->x = d->pos[3 * a] + sx;
                tm->y = d->pos[3 * a + 1] + sy;
                tm->z = d->pos[3 * a + 2] + sz;
                tm->kind = p->kind;
                tm->p0 = p->p[0]; tm->p1 = p->p[1]; tm->p2 = p->p[2];
                tm->coul = d->coulomb && !d->vdw_pbc && d->tip_charge != 0 && d->charge[a] != 0;
                tm->qq = tm->coul ? d->qbase * d->tip_charge * d->charge[a] : 0.0;
            }
        }
    c->mode = 0;
    if (d->use_external_potential) {
        int st = build_es(c);
        if (st) return st;
        c->mode = 1;
    }
    if (d->rigidgrid) {
        build_grid(c);
        c->mode = 2;
    }
    return 0;
}

static void ctx_free(Ctx* c) {
    free(c->terms);
    free(c->es.fe);
    free(c->grid.fe);
}

/* ---- entry points (ctypes) ----------------------------------------------- */

/* Relax columns [col_begin, col_end); out[(col - col_begin)*nz + k]
 * (Simulation::run simulation.cpp:67-143, OpenMP over columns as the
 * reference's schedule(dynamic, 1)).  nthreads <= 0 keeps the OpenMP default. */
int oracle_run(const mafm_scan_desc* d, int col_begin, int col_end, mafm_point* out,
               int nthreads, uint64_t* total_steps) {
    Ctx c;
    int st = ctx_init(&c, d);
    if (st) { ctx_free(&c); return st; }
    unsigned long long steps = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : steps) num_threads(nthreads > 0 ? nthreads : omp_get_max_threads())
    for (int col = col_begin; col < col_end; ++col) {
        mafm_point* o = out + (size_t)(col - col_begin) * d->nz;
        column(&c, col, o);
        for (int k = 0; k < d->nz; ++k) steps += (unsigned long long)o[k].steps;
    }
    if (total_steps) *total_steps = steps;
    ctx_free(&c);
    return 0;
}

/* oracle_run over a list of columns: out[i*nz + k] for column cols[i] (a
 * seeded sample of pixels spread over the whole scan). */
int oracle_run_columns(const mafm_scan_desc* d, const int32_t* cols, int64_t n, mafm_point* out,
                       int nthreads, uint64_t* total_steps) {
    Ctx c;
    int st = ctx_init(&c, d);
    if (st) { ctx_free(&c); return st; }
    unsigned long long steps = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : steps) num_threads(nthreads > 0 ? nthreads : omp_get_max_threads())
    for (int64_t i = 0; i < n; ++i) {
        mafm_point* o = out + (size_t)i * d->nz;
        column(&c, cols[i], o);
        for (int k = 0; k < d->nz; ++k) steps += (unsigned long long)o[k].steps;
    }
    if (total_steps) *total_steps = steps;
    ctx_free(&c);
    return 0;
}

/* oracle_run with its wall time split into the set-up (terms, external field,
 * rigid grid: ctx_init) and the relaxation: t[0], t[1] in seconds. */
int oracle_run_split(const mafm_scan_desc* d, int col_begin, int col_end, mafm_point* out,
                     int nthreads, uint64_t* total_steps, double t[2]) {
    const double t0 = omp_get_wtime();
    Ctx c;
    int st = ctx_init(&c, d);
    if (st) { ctx_free(&c); return st; }
    const double t1 = omp_get_wtime();
    unsigned long long steps = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : steps) num_threads(nthreads > 0 ? nthreads : omp_get_max_threads())
    for (int col = col_begin; col < col_end; ++col) {
        mafm_point* o = out + (size_t)(col - col_begin) * d->nz;
        column(&c, col, o);
        for (int k = 0; k < d->nz; ++k) steps += (unsigned long long)o[k].steps;
    }
    if (total_steps) *total_steps = steps;
    ctx_free(&c);
    t[0] = t1 - t0;
    t[1] = omp_get_wtime() - t1;
    return 0;
}

/* Tip–surface F,E at tip positions (the tip-surface sum of System::getOutput,
 * system.cpp:28-51); what 1 = external field only
 * (ElectrostaticPotentialInteraction::eval interactions.cpp:236-242). */
int oracle_sample(const mafm_scan_desc* d, int what, const double* pts, int64_t n, double* out) {
    Ctx c;
    int st = ctx_init(&c, d);
    if (st) { ctx_free(&c); return st; }
    for (int64_t i = 0; i < n; ++i) {
        v3 tip = {pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]};
        v3 F = {0, 0, 0};
        double E = 0;
        int outside = 0;
        if (what == 1) {
            if (d->use_external_potential) grid_interp(&c, &c.es, tip, &F, &E, &outside);
        } else {
            eval_ts(&c, tip, &F, &E, &outside);
        }
        out[4 * i] = F.x; out[4 * i + 1] = F.y; out[4 * i + 2] = F.z; out[4 * i + 3] = E;
    }
    ctx_free(&c);
    return 0;
}

/* Copy a grid (what 0 = rigid grid of buildTipGridInteractions simulation.cpp:
 * 420-501, 1 = external field of interactions.cpp:53-234): n, then 4 doubles per node. */
int oracle_grid(const mafm_scan_desc* d, int what, int32_t n[3], double* out, int64_t cap) {
    Ctx c;
    int st = ctx_init(&c, d);
    if (st) { ctx_free(&c); return st; }
    const Grid* g = what == 1 ? &c.es : &c.grid;
    if (!g->fe) { ctx_free(&c); return MAFM_E_INVALID; }
    for (int a = 0; a < 3; ++a) n[a] = g->n[a];
    const int64_t N = (int64_t)g->n[0] * g->n[1] * g->n[2] * 4;
    if (out && cap >= N) memcpy(out, g->fe, (size_t)N * sizeof(double));
    ctx_free(&c);
    return 0;
}

/* ---- adjoint (implicit differentiation at the relaxed points) ------------
 * Same formulas as the product's adjoint kernel, written plainly: per point,
 * J = dF_total/dx, lambda = J^-T (row z of dF_ts/dx), mu = w (e_z - lambda),
 * and every term contributes mu . df/dtheta.  The reference itself has no
 * derivatives; this restatement is checked against central finite differences
 * of the oracle's own relaxation in tests/test_adjoint.py. */
/* Adjoint helpers: derivatives of interactions.cpp:15-51 (no counterpart in the
 * reference, which has no derivatives). */
static void pair_s_o(int kind, double p0, double p1, double p2, double r2, double* s, double* dsr) {
    if (kind == MAFM_PAIR_LJ) {
        double ir2 = 1.0 / r2, ir6 = ir2 * ir2 * ir2;
        double a12 = p1 * ir6 * ir6, a6 = p0 * ir6;
        *s = (12 * a12 - 6 * a6) * ir2;
        *dsr = (-168 * a12 + 48 * a6) * ir2 * ir2;
    } else {
        double r = sqrt(r2), d = exp(-p1 * (r - p2));
        double g = 2 * p0 * p1 * (d * d - d), dg = 2 * p0 * p1 * (2 * d - 1) * (-p1 * d);
        *s = g / r;
        *dsr = (dg / r - g / r2) / r;
    }
}

static void pair_dparam_o(int kind, double p0, double p1, double p2, double r2, double q[3]) {
    if (kind == MAFM_PAIR_LJ) {
        double ir2 = 1.0 / r2, ir6 = ir2 * ir2 * ir2;
        q[0] = -6 * ir6 * ir2;
        q[1] = 12 * ir6 * ir6 * ir2;
        q[2] = 0;
    } else {
        double r = sqrt(r2), x = r - p2, d = exp(-p1 * x), dd = d * d - d;
        q[0] = 2 * p1 * dd / r;
        q[1] = (2 * p0 * dd + 2 * p0 * p1 * (2 * d - 1) * (-x * d)) / r;
        q[2] = 2 * p0 * p1 * (2 * d - 1) * (p1 * d) / r;
    }
}

static void es_jac_o(const Grid* g, v3 pos, double Jg[9]) {
    double q[3] = {pos.x - g->origin[0], pos.y - g->origin[1], pos.z - g->origin[2]}, pb[3], d[3];
    int gp[3];
    for (int a = 0; a < 3; ++a) {
        pb[a] = g->inv[a][0] * q[0] + g->inv[a][1] * q[1] + g->inv[a][2] * q[2];
        gp[a] = (int)floor(pb[a]);
        d[a] = pb[a] - gp[a];
    }
    double dFd[3][3] = {{0}};
    for (int c = 0; c < 8; ++c) {
        int idx[3] = {gp[0] + (c >> 2), gp[1] + ((c >> 1) & 1), gp[2] + (c & 1)};
        for (int a = 0; a < 3; ++a) {
            idx[a] %= g->n[a];
            if (idx[a] < 0) idx[a] += g->n[a];
        }
        const double* v = g->fe + 4 * (((size_t)idx[0] * g->n[1] + idx[1]) * g->n[2] + idx[2]);
        double w[3] = {(c >> 2) ? d[0] : 1 - d[0], ((c >> 1) & 1) ? d[1] : 1 - d[1], (c & 1) ? d[2] : 1 - d[2]};
        double sg[3] = {(c >> 2) ? 1.0 : -1.0, ((c >> 1) & 1) ? 1.0 : -1.0, (c & 1) ? 1.0 : -1.0};
        double dw[3] = {sg[0] * w[1] * w[2], sg[1] * w[0] * w[2], sg[2] * w[0] * w[1]};
        for (int m = 0; m < 3; ++m)
            for (int a = 0; a < 3; ++a) dFd[m][a] += v[m] * dw[a];
    }
    for (int m = 0; m < 3; ++m)
        for (int j = 0; j < 3; ++j)
            Jg[3 * m + j] = dFd[m][0] * g->inv[0][j] + dFd[m][1] * g->inv[1][j] + dFd[m][2] * g->inv[2][j];
}

/* FP64 gradients of sum_p w_p Fz_p by implicit differentiation at each
 * relaxed point (no counterpart in the reference, which has no derivatives;
 * pinned by finite differences of the reference's own relaxation). */
int oracle_adjoint(const mafm_scan_desc* d, const mafm_point* pts, const double* w, double* dpos,
                   double* dcharge, double* dpair) {
    Ctx c;
    int st = ctx_init(&c, d);
    if (st) { ctx_free(&c); return st; }
    if (c.mode == 2) { ctx_free(&c); return MAFM_E_UNSUPPORTED; }
    const int na = d->n_atoms;
    memset(dpos, 0, sizeof(double) * 3 * na);
    memset(dcharge, 0, sizeof(double) * na);
    memset(dpair, 0, sizeof(double) * 3 * d->n_types);
    const double qbq = d->qbase * d->tip_charge;
    const long long npts = (long long)d->nx * d->ny * d->nz;
    for (long long p = 0; p < npts; ++p) {
        const long long col = p / d->nz;
        const int k = (int)(p % d->nz);
        double dx, dy;
        dummy_xy(&c, d->tip_pbc && !d->rigidgrid, (int)(col / d->ny) * d->dx, (int)(col % d->ny) * d->dy, &dx, &dy);
        double dz = d->zhigh;
        for (int s = 0; s < k; ++s) dz -= d->dz;
        v3 x = {pts[p].tip[0], pts[p].tip[1], pts[p].tip[2]};
        double J[9] = {0};
        for (int t = 0; t < c.nt; ++t) {
            const Term* tm = &c.terms[t];
            v3 r = {x.x - tm->x, x.y - tm->y, x.z - tm->z};
            double r2 = r.x * r.x + r.y * r.y + r.z * r.z, s, dsr;
            pair_s_o(tm->kind, tm->p0, tm->p1, tm->p2, r2, &s, &dsr);
            if (tm->coul) {
                double ir = 1.0 / sqrt(r2), ir3 = ir * ir * ir;
                s += tm->qq * ir3;
                dsr += -3 * tm->qq * ir3 * ir * ir;
            }
            double rv[3] = {r.x, r.y, r.z};
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) J[3 * a + b] += (a == b ? s : 0) + dsr * rv[a] * rv[b];
        }
        if (c.mode == 1) {
            double Jg[9];
            es_jac_o(&c.es, x, Jg);
            for (int m = 0; m < 9; ++m) J[m] += Jg[m];
        }
        double cz[3] = {J[6], J[7], J[8]};
        {
            v3 r = {x.x - dx, x.y - dy, x.z - dz};
            double r2 = r.x * r.x + r.y * r.y + r.z * r.z, s, dsr;
            pair_s_o(d->dummy_pair.kind, d->dummy_pair.p[0], d->dummy_pair.p[1], d->dummy_pair.p[2], r2, &s, &dsr);
            if (d->tip_dummy_coulomb && d->dummy_charge != 0 && d->tip_charge != 0) {
                double qq = d->qbase * d->dummy_charge * d->tip_charge;
                double ir = 1.0 / sqrt(r2), ir3 = ir * ir * ir;
                s += qq * ir3;
                dsr += -3 * qq * ir3 * ir * ir;
            }
            double rv[3] = {r.x, r.y, r.z};
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) J[3 * a + b] += (a == b ? s : 0) + dsr * rv[a] * rv[b];
            double rho = sqrt(r.x * r.x + r.y * r.y), k2 = 2 * d->harm_k;
            if (d->harm_r0 == 0.0 || rho <= 1e-10) {
                J[0] -= k2;
                J[4] -= k2;
            } else {
                double f = 1 - d->harm_r0 / rho, g = d->harm_r0 / (rho * rho * rho);
                J[0] -= k2 * (f + g * r.x * r.x);
                J[4] -= k2 * (f + g * r.y * r.y);
                J[1] -= k2 * g * r.x * r.y;
                J[3] -= k2 * g * r.x * r.y;
            }
        }
        /* lambda = J^-T cz by Gaussian elimination on J^T */
        double A[3][4];
        for (int a = 0; a < 3; ++a) {
            for (int b = 0; b < 3; ++b) A[a][b] = J[3 * b + a];
            A[a][3] = cz[a];
        }
        for (int col2 = 0; col2 < 3; ++col2) {
            int piv = col2;
            for (int r2 = col2 + 1; r2 < 3; ++r2)
                if (fabs(A[r2][col2]) > fabs(A[piv][col2])) piv = r2;
            for (int m = 0; m < 4; ++m) { double tmp = A[col2][m]; A[col2][m] = A[piv][m]; A[piv][m] = tmp; }
            for (int r2 = 0; r2 < 3; ++r2) {
                if (r2 == col2) continue;
                double f = A[r2][col2] / A[col2][col2];
                for (int m = col2; m < 4; ++m) A[r2][m] -= f * A[col2][m];
            }
        }
        double lam[3] = {A[0][3] / A[0][0], A[1][3] / A[1][1], A[2][3] / A[2][2]};
        double mu[3] = {-w[p] * lam[0], -w[p] * lam[1], w[p] * (1 - lam[2])};
        for (int t = 0; t < c.nt; ++t) {
            const Term* tm = &c.terms[t];
            const int a = t % na;
            v3 r = {x.x - tm->x, x.y - tm->y, x.z - tm->z};
            double r2 = r.x * r.x + r.y * r.y + r.z * r.z, s, dsr, ir3 = 0;
            pair_s_o(tm->kind, tm->p0, tm->p1, tm->p2, r2, &s, &dsr);
            if (tm->coul) {
                double ir = 1.0 / sqrt(r2);
                ir3 = ir * ir * ir;
                s += tm->qq * ir3;
                dsr += -3 * tm->qq * ir3 * ir * ir;
            }
            double rm = r.x * mu[0] + r.y * mu[1] + r.z * mu[2];
            dpos[3 * a] -= s * mu[0] + dsr * r.x * rm;
            dpos[3 * a + 1] -= s * mu[1] + dsr * r.y * rm;
            dpos[3 * a + 2] -= s * mu[2] + dsr * r.z * rm;
            double q[3];
            pair_dparam_o(tm->kind, tm->p0, tm->p1, tm->p2, r2, q);
            for (int m = 0; m < 3; ++m) dpair[3 * d->type[a] + m] += q[m] * rm;
            if (tm->coul) dcharge[a] += qbq * ir3 * rm;
        }
    }
    ctx_free(&c);
    return 0;
}

/* ---- flexible molecules ---------------------------------------------------
 * `flexible on`: every atom whose fixed flag is not 1 moves.  The interaction
 * list is built in the reference's order (Simulation::buildInteractions,
 * simulation.cpp:200-215: tip–surface, tip–dummy, bonds / angles / dihedrals /
 * non-bonded pairs of buildSurfaceSurfaceInteractions :557-693, substrate and
 * XY tethers of buildSubstrateInteractions :516-528) and evaluated into shared
 * force / energy arrays exactly as the reference's integrators do
 * (integrators.cpp:8-111), each term written as its eval() in
 * interactions.cpp:15-51, 252-370. */

enum { FI_LJ, FI_MORSE, FI_COUL, FI_TIPHARM, FI_XY, FI_SUB, FI_BOND, FI_ANGLE, FI_DIHED };

typedef struct {
    int type, ts;      /* ts: a tip–surface term (isTipSurface) */
    int a[4];          /* System indices */
    double p[6];
    v3 shift;
} FInt;

typedef struct {
    const mafm_scan_desc* d;
    int na;
    FInt* it;
    int nit;
    int* fixed;
    v3* pos0;
    double cell[3][3], cinv[3][3];
} FCtx;

static v3 vsub(v3 a, v3 b) { v3 r = {a.x - b.x, a.y - b.y, a.z - b.z}; return r; }
static v3 vadd(v3 a, v3 b) { v3 r = {a.x + b.x, a.y + b.y, a.z + b.z}; return r; }
static v3 vscal(double s, v3 a) { v3 r = {s * a.x, s * a.y, s * a.z}; return r; }
static v3 vmul(v3 a, double s) { v3 r = {a.x * s, a.y * s, a.z * s}; return r; }
static v3 vdiv(v3 a, double s) { v3 r = {a.x / s, a.y / s, a.z / s}; return r; }
static double vdot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static v3 vcross(v3 a, v3 b) {
    v3 r = {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
    return r;
}
static v3 vnorm(v3 a) {
    double l = len3(a);
    v3 z = {0, 0, 0};
    if (l > 1e-10) { v3 r = {a.x / l, a.y / l, a.z / l}; return r; }
    return z;
}

/* The flexible-mode interactions: interactions.cpp:15-51 (pairs), :252-266
 * (tip spring), :268-362 (XY tether, substrate, bond, angle, dihedral). */
static void fint_eval(const FCtx* c, const FInt* t, const v3* pos, v3* F, double* E) {
    switch (t->type) {
    case FI_LJ: {
        int i1 = t->a[0], i2 = t->a[1];
        v3 r = vsub(pos[i1], vadd(pos[i2], t->shift));
        double r_sqr = r.x * r.x + r.y * r.y + r.z * r.z;
        double r6 = r_sqr * r_sqr * r_sqr;
        double ta = t->p[1] / (r6 * r6), tb = t->p[0] / r6;
        double e = ta - tb;
        v3 f = vscal((12 * ta - 6 * tb) / r_sqr, r);
        E[i1] += e; E[i2] += e;
        F[i1] = vadd(F[i1], f); F[i2] = vsub(F[i2], f);
        break;
    }
    case FI_MORSE: {
        int i1 = t->a[0], i2 = t->a[1];
        v3 r = vsub(pos[i1], vadd(pos[i2], t->shift));
        double rl = len3(r);
        double d = exp(-t->p[1] * (rl - t->p[2]));
        double e = t->p[0] * (d * d - 2 * d + 1);
        double f_abs = 2 * t->p[0] * t->p[1] * (d * d - d);
        v3 f = vscal(f_abs / rl, r);
        E[i1] += e; E[i2] += e;
        F[i1] = vadd(F[i1], f); F[i2] = vsub(F[i2], f);
        break;
    }
    case FI_COUL: {
        int i1 = t->a[0], i2 = t->a[1];
        v3 r = vsub(pos[i1], pos[i2]);
        double rl = len3(r);
        double e = t->p[0] / rl;
        v3 f = vscal(t->p[0] / (rl * rl * rl), r);
        E[i1] += e; E[i2] += e;
        F[i1] = vadd(F[i1], f); F[i2] = vsub(F[i2], f);
        break;
    }
    case FI_TIPHARM: {
        int i1 = t->a[0], i2 = t->a[1];
        v3 rv = vsub(pos[i1], pos[i2]);
        double r = sqrt(rv.x * rv.x + rv.y * rv.y);
        double dr = r - t->p[1];
        double e = t->p[0] * dr * dr;
        v3 f = {0, 0, 0};
        if (r > TOL) {
            double s = -2 * t->p[0] * dr / r;
            f.x = s * rv.x; f.y = s * rv.y; f.z = 0;
        }
        E[i1] += e; E[i2] += e;
        F[i1] = vadd(F[i1], f); F[i2] = vsub(F[i2], f);
        break;
    }
    case FI_XY: {
        int i = t->a[0];
        double rx = pos[i].x - t->p[1], ry = pos[i].y - t->p[2];
        double r = sqrt(rx * rx + ry * ry);
        double e = t->p[0] * r * r;
        v3 f = {0, 0, 0};
        if (r > TOL) { double s = -2 * t->p[0]; f.x = s * rx; f.y = s * ry; f.z = 0; }
        E[i] += e;
        F[i] = vadd(F[i], f);
        break;
    }
    case FI_SUB: {
        int i = t->a[0];
        double mult = t->p[0], ulj = t->p[1], ushift = t->p[2], z0 = t->p[3], rc = t->p[4], sig = t->p[5];
        double dz = pos[i].z - z0;
        double sig_z = sig / dz;
        double sig_z2 = sig_z * sig_z;
        double sig_z4 = sig_z2 * sig_z2;
        double sig_z10 = sig_z4 * sig_z4 * sig_z2;
        double eterm = 0.0, fterm = 0.0;
        if (dz <= rc) {
            eterm += mult * (2. / 5 * sig_z10 - sig_z4) + ulj * dz * dz - ushift;
            fterm += 4 * mult / dz * (sig_z10 - sig_z4) + 2 * ulj * dz;
        }
        F[i].z += fterm;
        E[i] += eterm;
        break;
    }
    case FI_BOND: {
        int i1 = t->a[0], i2 = t->a[1];
        v3 rv = vsub(pos[i1], pos[i2]);
        double r = len3(rv);
        double dr = r - t->p[1];
        double e = t->p[0] * (dr * dr);
        v3 f = vscal(-2 * t->p[0] * dr / r, rv);
        E[i1] += e; E[i2] += e;
        F[i1] = vadd(F[i1], f); F[i2] = vsub(F[i2], f);
        break;
    }
    case FI_ANGLE: {
        int sh = t->a[0], i1 = t->a[1], i2 = t->a[2];
        v3 r1v = vsub(pos[i1], pos[sh]), r2v = vsub(pos[i2], pos[sh]);
        double r1 = len3(r1v), r2 = len3(r2v);
        double cos_t = vdot(r1v, r2v) / (r1 * r2);
        if (cos_t > 1) cos_t = 1;
        else if (cos_t < -1) cos_t = -1;
        double theta = acos(cos_t);
        double sin_t = sin(theta);
        double d_theta = theta - t->p[1];
        double fm = -2 * t->p[0] * d_theta / sin_t;
        v3 f1 = vscal(-fm / r1, vsub(vdiv(r2v, r2), vdiv(vmul(r1v, cos_t), r1)));
        v3 f2 = vscal(-fm / r2, vsub(vdiv(r1v, r1), vdiv(vmul(r2v, cos_t), r2)));
        double e = t->p[0] * (d_theta * d_theta);
        F[i1] = vadd(F[i1], f1);
        F[i2] = vadd(F[i2], f2);
        F[sh] = vsub(F[sh], vadd(f1, f2));
        E[i1] += e; E[i2] += e; E[sh] += e;
        break;
    }
    case FI_DIHED: {
        int a1 = t->a[0], a2 = t->a[1], a3 = t->a[2], a4 = t->a[3];
        v3 r12 = vsub(pos[a1], pos[a2]), r23v = vsub(pos[a2], pos[a3]), r43 = vsub(pos[a4], pos[a3]);
        double r23 = len3(r23v);
        v3 mv = vcross(r12, r23v), nv = vcross(r43, r23v);
        double m = len3(mv), n = len3(nv);
        double tan_s = vdot(nv, r12) * r23 / vdot(mv, nv);
        double sigma = atan(tan_s);
        double d_sigma = sigma - t->p[1];
        double fm = 2 * t->p[0] * d_sigma;
        v3 f1 = vscal(-fm * r23 / (m * m), mv);
        v3 f2 = vscal(-fm, vsub(vscal(vdot(r43, r23v) / (n * n * r23), nv),
                                vscal(((r23 * r23) + vdot(r12, r23v)) / (m * m * r23), mv)));
        v3 f3 = vscal(-fm, vadd(vscal(vdot(r12, r23v) / (m * m * r23), mv),
                                vscal(((r23 * r23) - vdot(r43, r23v)) / (n * n * r23), nv)));
        v3 f4 = vscal(fm * r23 / (n * n), nv);
        double e = t->p[0] * (d_sigma * d_sigma);
        F[a1] = vadd(F[a1], f1); F[a2] = vadd(F[a2], f2);
        F[a3] = vadd(F[a3], f3); F[a4] = vadd(F[a4], f4);
        E[a1] += e; E[a2] += e; E[a3] += e; E[a4] += e;
        break;
    }
    }
    (void)c;
}

static void fl_eval(const FCtx* c, const v3* pos, v3* F, double* E, int ts_only) {
    for (int i = 0; i < c->na; ++i) { F[i].x = F[i].y = F[i].z = 0; E[i] = 0; }
    for (int q = 0; q < c->nit; ++q)
        if (!ts_only || c->it[q].ts) fint_eval(c, &c->it[q], pos, F, E);
}

static int fl_push(FCtx* c, int* cap, FInt t) {
    if (c->nit == *cap) {
        *cap = *cap ? 2 * *cap : 256;
        FInt* n = (FInt*)realloc(c->it, sizeof(FInt) * (size_t)*cap);
        if (!n) return 1;
        c->it = n;
    }
    c->it[c->nit++] = t;
    return 0;
}

/* The interaction list of a flexible scan in the reference's order:
 * buildInteractions simulation.cpp:201-216 with buildSubstrateInteractions
 * :517-555 and buildSurfaceSurfaceInteractions :557-693. */
static int fctx_init(FCtx* c, const mafm_scan_desc* d, const mafm_flex_desc* f) {
    memset(c, 0, sizeof *c);
    c->d = d;
    c->na = d->n_atoms + 2;
    c->fixed = (int*)calloc((size_t)c->na, sizeof(int));
    c->pos0 = (v3*)calloc((size_t)c->na, sizeof(v3));
    if (!c->fixed || !c->pos0) return MAFM_E_NOMEM;
    c->fixed[0] = 1;
    for (int a = 0; a < d->n_atoms; ++a) {
        c->fixed[a + 2] = f->fixed[a];
        c->pos0[a + 2].x = d->pos[3 * a]; c->pos0[a + 2].y = d->pos[3 * a + 1]; c->pos0[a + 2].z = d->pos[3 * a + 2];
    }
    for (int r = 0; r < 3; ++r)
        for (int k = 0; k < 3; ++k) c->cell[r][k] = d->cell[3 * r + k];
    if (d->tip_pbc) inv3(c->cell, c->cinv);
    int cap = 0;
    FInt t;
    /* buildTipSurfaceInteractions (simulation.cpp:297-320) */
    for (int ia = -1; ia <= 1; ++ia)
        for (int ib = -1; ib <= 1; ++ib) {
            if (!d->vdw_pbc && (ia != 0 || ib != 0)) continue;
            v3 sh = {0, 0, 0};
            if (d->vdw_pbc) {
                sh.x = ia * c->cell[0][0] + ib * c->cell[0][1];
                sh.y = ia * c->cell[1][0] + ib * c->cell[1][1];
                sh.z = ia * c->cell[2][0] + ib * c->cell[2][1];
            }
            for (int a = 0; a < d->n_atoms; ++a) {
                const mafm_pair* pr = &d->tip_pair[d->type[a]];
                memset(&t, 0, sizeof t);
                t.type = pr->kind == MAFM_PAIR_LJ ? FI_LJ : FI_MORSE;
                t.ts = 1; t.a[0] = 1; t.a[1] = a + 2; t.shift = sh;
                for (int k = 0; k < 3; ++k) t.p[k] = pr->p[k];
                if (fl_push(c, &cap, t)) return MAFM_E_NOMEM;
                if (!d->vdw_pbc && d->coulomb && d->tip_charge != 0 && d->charge[a] != 0) {
                    memset(&t, 0, sizeof t);
                    t.type = FI_COUL; t.ts = 1; t.a[0] = 1; t.a[1] = a + 2;
                    t.p[0] = d->qbase * d->tip_charge * d->charge[a];
                    if (fl_push(c, &cap, t)) return MAFM_E_NOMEM;
                }
            }
        }
    /* buildTipDummyInteractions (simulation.cpp:503-515) */
    memset(&t, 0, sizeof t);
    t.type = d->dummy_pair.kind == MAFM_PAIR_LJ ? FI_LJ : FI_MORSE;
    t.a[0] = 0; t.a[1] = 1;
    for (int k = 0; k < 3; ++k) t.p[k] = d->dummy_pair.p[k];
    if (fl_push(c, &cap, t)) return MAFM_E_NOMEM;
    if (d->tip_dummy_coulomb && d->dummy_charge != 0 && d->tip_charge != 0) {
        memset(&t, 0, sizeof t);
        t.type = FI_COUL; t.a[0] = 0; t.a[1] = 1;
        t.p[0] = d->qbase * d->dummy_charge * d->tip_charge;
        if (fl_push(c, &cap, t)) return MAFM_E_NOMEM;
    }
    memset(&t, 0, sizeof t);
    t.type = FI_TIPHARM; t.a[0] = 0; t.a[1] = 1; t.p[0] = d->harm_k; t.p[1] = d->harm_r0;
    if (fl_push(c, &cap, t)) return MAFM_E_NOMEM;
    /* buildSurfaceSurfaceInteractions: bonds, angles, dihedrals, pairs */
    for (int b = 0; b < f->n_bonds; ++b) {
        memset(&t, 0, sizeof t);
        t.type = FI_BOND; t.a[0] = f->bond_atoms[2 * b] + 2; t.a[1] = f->bond_atoms[2 * b + 1] + 2;
        t.p[0] = f->bond_param[2 * b]; t.p[1] = f->bond_param[2 * b + 1];
        if (fl_push(c, &cap, t)) return MAFM_E_NOMEM;
    }
    for (int g = 0; g < f->n_angles; ++g) {
        memset(&t, 0, sizeof t);
        t.type = FI_ANGLE;
        for (int k = 0; k < 3; ++k) t.a[k] = f->angle_atoms[3 * g + k] + 2;
        t.p[0] = f->angle_param[2 * g]; t.p[1] = f->angle_param[2 * g + 1];
        if (fl_push(c, &cap, t)) return MAFM_E_NOMEM;
    }
    for (int g = 0; g < f->n_dihedrals; ++g) {
        memset(&t, 0, sizeof t);
        t.type = FI_DIHED;
        for (int k = 0; k < 4; ++k) t.a[k] = f->dihedral_atoms[4 * g + k] + 2;
        t.p[0] = f->dihedral_param[2 * g]; t.p[1] = f->dihedral_param[2 * g + 1];
        if (fl_push(c, &cap, t)) return MAFM_E_NOMEM;
    }
    for (int q = 0; q < f->n_pairs; ++q) {
        memset(&t, 0, sizeof t);
        t.type = f->pair_vdw[q].kind == MAFM_PAIR_LJ ? FI_LJ : FI_MORSE;
        t.a[0] = f->pair_atoms[2 * q] + 2; t.a[1] = f->pair_atoms[2 * q + 1] + 2;
        for (int k = 0; k < 3; ++k) t.p[k] = f->pair_vdw[q].p[k];
        if (fl_push(c, &cap, t)) return MAFM_E_NOMEM;
        if (f->pair_qq && f->pair_qq[q] != 0) {
            memset(&t, 0, sizeof t);
            t.type = FI_COUL; t.a[0] = f->pair_atoms[2 * q] + 2; t.a[1] = f->pair_atoms[2 * q + 1] + 2;
            t.p[0] = f->pair_qq[q];
            if (fl_push(c, &cap, t)) return MAFM_E_NOMEM;
        }
    }
    /* buildSubstrateInteractions; SubstrateInteraction ctor interactions.hpp:222-229 */
    double eps = f->substrate[0], sig = f->substrate[1], lam = f->substrate[2], rc = f->substrate[3];
    double mult = 2 * PI * eps * pow(sig / lam, 2);
    double ulj = (PI / (lam * lam)) * 4 * eps * (pow(sig / rc, 12) - pow(sig / rc, 6));
    double ushift = mult * ((12. / 5) * pow(sig / rc, 10) - 3 * pow(sig / rc, 4));
    for (int i = 2; i < c->na; ++i) {
        memset(&t, 0, sizeof t);
        t.type = FI_SUB; t.a[0] = i;
        t.p[0] = mult; t.p[1] = ulj; t.p[2] = ushift; t.p[3] = -sig; t.p[4] = rc; t.p[5] = sig;
        if (fl_push(c, &cap, t)) return MAFM_E_NOMEM;
        if (c->fixed[i] == 2) {
            memset(&t, 0, sizeof t);
            t.type = FI_XY; t.a[0] = i; t.p[0] = f->substrate[4];
            t.p[1] = c->pos0[i].x; t.p[2] = c->pos0[i].y;
            if (fl_push(c, &cap, t)) return MAFM_E_NOMEM;
        }
    }
    return 0;
}

static void fctx_free(FCtx* c) {
    free(c->it); free(c->fixed); free(c->pos0);
}

typedef struct {
    v3 *pos, *vel, *F, *p2, *v2, *p3, *v3b, *p4, *v4, *f1, *f2, *f3, *f4;
    double *E, *e1, *e2, *e3, *e4;
} FState;

/* one integrator step (integrators.cpp:8-111): forces_/energies_ in F/E */
/* eulerStep / midpointStep / rk4Step integrators.cpp:8-111 over every free atom. */
static void fl_step(const FCtx* c, FState* s, double dt) {
    const int n = c->na;
    const mafm_scan_desc* d = c->d;
    if (d->integrator == MAFM_INT_EULER) {
        fl_eval(c, s->pos, s->F, s->E, 0);
        for (int i = 0; i < n; ++i)
            if (c->fixed[i] != 1) {
                s->pos[i] = vadd(s->pos[i], vscal(dt, s->vel[i]));
                s->vel[i] = vadd(s->vel[i], vdiv(vscal(dt, s->F[i]), 1.0));
            }
    } else if (d->integrator == MAFM_INT_MIDPOINT) {
        memcpy(s->p2, s->pos, sizeof(v3) * n);
        memcpy(s->v2, s->vel, sizeof(v3) * n);
        fl_eval(c, s->pos, s->f1, s->e1, 0);
        for (int i = 0; i < n; ++i)
            if (c->fixed[i] != 1) {
                s->p2[i] = vadd(s->p2[i], vscal(dt / 2, s->vel[i]));
                s->v2[i] = vadd(s->v2[i], vdiv(vscal(dt / 2, s->f1[i]), 1.0));
            }
        fl_eval(c, s->p2, s->f2, s->e2, 0);
        for (int i = 0; i < n; ++i) {
            if (c->fixed[i] != 1) {
                s->pos[i] = vadd(s->pos[i], vscal(dt, s->v2[i]));
                s->vel[i] = vadd(s->vel[i], vdiv(vscal(dt, s->f2[i]), 1.0));
            }
            s->F[i] = s->f2[i];
            s->E[i] = s->e2[i];
        }
    } else {
        memcpy(s->p2, s->pos, sizeof(v3) * n); memcpy(s->p3, s->pos, sizeof(v3) * n);
        memcpy(s->p4, s->pos, sizeof(v3) * n);
        memcpy(s->v2, s->vel, sizeof(v3) * n); memcpy(s->v3b, s->vel, sizeof(v3) * n);
        memcpy(s->v4, s->vel, sizeof(v3) * n);
        fl_eval(c, s->pos, s->f1, s->e1, 0);
        for (int i = 0; i < n; ++i)
            if (c->fixed[i] != 1) {
                s->p2[i] = vadd(s->p2[i], vscal(dt / 2, s->vel[i]));
                s->v2[i] = vadd(s->v2[i], vdiv(vscal(dt / 2, s->f1[i]), 1.0));
            }
        fl_eval(c, s->p2, s->f2, s->e2, 0);
        for (int i = 0; i < n; ++i)
            if (c->fixed[i] != 1) {
                s->p3[i] = vadd(s->p3[i], vscal(dt / 2, s->v2[i]));
                s->v3b[i] = vadd(s->v3b[i], vdiv(vscal(dt / 2, s->f2[i]), 1.0));
            }
        fl_eval(c, s->p3, s->f3, s->e3, 0);
        for (int i = 0; i < n; ++i)
            if (c->fixed[i] != 1) {
                s->p4[i] = vadd(s->p4[i], vscal(dt, s->v3b[i]));
                s->v4[i] = vadd(s->v4[i], vdiv(vscal(dt, s->f3[i]), 1.0));
            }
        fl_eval(c, s->p4, s->f4, s->e4, 0);
        for (int i = 0; i < n; ++i) {
            v3 fs = vadd(vadd(vadd(s->f1[i], vscal(2, s->f2[i])), vscal(2, s->f3[i])), s->f4[i]);
            if (c->fixed[i] != 1) {
                v3 vs = vadd(vadd(vadd(s->vel[i], vscal(2, s->v2[i])), vscal(2, s->v3b[i])), s->v4[i]);
                s->pos[i] = vadd(s->pos[i], vscal(dt / 6, vs));
                s->vel[i] = vadd(s->vel[i], vdiv(vscal(dt / 6, fs), 1.0));
            }
            s->F[i] = vdiv(fs, 6);
            s->E[i] = (s->e1[i] + 2 * s->e2[i] + 2 * s->e3[i] + s->e4[i]) / 6;
        }
    }
}

static int fl_converged(const mafm_scan_desc* d, v3 F, double ediff) {
    return converged(d, F, ediff);
}

/* FIREMinimisation / SDMinimisation over all atoms (minimiser.cpp:39-129) */
/* FIREMinimisation / SDMinimisation minimiser.cpp:39-129 over every free atom. */
static int fl_minimise(const FCtx* c, FState* s) {
    const mafm_scan_desc* d = c->d;
    const int n = c->na;
    if (d->minimiser == MAFM_MIN_SD) {
        double prev = -10e6;
        int k = 1;
        for (; k < d->maxsteps; ++k) {
            prev = s->E[1];
            fl_eval(c, s->pos, s->F, s->E, 0);
            if (fl_converged(d, s->F[1], s->E[1] - prev)) break;
            for (int i = 0; i < n; ++i)
                if (c->fixed[i] != 1) s->pos[i] = vadd(s->pos[i], vscal(d->dt, s->F[i]));
        }
        (void)prev;
        return k;
    }
    double alpha = 0.1, dt = d->dt, dt_max = 10 * d->dt, prev = -10e6;
    int n_non_neg = 0, k = 1;
    for (; k < d->maxsteps; ++k) {
        prev = s->E[1];
        fl_step(c, s, dt);
        if (fl_converged(d, s->F[1], s->E[1] - prev)) break;
        double p = 0;
        for (int i = 0; i < n; ++i) {
            p += vdot(s->vel[i], s->F[i]);
            if (c->fixed[i] != 1)
                s->vel[i] = vadd(vscal(1 - alpha, s->vel[i]), vmul(vscal(alpha, vnorm(s->F[i])), len3(s->vel[i])));
        }
        if (p < 0) {
            for (int i = 0; i < n; ++i) s->vel[i].x = s->vel[i].y = s->vel[i].z = 0;
            n_non_neg = 0;
            dt *= 0.5;
            alpha = 0.1;
        } else {
            if (n_non_neg > 5) {
                dt = fmin(dt * 1.1, dt_max);
                alpha *= 0.99;
            }
            n_non_neg++;
        }
    }
    (void)prev;
    return k;
}

/* Relax columns [col_begin, col_end) of a flexible scan (Simulation::run
 * simulation.cpp:67-143 with flexible on); states (optional) receives every
 * atom's position after each height of column state_column, as
 * System::makeXYZFile writes them (system.cpp:54-66, simulation.cpp:114-116). */
int oracle_flex_run(const mafm_scan_desc* d, const mafm_flex_desc* f, int col_begin, int col_end,
                    mafm_point* out, int nthreads, uint64_t* total_steps, int state_column,
                    double* states) {
    FCtx c;
    int st = fctx_init(&c, d, f);
    if (st) { fctx_free(&c); return st; }
    unsigned long long steps = 0;
    const int n = c.na;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : steps) num_threads(nthreads > 0 ? nthreads : omp_get_max_threads())
    for (int col = col_begin; col < col_end; ++col) {
        FState s;
        v3** vs[] = {&s.pos, &s.vel, &s.F, &s.p2, &s.v2, &s.p3, &s.v3b, &s.p4, &s.v4, &s.f1, &s.f2, &s.f3, &s.f4};
        for (size_t q = 0; q < sizeof vs / sizeof vs[0]; ++q) *vs[q] = (v3*)calloc((size_t)n, sizeof(v3));
        double** es[] = {&s.E, &s.e1, &s.e2, &s.e3, &s.e4};
        for (size_t q = 0; q < sizeof es / sizeof es[0]; ++q) *es[q] = (double*)calloc((size_t)n, sizeof(double));
        memcpy(s.pos, c.pos0, sizeof(v3) * n);
        const int i = col / d->ny, j = col % d->ny;
        double x = i * d->dx, y = j * d->dy, ox = x, oy = y;
        if (d->tip_pbc) {
            v3 t = {x - d->offset[0], y - d->offset[1], 0 - d->offset[2]};
            v3 cn = mulv(c.cinv, t);
            cn.x -= floor(cn.x);
            cn.y -= floor(cn.y);
            v3 pb = mulv(c.cell, cn);
            ox = pb.x + d->offset[0];
            oy = pb.y + d->offset[1];
        }
        s.pos[0].x = ox; s.pos[0].y = oy; s.pos[1].x = ox; s.pos[1].y = oy;
        s.pos[0].z = d->zhigh;
        s.pos[1].z = d->zhigh - d->tip_dummy_d;
        for (int k = 0; k < d->nz; ++k) {
            int nst = fl_minimise(&c, &s);
            v3* Fo = (v3*)calloc((size_t)n, sizeof(v3));
            double* Eo = (double*)calloc((size_t)n, sizeof(double));
            fl_eval(&c, s.pos, Fo, Eo, 1);
            mafm_point* r = out + (size_t)(col - col_begin) * d->nz + k;
            r->tip[0] = s.pos[1].x; r->tip[1] = s.pos[1].y; r->tip[2] = s.pos[1].z;
            r->force[0] = Fo[1].x; r->force[1] = Fo[1].y; r->force[2] = Fo[1].z;
            r->energy = Eo[1];
            r->steps = nst;
            r->status = nst >= d->maxsteps ? MAFM_PT_MAXSTEPS : 0;
            free(Fo); free(Eo);
            steps += (unsigned long long)nst;
            if (states && col == state_column)
                for (int a = 0; a < n; ++a) {
                    states[((size_t)k * n + a) * 3] = s.pos[a].x;
                    states[((size_t)k * n + a) * 3 + 1] = s.pos[a].y;
                    states[((size_t)k * n + a) * 3 + 2] = s.pos[a].z;
                }
            s.pos[0].z -= d->dz;
            s.pos[1].z -= d->dz;
        }
        for (size_t q = 0; q < sizeof vs / sizeof vs[0]; ++q) free(*vs[q]);
        for (size_t q = 0; q < sizeof es / sizeof es[0]; ++q) free(*es[q]);
    }
    if (total_steps) *total_steps = steps;
    fctx_free(&c);
    return 0;
}
