// flex.cu — flexible molecules (`flexible on`) on the GPU, FP64.
//
// With a flexible molecule every surface atom whose xyz "fixed" flag is not 1
// moves with the tip (parse.cpp:559-563), held by bonds, angles, dihedrals,
// non-bonded pairs between bonded fragments, a substrate wall and XY tethers
// (simulation.cpp:516-693, interactions.cpp:268-370).  FIRE / SD and the
// integrators then run over all atoms (minimiser.cpp:39-129,
// integrators.cpp:8-111); convergence looks at the tip only.
//
// Layout: one warp per pixel column, the atoms' positions, velocities and
// force accumulators in the warp's shared-memory slice; lane l owns atoms
// l, l + 32, ...  The reference sums each atom's force over its interaction
// list in list order; here every atom has its own list of (interaction kind,
// index, role) entries in that same order (built on the host), and the lane
// owning the atom evaluates the entries one after another, so every per-atom
// sum is formed in the reference's order.  Interactions with several atoms
// are evaluated once per atom that needs them.  FIRE's P = sum_i v_i . F_i
// is summed by one lane in atom order.  Expressions follow the reference's
// operation order (vectors.hpp:99-125); the transcendental functions (exp,
// acos, sin, atan) are CUDA's, so results agree with the reference to
// rounding, not bit for bit.
#include <cmath>
#include <cstring>
#include <vector>

#include "mafm_internal.h"

struct mafm_flex {
    int device = 0;
    mafm_scan_desc d{};
    mafm::ScanParams P{};   // pixel grid, cell, minimiser, tip–dummy terms
    int n_sys = 0;          // atoms incl. dummy (0) and tip (1)
    int n_bonds = 0, n_angles = 0, n_dihedrals = 0, n_pairs = 0, n_xy = 0, n_ts = 0;
    void* dev_block = nullptr;   // every device array, one allocation
    size_t block_bytes = 0;
    struct Dev {
        const double* pos0;         // [n_sys*3] initial positions
        const int* fixed;           // [n_sys]
        const void* ts;             // FlexTS[n_ts]
        const int* bonds;           // [2 n_bonds] system indices
        const double* bond_par;     // [2 n_bonds]
        const int* angles;          // [3 n_angles]
        const double* angle_par;
        const int* dihedrals;       // [4 n_dihedrals]
        const double* dihedral_par;
        const int* pairs;           // [2 n_pairs]
        const void* pair_par;       // FlexPair[n_pairs]
        const double* xy;           // [3 n_xy] atom (as double), x0, y0
        const int* list_begin;      // [n_sys + 1]
        const int* list;            // entries: kind | role << 8, index
    } dv{};
    mafm::RunCounters* ctr = nullptr;
    mafm::RunCounters* host_ctr = nullptr;
    double sub[6] = {0, 0, 0, 0, 0, 0};   // multiplier, ulj, ushift, z0, rc, sig
    double sub_k = 0;
};

namespace mafm {
namespace {

enum : int {
    FT_TS_VDW = 0, FT_TS_COUL, FT_TD_VDW, FT_TD_COUL, FT_TD_HARM, FT_BOND, FT_ANGLE,
    FT_DIHEDRAL, FT_PAIR_VDW, FT_PAIR_COUL, FT_SUBSTRATE, FT_XY
};

struct FlexTS {          // one tip–surface term: LJ / Morse (+ the image shift), or Coulomb
    int atom;            // system index of the surface atom
    int kind;            // MAFM_PAIR_LJ / MAFM_PAIR_MORSE
    double shift[3];
    double p[3];
    double qq;           // Coulomb term when coul
    int coul;
    int pad;
};

struct FlexPair {        // one non-bonded surface pair
    int kind;
    int pad;
    double p[3];
    double qq;
};

struct V3 {
    double x, y, z;
};

__device__ __forceinline__ V3 v3(const double* p) { return V3{p[0], p[1], p[2]}; }
__device__ __forceinline__ V3 sub3(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ V3 add3(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ V3 scal(double s, V3 a) { return V3{s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ V3 mul3(V3 a, double s) { return V3{a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ V3 div3(V3 a, double s) { return V3{a.x / s, a.y / s, a.z / s}; }
__device__ __forceinline__ double dot3(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ double len3(V3 a) { return sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
__device__ __forceinline__ V3 cross3(V3 a, V3 b) {
    return V3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ V3 normalized3(V3 a) {
    const double l = len3(a);
    if (l > 1e-10) return V3{a.x / l, a.y / l, a.z / l};
    return V3{0, 0, 0};
}

// LJ (interactions.cpp:15-27) / Morse (:29-40): force on atom 1 of r_vec = x1 - x2.
__device__ __forceinline__ V3 vdw_force(int kind, const double p[3], V3 r, double& e) {
    if (kind == MAFM_PAIR_LJ) {
        const double r_sqr = r.x * r.x + r.y * r.y + r.z * r.z;
        const double r6 = r_sqr * r_sqr * r_sqr;
        const double ta = p[1] / (r6 * r6);
        const double tb = p[0] / r6;
        e = ta - tb;
        return scal((12 * ta - 6 * tb) / r_sqr, r);
    }
    const double rl = len3(r);
    const double d = exp(-p[1] * (rl - p[2]));
    e = p[0] * (d * d - 2 * d + 1);
    const double f_abs = 2 * p[0] * p[1] * (d * d - d);
    return scal(f_abs / rl, r);
}

// Coulomb (interactions.cpp:42-51).
__device__ __forceinline__ V3 coul_force(double qq, V3 r, double& e) {
    const double rl = len3(r);
    e = qq / rl;
    return scal(qq / (rl * rl * rl), r);
}

struct FlexKernelArgs {
    mafm_flex::Dev dv;
    ScanParams P;
    double sub[6];
    double sub_k;
    int n_sys;
    int col_begin, col_end;
    mafm_point* out;
    int state_column;
    double* states;
    unsigned long long watchdog_ns;
    RunCounters* ctr;
};

__device__ __forceinline__ unsigned long long now_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Force (and, for the tip, energy) on atom `a` at positions pe: the atom's
// entries in list order.  tip_only keeps the tip–surface terms (the output
// evaluation, System::evalTipSurfaceForces, system.cpp:41-51).
__device__ V3 atom_force(const FlexKernelArgs& A, const double* pe, int a, bool tip_only, double& e_sum) {
    const auto& dv = A.dv;
    const FlexTS* ts = static_cast<const FlexTS*>(dv.ts);
    const FlexPair* pp = static_cast<const FlexPair*>(dv.pair_par);
    V3 F{0, 0, 0};
    double E = 0;
    auto P3 = [&](int i) { return v3(pe + 3 * i); };
    for (int q = dv.list_begin[a]; q < dv.list_begin[a + 1]; ++q) {
        const int kr = dv.list[2 * q], idx = dv.list[2 * q + 1];
        const int kind = kr & 0xff, role = kr >> 8;
        if (tip_only && kind != FT_TS_VDW && kind != FT_TS_COUL) continue;
        double e = 0;
        switch (kind) {
            case FT_TS_VDW: {   // LJInteraction(1, j, shift) / Morse
                const FlexTS& t = ts[idx];
                const V3 sh{t.shift[0], t.shift[1], t.shift[2]};
                const V3 f = vdw_force(t.kind, t.p, sub3(P3(1), add3(P3(t.atom), sh)), e);
                F = role == 0 ? add3(F, f) : sub3(F, f);
                break;
            }
            case FT_TS_COUL: {
                const FlexTS& t = ts[idx];
                const V3 f = coul_force(t.qq, sub3(P3(1), P3(t.atom)), e);
                F = role == 0 ? add3(F, f) : sub3(F, f);
                break;
            }
            case FT_TD_VDW: {   // addVDWInteraction(0, 1)
                const V3 f = vdw_force(A.P.td_kind, A.P.td_p, sub3(P3(0), P3(1)), e);
                F = role == 0 ? add3(F, f) : sub3(F, f);
                break;
            }
            case FT_TD_COUL: {
                const V3 f = coul_force(A.P.td_qq, sub3(P3(0), P3(1)), e);
                F = role == 0 ? add3(F, f) : sub3(F, f);
                break;
            }
            case FT_TD_HARM: {  // TipHarmonicInteraction (interactions.cpp:252-266)
                const V3 r_vec = sub3(P3(0), P3(1));
                const double r = sqrt(r_vec.x * r_vec.x + r_vec.y * r_vec.y);
                const double dr = r - A.P.harm_r0;
                e = A.P.harm_k * dr * dr;
                V3 f{0, 0, 0};
                if (r > 1e-10) {
                    const double c = -2 * A.P.harm_k * dr / r;
                    f = V3{c * r_vec.x, c * r_vec.y, 0};
                }
                F = role == 0 ? add3(F, f) : sub3(F, f);
                break;
            }
            case FT_BOND: {     // HarmonicInteraction (interactions.cpp:298-309)
                const int i = dv.bonds[2 * idx], j = dv.bonds[2 * idx + 1];
                const double k = dv.bond_par[2 * idx], r0 = dv.bond_par[2 * idx + 1];
                const V3 r_vec = sub3(P3(i), P3(j));
                const double r = len3(r_vec);
                const double dr = r - r0;
                e = k * (dr * dr);
                const V3 f = scal(-2 * k * dr / r, r_vec);
                F = role == 0 ? add3(F, f) : sub3(F, f);
                break;
            }
            case FT_ANGLE: {    // HarmonicAngleInteraction (interactions.cpp:311-338)
                const int sh = dv.angles[3 * idx], i1 = dv.angles[3 * idx + 1], i2 = dv.angles[3 * idx + 2];
                const double k = dv.angle_par[2 * idx], theta0 = dv.angle_par[2 * idx + 1];
                const V3 r1_vec = sub3(P3(i1), P3(sh));
                const V3 r2_vec = sub3(P3(i2), P3(sh));
                const double r1 = len3(r1_vec), r2 = len3(r2_vec);
                double cos_t = dot3(r1_vec, r2_vec) / (r1 * r2);
                if (cos_t > 1) cos_t = 1;
                else if (cos_t < -1) cos_t = -1;
                const double theta = acos(cos_t);
                const double sin_t = sin(theta);
                const double d_theta = theta - theta0;
                const double f_mul = -2 * k * d_theta / sin_t;
                const V3 f1 = scal(-f_mul / r1, sub3(div3(r2_vec, r2), div3(mul3(r1_vec, cos_t), r1)));
                const V3 f2 = scal(-f_mul / r2, sub3(div3(r1_vec, r1), div3(mul3(r2_vec, cos_t), r2)));
                e = k * (d_theta * d_theta);
                if (role == 1) F = add3(F, f1);
                else if (role == 2) F = add3(F, f2);
                else F = sub3(F, add3(f1, f2));
                break;
            }
            case FT_DIHEDRAL: { // HarmonicDihedralInteraction (interactions.cpp:340-370)
                const int* at = dv.dihedrals + 4 * idx;
                const double k = dv.dihedral_par[2 * idx], sigma0 = dv.dihedral_par[2 * idx + 1];
                const V3 r12 = sub3(P3(at[0]), P3(at[1]));
                const V3 r23v = sub3(P3(at[1]), P3(at[2]));
                const V3 r43 = sub3(P3(at[3]), P3(at[2]));
                const double r23 = len3(r23v);
                const V3 m_vec = cross3(r12, r23v);
                const V3 n_vec = cross3(r43, r23v);
                const double m = len3(m_vec), n = len3(n_vec);
                const double tan_s = dot3(n_vec, r12) * r23 / dot3(m_vec, n_vec);
                const double sigma = atan(tan_s);
                const double d_sigma = sigma - sigma0;
                const double f_mul = 2 * k * d_sigma;
                V3 f;
                if (role == 0) {
                    f = scal(-f_mul * r23 / (m * m), m_vec);
                } else if (role == 1) {
                    f = scal(-f_mul, sub3(scal(dot3(r43, r23v) / (n * n * r23), n_vec),
                                          scal(((r23 * r23) + dot3(r12, r23v)) / (m * m * r23), m_vec)));
                } else if (role == 2) {
                    f = scal(-f_mul, add3(scal(dot3(r12, r23v) / (m * m * r23), m_vec),
                                          scal(((r23 * r23) - dot3(r43, r23v)) / (n * n * r23), n_vec)));
                } else {
                    f = scal(f_mul * r23 / (n * n), n_vec);
                }
                e = k * (d_sigma * d_sigma);
                F = add3(F, f);
                break;
            }
            case FT_PAIR_VDW: {
                const int i = dv.pairs[2 * idx], j = dv.pairs[2 * idx + 1];
                const V3 f = vdw_force(pp[idx].kind, pp[idx].p, sub3(P3(i), P3(j)), e);
                F = role == 0 ? add3(F, f) : sub3(F, f);
                break;
            }
            case FT_PAIR_COUL: {
                const int i = dv.pairs[2 * idx], j = dv.pairs[2 * idx + 1];
                const V3 f = coul_force(pp[idx].qq, sub3(P3(i), P3(j)), e);
                F = role == 0 ? add3(F, f) : sub3(F, f);
                break;
            }
            case FT_SUBSTRATE: { // SubstrateInteraction (interactions.cpp:280-296)
                const double dz = pe[3 * a + 2] - A.sub[3];
                const double sig_z = A.sub[5] / dz;
                const double sig_z2 = sig_z * sig_z;
                const double sig_z4 = sig_z2 * sig_z2;
                const double sig_z10 = sig_z4 * sig_z4 * sig_z2;
                double fterm = 0.0;
                if (dz <= A.sub[4]) {
                    e = A.sub[0] * (2. / 5 * sig_z10 - sig_z4) + A.sub[1] * dz * dz - A.sub[2];
                    fterm += 4 * A.sub[0] / dz * (sig_z10 - sig_z4) + 2 * A.sub[1] * dz;
                }
                F.z += fterm;
                break;
            }
            case FT_XY: {       // XYHarmonicInteraction (interactions.cpp:268-278)
                const double rx = pe[3 * a] - dv.xy[3 * idx + 1];
                const double ry = pe[3 * a + 1] - dv.xy[3 * idx + 2];
                const double r = sqrt(rx * rx + ry * ry);
                e = A.sub_k * r * r;
                if (r > 1e-10) {
                    const double c = -2 * A.sub_k;
                    F.x += c * rx;
                    F.y += c * ry;
                    F.z += 0.0;
                } else {
                    F.x += 0.0;
                    F.y += 0.0;
                    F.z += 0.0;
                }
                break;
            }
            default:
                break;
        }
        E += e;
    }
    e_sum = E;
    return F;
}

// Per-warp shared arrays, 3 doubles per atom each.
struct Slice {
    double* pos;   // positions_
    double* vel;   // velocities_
    double* pe;    // positions of the current evaluation
    double* vk;    // RK4 v_k / midpoint v2
    double* fsum;  // RK4 force sum; forces_ of the last step otherwise
    double* vsum;  // RK4 velocity sum
    double* f;     // forces of the current evaluation
};

__global__ void flex_kernel(FlexKernelArgs A) {
    extern __shared__ __align__(16) double flex_smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int na = A.n_sys;
    const size_t per = (size_t)na * 3;
    double* base = flex_smem + (size_t)warp * 7 * per;
    Slice S{base, base + per, base + 2 * per, base + 3 * per, base + 4 * per, base + 5 * per,
            base + 6 * per};
    __shared__ int s_col[32];
    const ScanParams& P = A.P;
    const unsigned long long t0 = now_ns();
    unsigned long long my_steps = 0, my_evals = 0;
    unsigned err = 0;
    const int* fixed = A.dv.fixed;

    for (;;) {
        if (lane == 0) {
            const unsigned long long t = atomicAdd(&A.ctr->next_work, 1ull);
            s_col[warp] = (t < (unsigned long long)(A.col_end - A.col_begin)) ? A.col_begin + (int)t : -1;
        }
        __syncwarp();
        const int col = s_col[warp];
        __syncwarp();
        if (col < 0) break;
        if (__any_sync(0xffffffffu, now_ns() - t0 > A.watchdog_ns)) {
            err |= ERR_WATCHDOG;
            break;
        }
        // System min_system = system (simulation.cpp:93): the initial state
        for (int a = lane; a < na; a += 32)
            for (int d = 0; d < 3; ++d) {
                S.pos[3 * a + d] = A.dv.pos0[3 * a + d];
                S.vel[3 * a + d] = 0.0;
                S.fsum[3 * a + d] = 0.0;
            }
        __syncwarp();
        // setDummyXY / setDummyZ (system.cpp:139-162, system.hpp:46-49)
        const int i = col / P.ny, j = col % P.ny;
        double x = i * P.dx, y = j * P.dy;
        if (P.tip_pbc) {
            const double* ci = P.cell_inv;
            const double* c = P.cell;
            const double tx = x - P.offset[0], ty = y - P.offset[1], tz = 0 - P.offset[2];
            double cx = ci[0] * tx + ci[1] * ty + ci[2] * tz;
            double cy = ci[3] * tx + ci[4] * ty + ci[5] * tz;
            const double cz = ci[6] * tx + ci[7] * ty + ci[8] * tz;
            cx -= floor(cx);
            cy -= floor(cy);
            x = (c[0] * cx + c[1] * cy + c[2] * cz) + P.offset[0];
            y = (c[3] * cx + c[4] * cy + c[5] * cz) + P.offset[1];
        }
        if (lane == 0) {
            S.pos[0] = x; S.pos[1] = y; S.pos[2] = P.zhigh;
            S.pos[3] = x; S.pos[4] = y; S.pos[5] = P.zhigh - P.tip_dummy_d;
        }
        __syncwarp();
        double e_tip = 0.0;   // System::energies_[1], carried between heights
        for (int k = 0; k < P.nz; ++k) {
            // ---- FIREMinimisation / SDMinimisation (minimiser.cpp:39-129) ----
            double alpha = 0.1, dt = P.dt;
            const double dt_max = 10 * P.dt;
            int n_non_neg = 0;
            int n = 1;
            for (; n < P.maxsteps; ++n) {
                if (((n & 1023) == 0) && __any_sync(0xffffffffu, now_ns() - t0 > A.watchdog_ns)) {
                    err |= ERR_WATCHDOG;
                    break;
                }
                const double prev_tip_e = e_tip;
                double e_new = 0.0;
                // evaluation at positions src into S.f; returns the tip energy
                auto evaluate = [&](const double* src) {
                    double et = 0.0;
                    for (int a = lane; a < na; a += 32) {
                        double e;
                        const V3 F = atom_force(A, src, a, false, e);
                        S.f[3 * a] = F.x; S.f[3 * a + 1] = F.y; S.f[3 * a + 2] = F.z;
                        if (a == 1) et = e;
                    }
                    __syncwarp();
                    my_evals += (lane == 0);
                    return __shfl_sync(0xffffffffu, et, 1);
                };
                if (P.minimiser == MAFM_MIN_SD) {
                    e_new = evaluate(S.pos);
                    for (int a = lane; a < na; a += 32)
                        for (int d = 0; d < 3; ++d) S.fsum[3 * a + d] = S.f[3 * a + d];
                } else if (P.integrator == MAFM_INT_EULER) {
                    e_new = evaluate(S.pos);
                    for (int a = lane; a < na; a += 32) {
                        for (int d = 0; d < 3; ++d) S.fsum[3 * a + d] = S.f[3 * a + d];
                        if (fixed[a] != 1)
                            for (int d = 0; d < 3; ++d) {
                                S.pos[3 * a + d] += dt * S.vel[3 * a + d];
                                S.vel[3 * a + d] += dt * S.f[3 * a + d] / 1.0;
                            }
                    }
                } else if (P.integrator == MAFM_INT_MIDPOINT) {
                    (void)evaluate(S.pos);
                    for (int a = lane; a < na; a += 32)
                        for (int d = 0; d < 3; ++d) {
                            S.pe[3 * a + d] = S.pos[3 * a + d];
                            S.vk[3 * a + d] = S.vel[3 * a + d];
                            if (fixed[a] != 1) {
                                S.pe[3 * a + d] += dt / 2 * S.vel[3 * a + d];
                                S.vk[3 * a + d] += dt / 2 * S.f[3 * a + d] / 1.0;
                            }
                        }
                    __syncwarp();
                    e_new = evaluate(S.pe);
                    for (int a = lane; a < na; a += 32)
                        for (int d = 0; d < 3; ++d) {
                            if (fixed[a] != 1) {
                                S.pos[3 * a + d] += dt * S.vk[3 * a + d];
                                S.vel[3 * a + d] += dt * S.f[3 * a + d] / 1.0;
                            }
                            S.fsum[3 * a + d] = S.f[3 * a + d];
                        }
                } else {   // RK4 (integrators.cpp:56-111)
                    const double e1 = evaluate(S.pos);
                    for (int a = lane; a < na; a += 32)
                        for (int d = 0; d < 3; ++d) {
                            const int q = 3 * a + d;
                            S.fsum[q] = S.f[q];                 // f1
                            S.vsum[q] = S.vel[q];               // v
                            S.pe[q] = S.pos[q];
                            S.vk[q] = S.vel[q];
                            if (fixed[a] != 1) {
                                S.pe[q] += dt / 2 * S.vel[q];   // p2
                                S.vk[q] += dt / 2 * S.f[q] / 1.0;   // v2
                            }
                        }
                    __syncwarp();
                    const double e2 = evaluate(S.pe);
                    for (int a = lane; a < na; a += 32)
                        for (int d = 0; d < 3; ++d) {
                            const int q = 3 * a + d;
                            S.fsum[q] = S.fsum[q] + 2 * S.f[q];
                            S.vsum[q] = S.vsum[q] + 2 * S.vk[q];
                            const double v2 = S.vk[q];
                            S.pe[q] = S.pos[q];
                            S.vk[q] = S.vel[q];
                            if (fixed[a] != 1) {
                                S.pe[q] += dt / 2 * v2;             // p3
                                S.vk[q] += dt / 2 * S.f[q] / 1.0;   // v3
                            }
                        }
                    __syncwarp();
                    const double e3 = evaluate(S.pe);
                    for (int a = lane; a < na; a += 32)
                        for (int d = 0; d < 3; ++d) {
                            const int q = 3 * a + d;
                            S.fsum[q] = S.fsum[q] + 2 * S.f[q];
                            S.vsum[q] = S.vsum[q] + 2 * S.vk[q];
                            const double v3 = S.vk[q];
                            S.pe[q] = S.pos[q];
                            S.vk[q] = S.vel[q];
                            if (fixed[a] != 1) {
                                S.pe[q] += dt * v3;             // p4
                                S.vk[q] += dt * S.f[q] / 1.0;   // v4
                            }
                        }
                    __syncwarp();
                    const double e4 = evaluate(S.pe);
                    for (int a = lane; a < na; a += 32)
                        for (int d = 0; d < 3; ++d) {
                            const int q = 3 * a + d;
                            const double fs = S.fsum[q] + S.f[q];    // f1 + 2f2 + 2f3 + f4
                            const double vs = S.vsum[q] + S.vk[q];   // v + 2v2 + 2v3 + v4
                            if (fixed[a] != 1) {
                                S.pos[q] += dt / 6 * vs;
                                S.vel[q] += dt / 6 * fs / 1.0;
                            }
                            S.fsum[q] = fs / 6;
                        }
                    e_new = (e1 + 2 * e2 + 2 * e3 + e4) / 6;
                }
                __syncwarp();
                e_tip = e_new;
                // checkConvergence on the tip (minimiser.cpp:15-37)
                const V3 ft = v3(S.fsum + 3);
                const double fl = len3(ft);
                const double ediff = e_tip - prev_tip_e;
                bool conv;
                if (P.minterm == MAFM_TERM_E) conv = fabs(ediff) < P.etol;
                else if (P.minterm == MAFM_TERM_F) conv = fl < P.ftol;
                else conv = fabs(ediff) < P.etol && fl < P.ftol;
                if (conv) break;
                if (P.minimiser == MAFM_MIN_SD) {
                    for (int a = lane; a < na; a += 32)
                        if (fixed[a] != 1)
                            for (int d = 0; d < 3; ++d) S.pos[3 * a + d] += P.dt * S.fsum[3 * a + d];
                    __syncwarp();
                    continue;
                }
                // FIRE: P = sum_i v_i . F_i in atom order, then the mixing
                double pw = 0;
                if (lane == 0)
                    for (int a = 0; a < na; ++a) pw += dot3(v3(S.vel + 3 * a), v3(S.fsum + 3 * a));
                pw = __shfl_sync(0xffffffffu, pw, 0);
                __syncwarp();
                for (int a = lane; a < na; a += 32) {
                    if (fixed[a] == 1) continue;
                    // (1 - alpha) v + alpha F.normalized() |v|  (minimiser.cpp:112-113)
                    const V3 v = v3(S.vel + 3 * a);
                    const V3 mixed = add3(scal(1 - alpha, v),
                                          mul3(scal(alpha, normalized3(v3(S.fsum + 3 * a))), len3(v)));
                    S.vel[3 * a] = mixed.x;
                    S.vel[3 * a + 1] = mixed.y;
                    S.vel[3 * a + 2] = mixed.z;
                }
                __syncwarp();
                if (pw < 0) {
                    for (int a = lane; a < na; a += 32)
                        for (int d = 0; d < 3; ++d) S.vel[3 * a + d] = 0.0;
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
                __syncwarp();
            }
            if (err & ERR_WATCHDOG) break;
            // System::getOutput (system.cpp:28-51)
            double et = 0;
            V3 ft{0, 0, 0};
            if (lane == 1) ft = atom_force(A, S.pos, 1, true, et);
            et = __shfl_sync(0xffffffffu, et, 1);
            ft.x = __shfl_sync(0xffffffffu, ft.x, 1);
            ft.y = __shfl_sync(0xffffffffu, ft.y, 1);
            ft.z = __shfl_sync(0xffffffffu, ft.z, 1);
            if (lane == 0) {
                int st = n >= P.maxsteps ? MAFM_PT_MAXSTEPS : 0;
                if (!isfinite(ft.x) || !isfinite(ft.y) || !isfinite(ft.z) || !isfinite(et))
                    st |= MAFM_PT_NONFINITE;
                mafm_point r;
                r.tip[0] = S.pos[3]; r.tip[1] = S.pos[4]; r.tip[2] = S.pos[5];
                r.force[0] = ft.x; r.force[1] = ft.y; r.force[2] = ft.z;
                r.energy = et;
                r.steps = n;
                r.status = st;
                A.out[(size_t)(col - A.col_begin) * P.nz + k] = r;
                my_steps += (unsigned long long)n;
            }
            if (A.states && col == A.state_column)
                for (int a = lane; a < na; a += 32)
                    for (int d = 0; d < 3; ++d) A.states[((size_t)k * na + a) * 3 + d] = S.pos[3 * a + d];
            __syncwarp();
            // System::lowerTip (system.hpp:51-54)
            if (lane == 0) {
                S.pos[2] -= P.dz;
                S.pos[5] -= P.dz;
            }
            __syncwarp();
            // the time limit once per height too: a height usually converges in
            // far fewer than the 1024 steps between the checks above
            if (__any_sync(0xffffffffu, now_ns() - t0 > A.watchdog_ns)) {
                err |= ERR_WATCHDOG;
                break;
            }
        }
        if (err & ERR_WATCHDOG) break;
    }
    for (int off = 16; off > 0; off >>= 1) {
        my_steps += __shfl_xor_sync(0xffffffffu, my_steps, off);
        my_evals += __shfl_xor_sync(0xffffffffu, my_evals, off);
        err |= __shfl_xor_sync(0xffffffffu, err, off);
    }
    if (lane == 0) {
        atomicAdd(&A.ctr->total_steps, my_steps);
        atomicAdd(&A.ctr->force_evals, my_evals);
        if (err) atomicOr(&A.ctr->error_word, err);
    }
}

}  // namespace
}  // namespace mafm

using namespace mafm;

extern "C" int mafm_flex_create(int device, const mafm_scan_desc* d, const mafm_flex_desc* f,
                                mafm_flex** out) {
    return guarded([&] {
        if (!d || !f || !out) fail(MAFM_E_INVALID, "null argument");
        *out = nullptr;
        if (!d->flexible) fail(MAFM_E_INVALID, "the descriptor is not a flexible molecule");
        if (d->rigidgrid || d->use_external_potential)
            fail(MAFM_E_UNSUPPORTED, "flexible molecules run with pair and Coulomb terms only");
        if (d->n_atoms < 1 || !d->pos || !d->type || !d->tip_pair || !f->fixed)
            fail(MAFM_E_INVALID, "flexible descriptor without atoms");
        if (d->n_atoms + 2 > 1024) fail(MAFM_E_RANGE, "flexible molecules of up to 1022 atoms");
        if (device >= 0) cuda_check(cudaSetDevice(device), "cudaSetDevice");
        auto* s = new mafm_flex();
        try {
            cuda_check(cudaGetDevice(&s->device), "cudaGetDevice");
            s->d = *d;
            const int ns = d->n_atoms, na = ns + 2;
            s->n_sys = na;
            // scan parameters shared with the rigid kernels
            ScanParams& P = s->P;
            P.td_kind = d->dummy_pair.kind;
            for (int k = 0; k < 3; ++k) P.td_p[k] = d->dummy_pair.p[k];
            P.td_coul = d->tip_dummy_coulomb && d->dummy_charge != 0 && d->tip_charge != 0;
            P.td_qq = P.td_coul ? d->qbase * d->dummy_charge * d->tip_charge : 0.0;
            P.harm_k = d->harm_k;
            P.harm_r0 = d->harm_r0;
            P.tip_dummy_d = d->tip_dummy_d;
            P.nx = d->nx; P.ny = d->ny; P.nz = d->nz;
            P.tip_pbc = d->tip_pbc;
            P.dx = d->dx; P.dy = d->dy; P.dz = d->dz; P.zhigh = d->zhigh;
            std::memcpy(P.cell, d->cell, sizeof P.cell);
            if (d->tip_pbc) {
                // the inverse in the reference's order (matrices.hpp:117-133)
                const double* m = d->cell;
                const double a = m[0], b = m[1], c = m[2], dd = m[3], e = m[4], ff = m[5], g = m[6],
                             h = m[7], ii = m[8];
                double det = a * (e * ii - ff * h);
                det += b * (ff * g - dd * ii);
                det += c * (dd * h - e * g);
                const double id = 1 / det;
                const double inv[9] = {id * (e * ii - ff * h), -id * (b * ii - c * h), id * (b * ff - c * e),
                                       -id * (dd * ii - ff * g), id * (a * ii - c * g), -id * (a * ff - c * dd),
                                       id * (dd * h - e * g), -id * (a * h - b * g), id * (a * e - b * dd)};
                std::memcpy(P.cell_inv, inv, sizeof inv);
            }
            std::memcpy(P.offset, d->offset, sizeof P.offset);
            P.minimiser = d->minimiser;
            P.integrator = d->integrator;
            P.minterm = d->minterm;
            P.maxsteps = d->maxsteps;
            P.etol = d->etol; P.ftol = d->ftol; P.dt = d->dt;

            // ---- host-side lists, in the reference's interaction order ----
            std::vector<double> pos0(3 * (size_t)na, 0.0);
            for (int a = 0; a < ns; ++a)
                for (int k = 0; k < 3; ++k) pos0[3 * (size_t)(a + 2) + k] = d->pos[3 * (size_t)a + k];
            std::vector<int> fixed(na, 0);
            fixed[0] = 1;
            for (int a = 0; a < ns; ++a) fixed[a + 2] = f->fixed[a];
            std::vector<std::vector<std::pair<int, int>>> lists(na);   // (kind | role << 8, index)
            auto add = [&](int atom, int kind, int role, int idx) { lists[atom].push_back({kind | (role << 8), idx}); };
            std::vector<FlexTS> ts;
            // buildTipSurfaceInteractions (simulation.cpp:297-320)
            const int images = d->vdw_pbc ? 9 : 1;
            for (int im = 0; im < 9; ++im) {
                const int ia = im / 3 - 1, ib = im % 3 - 1;
                if (images == 1 && (ia != 0 || ib != 0)) continue;
                double sh[3] = {0, 0, 0};
                if (d->vdw_pbc)
                    for (int k = 0; k < 3; ++k) sh[k] = ia * d->cell[3 * k] + ib * d->cell[3 * k + 1];
                for (int a = 0; a < ns; ++a) {
                    const mafm_pair& pr = d->tip_pair[d->type[a]];
                    FlexTS t{};
                    t.atom = a + 2;
                    t.kind = pr.kind;
                    for (int k = 0; k < 3; ++k) { t.shift[k] = sh[k]; t.p[k] = pr.p[k]; }
                    ts.push_back(t);
                    add(1, FT_TS_VDW, 0, (int)ts.size() - 1);
                    add(a + 2, FT_TS_VDW, 1, (int)ts.size() - 1);
                    if (!d->vdw_pbc && d->coulomb && d->tip_charge != 0 && d->charge[a] != 0) {
                        FlexTS c{};
                        c.atom = a + 2;
                        c.coul = 1;
                        c.qq = d->qbase * d->tip_charge * d->charge[a];
                        ts.push_back(c);
                        add(1, FT_TS_COUL, 0, (int)ts.size() - 1);
                        add(a + 2, FT_TS_COUL, 1, (int)ts.size() - 1);
                    }
                }
            }
            // buildTipDummyInteractions (simulation.cpp:503-515)
            add(0, FT_TD_VDW, 0, 0);
            add(1, FT_TD_VDW, 1, 0);
            if (P.td_coul) {
                add(0, FT_TD_COUL, 0, 0);
                add(1, FT_TD_COUL, 1, 0);
            }
            add(0, FT_TD_HARM, 0, 0);
            add(1, FT_TD_HARM, 1, 0);
            // buildSurfaceSurfaceInteractions (simulation.cpp:557-693): bonds,
            // angles, dihedrals, then the non-bonded pairs
            std::vector<int> bonds, angles, dihedrals, pairs;
            for (int b = 0; b < f->n_bonds; ++b) {
                const int i = f->bond_atoms[2 * b] + 2, j = f->bond_atoms[2 * b + 1] + 2;
                bonds.insert(bonds.end(), {i, j});
            }
            for (int g = 0; g < f->n_angles; ++g)
                for (int k = 0; k < 3; ++k) angles.push_back(f->angle_atoms[3 * g + k] + 2);
            for (int g = 0; g < f->n_dihedrals; ++g)
                for (int k = 0; k < 4; ++k) dihedrals.push_back(f->dihedral_atoms[4 * g + k] + 2);
            std::vector<FlexPair> pp;
            for (int q = 0; q < f->n_pairs; ++q) {
                pairs.insert(pairs.end(), {f->pair_atoms[2 * q] + 2, f->pair_atoms[2 * q + 1] + 2});
                FlexPair x{};
                x.kind = f->pair_vdw[q].kind;
                for (int k = 0; k < 3; ++k) x.p[k] = f->pair_vdw[q].p[k];
                x.qq = f->pair_qq ? f->pair_qq[q] : 0.0;
                pp.push_back(x);
            }
            for (int a : bonds)
                if (a < 2 || a >= na) fail(MAFM_E_INVALID, "bond atom out of range");
            for (int a : angles)
                if (a < 2 || a >= na) fail(MAFM_E_INVALID, "angle atom out of range");
            for (int a : dihedrals)
                if (a < 2 || a >= na) fail(MAFM_E_INVALID, "dihedral atom out of range");
            for (int a : pairs)
                if (a < 2 || a >= na) fail(MAFM_E_INVALID, "pair atom out of range");
            for (int b = 0; b < f->n_bonds; ++b) {
                add(bonds[2 * b], FT_BOND, 0, b);
                add(bonds[2 * b + 1], FT_BOND, 1, b);
            }
            for (int g = 0; g < f->n_angles; ++g) {
                add(angles[3 * g + 1], FT_ANGLE, 1, g);
                add(angles[3 * g + 2], FT_ANGLE, 2, g);
                add(angles[3 * g], FT_ANGLE, 0, g);
            }
            for (int g = 0; g < f->n_dihedrals; ++g)
                for (int r = 0; r < 4; ++r) add(dihedrals[4 * g + r], FT_DIHEDRAL, r, g);
            for (int q = 0; q < f->n_pairs; ++q) {
                add(pairs[2 * q], FT_PAIR_VDW, 0, q);
                add(pairs[2 * q + 1], FT_PAIR_VDW, 1, q);
                if (pp[q].qq != 0) {
                    add(pairs[2 * q], FT_PAIR_COUL, 0, q);
                    add(pairs[2 * q + 1], FT_PAIR_COUL, 1, q);
                }
            }
            // buildSubstrateInteractions (simulation.cpp:516-528)
            const double eps = f->substrate[0], sig = f->substrate[1], lambda = f->substrate[2],
                         rc = f->substrate[3];
            const double kPi = 3.14159265358979323846;
            s->sub[0] = 2 * kPi * eps * pow(sig / lambda, 2);
            s->sub[1] = (kPi / (lambda * lambda)) * 4 * eps * (pow(sig / rc, 12) - pow(sig / rc, 6));
            s->sub[2] = s->sub[0] * ((12. / 5) * pow(sig / rc, 10) - 3 * pow(sig / rc, 4));
            s->sub[3] = -sig;
            s->sub[4] = rc;
            s->sub[5] = sig;
            s->sub_k = f->substrate[4];
            std::vector<double> xy;
            for (int a = 2; a < na; ++a) {
                add(a, FT_SUBSTRATE, 0, 0);
                if (fixed[a] == 2) {
                    xy.insert(xy.end(), {(double)a, pos0[3 * (size_t)a], pos0[3 * (size_t)a + 1]});
                    add(a, FT_XY, 0, (int)xy.size() / 3 - 1);
                }
            }
            // the (kind, index) entries of every atom, atom after atom
            std::vector<int> begin(na + 1, 0), list;
            for (int a = 0; a < na; ++a) {
                begin[a] = (int)list.size() / 2;
                for (const auto& e : lists[a]) list.insert(list.end(), {e.first, e.second});
            }
            begin[na] = (int)list.size() / 2;
            s->n_ts = (int)ts.size();
            s->n_bonds = f->n_bonds; s->n_angles = f->n_angles; s->n_dihedrals = f->n_dihedrals;
            s->n_pairs = f->n_pairs; s->n_xy = (int)xy.size() / 3;

            // one device block for every array (256-byte aligned pieces)
            struct Piece { const void* src; size_t bytes; size_t off; };
            std::vector<Piece> pieces;
            size_t off = 0;
            auto piece = [&](const void* src, size_t bytes) {
                pieces.push_back({src, bytes, off});
                const size_t at = off;
                off += (bytes + 255) & ~(size_t)255;
                return at;
            };
            const size_t o_pos = piece(pos0.data(), pos0.size() * sizeof(double));
            const size_t o_fixed = piece(fixed.data(), fixed.size() * sizeof(int));
            const size_t o_ts = piece(ts.data(), ts.size() * sizeof(FlexTS));
            const size_t o_b = piece(bonds.data(), bonds.size() * sizeof(int));
            const size_t o_bp = piece(f->bond_param, (size_t)f->n_bonds * 2 * sizeof(double));
            const size_t o_a = piece(angles.data(), angles.size() * sizeof(int));
            const size_t o_ap = piece(f->angle_param, (size_t)f->n_angles * 2 * sizeof(double));
            const size_t o_dh = piece(dihedrals.data(), dihedrals.size() * sizeof(int));
            const size_t o_dp = piece(f->dihedral_param, (size_t)f->n_dihedrals * 2 * sizeof(double));
            const size_t o_pr = piece(pairs.data(), pairs.size() * sizeof(int));
            const size_t o_pp = piece(pp.data(), pp.size() * sizeof(FlexPair));
            const size_t o_xy = piece(xy.data(), xy.size() * sizeof(double));
            const size_t o_lb = piece(begin.data(), begin.size() * sizeof(int));
            const size_t o_l = piece(list.data(), list.size() * sizeof(int));
            s->block_bytes = std::max<size_t>(off, 256);
            cuda_check(cudaMalloc(&s->dev_block, s->block_bytes), "cudaMalloc");
            char* dev = static_cast<char*>(s->dev_block);
            for (const Piece& p : pieces)
                if (p.bytes)
                    cuda_check(cudaMemcpy(dev + p.off, p.src, p.bytes, cudaMemcpyHostToDevice), "upload");
            s->dv.pos0 = reinterpret_cast<const double*>(dev + o_pos);
            s->dv.fixed = reinterpret_cast<const int*>(dev + o_fixed);
            s->dv.ts = dev + o_ts;
            s->dv.bonds = reinterpret_cast<const int*>(dev + o_b);
            s->dv.bond_par = reinterpret_cast<const double*>(dev + o_bp);
            s->dv.angles = reinterpret_cast<const int*>(dev + o_a);
            s->dv.angle_par = reinterpret_cast<const double*>(dev + o_ap);
            s->dv.dihedrals = reinterpret_cast<const int*>(dev + o_dh);
            s->dv.dihedral_par = reinterpret_cast<const double*>(dev + o_dp);
            s->dv.pairs = reinterpret_cast<const int*>(dev + o_pr);
            s->dv.pair_par = dev + o_pp;
            s->dv.xy = reinterpret_cast<const double*>(dev + o_xy);
            s->dv.list_begin = reinterpret_cast<const int*>(dev + o_lb);
            s->dv.list = reinterpret_cast<const int*>(dev + o_l);
            cuda_check(cudaMalloc(&s->ctr, sizeof(RunCounters)), "cudaMalloc");
            cuda_check(cudaMallocHost(&s->host_ctr, sizeof(RunCounters)), "cudaMallocHost");
        } catch (...) {
            if (s->dev_block) cudaFree(s->dev_block);
            if (s->ctr) cudaFree(s->ctr);
            if (s->host_ctr) cudaFreeHost(s->host_ctr);
            delete s;
            throw;
        }
        *out = s;
    });
}

extern "C" int mafm_flex_destroy(mafm_flex* s) {
    if (s) {
        cudaSetDevice(s->device);
        if (s->dev_block) cudaFree(s->dev_block);
        if (s->ctr) cudaFree(s->ctr);
        if (s->host_ctr) cudaFreeHost(s->host_ctr);
        delete s;
    }
    return MAFM_OK;
}

extern "C" int mafm_flex_run(mafm_flex* s, int32_t col_begin, int32_t col_end, mafm_point* out,
                             mafm_run_stats* stats, int32_t state_column, double* states,
                             void* stream) {
    return guarded([&] {
        if (!s || !out) fail(MAFM_E_INVALID, "null argument");
        cuda_check(cudaSetDevice(s->device), "cudaSetDevice");
        const int n_cols = s->d.nx * s->d.ny;
        if (col_begin == 0 && col_end == 0) col_end = n_cols;
        if (col_begin < 0 || col_end > n_cols || col_begin > col_end)
            fail(MAFM_E_INVALID, "column range [%d, %d) outside [0, %d)", col_begin, col_end, n_cols);
        const size_t n_pts = (size_t)(col_end - col_begin) * s->d.nz;
        cudaStream_t st = (cudaStream_t)stream;
        // outputs: device or pinned memory directly, pageable through a copy
        mafm_point* dout = out;
        double* dstates = states;
        void* tmp_out = nullptr;
        void* tmp_states = nullptr;
        const size_t states_bytes = (size_t)s->d.nz * s->n_sys * 3 * sizeof(double);
        auto device_view = [](void* p) -> void* {
            cudaPointerAttributes a{};
            if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
                cudaGetLastError();
                return nullptr;
            }
            if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) return p;
            if (a.type == cudaMemoryTypeHost) return a.devicePointer;
            return nullptr;
        };
        struct Frees {
            void* a = nullptr;
            void* b = nullptr;
            ~Frees() {
                if (a) cudaFree(a);
                if (b) cudaFree(b);
            }
        } frees;
        if (void* v = device_view(out)) {
            dout = static_cast<mafm_point*>(v);
        } else {
            cuda_check(cudaMalloc(&tmp_out, n_pts * sizeof(mafm_point)), "cudaMalloc");
            frees.a = tmp_out;
            dout = static_cast<mafm_point*>(tmp_out);
        }
        if (states) {
            if (void* v = device_view(states)) {
                dstates = static_cast<double*>(v);
            } else {
                cuda_check(cudaMalloc(&tmp_states, states_bytes), "cudaMalloc");
                frees.b = tmp_states;
                dstates = static_cast<double*>(tmp_states);
                cuda_check(cudaMemsetAsync(tmp_states, 0, states_bytes, st), "memset states");
            }
        }
        FlexKernelArgs A{};
        A.dv = s->dv;
        A.P = s->P;
        std::memcpy(A.sub, s->sub, sizeof A.sub);
        A.sub_k = s->sub_k;
        A.n_sys = s->n_sys;
        A.col_begin = col_begin;
        A.col_end = col_end;
        A.out = dout;
        A.state_column = state_column;
        A.states = dstates;
        A.watchdog_ns = watchdog_ns_from_env();
        A.ctr = s->ctr;
        cuda_check(cudaMemsetAsync(s->ctr, 0, sizeof(RunCounters), st), "reset counters");
        const size_t per_warp = (size_t)7 * s->n_sys * 3 * sizeof(double);
        int warps = (int)std::min<size_t>(4, std::max<size_t>(1, (200u * 1024u) / per_warp));
        const size_t smem = per_warp * warps;
        cuda_check(cudaFuncSetAttribute(flex_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                   "flex smem");
        const int cols = col_end - col_begin;
        int blocks = (cols + warps - 1) / warps;
        blocks = std::max(1, std::min(blocks, sm_count() * 8));
        if (cols > 0) {
            flex_kernel<<<blocks, 32 * warps, smem, st>>>(A);
            cuda_check(cudaGetLastError(), "flex launch");
        }
        if (tmp_out)
            cuda_check(cudaMemcpyAsync(out, tmp_out, n_pts * sizeof(mafm_point), cudaMemcpyDeviceToHost, st),
                       "copy points");
        if (tmp_states)
            cuda_check(cudaMemcpyAsync(states, tmp_states, states_bytes, cudaMemcpyDeviceToHost, st),
                       "copy states");
        cuda_check(cudaMemcpyAsync(s->host_ctr, s->ctr, sizeof(RunCounters), cudaMemcpyDeviceToHost, st),
                   "counters");
        cuda_check(cudaStreamSynchronize(st), "flex relax");
        const RunCounters c = *s->host_ctr;
        if (stats) {
            *stats = mafm_run_stats{};
            stats->total_steps = c.total_steps;
            stats->force_evals = c.force_evals;
            stats->error_word = c.error_word;
        }
        if (c.error_word & ERR_WATCHDOG)
            fail(MAFM_E_DEVICE, "the flexible relaxation exceeded its time limit (MAFM_WATCHDOG_S)");
    });
}
