// adjoint.cu — gradients of a loss on the Fz image through the relaxation.
//
// The reference has no derivatives; this is the differentiation the scan's
// users need for fitting (positions, pair parameters, charges to a measured
// image).  Per relaxed point p the tip sits at x_p with the total force
//   F(x) = F_ts(x; theta) + F_td(x; dummy) = 0        (FIRE's minimum)
// and the recorded output is Fz_p = F_ts,z(x_p; theta) (system.cpp:41-51).
// Implicit differentiation at the minimum (no unrolling of FIRE):
//   dx_p/dtheta = -J^-1 dF_ts/dtheta,   J = dF/dx (3x3, symmetric),
//   dL/dtheta = sum_p mu_p . dF_ts(x_p)/dtheta,
//   mu_p = w_p (e_z - lambda_p),  J lambda_p = (dF_ts,z/dx)^T,
// with w_p = dL/dFz_p.  The relaxed positions of every z-slice are the
// checkpoints (the forward pass's point records), so the reverse sweep reads
// them instead of replaying FIRE; at a minimum the start of a slice (the
// previous slice's position) does not enter.
//
// One thread per point.  MAFM_FP64: every step in FP64.  MAFM_FP32C: the
// per-term work in FP32 with compensated sums, the per-point 3x3 part in FP64.
// Per-term contributions are reduced across the warp with shuffles and
// accumulated in shared memory per block when the terms fit, in global memory
// otherwise.
#include "mafm_internal.h"

namespace mafm {
namespace {

struct V3 {
    double x, y, z;
};

// s(r) and s'(r)/r of a pair force f = s(r) r_vec (r_vec = tip - atom).
__device__ __forceinline__ void pair_s(int kind, double p0, double p1, double p2, double r2,
                                       double& s, double& dsr) {
    if (kind == MAFM_PAIR_LJ) {
        const double ir2 = 1.0 / r2;
        const double ir6 = ir2 * ir2 * ir2;
        const double a12 = p1 * ir6 * ir6, a6 = p0 * ir6;
        s = (12 * a12 - 6 * a6) * ir2;
        dsr = (-168 * a12 + 48 * a6) * ir2 * ir2;
    } else {
        const double r = sqrt(r2);
        const double d = exp(-p1 * (r - p2));
        const double g = 2 * p0 * p1 * (d * d - d);       // |f|
        const double dg = 2 * p0 * p1 * (2 * d - 1) * (-p1 * d);   // d|f|/dr
        s = g / r;
        dsr = (dg / r - g / r2) / r;
    }
}

// d f / d(p0, p1, p2) of a vdW term, as multiples of r_vec.
__device__ __forceinline__ void pair_dparam(int kind, double p0, double p1, double p2, double r2,
                                            double q[3]) {
    if (kind == MAFM_PAIR_LJ) {
        const double ir2 = 1.0 / r2;
        const double ir6 = ir2 * ir2 * ir2;
        q[0] = -6 * ir6 * ir2;          // d s / d es6
        q[1] = 12 * ir6 * ir6 * ir2;    // d s / d es12
        q[2] = 0;
    } else {
        const double r = sqrt(r2);
        const double x = r - p2;
        const double d = exp(-p1 * x);
        const double dd = d * d - d;
        q[0] = 2 * p1 * dd / r;                                           // d s / d De
        q[1] = (2 * p0 * dd + 2 * p0 * p1 * (2 * d - 1) * (-x * d)) / r;  // d s / d a
        q[2] = 2 * p0 * p1 * (2 * d - 1) * (p1 * d) / r;                  // d s / d re
    }
}

// Accumulate s I + dsr r r^T into a symmetric 3x3 (xx, yy, zz, xy, xz, yz).
__device__ __forceinline__ void add_jac(double J[6], double s, double dsr, V3 r) {
    J[0] += s + dsr * r.x * r.x;
    J[1] += s + dsr * r.y * r.y;
    J[2] += s + dsr * r.z * r.z;
    J[3] += dsr * r.x * r.y;
    J[4] += dsr * r.x * r.z;
    J[5] += dsr * r.y * r.z;
}

// Jacobian of a periodic trilinear grid lookup (the external field).
__device__ void es_jacobian(const GridView& g, V3 pos, double Jg[9]) {
    const double qx = pos.x - g.origin[0], qy = pos.y - g.origin[1], qz = pos.z - g.origin[2];
    double pb[3];
    for (int a = 0; a < 3; ++a) pb[a] = g.inv[3 * a] * qx + g.inv[3 * a + 1] * qy + g.inv[3 * a + 2] * qz;
    int gp[3];
    double d[3];
    for (int a = 0; a < 3; ++a) {
        gp[a] = (int)floor(pb[a]);
        d[a] = pb[a] - gp[a];
    }
    double dFd[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};   // dF_comp / d d_axis
    for (int c = 0; c < 8; ++c) {
        int idx[3] = {gp[0] + (c >> 2), gp[1] + ((c >> 1) & 1), gp[2] + (c & 1)};
        for (int a = 0; a < 3; ++a) {
            idx[a] %= g.n[a];
            if (idx[a] < 0) idx[a] += g.n[a];
        }
        const Node64 v = g.g64[((long long)idx[0] * g.n[1] + idx[1]) * g.n[2] + idx[2]];
        const double w[3] = {(c >> 2) ? d[0] : 1 - d[0], ((c >> 1) & 1) ? d[1] : 1 - d[1],
                             (c & 1) ? d[2] : 1 - d[2]};
        const double sgn[3] = {(c >> 2) ? 1.0 : -1.0, ((c >> 1) & 1) ? 1.0 : -1.0, (c & 1) ? 1.0 : -1.0};
        const double dw[3] = {sgn[0] * w[1] * w[2], sgn[1] * w[0] * w[2], sgn[2] * w[0] * w[1]};
        const double F[3] = {v.x, v.y, v.z};
        for (int m = 0; m < 3; ++m)
            for (int a = 0; a < 3; ++a) dFd[m][a] += F[m] * dw[a];
    }
    for (int m = 0; m < 3; ++m)
        for (int j = 0; j < 3; ++j)
            Jg[3 * m + j] = dFd[m][0] * g.inv[j] + dFd[m][1] * g.inv[3 + j] + dFd[m][2] * g.inv[6 + j];
}

__device__ __forceinline__ double warp_sum(double v) {
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}

__device__ __forceinline__ float warp_sum(float v) {
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}

constexpr int kG = 7;   // per-term gradient values: position (3), p0..p2 (3), charge (1)

// mu of one relaxed point (index idx, tip x, w = dL/dFz) from the summed
// tip–surface Jacobian Jts (xx, yy, zz, xy, xz, yz): adds the external field,
// the tip–dummy terms and the XY spring, solves J^T lambda = (row z of
// dF_ts/dx) and returns mu = w (e_z - lambda); false when J is singular.
__device__ bool point_mu(const ScanParams& p, long long idx, V3 x, double wp, const double Jts[6],
                         V3& mu) {
    const long long col = idx / p.nz;
    const int k = (int)(idx % p.nz);
    const int i = (int)(col / p.ny), j = (int)(col % p.ny);
    // dummy position (System::setDummyXY / setDummyZ / lowerTip)
    double dxp = i * p.dx, dyp = j * p.dy;
    if (p.tip_pbc && p.ts_mode != 2) {
        const double* ci = p.cell_inv;
        const double* c = p.cell;
        const double tx = dxp - p.offset[0], ty = dyp - p.offset[1], tz = 0 - p.offset[2];
        double cx = ci[0] * tx + ci[1] * ty + ci[2] * tz;
        double cy = ci[3] * tx + ci[4] * ty + ci[5] * tz;
        const double cz = ci[6] * tx + ci[7] * ty + ci[8] * tz;
        cx -= floor(cx);
        cy -= floor(cy);
        dxp = (c[0] * cx + c[1] * cy + c[2] * cz) + p.offset[0];
        dyp = (c[3] * cx + c[4] * cy + c[5] * cz) + p.offset[1];
    }
    double dzp = p.zhigh;
    for (int s = 0; s < k; ++s) dzp -= p.dz;
    double J[9] = {Jts[0], Jts[3], Jts[4], Jts[3], Jts[1], Jts[5], Jts[4], Jts[5], Jts[2]};
    if (p.ts_mode == 1) {
        double Jg[9];
        es_jacobian(p.es, x, Jg);
        for (int m = 0; m < 9; ++m) J[m] += Jg[m];
    }
    const double cz[3] = {J[6], J[7], J[8]};   // row z of dF_ts/dx
    // tip–dummy coupling: F_td = s(|x-d|)(x-d) for the vdW / Coulomb terms
    {
        const V3 r = {x.x - dxp, x.y - dyp, x.z - dzp};
        const double r2 = r.x * r.x + r.y * r.y + r.z * r.z;
        double s, dsr;
        pair_s(p.td_kind, p.td_p[0], p.td_p[1], p.td_p[2], r2, s, dsr);
        if (p.td_coul) {
            const double ir = 1.0 / sqrt(r2);
            const double ir3 = ir * ir * ir;
            s += p.td_qq * ir3;
            dsr += -3 * p.td_qq * ir3 * ir * ir;
        }
        double Jd[6] = {0, 0, 0, 0, 0, 0};
        add_jac(Jd, s, dsr, r);
        J[0] += Jd[0]; J[4] += Jd[1]; J[8] += Jd[2];
        J[1] += Jd[3]; J[3] += Jd[3];
        J[2] += Jd[4]; J[6] += Jd[4];
        J[5] += Jd[5]; J[7] += Jd[5];
        // XY spring: F_xy = -2k (1 - r0/rho) u, u = (x-d)_xy
        const double ux = r.x, uy = r.y;
        const double rho = sqrt(ux * ux + uy * uy);
        const double k2 = 2 * p.harm_k;
        if (p.harm_r0 == 0.0 || rho <= 1e-10) {
            J[0] -= k2;
            J[4] -= k2;
        } else {
            const double f = 1 - p.harm_r0 / rho;
            const double g = p.harm_r0 / (rho * rho * rho);
            J[0] -= k2 * (f + g * ux * ux);
            J[4] -= k2 * (f + g * uy * uy);
            J[1] -= k2 * g * ux * uy;
            J[3] -= k2 * g * ux * uy;
        }
    }
    // solve J^T lambda = cz (Cramer / adjugate)
    const double a = J[0], b = J[1], c = J[2], d = J[3], e = J[4], f = J[5], g = J[6], h = J[7],
                 ii = J[8];
    const double det = a * (e * ii - f * h) - b * (d * ii - f * g) + c * (d * h - e * g);
    if (!isfinite(det) || fabs(det) < 1e-300) return false;
    // inverse of J^T = (J^-1)^T
    const double inv[9] = {(e * ii - f * h) / det, -(b * ii - c * h) / det, (b * f - c * e) / det,
                           -(d * ii - f * g) / det, (a * ii - c * g) / det, -(a * f - c * d) / det,
                           (d * h - e * g) / det, -(a * h - b * g) / det, (a * e - b * d) / det};
    // lambda = (J^T)^-1 cz = (J^-1)^T cz
    const V3 lam = {inv[0] * cz[0] + inv[3] * cz[1] + inv[6] * cz[2],
                    inv[1] * cz[0] + inv[4] * cz[1] + inv[7] * cz[2],
                    inv[2] * cz[0] + inv[5] * cz[1] + inv[8] * cz[2]};
    mu = {-wp * lam.x, -wp * lam.y, wp * (1.0 - lam.z)};
    return true;
}

__global__ void __launch_bounds__(256) adjoint_kernel(const ScanParams p, const mafm_point* pts,
                                                      const double* w, long long n_points,
                                                      double qbase_qtip, double* gterm,
                                                      int use_smem, RunCounters* ctr) {
    extern __shared__ __align__(16) double sacc[];
    const int n = p.n_terms_direct;
    if (use_smem) {
        for (int i = threadIdx.x; i < n * kG; i += blockDim.x) sacc[i] = 0.0;
        __syncthreads();
    }
    double* acc = use_smem ? sacc : gterm;
    const int lane = threadIdx.x & 31;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long first = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    // every warp runs the same number of rounds so that shuffles see all lanes
    const long long rounds = (n_points + stride - 1) / stride;
    unsigned err = 0;
    for (long long rd = 0; rd < rounds; ++rd) {
        const long long idx = first + rd * stride;
        const bool live = idx < n_points;
        V3 x = {0, 0, 0}, mu = {0, 0, 0};
        if (live) {
            const mafm_point pt = pts[idx];
            x = {pt.tip[0], pt.tip[1], pt.tip[2]};
            double Jts[6] = {0, 0, 0, 0, 0, 0};
            for (int t = 0; t < n; ++t) {
                const AtomRec64 a = p.atoms64[t];
                const V3 r = {x.x - a.x, x.y - a.y, x.z - a.z};
                const double r2 = r.x * r.x + r.y * r.y + r.z * r.z;
                double s, dsr;
                pair_s(a.kind, a.p0, a.p1, a.p2, r2, s, dsr);
                if (a.coul) {
                    const double ir = 1.0 / sqrt(r2);
                    const double ir3 = ir * ir * ir;
                    s += a.qq * ir3;
                    dsr += -3 * a.qq * ir3 * ir * ir;
                }
                add_jac(Jts, s, dsr, r);
            }
            if (!point_mu(p, idx, x, w[idx], Jts, mu)) {
                err |= MAFM_PT_NONFINITE;
                mu = {0, 0, 0};
            }
        }
        // per-term contributions: d/d(atom position) = -J_t mu, d/dparams = mu . df/dparams
        for (int t = 0; t < n; ++t) {
            double gv[kG] = {0, 0, 0, 0, 0, 0, 0};
            if (live) {
                const AtomRec64 a = p.atoms64[t];
                const V3 r = {x.x - a.x, x.y - a.y, x.z - a.z};
                const double r2 = r.x * r.x + r.y * r.y + r.z * r.z;
                double s, dsr;
                pair_s(a.kind, a.p0, a.p1, a.p2, r2, s, dsr);
                double ir3 = 0;
                if (a.coul) {
                    const double ir = 1.0 / sqrt(r2);
                    ir3 = ir * ir * ir;
                    s += a.qq * ir3;
                    dsr += -3 * a.qq * ir3 * ir * ir;
                }
                const double rm = r.x * mu.x + r.y * mu.y + r.z * mu.z;
                gv[0] = -(s * mu.x + dsr * r.x * rm);
                gv[1] = -(s * mu.y + dsr * r.y * rm);
                gv[2] = -(s * mu.z + dsr * r.z * rm);
                double q[3];
                pair_dparam(a.kind, a.p0, a.p1, a.p2, r2, q);
                gv[3] = q[0] * rm;
                gv[4] = q[1] * rm;
                gv[5] = q[2] * rm;
                gv[6] = a.coul ? qbase_qtip * ir3 * rm : 0.0;
            }
#pragma unroll
            for (int m = 0; m < kG; ++m) {
                const double v = warp_sum(gv[m]);
                if (lane == 0 && v != 0.0) atomicAdd(acc + (size_t)t * kG + m, v);
            }
        }
    }
    if (use_smem) {
        __syncthreads();
        for (int i = threadIdx.x; i < n * kG; i += blockDim.x)
            if (sacc[i] != 0.0) atomicAdd(gterm + i, sacc[i]);
    }
    if (err) atomicOr(&ctr->error_word, err);
}

// ---- FP32C adjoint ----------------------------------------------------------
// The same quantities with the per-term work in FP32 (FP64 costs 64x FP32 on
// this GPU): s(r), s'(r)/r and the parameter derivatives from rsqrt.approx and
// __expf, the 6 entries of the summed Jacobian with Kahan compensation, the
// per-point part (field, tip–dummy, spring, 3x3 solve) in FP64 (point_mu),
// and per-term gradients summed over the warp in FP32, then in FP64.

__device__ __forceinline__ void pair_s32(bool lj, float p0, float p1, float p2, float r2, float ir,
                                         float& s, float& dsr) {
    const float ir2 = ir * ir;
    if (lj) {
        const float ir6 = ir2 * ir2 * ir2;
        const float a12 = p1 * ir6 * ir6, a6 = p0 * ir6;
        s = (12.f * a12 - 6.f * a6) * ir2;
        dsr = (-168.f * a12 + 48.f * a6) * ir2 * ir2;
    } else {
        const float r = r2 * ir;
        const float d = __expf(-p1 * (r - p2));
        const float g = 2.f * p0 * p1 * (d * d - d);
        const float dg = 2.f * p0 * p1 * (2.f * d - 1.f) * (-p1 * d);
        s = g * ir;
        dsr = (dg * ir - g * ir2) * ir;
    }
}

__device__ __forceinline__ void pair_dparam32(bool lj, float p0, float p1, float p2, float r2,
                                              float ir, float q[3]) {
    const float ir2 = ir * ir;
    if (lj) {
        const float ir6 = ir2 * ir2 * ir2;
        q[0] = -6.f * ir6 * ir2;
        q[1] = 12.f * ir6 * ir6 * ir2;
        q[2] = 0.f;
    } else {
        const float r = r2 * ir;
        const float x = r - p2;
        const float d = __expf(-p1 * x);
        const float dd = d * d - d;
        q[0] = 2.f * p1 * dd * ir;
        q[1] = (2.f * p0 * dd + 2.f * p0 * p1 * (2.f * d - 1.f) * (-x * d)) * ir;
        q[2] = 2.f * p0 * p1 * (2.f * d - 1.f) * (p1 * d) * ir;
    }
}

__device__ __forceinline__ void kahan_add(float& sum, float& c, float v) {
    const float y = v - c;
    const float t = sum + y;
    c = (t - sum) - y;
    sum = t;
}

__global__ void __launch_bounds__(256) adjoint32_kernel(const ScanParams p, const mafm_point* pts,
                                                        const double* w, long long n_points,
                                                        float qbase_qtip, const int* index32,
                                                        double* gterm, int use_smem,
                                                        RunCounters* ctr) {
    extern __shared__ __align__(16) double sacc[];
    const int n = p.n_terms_direct;
    if (use_smem) {
        for (int i = threadIdx.x; i < n * kG; i += blockDim.x) sacc[i] = 0.0;
        __syncthreads();
    }
    double* acc = use_smem ? sacc : gterm;
    const int lane = threadIdx.x & 31;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long first = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long rounds = (n_points + stride - 1) / stride;
    unsigned err = 0;
    for (long long rd = 0; rd < rounds; ++rd) {
        const long long idx = first + rd * stride;
        const bool live = idx < n_points;
        float xf = 0.f, yf = 0.f, zf = 0.f, mx = 0.f, my = 0.f, mz = 0.f;
        if (live) {
            const mafm_point pt = pts[idx];
            const V3 x = {pt.tip[0], pt.tip[1], pt.tip[2]};
            xf = (float)x.x;
            yf = (float)x.y;
            zf = (float)x.z;
            float js[6] = {0, 0, 0, 0, 0, 0}, jc[6] = {0, 0, 0, 0, 0, 0};
            for (int t = 0; t < n; ++t) {
                const AtomRec32 a = p.atoms32[t];
                const float rx = xf - a.a.x, ry = yf - a.a.y, rz = zf - a.a.z;
                const float r2 = rx * rx + ry * ry + rz * rz;
                const float ir = rsqrtf(r2);
                float s, dsr;
                pair_s32(__float_as_int(a.b.w) == MAFM_PAIR_LJ, a.b.x, a.b.y, a.b.z, r2, ir, s, dsr);
                if (a.a.w != 0.f) {
                    const float ir3 = ir * ir * ir;
                    s += a.a.w * ir3;
                    dsr += -3.f * a.a.w * ir3 * ir * ir;
                }
                kahan_add(js[0], jc[0], s + dsr * rx * rx);
                kahan_add(js[1], jc[1], s + dsr * ry * ry);
                kahan_add(js[2], jc[2], s + dsr * rz * rz);
                kahan_add(js[3], jc[3], dsr * rx * ry);
                kahan_add(js[4], jc[4], dsr * rx * rz);
                kahan_add(js[5], jc[5], dsr * ry * rz);
            }
            double Jts[6];
            for (int m = 0; m < 6; ++m) Jts[m] = (double)js[m] - (double)jc[m];
            V3 mu;
            if (point_mu(p, idx, x, w[idx], Jts, mu)) {
                mx = (float)mu.x;
                my = (float)mu.y;
                mz = (float)mu.z;
            } else {
                err |= MAFM_PT_NONFINITE;
            }
        }
        for (int t = 0; t < n; ++t) {
            float gv[kG] = {0, 0, 0, 0, 0, 0, 0};
            const AtomRec32 a = p.atoms32[t];
            if (live) {
                const float rx = xf - a.a.x, ry = yf - a.a.y, rz = zf - a.a.z;
                const float r2 = rx * rx + ry * ry + rz * rz;
                const float ir = rsqrtf(r2);
                const bool lj = __float_as_int(a.b.w) == MAFM_PAIR_LJ;
                float s, dsr;
                pair_s32(lj, a.b.x, a.b.y, a.b.z, r2, ir, s, dsr);
                float ir3 = 0.f;
                if (a.a.w != 0.f) {
                    ir3 = ir * ir * ir;
                    s += a.a.w * ir3;
                    dsr += -3.f * a.a.w * ir3 * ir * ir;
                }
                const float rm = rx * mx + ry * my + rz * mz;
                gv[0] = -(s * mx + dsr * rx * rm);
                gv[1] = -(s * my + dsr * ry * rm);
                gv[2] = -(s * mz + dsr * rz * rm);
                float q[3];
                pair_dparam32(lj, a.b.x, a.b.y, a.b.z, r2, ir, q);
                gv[3] = q[0] * rm;
                gv[4] = q[1] * rm;
                gv[5] = q[2] * rm;
                gv[6] = a.a.w != 0.f ? qbase_qtip * ir3 * rm : 0.f;
            }
            const int tt = index32[t];
#pragma unroll
            for (int m = 0; m < kG; ++m) {
                const float v = warp_sum(gv[m]);
                if (lane == 0 && v != 0.f) atomicAdd(acc + (size_t)tt * kG + m, (double)v);
            }
        }
    }
    if (use_smem) {
        __syncthreads();
        for (int i = threadIdx.x; i < n * kG; i += blockDim.x)
            if (sacc[i] != 0.0) atomicAdd(gterm + i, sacc[i]);
    }
    if (err) atomicOr(&ctr->error_word, err);
}

}  // namespace

cudaError_t launch_adjoint(const ScanParams& p, int precision, const int* index32,
                           const mafm_point* pts, const double* w, long long n_points,
                           double qbase_qtip, double* gterm, RunCounters* ctr, cudaStream_t s) {
    const int n = p.n_terms_direct;
    const size_t smem = (size_t)n * kG * sizeof(double);
    const int use_smem = smem <= 96 * 1024 ? 1 : 0;
    const size_t dyn = use_smem ? smem : 0;
    const bool fp32 = precision == MAFM_FP32C;
    cudaError_t e = fp32 ? cudaFuncSetAttribute(adjoint32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                (int)std::max<size_t>(dyn, 1))
                         : cudaFuncSetAttribute(adjoint_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                (int)std::max<size_t>(dyn, 1));
    if (e != cudaSuccess) return e;
    long long blocks = (n_points + 255) / 256;
    const long long cap = (long long)sm_count() * 4;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    if (fp32)
        adjoint32_kernel<<<(unsigned)blocks, 256, dyn, s>>>(p, pts, w, n_points, (float)qbase_qtip,
                                                             index32, gterm, use_smem, ctr);
    else
        adjoint_kernel<<<(unsigned)blocks, 256, dyn, s>>>(p, pts, w, n_points, qbase_qtip, gterm,
                                                          use_smem, ctr);
    return cudaGetLastError();
}

}  // namespace mafm
