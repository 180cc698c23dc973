// dfloat.cuh — double-float arithmetic on the FP32 pipes.
//
// A dfloat is the unevaluated sum h + l of two FP32 numbers with |l| at most
// half an ulp of h: 48 significant bits, about 3.6e-15 relative.  GB300 runs
// FP64 at 1/64 of its FP32 rate, so the FP64-faithful relaxation (MAFM_DF)
// computes with dfloats: every operation below costs 3-25 FP32 instructions.
//
// The building blocks are the error-free transformations of Dekker and Knuth
// (two_sum, fast_two_sum) and the FMA-based exact product; the compound
// operations follow the double-word algorithms analysed by Joldes, Muller and
// Popescu ("Tight and rigorous error bounds for basic building blocks of
// double-word arithmetic", ACM TOMS 44, 2017): the sloppy sum (relative error
// below 2^-44 without cancellation, absolute error below 2^-47 of the larger
// operand with it), the product with FMA (below 2^-45), quotient and square
// root by one Newton correction of the FP32 approximation.  Only the explicitly
// rounded intrinsics (__fadd_rn, __fmul_rn, __fmaf_rn) are used, which the
// compiler never contracts or reassociates, so the transformations stay exact
// under any optimisation flags.
#pragma once

#include <cuda_runtime.h>

namespace mafm {

struct dfloat {
    float h, l;
    dfloat() = default;
    __host__ __device__ constexpr dfloat(float hi, float lo) : h(hi), l(lo) {}
    // Split of a double: exact for the 48 leading bits.  constexpr, so a
    // literal argument is split at compile time (no FP64 instruction).
    __host__ __device__ constexpr explicit dfloat(double x)
        : h((float)x), l((float)(x - (double)(float)x)) {}
    __host__ __device__ constexpr explicit dfloat(int x) : h((float)x), l(0.0f) {}
};

// ---- error-free transformations -------------------------------------------

__device__ __forceinline__ dfloat dfl_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return dfloat(s, e);
}

// a + b exactly, for |a| >= |b| (or a = 0)
__device__ __forceinline__ dfloat dfl_fast_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    return dfloat(s, __fsub_rn(b, __fsub_rn(s, a)));
}

__device__ __forceinline__ dfloat dfl_two_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    return dfloat(p, __fmaf_rn(a, b, -p));
}

// ---- arithmetic ------------------------------------------------------------

__device__ __forceinline__ dfloat operator+(dfloat a, dfloat b) {
    const dfloat s = dfl_two_sum(a.h, b.h);
    return dfl_fast_two_sum(s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l)));
}
__device__ __forceinline__ dfloat operator-(dfloat a) { return dfloat(-a.h, -a.l); }
__device__ __forceinline__ dfloat operator-(dfloat a, dfloat b) { return a + (-b); }

__device__ __forceinline__ dfloat operator*(dfloat a, dfloat b) {
    const float p = __fmul_rn(a.h, b.h);
    float e = __fmaf_rn(a.h, b.h, -p);
    e = __fmaf_rn(a.h, b.l, e);
    e = __fmaf_rn(a.l, b.h, e);
    return dfl_fast_two_sum(p, e);
}

__device__ __forceinline__ float dfl_rcp_approx(float x) {
    float r;
    asm("rcp.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

__device__ __forceinline__ float dfl_rsqrt_approx(float x) {
    float r;
    asm("rsqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// a / b: q1 = a.h / b.h to FP32 accuracy, then q2 = (a - q1 b) / b corrects it.
__device__ __forceinline__ dfloat operator/(dfloat a, dfloat b) {
    const float y = dfl_rcp_approx(b.h);
    const float q1 = __fmul_rn(a.h, y);
    const dfloat r = a - b * dfloat(q1, 0.0f);
    const float q2 = __fmul_rn(r.h, y);
    const dfloat q = dfl_fast_two_sum(q1, q2);
    // second correction: the approximate reciprocal has an FP32 error
    const dfloat r2 = a - b * q;
    return q + dfloat(__fmul_rn(r2.h, y), 0.0f);
}

// a x for a float x
__device__ __forceinline__ dfloat operator*(dfloat a, float x) {
    const float p = __fmul_rn(a.h, x);
    float e = __fmaf_rn(a.h, x, -p);
    e = __fmaf_rn(a.l, x, e);
    return dfl_fast_two_sum(p, e);
}

__device__ __forceinline__ dfloat& operator+=(dfloat& a, dfloat b) { return a = a + b; }
__device__ __forceinline__ dfloat& operator-=(dfloat& a, dfloat b) { return a = a - b; }
__device__ __forceinline__ dfloat& operator*=(dfloat& a, dfloat b) { return a = a * b; }

// 1 / a
__device__ __forceinline__ dfloat dfl_rcp(dfloat a) { return dfloat(1.0f, 0.0f) / a; }

// sqrt(a) for a >= 0: s = a.h rsqrt(a.h), then s + (a - s^2) / (2 s)
__device__ __forceinline__ dfloat dfl_sqrt(dfloat a) {
    if (!(a.h > 0.0f)) return dfloat(0.0f, 0.0f);
    const float y = dfl_rsqrt_approx(a.h);
    const float s = __fmul_rn(a.h, y);
    const dfloat r = a - dfl_two_prod(s, s);
    const dfloat t = dfl_fast_two_sum(s, __fmul_rn(__fmul_rn(r.h, y), 0.5f));
    // one more correction step (the first s carries the rsqrt approximation error)
    const dfloat r2 = a - t * t;
    return t + dfloat(__fmul_rn(__fmul_rn(r2.h, y), 0.5f), 0.0f);
}

// 1 / sqrt(a) for a > 0: one Newton step y (1 + (1 - a y^2) / 2) in
// double-float from the FP32 approximation y, whose relative error e0 (about
// 2^-23) leaves (3/2) e0^2, about 3e-14
__device__ __forceinline__ dfloat dfl_rsqrt(dfloat a) {
    const float y = dfl_rsqrt_approx(a.h);
    const dfloat t = (a * y) * y;                        // about 1
    const float e = __fadd_rn(__fsub_rn(1.0f, t.h), -t.l);
    return dfl_fast_two_sum(y, __fmul_rn(__fmul_rn(y, e), 0.5f));
}

__device__ __forceinline__ bool operator<(dfloat a, dfloat b) {
    return a.h < b.h || (a.h == b.h && a.l < b.l);
}
__device__ __forceinline__ bool operator>(dfloat a, dfloat b) { return b < a; }
__device__ __forceinline__ bool operator<=(dfloat a, dfloat b) { return !(b < a); }
__device__ __forceinline__ bool operator>=(dfloat a, dfloat b) { return !(a < b); }

__device__ __forceinline__ dfloat dfl_fabs(dfloat a) {
    return (a.h < 0.0f || (a.h == 0.0f && a.l < 0.0f)) ? -a : a;
}

__device__ __forceinline__ bool dfl_isfinite(dfloat a) { return isfinite(a.h) && isfinite(a.l); }

__device__ __forceinline__ double to_double(dfloat a) { return (double)a.h + (double)a.l; }

// floor for the cell wrap of pixel positions (System::setDummyXY)
__device__ __forceinline__ dfloat dfl_floor(dfloat a) {
    const float fh = floorf(a.h);
    if (fh != a.h) return dfloat(fh, 0.0f);
    // a.h is an integer: the low part decides
    return dfl_fast_two_sum(fh, floorf(a.l));
}

// exp(x): x = n ln2 + r with a three-part ln2 (Cody and Waite), r / 16 into a
// degree-9 Taylor series of expm1, four doublings e <- e (2 + e), then
// 2^n (1 + e).  For |x| > 87 the FP32 range ends: 0 or infinity.
__device__ __forceinline__ dfloat dfl_exp(dfloat x) {
    constexpr double kLn2 = 0.69314718055994530942;
    constexpr float kLn2Hi = 0.693145751953125f;            // 15 significant bits
    constexpr double kRest = kLn2 - (double)kLn2Hi;
    constexpr float kLn2Mid = (float)kRest;
    constexpr float kLn2Lo = (float)(kRest - (double)kLn2Mid);
    if (x.h > 87.0f) return dfloat(__int_as_float(0x7f800000), 0.0f);
    if (x.h < -87.0f) return dfloat(0.0f, 0.0f);
    const float n = rintf(__fmul_rn(x.h, 1.44269504088896341f));
    dfloat r = x - dfloat(__fmul_rn(n, kLn2Hi), 0.0f);       // n kLn2Hi is exact
    r = r - dfl_two_prod(n, kLn2Mid);
    r = r - dfloat(__fmul_rn(n, kLn2Lo), 0.0f);
    r = dfloat(__fmul_rn(r.h, 0.0625f), __fmul_rn(r.l, 0.0625f));   // |r| < 0.022
    // expm1(r) = r (1 + r/2 (1 + r/3 (1 + ... (1 + r/9))))
    constexpr dfloat kInv[10] = {dfloat(0.0), dfloat(1.0), dfloat(1.0 / 2), dfloat(1.0 / 3),
                                 dfloat(1.0 / 4), dfloat(1.0 / 5), dfloat(1.0 / 6),
                                 dfloat(1.0 / 7), dfloat(1.0 / 8), dfloat(1.0 / 9)};
    dfloat p = dfloat(1.0f, 0.0f);
#pragma unroll
    for (int k = 9; k >= 2; --k) p = dfloat(1.0f, 0.0f) + (r * p) * kInv[k];
    dfloat e = r * p;
#pragma unroll
    for (int k = 0; k < 4; ++k) e = e * (dfloat(2.0f, 0.0f) + e);
    const dfloat y = dfloat(1.0f, 0.0f) + e;
    const int ni = (int)n;
    return dfloat(ldexpf(y.h, ni), ldexpf(y.l, ni));
}

// ---- two double-floats per instruction (packed f32x2) ---------------------
//
// A dfloat2 is two independent double-floats, element .x and element .y of
// each part.  Its operations are the scalar ones above applied to both
// elements by the packed FP32 instructions of the sm_100 family
// (add / mul / fma .rn .f32x2, which round each element as the scalar
// instruction does), so one instruction stream evaluates two tip–atom terms.

struct dfloat2 {
    float2 h, l;
};

__device__ __forceinline__ float2 p_add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 p_neg(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 p_sub(float2 a, float2 b) { return __fadd2_rn(a, p_neg(b)); }
__device__ __forceinline__ float2 p_mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 p_fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 p_bcast(float a) { return make_float2(a, a); }

__device__ __forceinline__ dfloat2 dfl2(dfloat a) { return {p_bcast(a.h), p_bcast(a.l)}; }
__device__ __forceinline__ dfloat dfl2_x(dfloat2 a) { return dfloat(a.h.x, a.l.x); }
__device__ __forceinline__ dfloat dfl2_y(dfloat2 a) { return dfloat(a.h.y, a.l.y); }

__device__ __forceinline__ dfloat2 dfl2_two_sum(float2 a, float2 b) {
    const float2 s = p_add(a, b);
    const float2 bb = p_sub(s, a);
    return {s, p_add(p_sub(a, p_sub(s, bb)), p_sub(b, bb))};
}

__device__ __forceinline__ dfloat2 dfl2_fast_two_sum(float2 a, float2 b) {
    const float2 s = p_add(a, b);
    return {s, p_sub(b, p_sub(s, a))};
}

__device__ __forceinline__ dfloat2 operator+(dfloat2 a, dfloat2 b) {
    const dfloat2 s = dfl2_two_sum(a.h, b.h);
    return dfl2_fast_two_sum(s.h, p_add(s.l, p_add(a.l, b.l)));
}
__device__ __forceinline__ dfloat2 operator-(dfloat2 a) { return {p_neg(a.h), p_neg(a.l)}; }
__device__ __forceinline__ dfloat2 operator-(dfloat2 a, dfloat2 b) { return a + (-b); }

__device__ __forceinline__ dfloat2 operator*(dfloat2 a, dfloat2 b) {
    const float2 p = p_mul(a.h, b.h);
    float2 e = p_fma(a.h, b.h, p_neg(p));
    e = p_fma(a.h, b.l, e);
    e = p_fma(a.l, b.h, e);
    return dfl2_fast_two_sum(p, e);
}

// a x for FP32 x (per element)
__device__ __forceinline__ dfloat2 operator*(dfloat2 a, float2 x) {
    const float2 p = p_mul(a.h, x);
    float2 e = p_fma(a.h, x, p_neg(p));
    e = p_fma(a.l, x, e);
    return dfl2_fast_two_sum(p, e);
}
__device__ __forceinline__ dfloat2 operator*(dfloat2 a, float x) { return a * p_bcast(x); }

// Operations whose result only feeds further arithmetic skip the final
// renormalisation (fast_two_sum): the low part may then exceed half an ulp
// of the high part by a few ulps, which the next operation absorbs.  The
// value h + l keeps the double-float accuracy (the dropped low x low
// product stays below 2^-44 of the operands' product); dfl2_norm restores the
// canonical form where a chain gets long.
__device__ __forceinline__ dfloat2 dfl2_mul_u(dfloat2 a, dfloat2 b) {
    const float2 p = p_mul(a.h, b.h);
    float2 e = p_fma(a.h, b.h, p_neg(p));
    e = p_fma(a.h, b.l, e);
    e = p_fma(a.l, b.h, e);
    return {p, e};
}
__device__ __forceinline__ dfloat2 dfl2_mulf_u(dfloat2 a, float2 x) {
    const float2 p = p_mul(a.h, x);
    float2 e = p_fma(a.h, x, p_neg(p));
    e = p_fma(a.l, x, e);
    return {p, e};
}
__device__ __forceinline__ dfloat2 dfl2_add_u(dfloat2 a, dfloat2 b) {
    const dfloat2 s = dfl2_two_sum(a.h, b.h);
    return {s.h, p_add(s.l, p_add(a.l, b.l))};
}
__device__ __forceinline__ dfloat2 dfl2_sub_u(dfloat2 a, dfloat2 b) { return dfl2_add_u(a, -b); }
__device__ __forceinline__ dfloat2 dfl2_norm(dfloat2 a) { return dfl2_fast_two_sum(a.h, a.l); }

// 1 / sqrt(a), as dfl_rsqrt
__device__ __forceinline__ dfloat2 dfl2_rsqrt(dfloat2 a) {
    const float2 y = make_float2(dfl_rsqrt_approx(a.h.x), dfl_rsqrt_approx(a.h.y));
    const dfloat2 t = (a * y) * y;
    const float2 e = p_sub(p_sub(p_bcast(1.0f), t.h), t.l);
    return dfl2_fast_two_sum(y, p_mul(p_mul(y, e), p_bcast(0.5f)));
}

// exp(x) per element: the range reduction of dfl_exp (Cody and Waite, then
// r / 16), a degree-7 Taylor polynomial of expm1 in Horner form with 1/k! as
// double-float constants, four doublings e <- e (2 + e), then 2^n (1 + e),
// all but the last sum in unnormalised form.  |r| < 0.022, so the truncation
// is below 2^-60 of the result before the doublings multiply it by 16; in an
// FP32 emulation against 120-bit arithmetic the relative error stays near
// 1.4e-14 over [-20, 8] (dfl_exp's degree-9 nested form: 3e-15) at about half
// the instructions.
__device__ __forceinline__ dfloat2 dfl2_exp(dfloat2 x) {
    constexpr double kLn2 = 0.69314718055994530942;
    constexpr float kLn2Hi = 0.693145751953125f;
    constexpr double kRest = kLn2 - (double)kLn2Hi;
    constexpr float kLn2Mid = (float)kRest;
    constexpr float kLn2Lo = (float)(kRest - (double)kLn2Mid);
    // outside [-87, 87] the element's result is replaced at the end; reduce a
    // clamped argument meanwhile so that no element overflows on the way
    const float2 xc = make_float2(fminf(fmaxf(x.h.x, -87.0f), 87.0f), fminf(fmaxf(x.h.y, -87.0f), 87.0f));
    const dfloat2 xr = {xc, make_float2(xc.x == x.h.x ? x.l.x : 0.0f, xc.y == x.h.y ? x.l.y : 0.0f)};
    const float2 n = make_float2(rintf(__fmul_rn(xc.x, 1.44269504088896341f)),
                                 rintf(__fmul_rn(xc.y, 1.44269504088896341f)));
    dfloat2 r = xr - dfloat2{p_mul(n, p_bcast(kLn2Hi)), p_bcast(0.0f)};
    {
        const float2 p = p_mul(n, p_bcast(kLn2Mid));
        r = r - dfloat2{p, p_fma(n, p_bcast(kLn2Mid), p_neg(p))};
    }
    r = r - dfloat2{p_mul(n, p_bcast(kLn2Lo)), p_bcast(0.0f)};
    r = {p_mul(r.h, p_bcast(0.0625f)), p_mul(r.l, p_bcast(0.0625f))};
    constexpr dfloat kC[8] = {dfloat(1.0), dfloat(1.0), dfloat(1.0 / 2), dfloat(1.0 / 6),
                              dfloat(1.0 / 24), dfloat(1.0 / 120), dfloat(1.0 / 720),
                              dfloat(1.0 / 5040)};
    dfloat2 p = dfl2(kC[7]);
#pragma unroll
    for (int k = 6; k >= 1; --k) p = dfl2_add_u(dfl2_mul_u(p, r), dfl2(kC[k]));
    dfloat2 e = dfl2_mul_u(p, r);
    const dfloat2 two = {p_bcast(2.0f), p_bcast(0.0f)};
#pragma unroll
    for (int k = 0; k < 4; ++k) e = dfl2_mul_u(e, dfl2_add_u(two, e));
    const dfloat2 y = dfl2_norm(dfl2_add_u(dfloat2{p_bcast(1.0f), p_bcast(0.0f)}, e));
    const int nx = (int)n.x, ny = (int)n.y;
    dfloat2 out = {make_float2(ldexpf(y.h.x, nx), ldexpf(y.h.y, ny)),
                   make_float2(ldexpf(y.l.x, nx), ldexpf(y.l.y, ny))};
    if (x.h.x > 87.0f) { out.h.x = __int_as_float(0x7f800000); out.l.x = 0.0f; }
    if (x.h.x < -87.0f) { out.h.x = 0.0f; out.l.x = 0.0f; }
    if (x.h.y > 87.0f) { out.h.y = __int_as_float(0x7f800000); out.l.y = 0.0f; }
    if (x.h.y < -87.0f) { out.h.y = 0.0f; out.l.y = 0.0f; }
    return out;
}

}  // namespace mafm
