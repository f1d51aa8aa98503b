/*
 * FP64 divisions that cost fewer FP64 instructions than the IEEE division.
 *
 * div_rcp: division by a tabulated reciprocal, rounded exactly as x / d.
 *
 * A march that divides many times by grid-only quantities (widths,
 * spacings) can store r = 1 / d once, rounded to nearest, and recover the
 * correctly rounded quotient from it with Markstein's method (P. Markstein,
 * "Computation of elementary functions on the IBM RISC System/6000
 * processor", IBM J. Res. Dev. 34(1), 1990; the theorem is also stated in
 * Muller et al., "Handbook of Floating-Point Arithmetic"):
 *
 *   q0 = x r                  within 1.5 ulp of x / d (r within half an ulp)
 *   q1 = q0 + (x - q0 d) r    within one ulp (the correction's own error is
 *                             about 2^-53 of q0's)
 *   q2 = q1 + (x - q1 d) r    = x / d rounded to nearest (Markstein's
 *                             theorem: r within half an ulp of 1 / d, q1
 *                             within one ulp, the remainder x - q1 d exact
 *                             in a fused multiply-add)
 *
 * one multiplication and four fused multiply-adds, all on values of the
 * march.  The theorem needs the operands away from the ends of the exponent
 * range (no overflow or underflow in q, the remainder or the correction), so
 * both |x| and |d| must lie in [2^-400, 2^400); a zero x is exact too (q0
 * carries its sign, which the corrections would lose).  Anything else
 * (denormals, infinities, NaN, a d whose reciprocal was not tabulated)
 * divides.  The results equal CUDA's IEEE division bit for bit; the device
 * check scg_divide_check compares the two.
 *
 * recip: a reciprocal within one ulp, for the marches whose results are
 * compared to round-off (below).
 */
#pragma once

#include <cuda_runtime.h>

namespace scg
{
namespace dev
{

// High word of |v| against [2^-400, 2^400): biased exponents 623 to 1422.
constexpr unsigned RCP_EXP_LO = (1023u - 400u) << 20;
constexpr unsigned RCP_EXP_SPAN = 800u << 20;

__device__ __forceinline__ bool rcp_window(double v)
{
    unsigned const h = static_cast<unsigned>(__double2hiint(v)) & 0x7fffffffu;
    return h - RCP_EXP_LO < RCP_EXP_SPAN;
}

// The tabulated reciprocal of d: 1 / d rounded to nearest when d is in the
// window, else 0 (div_rcp then divides).
__device__ __forceinline__ double rcp_tab(double d) { return rcp_window(d) ? 1.0 / d : 0.0; }

static __device__ __noinline__ double div_plain(double x, double d) { return x / d; }

// x / d, rounded to nearest, from r = rcp_tab(d).
__device__ __forceinline__ double div_rcp(double x, double d, double r)
{
    double const q0 = x * r;
    unsigned const hx = static_cast<unsigned>(__double2hiint(x)) & 0x7fffffffu;
    bool const xok = hx - RCP_EXP_LO < RCP_EXP_SPAN || (hx | static_cast<unsigned>(__double2loint(x))) == 0u;
    if (__double2hiint(r) != 0 && xok)
    {
        double const q1 = __fma_rn(__fma_rn(-q0, d, x), r, q0);
        double const q2 = __fma_rn(__fma_rn(-q1, d, x), r, q1);
        return copysign(q2, q0);
    }
    return div_plain(x, d);
}

// Reciprocal.  FP64: Newton's iteration r <- r + r (1 - d r) from the FP32
// hardware approximation of the reciprocal of d's significand (its top 23
// bits), rescaled by d's exponent; each step squares the relative error, so
// two take it from ~2^-22 below 2^-86 and r is within one ulp of 1 / d, in
// four fused multiply-adds (a correctly rounded division takes about twice
// as many FP64 instructions).  That holds for |d| in [2^-1022, 2^1022);
// outside it (zero, subnormals, the largest magnitudes, infinities, NaN) the
// division replaces the result, behind a branch inside one asm statement.
// The compiler then sees no branch, as it sees none in a division
// instruction: with the edges taken by branches or selects it could see,
// kernels inlining this in different code contracted the callers'
// multiply-adds differently, and batched and single-core marches no longer
// rounded alike.  A predicated division instead of the branch was issued at
// every call.  FP32: the division.
__device__ __forceinline__ double recip(double d)
{
    unsigned const hi = static_cast<unsigned>(__double2hiint(d));
    unsigned const e = (hi >> 20) & 0x7ffu;
    float const m =
        __uint_as_float((127u << 23) | ((hi & 0xfffffu) << 3) | (static_cast<unsigned>(__double2loint(d)) >> 29));
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(m));
    unsigned const yb = __float_as_uint(y);
    double r = __hiloint2double(static_cast<int>(((yb >> 3) + (896u << 20) - ((e - 1023u) << 20)) | (hi & 0x80000000u)),
                                static_cast<int>(yb << 29));
    double t = __fma_rn(-d, r, 1.0);
    r = __fma_rn(r, t, r);
    t = __fma_rn(-d, r, 1.0);
    r = __fma_rn(r, t, r);
    asm("{\n\t"
        ".reg .pred p;\n\t"
        "setp.le.u32 p, %2, 2043;\n\t"
        "@p bra RCP_DONE;\n\t"
        "div.rn.f64 %0, 0d3FF0000000000000, %1;\n\t"
        "RCP_DONE:\n\t"
        "}"
        : "+d"(r)
        : "d"(d), "r"(e - 1u));
    return r;
}
__device__ __forceinline__ float recip(float d) { return 1.0f / d; }

} // namespace dev
} // namespace scg
