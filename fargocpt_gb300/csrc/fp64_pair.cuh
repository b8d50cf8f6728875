// FP64-accurate arithmetic from pairs of FP32 values, for the FP64 kernels
// whose cost is all arithmetic (the potential and the disk force): a value is
// the unevaluated sum hi + lo of two floats with |lo| <= ulp(hi) / 2, about
// 48 significant bits.  GB300 issues FP32 operations at 64 times its FP64
// rate, so a pair operation of 5 to 20 FP32 operations is several times
// cheaper than one FP64 operation.
//
// The building blocks are the error-free transformations TwoSum (Knuth 1969),
// Fast2Sum (Dekker 1971) and TwoProduct by fused multiply-add, combined as in
// Joldes, Muller and Popescu, "Tight and rigorous error bounds for basic
// building blocks of double-word arithmetic" (ACM TOMS 44, 2017): the sum of
// two pairs (their algorithm 6, relative error below 3 u^2, u = 2^-24), the
// product of two pairs (algorithm 12, below 5 u^2) and of a pair and a float
// (algorithm 9).  Every operation is spelled with the round-to-nearest
// intrinsics so that the compiler neither contracts nor reorders them.
#pragma once

#include <cuda_runtime.h>

namespace fgpu {

struct f2 {
    float h, l;
};

__device__ __forceinline__ f2 f2_of(double x)
{
    const float h = __double2float_rn(x);
    return f2{h, __double2float_rn(x - (double)h)};
}
__device__ __forceinline__ double f2_value(f2 a) { return (double)a.h + (double)a.l; }

// a + b exactly as s + e, for |a| >= |b| or a = 0
__device__ __forceinline__ f2 fast_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    return f2{s, __fsub_rn(b, __fsub_rn(s, a))};
}
// a + b exactly as s + e, any magnitudes
__device__ __forceinline__ f2 two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return f2{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
// a b exactly as p + e
__device__ __forceinline__ f2 two_prod(float a, float b)
{
    const float p = __fmul_rn(a, b);
    return f2{p, __fmaf_rn(a, b, -p)};
}

__device__ __forceinline__ f2 f2_add(f2 x, f2 y)
{
    const f2 s = two_sum(x.h, y.h);
    const f2 t = two_sum(x.l, y.l);
    const f2 v = fast_two_sum(s.h, __fadd_rn(s.l, t.h));
    return fast_two_sum(v.h, __fadd_rn(t.l, v.l));
}
__device__ __forceinline__ f2 f2_neg(f2 x) { return f2{-x.h, -x.l}; }
__device__ __forceinline__ f2 f2_sub(f2 x, f2 y) { return f2_add(x, f2_neg(y)); }

__device__ __forceinline__ f2 f2_mul(f2 x, f2 y)
{
    const f2 c = two_prod(x.h, y.h);
    const float t = __fmaf_rn(x.h, y.l, __fmul_rn(x.l, y.l));
    return fast_two_sum(c.h, __fadd_rn(c.l, __fmaf_rn(x.l, y.h, t)));
}
__device__ __forceinline__ f2 f2_mul_f(f2 x, float y)
{
    const f2 c = two_prod(x.h, y);
    return fast_two_sum(c.h, __fmaf_rn(x.l, y, c.l));
}

// 1 / sqrt(d) for d > 0: the hardware estimate, one FP32 Newton step, then
// one Newton step whose residual 1 - d r^2 is formed in pair arithmetic; the
// result is within a few units of 2^-46 of the exact value
__device__ __forceinline__ f2 f2_rsqrt(f2 d)
{
    float r = rsqrtf(d.h);
    r = __fmul_rn(r, __fmaf_rn(__fmul_rn(-0.5f, d.h), __fmul_rn(r, r), 1.5f));
    const f2 p = f2_mul(d, two_prod(r, r));  // about 1
    const float e = __fsub_rn(__fsub_rn(1.0f, p.h), p.l);
    return fast_two_sum(r, __fmul_rn(__fmul_rn(0.5f, r), e));
}

// running sum hi + lo of pairs, one TwoSum per term (the low parts are small
// against the sum, their float addition loses only below 2^-48 of it)
__device__ __forceinline__ void f2_accumulate(float &hi, float &lo, f2 x)
{
    const f2 s = two_sum(hi, x.h);
    hi = s.h;
    lo = __fadd_rn(lo, __fadd_rn(s.l, x.l));
}

// ---------------------------------------------------------------------------
// Conversions on the integer pipe.  GB300 converts between FP64 and FP32
// (F2F) at about one result per clock per SM, slower than its FP64
// arithmetic, so the transports split doubles into pairs and join pairs into
// doubles with bit operations and one integer-to-float conversion.
// ---------------------------------------------------------------------------

// x as a normalised pair, |x - (h + l)| <= 2^-48 |x|: h is x truncated to
// 24 significant bits (the sign, the rebased exponent and the top 23
// mantissa bits, shifted into place), l the remaining 29 mantissa bits
// converted to float and scaled by 2^(e - 1075).  Both are normal floats for
// biased exponents e in [949, 1150] (2^-74 <= |x| < 2^128).  Below that range
// x becomes zero (an absolute error under 2^-74); at or above it, and for
// infinities and NaN, a NaN of x's sign, so that a state out of the pairs'
// range shows as non-finite.  Branch-free: the callers' loops over a thread's
// cells stay one instruction stream.
__device__ __forceinline__ f2 f2_split(double x)
{
    const unsigned w1 = (unsigned)__double2hiint(x), w0 = (unsigned)__double2loint(x);
    const unsigned ax = w1 & 0x7fffffffu, sign = w1 & 0x80000000u;
    const unsigned hb = __funnelshift_l(w0, ax - (896u << 20), 3);
    const float scale = __uint_as_float((hb & 0x7f800000u) - (52u << 23));
    const float l = __fmul_rn(__uint2float_rn(w0 & 0x1fffffffu), scale);
    const f2 p = fast_two_sum(__uint_as_float(hb | sign), __uint_as_float(__float_as_uint(l) | sign));
    const bool tiny = ax < (949u << 20), huge = ax >= (1151u << 20);
    const float nan = __uint_as_float(0x7fc00000u | sign);
    return f2{tiny ? 0.0f : (huge ? nan : p.h), tiny ? 0.0f : (huge ? nan : p.l)};
}

// a float as a double, exactly: the exponent rebased, the mantissa shifted;
// zero and subnormal floats (below 2^-126) give a signed zero, infinities an
// infinity, NaN a NaN.  Branch-free.
__device__ __forceinline__ double f_to_d(float f)
{
    const unsigned b = __float_as_uint(f);
    const unsigned ef = (b >> 23) & 0xffu, sign = b & 0x80000000u;
    const unsigned hi = sign | (((b & 0x7fffffffu) >> 3) + (896u << 20));
    const unsigned special = sign | ((b & 0x7fffffu) ? 0x7ff80000u : 0x7ff00000u);
    const unsigned w1 = ef == 0u ? sign : (ef == 255u ? special : hi);
    const unsigned w0 = (ef == 0u || ef == 255u) ? 0u : (b << 29);
    return __hiloint2double((int)w1, (int)w0);
}

// h + l as a double (one FP64 addition of the two exact conversions)
__device__ __forceinline__ double f2_to_double(f2 a) { return f_to_d(a.h) + f_to_d(a.l); }

// ---------------------------------------------------------------------------
// Cheaper pair operations for the transports, whose error bars are relative
// to the operands' magnitudes (the pair representation itself carries 2^-48
// of each value): the sloppy sum (Joldes, Muller and Popescu, algorithm 5),
// absolute error within a few 2^-48 (|x| + |y|); the product without the
// low-by-low term; quotient and reciprocal from the hardware reciprocal
// estimate (rcp.approx, within 2^-22) with one correction in pair
// arithmetic, relative error within a few 2^-46.
// ---------------------------------------------------------------------------
__device__ __forceinline__ f2 f2_sadd(f2 x, f2 y)
{
    const f2 s = two_sum(x.h, y.h);
    return fast_two_sum(s.h, __fadd_rn(s.l, __fadd_rn(x.l, y.l)));
}
__device__ __forceinline__ f2 f2_ssub(f2 x, f2 y) { return f2_sadd(x, f2_neg(y)); }

__device__ __forceinline__ f2 f2_smul(f2 x, f2 y)
{
    const f2 c = two_prod(x.h, y.h);
    return fast_two_sum(c.h, __fadd_rn(c.l, __fmaf_rn(x.l, y.h, __fmul_rn(x.h, y.l))));
}

__device__ __forceinline__ float rcp_approx(float x)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// 1 / d for a normal d: r = rcp(d.h), then r + r (1 - d r)
__device__ __forceinline__ f2 f2_rcp(f2 d)
{
    const float r = rcp_approx(d.h);
    const f2 p = f2_mul_f(d, r);  // about 1
    const float e = __fsub_rn(__fsub_rn(1.0f, p.h), p.l);
    return fast_two_sum(r, __fmul_rn(r, e));
}

// p / s for a normal s: q = p.h rcp(s.h), then q + (p - q s) rcp(s.h)
__device__ __forceinline__ f2 f2_sdiv(f2 p, f2 s)
{
    const float r = rcp_approx(s.h);
    const float q = __fmul_rn(p.h, r);
    const f2 qs = two_prod(q, s.h);
    const float d = __fmaf_rn(-q, s.l, __fadd_rn(__fsub_rn(__fsub_rn(p.h, qs.h), qs.l), p.l));
    return fast_two_sum(q, __fmul_rn(d, r));
}

}  // namespace fgpu
