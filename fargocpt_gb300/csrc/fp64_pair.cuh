// FP64-accurate arithmetic from pairs of FP32 values for the FP64 form's
// kernels: a value is the unevaluated sum hi + lo of two floats with |lo|
// at most about ulp(hi) / 2, about 48 significant bits.  GB300 issues FP32
// operations at about 70 times its FP64 rate (measured: 113 against 1.6
// results per clock per SM), so a pair operation of 5 to 20 FP32 operations
// is several times cheaper than one FP64 operation.
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

// x as a pair, |x - (h + l)| <= 2^-48 |x|, |l| < ulp(h): h is x truncated to
// 24 significant bits (the sign, the rebased exponent and the top 23
// mantissa bits, shifted into place), l the remaining 29 mantissa bits
// converted to float and scaled by 2^(e - 1075).  (The pair is not
// renormalised: the pair operations take |l| < ulp(h) with error bounds at
// most twice those for |l| <= ulp(h) / 2, and the sign of h is the sign of
// x.)  Both are normal floats for biased exponents e in [949, 1150]
// (2^-74 <= |x| < 2^128).  Below that range x becomes zero (an absolute
// error under 2^-74); at or above it, and for infinities and NaN, a NaN of
// x's sign, so that a state out of the pairs' range shows as non-finite.
// Branch-free: the callers' loops over a thread's cells stay one
// instruction stream.
__device__ __forceinline__ f2 f2_split(double x)
{
    const unsigned w1 = (unsigned)__double2hiint(x), w0 = (unsigned)__double2loint(x);
    const unsigned ax = w1 & 0x7fffffffu, sign = w1 & 0x80000000u;
    const unsigned hb = __funnelshift_l(w0, ax - (896u << 20), 3);
    const float scale = __uint_as_float((hb & 0x7f800000u) - (52u << 23));
    const unsigned lb = __float_as_uint(__fmul_rn(__uint2float_rn(w0 & 0x1fffffffu), scale));
    const bool in = ax - (949u << 20) < (202u << 20);
    const unsigned out = ax < (949u << 20) ? 0u : (0x7fc00000u | sign);
    return f2{__uint_as_float(in ? (hb | sign) : out), __uint_as_float(in ? (lb | sign) : out)};
}

// a float as a double, exactly: the exponent rebased, the mantissa shifted;
// zero and subnormal floats (below 2^-126) give a signed zero, infinities and
// NaN a NaN.  Branch-free.
__device__ __forceinline__ double f_to_d(float f)
{
    const unsigned b = __float_as_uint(f);
    const unsigned mag = b & 0x7fffffffu, sign = b & 0x80000000u;
    const bool normal = mag - 0x00800000u < 0x7f000000u;
    const unsigned w1 = normal ? (sign | ((mag >> 3) + (896u << 20)))
                               : (sign | (mag < 0x00800000u ? 0u : 0x7ff80000u));
    return __hiloint2double((int)w1, (int)(normal ? b << 29 : 0u));
}
// the same for the low part of a pair, which is finite when the high part
// is (a NaN pair has a NaN high part): zero and subnormals give zero
__device__ __forceinline__ double f_to_d_lo(float f)
{
    const unsigned b = __float_as_uint(f);
    const unsigned mag = b & 0x7fffffffu;
    const bool tiny = mag < 0x00800000u;
    const unsigned w1 = (b & 0x80000000u) | (tiny ? 0u : (mag >> 3) + (896u << 20));
    return __hiloint2double((int)w1, (int)(tiny ? 0u : b << 29));
}

// h + l as a double (one FP64 addition of the two exact conversions)
__device__ __forceinline__ double f2_to_double(f2 a) { return f_to_d(a.h) + f_to_d_lo(a.l); }

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
// x + a d in one: the product's error-free high part, the sum's TwoSum, one
// renormalisation
__device__ __forceinline__ f2 f2_sfma(f2 x, f2 a, f2 d)
{
    const f2 p = two_prod(a.h, d.h);
    const float pl = __fmaf_rn(a.l, d.h, __fmaf_rn(a.h, d.l, p.l));
    const f2 s = two_sum(x.h, p.h);
    return fast_two_sum(s.h, __fadd_rn(s.l, __fadd_rn(x.l, pl)));
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

// sqrt(x) for x > 0: x rsqrt(x)
__device__ __forceinline__ f2 f2_sqrt(f2 x) { return f2_smul(x, f2_rsqrt(x)); }

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
