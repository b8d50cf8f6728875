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

}  // namespace fgpu
