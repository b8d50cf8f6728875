// Reproducible compensated sum of per-ring partial sums (disk force, mass).
#pragma once

#include <cuda_runtime.h>

// Component w of `rows` rows of `width` partial sums, summed by one warp:
// lane l adds rows l, l + 32, ... with Kahan compensation, then the 32
// (sum, compensation) pairs are combined along a fixed shuffle tree with
// Knuth's TwoSum, which recovers the rounding error of each addition
// exactly.  The order of operations is fixed, so the result is the same on
// every run.  Every lane of the warp must call it with the same w.
__device__ __forceinline__ void warp_compensated_rows(const double *__restrict__ partial, int rows,
                                                      int width, int w, double *__restrict__ out)
{
    const int lane = threadIdx.x & 31;
    double s = 0.0, c = 0.0;  // the sum is s - c
    for (int r = lane; r < rows; r += 32) {
        const double y = partial[(size_t)r * width + w] - c;
        const double t = s + y;
        c = (t - s) - y;
        s = t;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const double s2 = __shfl_down_sync(0xffffffffu, s, o);
        const double c2 = __shfl_down_sync(0xffffffffu, c, o);
        const double t = s + s2;
        const double bp = t - s;
        const double e = (s - (t - bp)) + (s2 - bp);  // s + s2 = t + e exactly
        c = (c + c2) - e;
        s = t;
    }
    if (lane == 0) out[w] = s - c;
}
