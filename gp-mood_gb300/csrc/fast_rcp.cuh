// fast_rcp.cuh -- reciprocal for the fast floating-point mode.
//
// 1/d by Newton-Raphson iteration from the hardware's approximate reciprocal
// (PTX rcp.approx.ftz.f64): y <- y + y*(1 - d*y), twice, each step an FMA pair
// (the FMA form of Newton's iteration for 1/d, P. Markstein, IBM J. Res. Dev.
// 34(1):111-119, 1990).  Each step squares the relative error, so the result
// is within a few ulp of 1/d for normal d; it is not correctly rounded.  Four
// FP64 pipe instructions against about seven and a half for an IEEE division.
// A zero or subnormal d gives NaN (the approximation flushes it to zero).
#pragma once

__device__ __forceinline__ double gpm_fast_rcp(double d) {
    double y;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(d));
    double e = fma(-d, y, 1.0);
    y = fma(y, e, y);
    e = fma(-d, y, 1.0);
    return fma(y, e, y);
}
