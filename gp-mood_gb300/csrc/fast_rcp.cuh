// fast_rcp.cuh -- reciprocal and square root for the fast floating-point mode.
//
// 1/d by Newton-Raphson iteration from the hardware's approximate reciprocal
// (PTX rcp.approx.ftz.f64): y <- y + y*(1 - d*y), twice, each step an FMA pair
// (the FMA form of Newton's iteration for 1/d, P. Markstein, IBM J. Res. Dev.
// 34(1):111-119, 1990).  Each step squares the relative error, so the result
// is within a few ulp of 1/d for normal d; it is not correctly rounded.  Four
// FP64 pipe instructions against about seven and a half for an IEEE division.
// A zero or subnormal d gives NaN (the approximation flushes it to zero).
//
// sqrt(x) from the hardware's approximate reciprocal square root y ~ 1/sqrt(x)
// (PTX rsqrt.approx.ftz.f64) by the coupled iteration of the same paper: with
// g ~ sqrt(x) = x*y and h ~ 1/(2 sqrt(x)) = y/2, the residual r = 1/2 - g*h
// corrects both (g += g*r, h += h*r), which squares the relative error; a last
// step g += h*(x - g*g) (Newton's step for g^2 = x, its residual by one FMA)
// squares it again.  Seven FP64 pipe instructions and one approximation, no
// branch; within a few ulp of sqrt(x) for positive normal x, not correctly
// rounded.  Zero, subnormal and infinite x give NaN, and so do negative x (as
// sqrt does); the solver takes it only of a pressure over a density that it
// has already tested, or will test, for positivity.
#pragma once

__device__ __forceinline__ double gpm_fast_rcp(double d) {
    double y;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(d));
    double e = fma(-d, y, 1.0);
    y = fma(y, e, y);
    e = fma(-d, y, 1.0);
    return fma(y, e, y);
}

__device__ __forceinline__ double gpm_fast_sqrt(double x) {
    double y;
    asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    double g = x * y, h = 0.5 * y;
    const double r = fma(-g, h, 0.5);
    g = fma(g, r, g);
    h = fma(h, r, h);
    const double e = fma(-g, g, x);
    return fma(h, e, g);
}
