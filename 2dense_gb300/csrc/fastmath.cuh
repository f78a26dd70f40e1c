// fastmath.cuh — reciprocal and inverse square root on the FP64 pipe without IEEE divide or
// sqrt sequences: the hardware seeds (rcp.approx.ftz.f64, rsqrt.approx.ftz.f64) refined by two
// Newton-Raphson steps (for 1/d: r <- r + r(1 - d r); for 1/sqrt(x): y <- y + y(1 - x y^2)/2),
// which lands within an ulp of the correctly rounded result for positive normal arguments.
// On GB300 an IEEE double divide costs about ten FMA slots; these cost five.
#pragma once

namespace dense {

__device__ __forceinline__ double rcp_nr(double d) {
    double r;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(d));
    double e = fma(-d, r, 1.0);
    r = fma(r, e, r);
    e = fma(-d, r, 1.0);
    return fma(r, e, r);
}

__device__ __forceinline__ double rsqrt_nr(double x) {
    double y;
    asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    double e = fma(-x * y, y, 1.0);
    y = fma(0.5 * y, e, y);
    e = fma(-x * y, y, 1.0);
    return fma(0.5 * y, e, y);
}

}  // namespace dense
