// fastmath.cuh — reciprocal and inverse square root on the FP64 pipe without IEEE divide or
// sqrt sequences: the hardware seeds (rcp.approx.ftz.f64, rsqrt.approx.ftz.f64, relative error
// below 1e-6) refined by one third-order step each, which lands within an ulp of the correctly
// rounded result for positive normal arguments.
//  * 1/d: with e = 1 - d r, 1/d = r/(1 - e) = r (1 + e + e^2 + ...), so r <- r + r (e + e^2)
//    leaves a relative error of e^3 (Householder's third-order iteration for the reciprocal);
//  * 1/sqrt(x): with e = 1 - x y^2, 1/sqrt(x) = y (1 - e)^(-1/2) = y (1 + e/2 + 3e^2/8 + ...),
//    so y <- y + y e (1/2 + 3e/8) leaves 5e^3/16.
// Each costs three (reciprocal) or five (inverse square root) FP64 operations after the seed,
// against two Newton-Raphson steps' four and eight; an IEEE double divide costs about ten FMA
// slots on GB300.
#pragma once

namespace dense {

__device__ __forceinline__ double rcp_nr(double d) {
    double r;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(d));
    const double e = fma(-d, r, 1.0);
    return fma(r, fma(e, e, e), r);
}

__device__ __forceinline__ double rsqrt_nr(double x) {
    double y;
    asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    const double e = fma(-x * y, y, 1.0);
    return fma(y, e * fma(0.375, e, 0.5), y);
}

}  // namespace dense
