// limiter_dual.cuh -- slope limiter value and derivative along the branch the
// forward takes (dual numbers through the same expressions and the same fmin/fmax
// operand selections as slopeLimiter in common.cuh).  Used by the adjoint.
#pragma once
#include "common.cuh"

namespace hgpu {

struct Dual {
    double v, d;
};
__device__ __forceinline__ Dual cst(double c) { return {c, 0.}; }
__device__ __forceinline__ Dual operator+(Dual a, Dual b) { return {a.v + b.v, a.d + b.d}; }
__device__ __forceinline__ Dual operator-(Dual a, Dual b) { return {a.v - b.v, a.d - b.d}; }
__device__ __forceinline__ Dual operator*(Dual a, Dual b) { return {a.v * b.v, a.d * b.v + a.v * b.d}; }
__device__ __forceinline__ Dual operator/(Dual a, Dual b) {
    double q = a.v / b.v;
    return {q, (a.d - q * b.d) / b.v};
}
__device__ __forceinline__ Dual operator+(Dual a, double b) { return {a.v + b, a.d}; }
__device__ __forceinline__ Dual operator+(double a, Dual b) { return {a + b.v, b.d}; }
__device__ __forceinline__ Dual operator*(double a, Dual b) { return {a * b.v, a * b.d}; }
__device__ __forceinline__ Dual operator/(double a, Dual b) { return cst(a) / b; }
__device__ __forceinline__ Dual dabs(Dual a) { return signbit(a.v) ? Dual{-a.v, -a.d} : a; }
// the operand fminLibm / fmaxLibm return: NaN yields the other, ties the second
// (chosen on the bits and selected as integers, like fminLibm / fmaxLibm)
__device__ __forceinline__ Dual dsel(bool c, Dual a, Dual b) { return {selectD(c, a.v, b.v), selectD(c, a.d, b.d)}; }
__device__ __forceinline__ Dual dmin(Dual a, Dual b) { return dsel(fminTakesFirst(a.v, b.v), a, b); }
__device__ __forceinline__ Dual dmax(Dual a, Dual b) { return dsel(fmaxTakesFirst(a.v, b.v), a, b); }

// res/SlopeLimiter.cl, same expressions and min/max operand order as slopeLimiter()
__device__ __forceinline__ Dual limiterDual(int lim, Dual r) {
    const Dual z = cst(0.), one = cst(1.);
    if (lim == 8) {
        // MinMod, max(0, min(r, 1)): the derivative is r's where min takes r and max
        // takes that, i.e. r in [-0, 1) on the bit pattern (minmodBits for the value)
        const long long b = bitsOf(r.v);
        const bool takesR = (b >= 0 && b < 0x3FF0000000000000LL) || b == (long long)0x8000000000000000ULL;
        return {minmodBits(r.v), selectD(takesR, r.d, 0.)};
    }
    switch (lim) {
    case 0: return z;
    case 1: return one;
    case 2: return r;
    case 3: return .5 * (1. + r);
    case 4: return dmax(z, r) * (3. * r + 1.) / ((r + 1.) * (r + 1.));
    case 5: return dmax(z, 1.5 * (r + dabs(r)) / (r + 2.));
    case 6: return dmax(z, 2. * (r + dabs(r)) / (r + 3.));
    case 7: return dmax(z, dmin(2. * r, dmin((1. + 2. * r) / cst(3.), cst(2.))));
    case 8: return dmax(z, dmin(r, one));
    case 9: return dmax(z, dmin(r, cst(1.5)));
    case 10: return .5 * (r * r + r) / ((r * r + r) + 1.);
    case 11: return dmax(z, dmin(2. * r, dmin(.25 + .75 * r, cst(4.))));
    case 12: return dmax(z, dmax(dmin(1.5 * r, one), dmin(r, cst(1.5))));
    case 13: return dmax(z, dmin(dmin(2. * r, .75 + .25 * r), dmin(.25 + .75 * r, cst(2.))));
    case 14: return (r * r + r) / (r * r + 1.);
    case 15: return 2. * r / (r * r + 1.);
    case 16: return dmax(z, r) * cst(2.) / (1. + r);
    case 17: return dmax(z, dmin(cst(2.), dmin(.5 * (1. + r), 2. * r)));
    case 18: return dmax(z, dmax(dmin(one, 2. * r), dmin(cst(2.), r)));
    case 19: return .5 * (r + 1.) * dmin(one, dmin(4. * r / (r + 1.), 4. / (r + 1.)));
    }
    return z;
}

}  // namespace hgpu
