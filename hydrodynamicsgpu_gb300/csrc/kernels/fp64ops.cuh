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

// Class tests on the two 32-bit words: a test of the whole 64-bit pattern is
// recognised by the compiler as a floating-point class test or compare and issued to
// the FP64 unit; on the words it stays on the integer pipes.
__device__ __forceinline__ bool isNaNBits(double x) {
    const int hi = __double2hiint(x) & 0x7FFFFFFF, lo = __double2loint(x);
    return hi > 0x7FF00000 || (hi == 0x7FF00000 && lo != 0);
}

__device__ __forceinline__ bool isNaNBits(float x) { return x != x; }

// x >= 0.  (-0 >= 0 is true, NaN >= 0 is false)
__device__ __forceinline__ bool geZero(double x) {
    const int hi = __double2hiint(x), lo = __double2loint(x);
    return hi >= 0 ? (hi < 0x7FF00000 || (hi == 0x7FF00000 && lo == 0)) : (hi == (int)0x80000000 && lo == 0);
}
// x is +0 or -0
__device__ __forceinline__ bool isZeroBits(double x) {
    return ((__double2hiint(x) & 0x7FFFFFFF) | __double2loint(x)) == 0;
}
__device__ __forceinline__ bool geZero(float x) { return x >= 0.f; }
__device__ __forceinline__ bool isZeroBits(float x) { return (__float_as_int(x) & 0x7FFFFFFF) == 0; }

// .5 * x exactly: decrement the exponent of a normal x whose half is normal.  The
// rare other operands (zero, subnormal, Inf, NaN) take the FP64 unit out of line, so
// the compiler cannot issue that product for every operand and select.
static __device__ __noinline__ double halfNative(double x) { return x * .5; }
__device__ __forceinline__ double halfOf(double x) {
    long long b = bitsOf(x);
    int e = (int)((b >> 52) & 0x7FF);
    if (e >= 2 && e <= 0x7FE) return fromBits(b - (1LL << 52));
    return halfNative(x);
}
__device__ __forceinline__ float halfOf(float x) { return x * .5f; }

// total-order key of a non-NaN double (-0 < +0 here; callers treat zeros as equal)
__device__ __forceinline__ long long orderKey(long long b) { return b ^ ((b >> 63) & 0x7FFFFFFFFFFFFFFFLL); }

// C library fmin/fmax semantics (the oracle's): a NaN operand yields the other
// operand; equal operands (including -0 and +0) yield the second one.  The choice is
// made on the bit patterns and the result selected as an integer: a select between
// two doubles issues FP64-unit instructions on this part.
__device__ __forceinline__ bool fminTakesFirst(double x, double y) {
    const long long bx = bitsOf(x), by = bitsOf(y);
    const bool bothZero = ((bx | by) & 0x7FFFFFFFFFFFFFFFLL) == 0;
    return isNaNBits(y) || (!isNaNBits(x) && !bothZero && orderKey(bx) < orderKey(by));
}
__device__ __forceinline__ bool fmaxTakesFirst(double x, double y) {
    const long long bx = bitsOf(x), by = bitsOf(y);
    const bool bothZero = ((bx | by) & 0x7FFFFFFFFFFFFFFFLL) == 0;
    return isNaNBits(y) || (!isNaNBits(x) && !bothZero && orderKey(bx) > orderKey(by));
}
// c ? a : b, selected as an integer
__device__ __forceinline__ double selectD(bool c, double a, double b) {
    return fromBits(c ? bitsOf(a) : bitsOf(b));
}
__device__ __forceinline__ double fminLibm(double x, double y) { return selectD(fminTakesFirst(x, y), x, y); }
__device__ __forceinline__ double fmaxLibm(double x, double y) { return selectD(fmaxTakesFirst(x, y), x, y); }
// c ? 1. : -1., selected as an integer
__device__ __forceinline__ double plusMinusOne(bool c) {
    return fromBits(c ? 0x3FF0000000000000LL : (long long)0xBFF0000000000000ULL);
}
// x <= 0 (-0 and +0 included, NaN false) and a <= b, on the words / bit patterns
__device__ __forceinline__ bool leZero(double x) { return isZeroBits(x) || (__double2hiint(x) < 0 && !isNaNBits(x)); }
__device__ __forceinline__ bool leZero(float x) { return x <= 0.f; }
__device__ __forceinline__ bool leD(double a, double b) {
    if (isNaNBits(a) || isNaNBits(b)) return false;
    return (isZeroBits(a) && isZeroBits(b)) || orderKey(bitsOf(a)) <= orderKey(bitsOf(b));
}
__device__ __forceinline__ bool leD(float a, float b) { return a <= b; }
// x is finite / x is finite and nonzero, on the words
__device__ __forceinline__ bool finiteD(double x) { return (__double2hiint(x) & 0x7FF00000) != 0x7FF00000; }
__device__ __forceinline__ bool finiteNonzeroD(double x) { return finiteD(x) && !isZeroBits(x); }
__device__ __forceinline__ float fminLibm(float x, float y) { return (x < y || y != y) ? x : y; }
__device__ __forceinline__ float fmaxLibm(float x, float y) { return (x > y || y != y) ? x : y; }



// x * y computed on the integer pipes, bit-identical to the FP64 unit's product.
// The FP64 unit issues 2 operations per SM per clock on this part while the integer
// and FP32 pipes stand idle in the FP64-bound kernels; products routed here run on
// those pipes, concurrently with the native adds.  Fast path: both operands normal
// and the biased exponent sum in [1, 2045]; the 53 x 53-bit significand product is
// formed exactly (106 bits) and rounded to nearest, ties to even; the carry of a
// round-up into bit 53 increments the exponent field (to +-Inf only from the largest
// binade, as IEEE 754 requires).  Zeros, subnormals, Inf, NaN and products that could
// leave the normal range take the FP64 unit.  Checked against the FP64 unit on 4.3e9
// random operand pairs (all exponent ranges, short significands, extremes).
// the rare native product, kept out of line: inlined, it would be if-converted and
// issued to the FP64 unit for every operand pair
static __device__ __noinline__ double mulNative(double x, double y) { return x * y; }

__device__ __forceinline__ double mulI(double x, double y) {
    const unsigned long long ux = (unsigned long long)bitsOf(x), uy = (unsigned long long)bitsOf(y);
    const unsigned ex = (unsigned)(ux >> 52) & 0x7FF, ey = (unsigned)(uy >> 52) & 0x7FF;
    int e = (int)ex + (int)ey - 1023;
    if (ex - 1u >= 2046u || ey - 1u >= 2046u || (unsigned)(e - 1) >= 2045u) return mulNative(x, y);
    const unsigned long long mx = (ux & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    const unsigned long long my = (uy & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    const unsigned long long lo = mx * my, hi = __umul64hi(mx, my);   // product in [2^104, 2^106)
    unsigned long long mant, rest;
    if (hi >> 41) {
        mant = (hi << 11) | (lo >> 53);
        rest = lo << 11;
        e += 1;
    } else {
        mant = (hi << 12) | (lo >> 52);
        rest = lo << 12;
    }
    // rest: the round bit on top, the sticky bits below it
    mant += (rest > 0x8000000000000000ull) || (rest == 0x8000000000000000ull && (mant & 1));
    const unsigned long long r = (((unsigned long long)(e - 1) << 52) + mant) | ((ux ^ uy) & 0x8000000000000000ull);
    return fromBits((long long)r);
}
__device__ __forceinline__ float mulI(float x, float y) { return x * y; }

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
    if (isZeroBits(x) && eb != 0 && eb != 0x7FF) return fromBits((bx ^ bb) & (long long)0x8000000000000000ULL);
    if (ex < 623 || ex > 1423 || eb < 623 || eb > 1423) return x / b;
    double q = mulI(x, rb);
    double r = fma(-b, q, x);
    return fma(r, rb, q);
}
__device__ __forceinline__ float divByRecip(float x, float b, float rb) { return x / b; }

static __device__ __noinline__ double divNative(double x, double y) { return x / y; }

// x / y on the integer pipes, bit-identical to the IEEE quotient (round to nearest
// even).  Fast path: both operands normal and the quotient's biased exponent safely
// inside [1, 2046].  With m_x, m_y the 53-bit significands and s = [m_x < m_y], the
// truncated quotient q = floor(m_x 2^(52+s) / m_y) lies in [2^52, 2^53).  A reciprocal
// v ~ 2^126 / (m_y 2^11) is seeded from the FP32 reciprocal of m_y's top 24 bits
// (relative error below 2^-22) and refined by two fixed-point Newton steps
// v += v (2^126 - m_y 2^11 v) / 2^126; q is estimated as (m_x v) >> (63 - s), the
// remainder r = m_x 2^(52+s) - q m_y is formed exactly modulo 2^64 (|r| < 2^63) and
// q corrected until 0 <= r < m_y; then q is rounded up when 2r > m_y, or 2r = m_y
// and q is odd.  A zero operand beside a finite one is resolved with integer
// operations; everything else takes the FP64 unit.  Checked against the FP64 unit's
// quotient on 4.3e9 random operand pairs.
__device__ __forceinline__ double divI(double x, double y) {
    const unsigned long long ux = (unsigned long long)bitsOf(x), uy = (unsigned long long)bitsOf(y);
    const unsigned ex = (unsigned)(ux >> 52) & 0x7FF, ey = (unsigned)(uy >> 52) & 0x7FF;
    int e = (int)ex - (int)ey + 1023;
    if (ex - 1u >= 2046u || ey - 1u >= 2046u || (unsigned)(e - 2) >= 2044u) {
        // a zero operand beside a finite one: 0/0 = NaN, x/0 = +-Inf, 0/y = +-0 (the
        // limiter ratios of flat states are mostly these); the rest on the FP64 unit
        const bool xz = (ux << 1) == 0, yz = (uy << 1) == 0;
        if ((xz || yz) && ex != 0x7FF && ey != 0x7FF) {
            const unsigned long long sgn = (ux ^ uy) & 0x8000000000000000ull;
            return fromBits((long long)(xz && yz ? 0x7FFFFFFFFFFFFFFFull : xz ? sgn : (sgn | 0x7FF0000000000000ull)));
        }
        return divNative(x, y);
    }
    const unsigned long long mx = (ux & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    const unsigned long long d = (uy & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    const unsigned s = mx < d;
    e -= (int)s;
    const unsigned long long dn = d << 11;                                   // [2^63, 2^64)
    // The seed's two conversions are exact and done on the bits (the conversion
    // instructions would issue to the FP64 unit): the top 24 bits t in [2^23, 2^24)
    // are the float with exponent field 150 and fraction t - 2^23; rf = RN(1/t) lies
    // in (2^-24, 2^-23], so rf * 2^86 = (its 24-bit significand) << (exponent field - 64).
    const unsigned top = (unsigned)(dn >> 40);
    const float rf = __frcp_rn(__uint_as_float((150u << 23) | (top & 0x7FFFFFu)));
    const unsigned rb = __float_as_uint(rf);
    unsigned long long v = (unsigned long long)((rb & 0x7FFFFFu) | 0x800000u) << (((rb >> 23) & 0xFFu) - 64u);
#pragma unroll
    for (int it = 0; it < 2; ++it) {
        const unsigned long long plo = dn * v, phi = __umul64hi(dn, v);
        const long long eh = (long long)(0x4000000000000000ull - phi) - (plo != 0);   // floor((2^126 - dn v) / 2^64)
        const unsigned long long mag = (unsigned long long)(eh < 0 ? -eh : eh);
        const unsigned long long corr = (__umul64hi(v, mag) << 2) | ((v * mag) >> 62);   // v |eh| / 2^62
        v = eh < 0 ? v - corr : v + corr;
    }
    const unsigned long long hi = __umul64hi(mx, v), lo = mx * v;
    unsigned long long q = s ? ((hi << 2) | (lo >> 62)) : ((hi << 1) | (lo >> 63));
    long long r = (long long)((mx << (52 + s)) - q * d);
    if (r < 0) { q -= 1; r += (long long)d; }
    if (r < 0) { q -= 1; r += (long long)d; }
    if (r >= (long long)d) { q += 1; r -= (long long)d; }
    if (r >= (long long)d) { q += 1; r -= (long long)d; }
    const unsigned long long r2 = (unsigned long long)r << 1;
    q += (r2 > d) || (r2 == d && (q & 1));
    return fromBits((long long)((((unsigned long long)(e - 1) << 52) + q) | ((ux ^ uy) & 0x8000000000000000ull)));
}
__device__ __forceinline__ float divI(float x, float y) { return x / y; }



}  // namespace hgpu
