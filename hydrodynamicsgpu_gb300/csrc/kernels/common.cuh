// common.cuh -- device-side building blocks shared by the Euler kernels (sm_103a).
//
// Arithmetic conventions (parity with the reference OpenCL kernels):
//  * the .cu files are compiled with --fmad=false, so a*b+c is two roundings as in
//    the reference source; deliberate fused operations call fma() explicitly;
//  * a dot/matrix product `sum = 0; sum += M[i][j]*x[j]` (res/RoeEigenfieldLinear.cl:16-54)
//    is evaluated with its structurally-zero and unit coefficients skipped.  For
//    finite inputs this is exact: the running sum starts as +0 + first term (which
//    turns -0 into +0, see zfix) and a running sum started from +0 is never -0, so
//    adding +/-0 or multiplying by exactly 1 never changes it.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "fp64ops.cuh"

namespace hgpu {

// ---- grid geometry (reference layout: INDEX(x,y,z) = x + SX*(y + SY*z)) ----
struct Grid {
    int S[3];            // cells per axis incl. 2 ghost layers per side (1 = unused axis)
    int dim;
    long long step[3];   // cell stride per axis
    long long V;         // S[0]*S[1]*S[2]
    unsigned* check = nullptr;   // checked builds: device word for index violations
};

// ---- checked build (compiled with HGPU_CHECKED): every cell index a kernel body
// computes is tested against the grid before it is used; a violation ORs
// CHECK_INDEX into *g.check and the access is skipped (no trap).  In the normal build
// the test is the constant true and compiles away. ----
enum : unsigned int { CHECK_INDEX = 1u, CHECK_GUARD = 2u };
#ifdef HGPU_CHECKED
__device__ __forceinline__ bool cellOk(const Grid& g, long long c) {
    if (c >= 0 && c < g.V) return true;
    if (g.check) atomicOr(g.check, CHECK_INDEX);
    return false;
}
#else
__device__ __forceinline__ constexpr bool cellOk(const Grid&, long long) { return true; }
#endif

__host__ __device__ inline void cellCoords(const Grid& g, long long c, int& x, int& y, int& z) {
    x = (int)(c % g.S[0]);
    long long r = c / g.S[0];
    y = (int)(r % g.S[1]);
    z = (int)(r / g.S[1]);
}

// every active coordinate in [lo, S-hi)
__host__ __device__ inline bool inRange(const Grid& g, int x, int y, int z, int lo, int hi) {
    if (x < lo || x >= g.S[0] - hi) return false;
    if (g.dim > 1 && (y < lo || y >= g.S[1] - hi)) return false;
    if (g.dim > 2 && (z < lo || z >= g.S[2] - hi)) return false;
    return true;
}

// face (side, c) is "along" coordinate lo..S-hiA along `side`, transverse lo..S-hiT
__host__ __device__ inline bool faceInRange(const Grid& g, int side, int x, int y, int z, int hiAlong, int hiTrans) {
    int c[3] = {x, y, z};
    for (int a = 0; a < g.dim; ++a) {
        int hi = (a == side) ? hiAlong : hiTrans;
        if (c[a] < 2 || c[a] >= g.S[a] - hi) return false;
    }
    return true;
}

// ---- -0 -> +0 (the effect of `+0 + x` in round-to-nearest), integer ops only ----
__device__ __forceinline__ double zfix(double x) {
    long long b = __double_as_longlong(x);
    return __longlong_as_double(b == (long long)0x8000000000000000ULL ? 0LL : b);
}
__device__ __forceinline__ float zfix(float x) {
    int b = __float_as_int(x);
    return __int_as_float(b == (int)0x80000000u ? 0 : b);
}

// ---- finiteness by exponent bits (integer pipe) ----
// Tested on the high 32-bit word: a test of the whole 64-bit pattern is recognised by
// the compiler as a floating-point class test and issued to the FP64 unit.
__device__ __forceinline__ bool finiteBits(double x) {
    return (__double2hiint(x) & 0x7FF00000) != 0x7FF00000;
}
__device__ __forceinline__ bool finiteBits(float x) { return (__float_as_int(x) & 0x7F800000) != 0x7F800000; }
template <typename real, int N>
__device__ __forceinline__ bool allFinite(const real* v) {
    bool ok = true;
#pragma unroll
    for (int i = 0; i < N; ++i) ok &= finiteBits(v[i]);
    return ok;
}

// ---- ordered-bit atomic minimum of non-negative reals (NaN ignored by construction) ----
__device__ __forceinline__ unsigned long long realBits(double x) { return (unsigned long long)__double_as_longlong(x); }
__device__ __forceinline__ unsigned long long realBits(float x) { return (unsigned long long)(unsigned int)__float_as_int(x); }
__host__ __device__ inline double bitsToDouble(unsigned long long b, bool isFloat) {
#ifdef __CUDA_ARCH__
    return isFloat ? (double)__int_as_float((int)(unsigned int)b) : __longlong_as_double((long long)b);
#else
    if (isFloat) { unsigned int u = (unsigned int)b; float f; memcpy(&f, &u, 4); return f; }
    double d; memcpy(&d, &b, 8); return d;
#endif
}

// ---- health word bits (hgpu_health) ----
// (HGPU_HEALTH_* in include/hgpu/hgpu.h)
enum : unsigned int {
    HEALTH_NONFINITE_DT = 1u,       // a NaN in the CFL reduction
    HEALTH_HLLC_NOBRANCH = 2u,      // an HLLC interface where no flux branch was taken
    HEALTH_STATE_NONFINITE = 4u,    // a checked state holds a NaN or an infinity
    HEALTH_STATE_DENSITY = 8u,      // a checked state has density <= 0
    HEALTH_STATE_PRESSURE = 16u,    // a checked state has pressure <= 0
    HEALTH_COPY_TIMEOUT = 32u,      // a bounded wait for a bulk copy (TMA) gave up
    HEALTH_STATE_BITS = 28u
};

// ---- slope limiters: res/SlopeLimiter.cl:5-68, min/max with C-library fmin/fmax semantics ----
// Literal types follow the reference source: `2.` is a double literal, so in the FP32
// program those sub-expressions are evaluated in double and converted back, exactly
// as C/OpenCL promote them; the FP64 program is unaffected.
// MinMod, max(0, min(r, 1)) with those semantics, decided on the bit pattern: NaN and
// r >= 1 give 1, [+0, 1) gives r, -0 gives -0 (fmax(0, -0) is its second operand), any
// other negative gives +0.  (Through fminLibm/fmaxLibm the compiler issues FP64
// instructions for it; this form stays on the integer pipes.)
__device__ __forceinline__ double minmodBits(double r) {
    const long long b = bitsOf(r), one = 0x3FF0000000000000LL;   // the bits of 1.
    const long long out = (isNaNBits(r) || b >= one) ? one : ((b >= 0 || b == (long long)0x8000000000000000ULL) ? b : 0LL);
    return fromBits(out);
}
__device__ __forceinline__ float minmodBits(float r) { return fmaxLibm(0.f, fminLibm(r, 1.f)); }

// Superbee, max(0, max(min(1, 2r), min(2, r))) with the same semantics, decided on the
// bit pattern: NaN and r >= 2 give 2, (1, 2) gives r, [1/2, 1] gives 1, (+0, 1/2) gives
// 2r (exact: the exponent field + 1, or the pattern doubled for a subnormal r), +0
// gives +0, -0 gives -0 (every fmin/fmax of the chain then takes its second, equal
// operand), any other negative gives +0.
__device__ __forceinline__ double superbeeBits(double r) {
    const long long b = bitsOf(r);
    const long long half = 0x3FE0000000000000LL, one = 0x3FF0000000000000LL, two = 0x4000000000000000LL;
    long long out;
    if (isNaNBits(r) || b >= two) out = two;
    else if (b >= one) out = b;
    else if (b >= half) out = one;
    else if (b > 0) out = b < (1LL << 52) ? b << 1 : b + (1LL << 52);
    else out = b == (long long)0x8000000000000000ULL ? b : 0LL;
    return fromBits(out);
}
__device__ __forceinline__ float superbeeBits(float r) {
    return fmaxLibm(0.f, fmaxLibm(fminLibm(1.f, 2.f * r), fminLibm(2.f, r)));
}

template <typename real>
__device__ __forceinline__ real slopeLimiter(int lim, real r) {
    typedef double W;
    if (lim == 8) return minmodBits(r);                                                         // MinMod
    if (lim == 18) return superbeeBits(r);                                                      // Superbee
#define MN fminLibm
#define MX fmaxLibm
    switch (lim) {
    case 0: return (real)0.;                                                                     // DonorCell
    case 1: return (real)1.;                                                                     // LaxWendroff
    case 2: return r;                                                                            // BeamWarming
    case 3: return (real)(.5 * (1. + (W)r));                                                     // Fromm
    case 4: return (real)((W)(real)MX((real)0., r) * (3. * (W)r + 1.) / (((W)r + 1.) * ((W)r + 1.)));  // CHARM
    case 5: return (real)MX((real)0., (real)(1.5 * (W)(r + (real)fabs(r)) / ((W)r + 2.)));       // HCUS
    case 6: return (real)MX((real)0., (real)(2. * (W)(r + (real)fabs(r)) / ((W)r + 3.)));        // HQUICK
    case 7: return (real)MX((real)0., (real)MN(2. * (W)r, (W)(real)MN((1. + 2. * (W)r) / 3., 2.)));  // Koren
    case 8: return (real)MX((real)0., (real)MN(r, (real)1.));                                    // MinMod
    case 9: return (real)MX((real)0., (real)MN(r, (real)1.5));                                   // Oshker
    case 10: return (real)(.5 * (W)(r * r + r) / ((W)(r * r + r) + 1.));                         // Ospre
    case 11: return (real)MX((real)0., (real)MN(2. * (W)r, (W)(real)MN(.25 + .75 * (W)r, 4.)));  // Smart
    case 12: return (real)MX((real)0., (real)MX((real)MN(1.5 * (W)r, 1.), (real)MN((W)r, 1.5)));  // Sweby
    case 13: return (real)MX((real)0., (real)MN((real)MN(2. * (W)r, .75 + .25 * (W)r),
                                                (real)MN(.25 + .75 * (W)r, 2.)));               // UMIST
    case 14: return (real)((W)(r * r + r) / ((W)(r * r) + 1.));                                 // VanAlbada1
    case 15: return (real)(2. * (W)r / ((W)(r * r) + 1.));                                      // VanAlbada2
    case 16: return (real)((W)(real)MX((real)0., r) * 2. / (1. + (W)r));                        // VanLeer
    case 17: return (real)MX((real)0., (real)MN(2., (W)(real)MN(.5 * (1. + (W)r), 2. * (W)r)));  // MonotizedCentral
    case 18: return (real)MX((real)0., (real)MX((real)MN((real)1., (real)2. * r), (real)MN((real)2., r)));  // Superbee
    case 19: return (real)(.5 * ((W)r + 1.) *
                           (W)(real)MN((real)1., (real)MN(4. * (W)r / ((W)r + 1.), 4. / ((W)r + 1.))));  // BarthJespersen
    }
#undef MN
#undef MX
    return (real)0.;
}

// ---- per-step constants kept on the device (dt never leaves the GPU during a step) ----
template <typename real>
struct StepConst {
    real dt;             // this step's dt (min * cfl, or the fixed dt)
    real dt_dx[3];       // dt / dx[side]   (res/Roe.cl:206)
    real coef[4][4];     // beta(m,k) * dt  (RungeKutta.h:86-99, computed in `real`)
    double dt_f64;       // dt widened, for the host
};

}  // namespace hgpu
