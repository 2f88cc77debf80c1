// health.cuh -- per-cell check of a conserved state (failure detection).
//
// The reference has no run-time detection: a NaN, a negative density or a negative
// pressure propagates silently (its only errors are thrown at set-up,
// src/Solver/Solver.cpp:150-153, 201).  Here every step ends with this check over the
// interior cells of the state it wrote, and so does every upload; the result is a set
// of health bits the host reads (hgpu_health, hgpu_batch_problem_health).
#pragma once
#include "kernels.h"

namespace hgpu {

// Bits of one interior cell of `s` (N = D + 2 conserved values, AoS):
//   HEALTH_STATE_NONFINITE  a NaN or an infinity in any conserved value;
//   HEALTH_STATE_DENSITY    density <= 0 (-0 included), the values finite;
//   HEALTH_STATE_PRESSURE   density > 0 and pressure <= 0, i.e. 2 rho (E - rho phi) <= |m|^2
//                           (p = (gamma - 1)(E - |m|^2 / (2 rho) - rho phi)), the products
//                           and sums rounded as binary64 (or binary32) operations.
// Ghost cells are copies of interior ones (or stale stage values) and are not checked.
// The class tests are on the bit patterns (integer pipes); the products use mulI.
template <typename real, int D>
__device__ __forceinline__ unsigned stateCheckCell(const Grid& g, const real* __restrict__ s,
                                                   const real* __restrict__ pot, long long c, int x, int y, int z) {
    if (!inRange(g, x, y, z, 2, 2) || !cellOk(g, c)) return 0u;
    const int N = D + 2;
    real u[N];
#pragma unroll
    for (int j = 0; j < N; ++j) u[j] = s[(long long)N * c + j];
    if (!allFinite<real, N>(u)) return HEALTH_STATE_NONFINITE;
    const real rho = u[0];
    if (!geZero(rho) || isZeroBits(rho)) return HEALTH_STATE_DENSITY;
    real m2 = mulI(u[1], u[1]);
#pragma unroll
    for (int j = 2; j < N - 1; ++j) m2 = m2 + mulI(u[j], u[j]);
    real twoRhoE = mulI((real)2, mulI(rho, u[N - 1]));
    if (pot) twoRhoE = twoRhoE - mulI((real)2, mulI(mulI(rho, rho), pot[c]));
    if (!(twoRhoE > m2)) return HEALTH_STATE_PRESSURE;
    return 0u;
}

// OR of `bits` over the warp; lane 0 of a warp with a nonzero result ORs it into w0
// (and w1 if given).  All 32 lanes must call it.
__device__ __forceinline__ void warpHealthOr(unsigned bits, unsigned* w0, unsigned* w1 = nullptr) {
    const unsigned all = __reduce_or_sync(0xffffffffu, bits);
    if (all && (threadIdx.x & 31) == 0) {
        atomicOr(w0, all);
        if (w1) atomicOr(w1, all);
    }
}

}  // namespace hgpu
