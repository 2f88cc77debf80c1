// hllc_cells.cuh -- per-cell bodies of the EulerHLLC kernels (res/EulerHLLC.cl),
// shared by the single-problem kernels (hllc.cu) and the batched kernels (batch.cu).
#pragma once
#include "kernels.h"

namespace hgpu {

// state rotated so the normal momentum is component 1 (EulerHLLC.cl:32-47)
template <typename real, int D, int SIDE>
__device__ __forceinline__ void loadRotated(const real* __restrict__ s, long long c, real* out) {
#pragma unroll
    for (int j = 0; j < D + 2; ++j) out[j] = s[(long long)(D + 2) * c + j];
    if (SIDE > 0) { real t = out[1]; out[1] = out[1 + SIDE]; out[1 + SIDE] = t; }
}

template <typename real, int D>
struct Prim {
    real density, invDensity, v[3], velocitySq, energyTotal, pressure, enthalpyTotal, potential;
};

// the part of primitives() that follows the velocities: |v|^2 (components in order),
// the internal energy, pressure and total enthalpy
template <typename real, int D, bool GRAV = false>
__device__ __forceinline__ void primitivesFromVelocity(real gamma, Prim<real, D>& p) {
    p.velocitySq = mulI(p.v[0], p.v[0]);
#pragma unroll
    for (int k = 1; k < D; ++k) p.velocitySq = p.velocitySq + mulI(p.v[k], p.v[k]);
    real energyKinetic = halfOf(p.velocitySq);                          // .5f * velocitySq
    real energyInternal = p.energyTotal - energyKinetic;
    if (GRAV) energyInternal = energyInternal - p.potential;
    p.pressure = (real)mulI(mulI((double)gamma - 1., (double)p.density), (double)energyInternal);
    p.enthalpyTotal = p.energyTotal + mulI(p.pressure, p.invDensity);
}

// primitive variables of a rotated state (EulerHLLC.cl:54-64 / :218-238).  GRAV: with
// the cell's potential phi (energyInternal = energyTotal - energyKinetic - phi);
// otherwise the potential is zero and that term, which would change no bit, is left out.
// `1. / densityL` and `(gamma - 1.) * ...` use double literals: FP32 promotes them.
template <typename real, int D, bool GRAV = false>
__device__ __forceinline__ void primitives(const real* st, real gamma, Prim<real, D>& p, real phi = (real)0) {
    const int E = D + 1;
    p.density = st[0];
    p.invDensity = (real)divI(1., (double)p.density);
    // VELOCITY: m/rho, by the correction step on RN(1/rho) in FP64 (fp64ops.cuh)
#pragma unroll
    for (int k = 0; k < D; ++k) p.v[k] = divByRecip(st[1 + k], p.density, p.invDensity);
    p.energyTotal = mulI(st[E], p.invDensity);
    p.potential = phi;
    primitivesFromVelocity<real, D, GRAV>(gamma, p);
}

// a face's primitives from its cell's, staged unrotated (hllcFluxTile): the velocities
// permuted as loadRotated permutes the momenta.  |v|^2 sums the rotated components in
// order; it changes only where the rotation moves the last component (3D, SIDE 2: v_z
// first), and there |v|^2, pressure and enthalpy are formed again from the rotated
// velocities, so every value is what primitives() gives for the rotated state.
template <typename real, int D, int SIDE, bool GRAV = false>
__device__ __forceinline__ void rotatePrim(const Prim<real, D>& p, real gamma, Prim<real, D>& r) {
    r = p;
    if (SIDE > 0) {
        r.v[0] = p.v[SIDE];
        r.v[SIDE] = p.v[0];
    }
    if (D == 3 && SIDE == 2) primitivesFromVelocity<real, D, GRAV>(gamma, r);
}

// sl, sr of one face (EulerHLLC.cl:85-97)
template <typename real, int D, int SIDE>
__device__ __forceinline__ void waveFaceFromPrim(const Grid& g, const Phys<real>& ph, double gq,
                                                 const Prim<real, D>& L, const Prim<real, D>& R,
                                                 real* __restrict__ waves, long long c);
template <typename real, int D, int SIDE, bool GRAV>
__device__ __forceinline__ void hllWaveFaceFromPrim(const Grid& g, const Phys<real>& ph, const Prim<real, D>& L,
                                                    const Prim<real, D>& R, real* __restrict__ waves, long long c);

template <typename real, int D, int SIDE, bool GRAV = false>
__device__ __forceinline__ void waveFace(const Grid& g, const Phys<real>& ph, double gq, const real* __restrict__ state,
                                         real* __restrict__ waves, long long c,
        const real* __restrict__ pot = nullptr) {
    if (!cellOk(g, c) || !cellOk(g, c - g.step[SIDE])) return;
    real sL[D + 2], sR[D + 2];
    loadRotated<real, D, SIDE>(state, c - g.step[SIDE], sL);
    loadRotated<real, D, SIDE>(state, c, sR);
    Prim<real, D> L, R;
    primitives<real, D, GRAV>(sL, ph.gamma, L, GRAV ? pot[c - g.step[SIDE]] : (real)0);
    primitives<real, D, GRAV>(sR, ph.gamma, R, GRAV ? pot[c] : (real)0);
    waveFaceFromPrim<real, D, SIDE>(g, ph, gq, L, R, waves, c);
}

// the rest of waveFace, given the face's two cells' primitives (rotated to the face)
template <typename real, int D, int SIDE>
__device__ __forceinline__ void waveFaceFromPrim(const Grid& g, const Phys<real>& ph, double gq,
                                                 const Prim<real, D>& L, const Prim<real, D>& R,
                                                 real* __restrict__ waves, long long c) {
    const double gm1 = (double)ph.gamma - 1.;
    real cL = (real)sqrt(mulI(gm1, (double)(L.enthalpyTotal - halfOf(L.velocitySq))));
    real cR = (real)sqrt(mulI(gm1, (double)(R.enthalpyTotal - halfOf(R.velocitySq))));
    // .5f * (pL + pR) - .5f * (vR - vL) * .5f * (rhoL + rhoR) * .5f * (cL + cR), halvings exact
    real pressureStar = (real)fmaxLibm(0., (double)(halfOf(L.pressure + R.pressure) -
                                                    mulI(halfOf(mulI(halfOf(halfOf(R.v[0] - L.v[0])),
                                                                     L.density + R.density)),
                                                         cL + cR)));
    real qL = leD(pressureStar, L.pressure) ? (real)1.
                                         : (real)sqrt(1. + mulI(gq, (double)divI(pressureStar, L.pressure) - 1.));
    real qR = leD(pressureStar, R.pressure) ? (real)1.
                                         : (real)sqrt(1. + mulI(gq, (double)divI(pressureStar, R.pressure) - 1.));
    waves[((long long)SIDE * 2 + 0) * g.V + c] = L.v[0] - mulI(cL, qL);
    waves[((long long)SIDE * 2 + 1) * g.V + c] = R.v[0] + mulI(cR, qR);
}

// EulerHLL sl, sr of one face (EulerHLL.cl:17-116): Davis direct bounded,
// sl = min(vL - cL, v - c), sr = max(vR + cR, v + c) with v, c from the Roe averages.
// `.5 * velocitySq` and `(gamma - 1.)` are double literals there (FP32 promotes).
template <typename real, int D, int SIDE, bool GRAV = false>
__device__ __forceinline__ void hllWaveFace(const Grid& g, const Phys<real>& ph, const real* __restrict__ state,
                                            real* __restrict__ waves, long long c,
        const real* __restrict__ pot = nullptr) {
    if (!cellOk(g, c) || !cellOk(g, c - g.step[SIDE])) return;
    real sL[D + 2], sR[D + 2];
    loadRotated<real, D, SIDE>(state, c - g.step[SIDE], sL);
    loadRotated<real, D, SIDE>(state, c, sR);
    Prim<real, D> L, R;
    primitives<real, D, GRAV>(sL, ph.gamma, L, GRAV ? pot[c - g.step[SIDE]] : (real)0);
    primitives<real, D, GRAV>(sR, ph.gamma, R, GRAV ? pot[c] : (real)0);
    hllWaveFaceFromPrim<real, D, SIDE, GRAV>(g, ph, L, R, waves, c);
}

// the rest of hllWaveFace, given the face's two cells' primitives (rotated to the face)
template <typename real, int D, int SIDE, bool GRAV>
__device__ __forceinline__ void hllWaveFaceFromPrim(const Grid& g, const Phys<real>& ph, const Prim<real, D>& L,
                                                    const Prim<real, D>& R, real* __restrict__ waves, long long c) {
    const double gm1 = (double)ph.gamma - 1.;
    const real cL = (real)sqrt(mulI(gm1, (double)L.enthalpyTotal - halfOf((double)L.velocitySq)));
    const real cR = (real)sqrt(mulI(gm1, (double)R.enthalpyTotal - halfOf((double)R.velocitySq)));
    const real wL = sqrt(L.density), wR = sqrt(R.density);
    const real norm = (real)divI(1., (double)(wL + wR));
    real v[3], vv;
#pragma unroll
    for (int k = 0; k < D; ++k) v[k] = mulI(mulI(wL, L.v[k]) + mulI(wR, R.v[k]), norm);
    const real H = mulI(mulI(wL, L.enthalpyTotal) + mulI(wR, R.enthalpyTotal), norm);
    vv = mulI(v[0], v[0]);
#pragma unroll
    for (int k = 1; k < D; ++k) vv = vv + mulI(v[k], v[k]);
    // - energyPotential, the Roe average of the potential (zero without GRAV: left out)
    double hc = (double)H - halfOf((double)vv);
    if (GRAV) hc = hc - (double)mulI(mulI(wL, L.potential) + mulI(wR, R.potential), norm);
    const real cs = (real)sqrt(mulI(gm1, hc));
    waves[((long long)SIDE * 2 + 0) * g.V + c] = fminLibm(L.v[0] - cL, v[0] - cs);
    waves[((long long)SIDE * 2 + 1) * g.V + c] = fmaxLibm(R.v[0] + cR, v[0] + cs);
}

// wave speeds of the faces of one cell: every axis in [2, S-2] (EulerHLLC.cl:110-131)
// (HLL: EulerHLL's wave speeds instead, EulerHLL.cl:118-138)
template <typename real, int D, bool HLL = false, bool GRAV = false>
__device__ __forceinline__ void hllcWaveCell(const Grid& g, const Phys<real>& ph, double gq,
                                             const real* __restrict__ state, real* __restrict__ waves, long long c,
                                             int x, int y, int z, const real* __restrict__ pot = nullptr) {
    if (!inRange(g, x, y, z, 2, 1)) return;
    if (HLL) {
        hllWaveFace<real, D, 0, GRAV>(g, ph, state, waves, c, pot);
        if (D > 1) hllWaveFace<real, D, (D > 1 ? 1 : 0), GRAV>(g, ph, state, waves, c, pot);
        if (D > 2) hllWaveFace<real, D, (D > 2 ? 2 : 0), GRAV>(g, ph, state, waves, c, pot);
        return;
    }
    waveFace<real, D, 0, GRAV>(g, ph, gq, state, waves, c, pot);
    if (D > 1) waveFace<real, D, (D > 1 ? 1 : 0), GRAV>(g, ph, gq, state, waves, c, pot);
    if (D > 2) waveFace<real, D, (D > 2 ? 2 : 0), GRAV>(g, ph, gq, state, waves, c, pot);
}

// cell timestep (EulerHLLC.cl:135-168): cells in [2, S-2], min over sides of
// dx / (max(0, sr(face c)) - min(0, sl(face c+1))); INFINITY elsewhere
template <typename real, int D>
__device__ __forceinline__ unsigned long long hllcDtCell(const Grid& g, const Phys<real>& ph,
                                                         const real* __restrict__ waves, long long c, int x, int y,
                                                         int z, bool& nan) {
    real result = (real)INFINITY;
    if (inRange(g, x, y, z, 2, 1)) {
#pragma unroll
        for (int side = 0; side < D; ++side) {
            if (!cellOk(g, c) || !cellOk(g, c + g.step[side])) continue;
            real srHere = waves[((long long)side * 2 + 1) * g.V + c];
            real slNext = waves[((long long)side * 2 + 0) * g.V + c + g.step[side]];
            real minLambda = (real)fminLibm(0., (double)slNext);
            real maxLambda = (real)fmaxLibm(0., (double)srHere);
            real dum = divI(ph.dx[side], maxLambda - minLambda);
            if (isNaNBits(dum)) nan = true;
            result = fminLibm(result, dum);
        }
    }
    return realBits(result);
}

template <typename real, int D, int SIDE>
__device__ __forceinline__ bool hllcFaceFromPrim(const Grid& g, const real* stL, const real* stR,
                                                 const Prim<real, D>& L, const Prim<real, D>& R,
                                                 const real* __restrict__ waves, real* __restrict__ fluxBuf,
                                                 long long c);
template <typename real, int D, int SIDE>
__device__ __forceinline__ bool hllFaceFromPrim(const Grid& g, const real* stL, const real* stR,
                                                const Prim<real, D>& L, const Prim<real, D>& R,
                                                const real* __restrict__ waves, real* __restrict__ fluxBuf,
                                                long long c);

// HLLC flux, HLLC_METHOD 2 (EulerHLLC.cl:240-418); `flux` holds the face's previous value.
template <typename real, int D, int SIDE, bool GRAV = false>
__device__ __forceinline__ bool hllcFace(const Grid& g, const Phys<real>& ph, const real* __restrict__ stage,
                                         const real* __restrict__ waves, real* __restrict__ fluxBuf, long long c,
        const real* __restrict__ pot = nullptr) {
    const int N = D + 2;
    if (!cellOk(g, c) || !cellOk(g, c - g.step[SIDE])) return true;
    real stL[N], stR[N];
    loadRotated<real, D, SIDE>(stage, c - g.step[SIDE], stL);
    loadRotated<real, D, SIDE>(stage, c, stR);
    Prim<real, D> L, R;
    primitives<real, D, GRAV>(stL, ph.gamma, L, GRAV ? pot[c - g.step[SIDE]] : (real)0);
    primitives<real, D, GRAV>(stR, ph.gamma, R, GRAV ? pot[c] : (real)0);
    return hllcFaceFromPrim<real, D, SIDE>(g, stL, stR, L, R, waves, fluxBuf, c);
}

// the rest of hllcFace, given the face's rotated states and their primitives
template <typename real, int D, int SIDE>
__device__ __forceinline__ bool hllcFaceFromPrim(const Grid& g, const real* stL, const real* stR,
                                                 const Prim<real, D>& L, const Prim<real, D>& R,
                                                 const real* __restrict__ waves, real* __restrict__ fluxBuf,
                                                 long long c) {
    const int N = D + 2, E = N - 1;
    real sl = waves[((long long)SIDE * 2 + 0) * g.V + c];
    real sr = waves[((long long)SIDE * 2 + 1) * g.V + c];
    real fL[N], fR[N], flux[N];
    fL[0] = mulI(L.density, L.v[0]);
    fL[1] = mulI(mulI(L.density, L.v[0]), L.v[0]) + L.pressure;
#pragma unroll
    for (int k = 1; k < D; ++k) fL[1 + k] = mulI(mulI(L.density, L.v[k]), L.v[0]);
    fL[E] = mulI(mulI(L.density, L.enthalpyTotal), L.v[0]);
    fR[0] = mulI(R.density, R.v[0]);
    fR[1] = mulI(mulI(R.density, R.v[0]), R.v[0]) + R.pressure;
#pragma unroll
    for (int k = 1; k < D; ++k) fR[1 + k] = mulI(mulI(R.density, R.v[k]), R.v[0]);
    fR[E] = mulI(mulI(R.density, R.enthalpyTotal), R.v[0]);
    real sStar = divI(mulI(mulI(R.density, R.v[0]), sr - R.v[0]) - mulI(mulI(L.density, L.v[0]), sl - L.v[0]) +
                          L.pressure - R.pressure,
                      mulI(R.density, sr - R.v[0]) - mulI(L.density, sl - L.v[0]));
    bool taken = true;
    // (the branch tests on the bit patterns: double compares issue to the FP64 unit)
    if (geZero(sl)) {
#pragma unroll
        for (int i = 0; i < N; ++i) flux[i] = fL[i];
    } else if (leZero(sl) && geZero(sStar)) {
        real pressureLR = halfOf(L.pressure + R.pressure + mulI(mulI(L.density, sl - L.v[0]), sStar - L.v[0]) +
                                 mulI(mulI(R.density, sr - R.v[0]), sStar - R.v[0]));
        // every component divides by (sl - sStar): one reciprocal, then exact corrected quotients
        real den = sl - sStar, rden = divI((real)1., den);
        flux[0] = divByRecip(mulI(sStar, mulI(sl, stL[0]) - fL[0]), den, rden);
        flux[1] = divByRecip(mulI(sStar, mulI(sl, stL[1]) - fL[1]) + mulI(sl, pressureLR), den, rden);
#pragma unroll
        for (int k = 1; k < D; ++k) flux[1 + k] = divByRecip(mulI(sStar, mulI(sl, stL[1 + k]) - fL[1 + k]), den, rden);
        flux[E] = divByRecip(mulI(sStar, mulI(sl, stL[E]) - fL[E]) + mulI(mulI(sl, pressureLR), sStar), den, rden);
    } else if (leZero(sStar) && geZero(sr)) {
        real pressureLR = halfOf(L.pressure + R.pressure + mulI(mulI(L.density, sl - L.v[0]), sStar - L.v[0]) +
                                 mulI(mulI(R.density, sr - R.v[0]), sStar - R.v[0]));
        real den = sr - sStar, rden = divI((real)1., den);
        flux[0] = divByRecip(mulI(sStar, mulI(sr, stR[0]) - fR[0]), den, rden);
        flux[1] = divByRecip(mulI(sStar, mulI(sr, stR[1]) - fR[1]) + mulI(sr, pressureLR), den, rden);
#pragma unroll
        for (int k = 1; k < D; ++k) flux[1 + k] = divByRecip(mulI(sStar, mulI(sr, stR[1 + k]) - fR[1 + k]), den, rden);
        flux[E] = divByRecip(mulI(sStar, mulI(sr, stR[E]) - fR[E]) + mulI(mulI(sr, pressureLR), sStar), den, rden);
    } else if (leZero(sr)) {
#pragma unroll
        for (int i = 0; i < N; ++i) flux[i] = fR[i];
    } else {
        // no branch: the reference leaves the buffer's previous (global-frame) value,
        // then applies the rotate-back swap to it
        taken = false;
#pragma unroll
        for (int j = 0; j < N; ++j) flux[j] = fluxBuf[((long long)SIDE * N + j) * g.V + c];
    }
    if (SIDE > 0) { real t = flux[1]; flux[1] = flux[1 + SIDE]; flux[1 + SIDE] = t; }
#pragma unroll
    for (int j = 0; j < N; ++j) fluxBuf[((long long)SIDE * N + j) * g.V + c] = flux[j];
    return taken;
}

// EulerHLL flux (EulerHLL.cl:185-346): fL, fR, or the two-state HLL flux
// (sr fL - sl fR + sl sr (uR - uL)) / (sr - sl); `flux` holds the face's previous value.
template <typename real, int D, int SIDE, bool GRAV = false>
__device__ __forceinline__ bool hllFace(const Grid& g, const Phys<real>& ph, const real* __restrict__ stage,
                                        const real* __restrict__ waves, real* __restrict__ fluxBuf, long long c,
        const real* __restrict__ pot = nullptr) {
    const int N = D + 2;
    if (!cellOk(g, c) || !cellOk(g, c - g.step[SIDE])) return true;
    real stL[N], stR[N];
    loadRotated<real, D, SIDE>(stage, c - g.step[SIDE], stL);
    loadRotated<real, D, SIDE>(stage, c, stR);
    Prim<real, D> L, R;
    primitives<real, D, GRAV>(stL, ph.gamma, L, GRAV ? pot[c - g.step[SIDE]] : (real)0);
    primitives<real, D, GRAV>(stR, ph.gamma, R, GRAV ? pot[c] : (real)0);
    return hllFaceFromPrim<real, D, SIDE>(g, stL, stR, L, R, waves, fluxBuf, c);
}

// the rest of hllFace, given the face's rotated states and their primitives
template <typename real, int D, int SIDE>
__device__ __forceinline__ bool hllFaceFromPrim(const Grid& g, const real* stL, const real* stR,
                                                const Prim<real, D>& L, const Prim<real, D>& R,
                                                const real* __restrict__ waves, real* __restrict__ fluxBuf,
                                                long long c) {
    const int N = D + 2, E = N - 1;
    const real sl = waves[((long long)SIDE * 2 + 0) * g.V + c];
    const real sr = waves[((long long)SIDE * 2 + 1) * g.V + c];
    real fL[N], fR[N], flux[N];
    fL[0] = mulI(L.density, L.v[0]);
    fL[1] = mulI(mulI(L.density, L.v[0]), L.v[0]) + L.pressure;
#pragma unroll
    for (int k = 1; k < D; ++k) fL[1 + k] = mulI(mulI(L.density, L.v[k]), L.v[0]);
    fL[E] = mulI(mulI(L.density, L.enthalpyTotal), L.v[0]);
    fR[0] = mulI(R.density, R.v[0]);
    fR[1] = mulI(mulI(R.density, R.v[0]), R.v[0]) + R.pressure;
#pragma unroll
    for (int k = 1; k < D; ++k) fR[1 + k] = mulI(mulI(R.density, R.v[k]), R.v[0]);
    fR[E] = mulI(mulI(R.density, R.enthalpyTotal), R.v[0]);
    bool taken = true;
    if (geZero(sl)) {
#pragma unroll
        for (int i = 0; i < N; ++i) flux[i] = fL[i];
    } else if (leZero(sl) && geZero(sr)) {
        const real invDenom = (real)divI(1., (double)(sr - sl));
        const real slsr = mulI(sl, sr);
#pragma unroll
        for (int i = 0; i < N; ++i)
            flux[i] = mulI(mulI(sr, fL[i]) - mulI(sl, fR[i]) + mulI(slsr, stR[i] - stL[i]), invDenom);
    } else if (leZero(sr)) {
#pragma unroll
        for (int i = 0; i < N; ++i) flux[i] = fR[i];
    } else {
        taken = false;                       // no branch: the previous (global-frame) value, swapped again
#pragma unroll
        for (int j = 0; j < N; ++j) flux[j] = fluxBuf[((long long)SIDE * N + j) * g.V + c];
    }
    if (SIDE > 0) { real t = flux[1]; flux[1] = flux[1 + SIDE]; flux[1 + SIDE] = t; }
#pragma unroll
    for (int j = 0; j < N; ++j) fluxBuf[((long long)SIDE * N + j) * g.V + c] = flux[j];
    return taken;
}

// HLLC fluxes of the faces of one cell: along [2, S-2], transverse interior [2, S-3]
// (the faces calcFluxDeriv reads).  Returns false if a face took no flux branch.
// (HLL: the EulerHLL flux instead)
template <typename real, int D, bool HLL = false, bool GRAV = false>
__device__ __forceinline__ bool hllcFluxCell(const Grid& g, const Phys<real>& ph, const real* __restrict__ stage,
                                             const real* __restrict__ waves, real* __restrict__ flux, long long c,
                                             int x, int y, int z, const real* __restrict__ pot = nullptr) {
    bool ok = true;
    int cc[3] = {x, y, z};
#pragma unroll
    for (int side = 0; side < D; ++side) {
        bool in = true;
        for (int a = 0; a < D; ++a) {
            int hi = a == side ? 1 : 2;
            if (cc[a] < 2 || cc[a] >= g.S[a] - hi) in = false;
        }
        if (!in) continue;
        if (HLL) {
            if (side == 0) ok &= hllFace<real, D, 0, GRAV>(g, ph, stage, waves, flux, c, pot);
            else if (side == 1) ok &= hllFace<real, D, (D > 1 ? 1 : 0), GRAV>(g, ph, stage, waves, flux, c, pot);
            else ok &= hllFace<real, D, (D > 2 ? 2 : 0), GRAV>(g, ph, stage, waves, flux, c, pot);
        } else {
            if (side == 0) ok &= hllcFace<real, D, 0, GRAV>(g, ph, stage, waves, flux, c, pot);
            else if (side == 1) ok &= hllcFace<real, D, (D > 1 ? 1 : 0), GRAV>(g, ph, stage, waves, flux, c, pot);
            else ok &= hllcFace<real, D, (D > 2 ? 2 : 0), GRAV>(g, ph, stage, waves, flux, c, pot);
        }
    }
    return ok;
}

// primitives of the tile's cells and of one cell below along every axis, into `prim`
// (HX*HY*HZ entries, x fastest); the caller synchronises
template <typename real, int D, bool GRAV>
__device__ __forceinline__ void stagePrims(const Grid& g, const Phys<real>& ph, const real* __restrict__ st,
                                           int x0, int y0, int z0, int HX, int HY, int HZ, Prim<real, D>* prim,
                                           const real* __restrict__ pot) {
    const int N = D + 2;
    const int ox = 1, oy = D > 1 ? 1 : 0, oz = D > 2 ? 1 : 0;
    for (int i = threadIdx.x; i < HX * HY * HZ; i += blockDim.x) {
        int hx = i % HX, hy = (i / HX) % HY, hz = i / (HX * HY);
        int gx = x0 - ox + hx, gy = y0 - oy + hy, gz = z0 - oz + hz;
        if (gx >= 0 && gx < g.S[0] && gy >= 0 && gy < g.S[1] && gz >= 0 && gz < g.S[2]) {
            long long c = gx + (long long)g.S[0] * (gy + (long long)g.S[1] * gz);
            if (cellOk(g, c)) {
                real s[N];
#pragma unroll
                for (int j = 0; j < N; ++j) s[j] = st[(long long)N * c + j];
                primitives<real, D, GRAV>(s, ph.gamma, prim[i], GRAV ? pot[c] : (real)0);
            }
        }
    }
}

// The wave speeds of a tile's cells' faces (hllcWaveCell) with each cell's primitives
// formed once and rotated to each face (rotatePrim), as hllcFluxTile does for the flux.
// Cells with slow-axis coordinate outside [s0, s1) are staged only.
template <typename real, int D, bool HLL = false, bool GRAV = false>
__device__ __forceinline__ void hllcWaveTile(const Grid& g, const Phys<real>& ph, double gq,
                                             const real* __restrict__ state, real* __restrict__ waves, int x0, int y0,
                                             int z0, int TX, int TY, int TZ, int s0, int s1, Prim<real, D>* prim,
                                             const real* __restrict__ pot = nullptr) {
    const int HX = TX + 1, HY = D > 1 ? TY + 1 : 1, HZ = D > 2 ? TZ + 1 : 1;
    const int ox = 1, oy = D > 1 ? 1 : 0, oz = D > 2 ? 1 : 0;
    stagePrims<real, D, GRAV>(g, ph, state, x0, y0, z0, HX, HY, HZ, prim, pot);
    __syncthreads();
    const int tx = threadIdx.x % TX, ty = (threadIdx.x / TX) % TY, tz = threadIdx.x / (TX * TY);
    const int x = x0 + tx, y = y0 + ty, z = z0 + tz;
    const int slow = D == 2 ? y : z;
    if (tz < TZ && x < g.S[0] && y < g.S[1] && z < g.S[2] && slow >= s0 && slow < s1 && inRange(g, x, y, z, 2, 1)) {
        const long long c = x + (long long)g.S[0] * (y + (long long)g.S[1] * z);
        const int self = (tz + oz) * HY * HX + (ty + oy) * HX + (tx + ox);
        const int below[3] = {1, HX, HX * HY};
#pragma unroll
        for (int side = 0; side < D; ++side) {
            if (!cellOk(g, c) || !cellOk(g, c - g.step[side])) continue;
            Prim<real, D> L, R;
            if (side == 0) {
                rotatePrim<real, D, 0, GRAV>(prim[self - below[0]], ph.gamma, L);
                rotatePrim<real, D, 0, GRAV>(prim[self], ph.gamma, R);
                if (HLL) hllWaveFaceFromPrim<real, D, 0, GRAV>(g, ph, L, R, waves, c);
                else waveFaceFromPrim<real, D, 0>(g, ph, gq, L, R, waves, c);
            } else if (side == 1) {
                constexpr int S1 = D > 1 ? 1 : 0;
                rotatePrim<real, D, S1, GRAV>(prim[self - below[1]], ph.gamma, L);
                rotatePrim<real, D, S1, GRAV>(prim[self], ph.gamma, R);
                if (HLL) hllWaveFaceFromPrim<real, D, S1, GRAV>(g, ph, L, R, waves, c);
                else waveFaceFromPrim<real, D, S1>(g, ph, gq, L, R, waves, c);
            } else {
                constexpr int S2 = D > 2 ? 2 : 0;
                rotatePrim<real, D, S2, GRAV>(prim[self - below[2]], ph.gamma, L);
                rotatePrim<real, D, S2, GRAV>(prim[self], ph.gamma, R);
                if (HLL) hllWaveFaceFromPrim<real, D, S2, GRAV>(g, ph, L, R, waves, c);
                else waveFaceFromPrim<real, D, S2>(g, ph, gq, L, R, waves, c);
            }
        }
    }
    __syncthreads();
}

// The HLLC (HLL) fluxes of a tile of cells with each cell's primitives formed once:
// the tile plus one cell below along every axis (each face's left cell) is staged in
// `prim` (HX*HY*HZ entries), then each cell takes its faces as hllcFluxCell does, the
// primitives rotated to the face (rotatePrim) instead of formed from the rotated
// state (every face otherwise formed its two cells' primitives).  Cells with slow-axis
// coordinate outside [s0, s1) (y in 2D, z in 3D) are staged only.  Returns through
// `ok` whether every face took a flux branch.
template <typename real, int D, bool HLL = false, bool GRAV = false>
__device__ __forceinline__ bool hllcFluxTile(const Grid& g, const Phys<real>& ph, const real* __restrict__ stage,
                                             const real* __restrict__ waves, real* __restrict__ flux, int x0, int y0,
                                             int z0, int TX, int TY, int TZ, int s0, int s1, Prim<real, D>* prim,
                                             const real* __restrict__ pot = nullptr) {
    const int N = D + 2;
    const int HX = TX + 1, HY = D > 1 ? TY + 1 : 1, HZ = D > 2 ? TZ + 1 : 1;
    const int ox = 1, oy = D > 1 ? 1 : 0, oz = D > 2 ? 1 : 0;
    stagePrims<real, D, GRAV>(g, ph, stage, x0, y0, z0, HX, HY, HZ, prim, pot);
    __syncthreads();
    bool ok = true;
    const int tx = threadIdx.x % TX, ty = (threadIdx.x / TX) % TY, tz = threadIdx.x / (TX * TY);
    const int x = x0 + tx, y = y0 + ty, z = z0 + tz;
    const int slow = D == 2 ? y : z;
    if (tz < TZ && x < g.S[0] && y < g.S[1] && z < g.S[2] && slow >= s0 && slow < s1) {
        const long long c = x + (long long)g.S[0] * (y + (long long)g.S[1] * z);
        const int self = (tz + oz) * HY * HX + (ty + oy) * HX + (tx + ox);
        const int cc[3] = {x, y, z};
        const int below[3] = {1, HX, HX * HY};
#pragma unroll
        for (int side = 0; side < D; ++side) {
            bool in = true;
            for (int a = 0; a < D; ++a) {
                int hi = a == side ? 1 : 2;
                if (cc[a] < 2 || cc[a] >= g.S[a] - hi) in = false;
            }
            if (!in || !cellOk(g, c) || !cellOk(g, c - g.step[side])) continue;
            real stL[N], stR[N];
            Prim<real, D> L, R;
            if (side == 0) {
                loadRotated<real, D, 0>(stage, c - g.step[0], stL);
                loadRotated<real, D, 0>(stage, c, stR);
                rotatePrim<real, D, 0, GRAV>(prim[self - below[0]], ph.gamma, L);
                rotatePrim<real, D, 0, GRAV>(prim[self], ph.gamma, R);
                ok &= HLL ? hllFaceFromPrim<real, D, 0>(g, stL, stR, L, R, waves, flux, c)
                          : hllcFaceFromPrim<real, D, 0>(g, stL, stR, L, R, waves, flux, c);
            } else if (side == 1) {
                constexpr int S1 = D > 1 ? 1 : 0;
                loadRotated<real, D, S1>(stage, c - g.step[1], stL);
                loadRotated<real, D, S1>(stage, c, stR);
                rotatePrim<real, D, S1, GRAV>(prim[self - below[1]], ph.gamma, L);
                rotatePrim<real, D, S1, GRAV>(prim[self], ph.gamma, R);
                ok &= HLL ? hllFaceFromPrim<real, D, S1>(g, stL, stR, L, R, waves, flux, c)
                          : hllcFaceFromPrim<real, D, S1>(g, stL, stR, L, R, waves, flux, c);
            } else {
                constexpr int S2 = D > 2 ? 2 : 0;
                loadRotated<real, D, S2>(stage, c - g.step[2], stL);
                loadRotated<real, D, S2>(stage, c, stR);
                rotatePrim<real, D, S2, GRAV>(prim[self - below[2]], ph.gamma, L);
                rotatePrim<real, D, S2, GRAV>(prim[self], ph.gamma, R);
                ok &= HLL ? hllFaceFromPrim<real, D, S2>(g, stL, stR, L, R, waves, flux, c)
                          : hllcFaceFromPrim<real, D, S2>(g, stL, stR, L, R, waves, flux, c);
            }
        }
    }
    __syncthreads();
    return ok;
}

}  // namespace hgpu
