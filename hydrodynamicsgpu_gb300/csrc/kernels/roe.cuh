// roe.cuh -- Roe eigenbasis, characteristic transforms and limited flux (device code).
//
// The scheme is HydroGPU's EulerRoe (res/EulerRoe.cl:18-259, res/Roe.cl:4-320,
// res/RoeEigenfieldLinear.cl:16-74): per interface the Roe-averaged state gives
// eigenvalues, right eigenvectors R and left eigenvectors L = R^-1, built in the
// frame whose x axis is the interface normal and rotated back by swapping the
// momentum-x and momentum-side rows/columns.  Here the basis of a face is kept in
// its normal frame as a compact record of the distinct matrix entries; the swap is
// applied as an index permutation when the matrices are used.  Every entry is
// computed with the reference's expression and operation order, so the values are
// bit-identical; sums over matrix columns keep the reference's column order in the
// global frame (see common.cuh for the zero/unit-coefficient rule).
#pragma once
#include "common.cuh"
#include "fp64ops.cuh"
#include "limiter_dual.cuh"

namespace hgpu {

// A product on the FP64 unit, never contracted into an fma (so the same in translation
// units built with and without --fmad=false).  The eigenbasis kernel issues far more
// integer than FP64 instructions (its quotients and the record's products on the
// integer pipes, the FP64 unit at ~59 %): its per-cell products and the left rows'
// products run here instead of through mulI, which balanced the pipes (KH 2048^2 step
// 7.703 -> 7.688 ms, the 512-problem batched sweep 24.42 -> 24.17 ms; every product
// through mulN was slower, 7.82 ms).
__device__ __forceinline__ double mulN(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float mulN(float a, float b) { return __fmul_rn(a, b); }

// record layout (per face, normal frame)
template <int D>
struct RoeRec {
    enum {
        N = D + 2,
        LAM0 = 0,   // vx - c              (= R[1][0])
        VX = 1,     // normal Roe velocity
        LAME = 2,   // vx + c              (= R[1][E])
        HM = 3,     // H - c*vx            (R[E][0])
        HV2 = 4,    // .5 * |v|^2          (R[E][1])
        HP = 5,     // H + c*vx            (R[E][E])
        VT = 6,     // tangential velocities vt[0..D-2]
        L0 = 6 + (D - 1),   // left row 0, N entries (normal frame columns)
        L1 = L0 + N,        // left row 1, N entries
        LE0 = L1 + N,       // left row E, column 0
        LE1 = LE0 + 1,      // left row E, column 1 (columns >= 2 equal row 0's)
        NB = LE1 + 1
    };
};

// global component j <-> normal-frame component for interface `side` (swap 1 <-> 1+side)
template <int SIDE>
__device__ __forceinline__ constexpr int perm(int j) { return j == 1 ? 1 + SIDE : (j == 1 + SIDE ? 1 : j); }

// Per-cell part of the Roe eigenbasis (res/EulerRoe.cl:51-83 with solid == 0,
// potential == 0): velocity, total enthalpy and Roe weight sqrt(rho).  Every face
// uses these for its two cells; computing them once per cell is exact.
template <typename real, int D>
struct RoePrim {
    real v[3];
    real h;     // enthalpyTotal
    real w;     // roeWeight = sqrt(density)
    real phi;   // energyPotential = potential of the cell (GRAV only)
};

// GRAV: a live gravitational potential phi (res/EulerRoe.cl:70-80); without it the
// potential is zero and its terms, which would change no bit, are left out.
template <typename real, int D, bool GRAV = false>
__device__ __forceinline__ void roePrim(const real* s, real gamma, RoePrim<real, D>& P, real phi = (real)0) {
    const int E = D + 1;
    const real gm1 = gamma - (real)1.f;
    real rho = s[0];
    real invDensity = divI((real)1.f, rho);                              // `1.f / density`
    // VELOCITY(ptr) = (m..., 0)/rho componentwise (res/include/HydroGPU/Euler.h:6-12);
    // m/rho by the correction step on RN(1/rho) (fp64ops.cuh) is the same quotient
#pragma unroll
    for (int k = 0; k < D; ++k) P.v[k] = divByRecip(s[1 + k], rho, invDensity);
    // dot(v,v) over 4 components; the zero components add +0 to a non-negative sum
    real vv = mulN(P.v[0], P.v[0]);
#pragma unroll
    for (int k = 1; k < D; ++k) vv = vv + mulN(P.v[k], P.v[k]);
    real energyTotal = mulN(s[E], invDensity);
    real energyKinetic = halfOf(vv);                                     // .5f * dot(v, v)
    real energyInternal = energyTotal - energyKinetic;                   // - energyPotential
    if (GRAV) energyInternal = energyInternal - phi;
    P.phi = phi;
    real pressure = mulN(mulN(gm1, rho), energyInternal);
    P.h = energyTotal + mulN(pressure, invDensity);
    P.w = sqrt(rho);
}

// Per-face part (res/EulerRoe.cl:85-226): Roe averages, eigenvalues, R and L.
template <typename real, int D, int SIDE, bool GRAV = false>
__device__ __forceinline__ void roeBasisFromPrim(const RoePrim<real, D>& L, const RoePrim<real, D>& R, real gamma,
                                                 real* rec) {
    typedef RoeRec<D> R_;
    const int E = D + 1;
    const real gm1 = gamma - (real)1.f;
    real norm = divI((real)1.f, L.w + R.w);
    real v[3];
#pragma unroll
    for (int k = 0; k < D; ++k) v[k] = mulI(mulI(L.w, L.v[k]) + mulI(R.w, R.v[k]), norm);
    real enthalpyTotal = mulI(mulI(L.w, L.h) + mulI(R.w, R.h), norm);
    real velocitySq = mulI(v[0], v[0]);
#pragma unroll
    for (int k = 1; k < D; ++k) velocitySq = velocitySq + mulI(v[k], v[k]);
    real hc = enthalpyTotal - halfOf(velocitySq);
    if (GRAV) {                                                          // - energyPotential (Roe average)
        const real energyPotential = mulI(mulI(L.w, L.phi) + mulI(R.w, R.phi), norm);
        hc = hc - energyPotential;
    }
    real c = sqrt(mulI(hc, gm1));
    // rotate: normal velocity first (res/EulerRoe.cl:101-110)
    real vx = v[SIDE];
    real vt[2] = {0, 0};
    if (D > 1) vt[0] = (SIDE == 1) ? v[0] : v[1];
    if (D > 2) vt[1] = (SIDE == 2) ? v[0] : v[2];
    real cvx = mulI(c, vx);
    rec[R_::LAM0] = vx - c;
    rec[R_::VX] = vx;
    rec[R_::LAME] = vx + c;
    rec[R_::HM] = enthalpyTotal - cvx;
    rec[R_::HV2] = halfOf(velocitySq);
#pragma unroll
    for (int t = 0; t < D - 1; ++t) rec[R_::VT + t] = vt[t];
    rec[R_::HP] = enthalpyTotal + cvx;
    real invDenom = divI((real).5f, mulI(c, c));
    real hv = mulN(mulN((real).5f, gm1), velocitySq);                    // .5f * (gamma - 1.f) * velocitySq
    real gvx = mulN(gm1, vx);
    rec[R_::L0 + 0] = mulN(hv + cvx, invDenom);
    rec[R_::L0 + 1] = mulN(-(c + gvx), invDenom);
#pragma unroll
    for (int t = 0; t < D - 1; ++t) rec[R_::L0 + 2 + t] = mulN(mulN(-gm1, vt[t]), invDenom);
    rec[R_::L0 + E] = mulN(gm1, invDenom);
    rec[R_::L1 + 0] = (real)1.f - mulN(mulN(gm1, velocitySq), invDenom);
    rec[R_::L1 + 1] = mulN(mulN(gvx, (real)2.f), invDenom);
#pragma unroll
    for (int t = 0; t < D - 1; ++t) rec[R_::L1 + 2 + t] = mulN(mulN(mulN(gm1, vt[t]), (real)2.f), invDenom);
    rec[R_::L1 + E] = mulN(mulN(-gm1, (real)2.f), invDenom);
    rec[R_::LE0] = mulN(hv - cvx, invDenom);
    rec[R_::LE1] = mulN(c - gvx, invDenom);
}

// Eigen basis of one interface from the two cell states.
template <typename real, int D, int SIDE>
__device__ __forceinline__ void roeBasis(const real* sL, const real* sR, real gamma, real* rec) {
    RoePrim<real, D> L, R;
    roePrim<real, D>(sL, gamma, L);
    roePrim<real, D>(sR, gamma, R);
    roeBasisFromPrim<real, D, SIDE>(L, R, gamma, rec);
}

// Normal-frame matrix entries, including the structural zeros and ones.
template <typename real, int D>
__device__ __forceinline__ real leftEntry(const real* rec, int i, int c) {
    typedef RoeRec<D> R_;
    const int E = D + 1;
    if (i == 0) return rec[R_::L0 + c];
    if (i == 1) return rec[R_::L1 + c];
    if (i == E) return c == 0 ? rec[R_::LE0] : (c == 1 ? rec[R_::LE1] : rec[R_::L0 + c]);
    return c == 0 ? -rec[R_::VT + i - 2] : (c == i ? (real)1.f : (real)0.f);
}
template <typename real, int D>
__device__ __forceinline__ real rightEntry(const real* rec, int i, int j) {
    typedef RoeRec<D> R_;
    const int E = D + 1;
    if (j == 0 || j == 1 || j == E) {
        if (i == 0) return (real)1.f;
        if (i == 1) return j == 0 ? rec[R_::LAM0] : (j == 1 ? rec[R_::VX] : rec[R_::LAME]);
        if (i == E) return j == 0 ? rec[R_::HM] : (j == 1 ? rec[R_::HV2] : rec[R_::HP]);
        return rec[R_::VT + i - 2];
    }
    if (i == j) return (real)1.f;
    if (i == E) return rec[R_::VT + j - 2];
    return (real)0.f;
}

// Dense forms, term for term as res/RoeEigenfieldLinear.cl:16-54 (used when an input
// is not finite: then 0 * Inf/NaN terms matter).
template <typename real, int D, int SIDE>
__device__ __forceinline__ void leftTransformDense(const real* rec, const real* x, real* y) {
    const int N = D + 2;
#pragma unroll
    for (int i = 0; i < N; ++i) {
        real s = (real)0.f;
#pragma unroll
        for (int j = 0; j < N; ++j) s = s + leftEntry<real, D>(rec, i, perm<SIDE>(j)) * x[j];
        y[i] = s;
    }
}
template <typename real, int D, int SIDE>
__device__ __forceinline__ void rightTransformDense(const real* rec, const real* f, real* F) {
    const int N = D + 2;
#pragma unroll
    for (int g = 0; g < N; ++g) {
        const int i = perm<SIDE>(g);
        real s = (real)0.f;
#pragma unroll
        for (int j = 0; j < N; ++j) s = s + rightEntry<real, D>(rec, i, j) * f[j];
        F[g] = s;
    }
}

// y = L x with L in the global frame: y_i = sum_j L[i][perm(j)] x_j, j ascending.
// FLAT: the caller's x is a difference of neighbouring states, often exactly zero.
template <typename real, int D, int SIDE, bool FLAT = false>
__device__ __forceinline__ void leftTransform(const real* rec, const real* x, real* y) {
    typedef RoeRec<D> R_;
    const int N = D + 2, E = N - 1;
    // FLAT, x zero in every component (either sign) and every record entry the rows
    // below read (VT .. LE1) finite: each product is a zero and every sum starts from
    // +0, so y is +0 throughout.  Flat states (equal neighbours) take this exit,
    // decided on the bit patterns, instead of N^2 zero products through the FP64 unit.
    if (FLAT) {
        bool flat = true;
#pragma unroll
        for (int j = 0; j < N; ++j) flat &= isZeroBits(x[j]);
        if (flat) {
#pragma unroll
            for (int k = R_::VT; k < R_::NB; ++k) flat &= finiteBits(rec[k]);
            if (flat) {
#pragma unroll
                for (int i = 0; i < N; ++i) y[i] = (real)0;
                return;
            }
        }
    }
    if (!allFinite<real, N>(x)) { leftTransformDense<real, D, SIDE>(rec, x, y); return; }
    // row 0 and row 1: dense
    {
        real s0 = zfix(mulI(rec[R_::L0 + perm<SIDE>(0)], x[0]));
        real s1 = zfix(mulI(rec[R_::L1 + perm<SIDE>(0)], x[0]));
#pragma unroll
        for (int j = 1; j < N; ++j) {
            s0 = s0 + mulI(rec[R_::L0 + perm<SIDE>(j)], x[j]);
            s1 = s1 + mulI(rec[R_::L1 + perm<SIDE>(j)], x[j]);
        }
        y[0] = s0;
        y[1] = s1;
    }
    // tangent rows t = 2..E-1: [-vt, 0, .., 1 (column t), .., 0] in the normal frame
#pragma unroll
    for (int t = 2; t < E; ++t) y[t] = zfix(mulI(-rec[R_::VT + t - 2], x[0])) + x[perm<SIDE>(t)];
    // row E: [LE0, LE1, L0[2..]] in the normal frame
    {
        real s = 0;
#pragma unroll
        for (int j = 0; j < N; ++j) {
            int c = perm<SIDE>(j);
            real m = c == 0 ? rec[R_::LE0] : (c == 1 ? rec[R_::LE1] : rec[R_::L0 + c]);
            s = (j == 0) ? zfix(mulI(m, x[0])) : s + mulI(m, x[j]);
        }
        y[E] = s;
    }
}

// F = R f in the global frame: F_rot = R_rot f (j ascending), F_glob[g] = F_rot[perm(g)].
template <typename real, int D, int SIDE>
__device__ __forceinline__ void rightTransform(const real* rec, const real* f, real* F) {
    typedef RoeRec<D> R_;
    const int N = D + 2, E = N - 1;
    if (!allFinite<real, N>(f)) { rightTransformDense<real, D, SIDE>(rec, f, F); return; }
    real Fr[5];
    // row 0: [1, 1, 0.., 1]
    Fr[0] = zfix(f[0]) + f[1] + f[E];
    // row 1: [lam0, vx, 0.., lamE]
    Fr[1] = zfix(mulI(rec[R_::LAM0], f[0])) + mulI(rec[R_::VX], f[1]) + mulI(rec[R_::LAME], f[E]);
    // tangent rows t: [vt, vt, (1 at column t), vt]
#pragma unroll
    for (int t = 2; t < E; ++t) {
        real vt = rec[R_::VT + t - 2];
        Fr[t] = ((zfix(mulI(vt, f[0])) + mulI(vt, f[1])) + f[t]) + mulI(vt, f[E]);
    }
    // row E: [H - c vx, .5 v^2, vt..., H + c vx]
    {
        real s = zfix(mulI(rec[R_::HM], f[0])) + mulI(rec[R_::HV2], f[1]);
#pragma unroll
        for (int t = 2; t < E; ++t) s = s + mulI(rec[R_::VT + t - 2], f[t]);
        Fr[E] = s + mulI(rec[R_::HP], f[E]);
    }
#pragma unroll
    for (int g = 0; g < N; ++g) F[g] = Fr[perm<SIDE>(g)];
}

template <typename real, int D>
__device__ __forceinline__ real roeEigenvalue(const real* rec, int i) {
    typedef RoeRec<D> R_;
    return i == 0 ? rec[R_::LAM0] : (i == D + 1 ? rec[R_::LAME] : rec[R_::VX]);
}

// Limited characteristic flux of one interface (res/Roe.cl:253-298).
// sL, sR: stage states; dqL, dq, dqR: Delta-q-tilde at the faces before/at/after.
// Per-wave values the adjoint reads back from a recording forward (REC): plane q of
// wave i of a face at tape[(q N + i) V] (the caller offsets tape to the face).
enum { FT_Y = 0, FT_A = 1, FT_PHI = 2, FT_DPHI = 3, FT_R = 4, FT_F = 5, FT_PLANES = 6 };

// LIM >= 0 fixes the slope limiter at compile time (the kernel then carries one
// limiter instead of all twenty at each of its wave sites); -1 dispatches on `lim`.
// REC (FP64 only) also stores the per-wave values above; the flux is the same.
template <typename real, int D, int SIDE, int LIM = -1, bool REC = false>
__device__ __forceinline__ void roeFlux(const real* rec, const real* sL, const real* sR, const real* dqL,
                                        const real* dq, const real* dqR, real dt_dx, int lim, real* F,
                                        real* __restrict__ tape = nullptr, long long V = 0) {
    typedef RoeRec<D> R_;
    const int N = D + 2;
    real avg[5], ft[5];
#pragma unroll
    for (int i = 0; i < N; ++i) avg[i] = (real)halfOf((double)(sR[i] + sL[i]));    // .5 * (stateR + stateL)
    leftTransform<real, D, SIDE>(rec, avg, ft);
    // waves 1..N-2 share the eigenvalue vx: their epsilon and theta are the same values
    const real vx = rec[R_::VX];
    const bool midUp = geZero(vx);
    const real midTheta = midUp ? (real)1. : (real)-1.;
    const real midEps = mulI(vx, dt_dx);
    const real midEpsTheta = midEps - midTheta;
#pragma unroll
    for (int i = 0; i < N; ++i) {
        const bool mid = i > 0 && i < N - 1;
        real eigenvalue = roeEigenvalue<real, D>(rec, i);
        if (REC) tape[((long long)FT_Y * N + i) * V] = ft[i];
        ft[i] = ft[i] * eigenvalue;
        bool up = mid ? midUp : geZero(eigenvalue);
        real rTilde = divI(up ? dqL[i] : dqR[i], dq[i]);
        real theta = mid ? midTheta : (up ? (real)1. : (real)-1.);
        real phi = slopeLimiter<real>(LIM >= 0 ? LIM : lim, rTilde);
        real epsMinusTheta = mid ? midEpsTheta : mulI(eigenvalue, dt_dx) - theta;
        real deltaFluxTilde = mulI(eigenvalue, dq[i]);
        // `fluxTilde[i] -= .5 * deltaFluxTilde * (theta + phi * (epsilon - theta))`
        // (the products on the path from L*avg to R*ft stay on the FP64 unit; eps and
        // lambda*dq, off that path, run on the integer pipes like the transforms)
        if (sizeof(real) == 8) {
            const real A = theta + phi * epsMinusTheta;
            ft[i] = ft[i] - halfOf(deltaFluxTilde) * A;
            if (REC) {
                tape[((long long)FT_A * N + i) * V] = A;
                tape[((long long)FT_PHI * N + i) * V] = phi;
                tape[((long long)FT_DPHI * N + i) * V] = limiterDual(LIM >= 0 ? LIM : lim, Dual{(double)rTilde, 1.}).d;
                tape[((long long)FT_R * N + i) * V] = rTilde;
                tape[((long long)FT_F * N + i) * V] = ft[i];
            }
        }
        else ft[i] -= .5 * deltaFluxTilde * (theta + phi * epsMinusTheta);   // double literal: FP32 promotes
    }
    rightTransform<real, D, SIDE>(rec, ft, F);
}


// The FP64 flux in two passes (same operations, same bits as roeFlux):
//   pass 1, per wave i: corr_i = (lambda_i dq_i / 2) (theta_i + phi(r_i) (eps_i - theta_i))
//   pass 2: ft = lambda (L avg) - corr, F = R ft
// Each pass keeps far fewer values live than the fused form, so more warps fit per SM.
// REC also stores the per-wave tape values of this pass (A, phi, phi', r; the caller
// offsets tape to the face, as for roeFlux).
// FLATQ: a wave whose Delta-q-tilde is +-0, with finite lambda and A, gets its
// correction (lambda (+-0) / 2) A as the signed zero it is (sign(lambda) xor sign(dq)
// xor sign(A)) on the bit patterns, skipping the product's and the halving's
// out-of-line FP64 calls for zero operands.  Piecewise-constant states (the batched
// four-quadrant problems) have such waves on most faces; the KH step measured it
// slower, so it is the batched kernel's choice.
template <int D, int SIDE, int LIM, bool REC = false, bool FLATQ = false>
__device__ __forceinline__ void roeFluxCorrections(const double* rec, const double* dqL, const double* dq,
                                                   const double* dqR, double dt_dx, int lim, double* corr,
                                                   double* __restrict__ tape = nullptr, long long V = 0) {
    typedef RoeRec<D> R_;
    const int N = D + 2;
    const double vx = rec[R_::VX];
    const bool midUp = geZero(vx);
    const double midTheta = plusMinusOne(midUp);
    const double midEpsTheta = mulI(vx, dt_dx) - midTheta;
#pragma unroll
    for (int i = 0; i < N; ++i) {
        const bool mid = i > 0 && i < N - 1;
        const double eigenvalue = roeEigenvalue<double, D>(rec, i);
        const bool up = mid ? midUp : geZero(eigenvalue);
        const double rTilde = divI(up ? dqL[i] : dqR[i], dq[i]);
        const double theta = plusMinusOne(up);
        const double phi = slopeLimiter<double>(LIM >= 0 ? LIM : lim, rTilde);
        const double epsMinusTheta = mid ? midEpsTheta : mulI(eigenvalue, dt_dx) - theta;
        const double A = theta + phi * epsMinusTheta;
        if (FLATQ && isZeroBits(dq[i]) && finiteD(eigenvalue) && finiteD(A))
            corr[i] = fromBits((bitsOf(eigenvalue) ^ bitsOf(dq[i]) ^ bitsOf(A)) & (long long)0x8000000000000000ULL);
        else
            corr[i] = halfOf(mulI(eigenvalue, dq[i])) * A;
        if (REC) {
            tape[((long long)FT_A * N + i) * V] = A;
            tape[((long long)FT_PHI * N + i) * V] = phi;
            tape[((long long)FT_DPHI * N + i) * V] = limiterDual(LIM >= 0 ? LIM : lim, Dual{rTilde, 1.}).d;
            tape[((long long)FT_R * N + i) * V] = rTilde;
        }
    }
}

// REC also stores the tape values of this pass (L avg, and ft after the correction)
template <int D, int SIDE, bool REC = false>
__device__ __forceinline__ void roeFluxTransforms(const double* rec, const double* sL, const double* sR,
                                                  const double* corr, double* F, double* __restrict__ tape = nullptr,
                                                  long long V = 0) {
    const int N = D + 2;
    double avg[5], ft[5];
#pragma unroll
    for (int i = 0; i < N; ++i) avg[i] = halfOf(sR[i] + sL[i]);
    leftTransform<double, D, SIDE>(rec, avg, ft);
#pragma unroll
    for (int i = 0; i < N; ++i) {
        if (REC) tape[((long long)FT_Y * N + i) * V] = ft[i];
        ft[i] = ft[i] * roeEigenvalue<double, D>(rec, i) - corr[i];
        if (REC) tape[((long long)FT_F * N + i) * V] = ft[i];
    }
    rightTransform<double, D, SIDE>(rec, ft, F);
}

}  // namespace hgpu
