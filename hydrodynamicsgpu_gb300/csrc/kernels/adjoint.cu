// adjoint.cu -- vector-Jacobian products of the EulerRoe step for sm_103a (FP64).
//
// Forward pieces being differentiated (all per face, normal frame of the face):
//   Delta-q-tilde  dq = L (u_R - u_L)                                  res/Roe.cl:152-168
//   flux           ft_i = lam_i (L avg)_i - .5 lam_i dq_i (theta_i + phi(r_i) (lam_i dt/dx - theta_i))
//                  F = R ft,  avg = .5 (u_L + u_R),  r_i = dq_upwind,i / dq_i    res/Roe.cl:170-320
//   divergence     dU_c/dt = -(F_{c+1} - F_c) / dx   (interior cells)         res/CalcFluxDeriv.cl:7-44
//   eigenbasis     Roe averages of (v, H) with weights sqrt(rho)               res/EulerRoe.cl:51-226
// The eigenvector matrices depend on the face parameters p = (vx, vt..., H, c).  With
// Q = (gamma-1)(.5|v|^2 x_0 - vx x_1 - vt.x_t + x_E), W = vx x_0 - x_1 and id = .5/c^2,
//   L x = [ (Q + cW) id,  x_0 - 2Q id,  x_t - vt x_0,  (Q - cW) id ]
// so  g.(L x) = a Q + b W + g_1 x_0 + sum_t g_t (x_t - vt x_0),  a = id (g_0 + g_E - 2 g_1),
// b = c id (g_0 - g_E), which gives L^T g and d(g.Lx)/dp in a few operations; R f is
// handled the same way from its rows.  The limiter's derivative is the derivative of
// the branch the forward selected (dual numbers through the same min/max choices).
// All cotangents are gathered, not scattered: every kernel writes only its own face or cell.
#include "adjoint.h"
#include "common.cuh"
#include "roe.cuh"
#include "roe_cells.cuh"
#include "limiter_dual.cuh"

namespace hgpu {
namespace {

constexpr int kT = 256;
inline unsigned blocksFor(long long n) { return (unsigned)((n + kT - 1) / kT); }

// face parameters from the compact record (normal frame)
template <int D>
struct FaceParams {
    double vx, vt[2], vv, H, c, id, lam0, lamE, hm, hp, hv2;
};
template <int D>
__device__ __forceinline__ void loadParams(const double* __restrict__ B, long long V, int side, long long f,
                                           FaceParams<D>& p) {
    typedef RoeRec<D> R_;
    const double* b = B + (long long)side * R_::NB * V + f;
    p.vx = b[R_::VX * V];
    p.vt[0] = p.vt[1] = 0.;
#pragma unroll
    for (int t = 0; t < D - 1; ++t) p.vt[t] = b[(R_::VT + t) * V];
    p.lam0 = b[R_::LAM0 * V];
    p.lamE = b[R_::LAME * V];
    p.hm = b[R_::HM * V];
    p.hp = b[R_::HP * V];
    p.hv2 = b[R_::HV2 * V];
    // (scalings by 1/2 and 2 by the exponent, exact, on the integer pipes)
    p.vv = p.hv2 + p.hv2;
    p.c = halfOf(p.lamE - p.lam0);
    p.H = halfOf(p.hm + p.hp);
    p.id = divI(.5, p.c * p.c);
}

// g.(L x): writes L^T g into gx and adds d(g.Lx)/d(vx, vt, c) into gp (H does not enter L)
template <int D>
__device__ __forceinline__ void leftVJP(const FaceParams<D>& p, double gm1, const double* g, const double* x,
                                        double* gx, double* gp) {
    const int E = D + 1;
    double vtx = 0., gvt = 0.;
#pragma unroll
    for (int t = 0; t < D - 1; ++t) {
        vtx += p.vt[t] * x[2 + t];
        gvt += g[2 + t] * p.vt[t];
    }
    const double Q = gm1 * (p.hv2 * x[0] - p.vx * x[1] - vtx + x[E]);        // .5 vv = hv2
    const double W = p.vx * x[0] - x[1];
    const double a = (g[0] + g[E] - 2. * g[1]) * p.id;
    const double b = (g[0] - g[E]) * p.id * p.c;
    const double ag = a * gm1;
    gx[0] = ag * p.hv2 + b * p.vx + g[1] - gvt;
    gx[1] = -ag * p.vx - b;
#pragma unroll
    for (int t = 0; t < D - 1; ++t) gx[2 + t] = -ag * p.vt[t] + g[2 + t];
    gx[E] = ag;
    gp[0] += ag * W + b * x[0];
#pragma unroll
    for (int t = 0; t < D - 1; ++t) gp[1 + t] += ag * (p.vt[t] * x[0] - x[2 + t]) - g[2 + t] * x[0];
    gp[D + 1] -= (2. * a * Q + b * W) * (2. * p.c * p.id);   // / c
}

// one face of the flux VJP (stage k): gn = cotangent of the face flux (global frame).
// The forward's per-wave values (L avg, A, phi, phi', r, ft) come from the recording
// forward's tape (roe_record.cu).
template <int D, int SIDE>
__device__ __forceinline__ void adjFluxFace(const Grid& g, double gm1, int lim, double k,
                                            const double* __restrict__ U, const double* __restrict__ DQ,
                                            const double* __restrict__ B, const double* __restrict__ FT,
                                            const double* gFc, const double* gFl, double rdx, const AdjScratch& S,
                                            int first, long long c) {
    const int N = D + 2, E = N - 1, P = D + 2;
    const long long V = g.V, st = g.step[SIDE];
    (void)lim;
    FaceParams<D> p;
    loadParams<D>(B, V, SIDE, c, p);
    double gn[N], avg[N];
#pragma unroll
    for (int j = 0; j < N; ++j) {
        const int pj = perm<SIDE>(j);
        gn[j] = (gFc[pj] - gFl[pj]) * rdx;
        avg[j] = halfOf(U[N * (c - st) + pj] + U[N * c + pj]);
    }
    const double* T = FT + (long long)SIDE * FT_PLANES * N * V + c;
    double ft[N];
#pragma unroll
    for (int i = 0; i < N; ++i) ft[i] = T[((long long)FT_F * N + i) * V];
    // reverse through F = R ft
    double gft[N], gp[P];
#pragma unroll
    for (int q = 0; q < P; ++q) gp[q] = 0.;
    {
        double sumT = 0.;
#pragma unroll
        for (int t = 0; t < D - 1; ++t) sumT += gn[2 + t] * p.vt[t];
        gft[0] = gn[0] + gn[1] * p.lam0 + sumT + gn[E] * p.hm;
        gft[1] = gn[0] + gn[1] * p.vx + sumT + gn[E] * p.hv2;
#pragma unroll
        for (int t = 0; t < D - 1; ++t) gft[2 + t] = gn[2 + t] + gn[E] * p.vt[t];
        gft[E] = gn[0] + gn[1] * p.lamE + sumT + gn[E] * p.hp;
        const double Sf = ft[0] + ft[1] + ft[E], Df = ft[E] - ft[0];
        gp[0] += gn[1] * Sf + gn[E] * (p.c * Df + p.vx * ft[1]);
#pragma unroll
        for (int t = 0; t < D - 1; ++t) gp[1 + t] += gn[2 + t] * Sf + gn[E] * (p.vt[t] * ft[1] + ft[2 + t]);
        gp[D] += gn[E] * (ft[0] + ft[E]);
        gp[D + 1] += (gn[1] + gn[E] * p.vx) * Df;
    }
    // reverse through the limited characteristic flux
    double gy[N], gq0[N], gqM[N], gqP[N];
#pragma unroll
    for (int i = 0; i < N; ++i) {
        // ft_i = lam (y - h A), h = dq0 / 2, A = theta + phi (lam k - theta):
        // d/dlam = y - h A - h lam phi k,  d/ddq0 = -lam A / 2,  d/dphi = -h lam (lam k - theta)
        const double lam = i == 0 ? p.lam0 : (i == E ? p.lamE : p.vx);
        const bool up = geZero(lam);
        const double em = lam * k - plusMinusOne(up);
        const double dq0 = DQ[((long long)SIDE * N + i) * V + c];
        const double y = T[((long long)FT_Y * N + i) * V], A = T[((long long)FT_A * N + i) * V];
        const double phi = T[((long long)FT_PHI * N + i) * V], dphi = T[((long long)FT_DPHI * N + i) * V];
        const double gf = gft[i], t = lam * gf, h = halfOf(dq0);
        gy[i] = t;
        const double gLam = gf * y - h * (A * gf + phi * k * t);
        gq0[i] = -halfOf(A * t);
        gqM[i] = 0.;
        gqP[i] = 0.;
        // (tests and selects on the bits: double compares and selects issue to the FP64 unit)
        if (finiteNonzeroD(dphi)) {
            const double r = T[((long long)FT_R * N + i) * V];
            if (finiteD(r)) {
                // d/d(upwind dq) = gphi phi' / dq0 with gphi = -h em t, h = dq0 / 2: the dq0
                // cancels (r finite, so dq0 != 0)
                const double gUp = -halfOf(em * t * dphi);
                gq0[i] -= gUp * r;
                gqM[i] = selectD(up, gUp, 0.);
                gqP[i] = selectD(up, 0., gUp);
            }
        }
        gp[0] += gLam;
        if (i == 0) gp[D + 1] -= gLam;
        if (i == E) gp[D + 1] += gLam;
    }
    // reverse through y = L avg
    double gavg[N];
    leftVJP<D>(p, gm1, gy, avg, gavg, gp);
    const long long o = (long long)SIDE * N * V + c;
#pragma unroll
    for (int j = 0; j < N; ++j) {
        S.gAvg[o + (long long)perm<SIDE>(j) * V] = halfOf(gavg[j]);
        S.gdqSelf[o + (long long)j * V] = gq0[j];
        S.gdqToM[o + (long long)j * V] = gqM[j];
        S.gdqToP[o + (long long)j * V] = gqP[j];
    }
    double* gP = S.gParam + (long long)SIDE * P * V + c;
#pragma unroll
    for (int q = 0; q < P; ++q) gP[q * V] = first ? gp[q] : gP[q * V] + gp[q];
}

// dL/dF_k at a cell: sum_i coefF[i] lam_i (zero outside the interior, where F is not formed)
template <int N>
__device__ __forceinline__ void stageCotangent(const AdjStage& st, long long c, bool interior, double* out) {
#pragma unroll
    for (int j = 0; j < N; ++j) out[j] = 0.;
    if (!interior) return;
#pragma unroll
    for (int i = 0; i < 4; ++i) {                 // constant indices keep `st` in registers
        if (i >= st.nlam) break;
        const double w = st.coefF[i];
        if (isZeroBits(w)) continue;
        const double* l = st.lam[i] + (long long)N * c;
#pragma unroll
        for (int j = 0; j < N; ++j) out[j] += w * l[j];
    }
}

// (4 blocks per SM: the register cap's few spills cost less than the occupancy gained;
// measured 0.996 ms per backward step against 0.998 with 3 and 1.008 uncapped)
template <int D>
__global__ void __launch_bounds__(kT, 4) adjFluxKernel(Grid g, Phys<double> ph, int lim, double k0, double k1, double k2,
                                                    const double* __restrict__ U, const double* __restrict__ DQ,
                                                    const double* __restrict__ B, const double* __restrict__ FT,
                                                    AdjStage st, AdjScratch S, int first) {
    const int N = D + 2;
    long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.V) return;
    int x, y, z;
    cellCoords(g, c, x, y, z);
    const double gm1 = ph.gamma - 1.;
    double gFc[N];
    stageCotangent<N>(st, c, inRange(g, x, y, z, 2, 2), gFc);
    const int co[3] = {x, y, z};
    const double ks[3] = {k0, k1, k2};
#pragma unroll
    for (int side = 0; side < D; ++side) {
        if (!roeFace(g, side, x, y, z, 2, 1)) continue;
        int cl[3] = {co[0], co[1], co[2]};
        cl[side] -= 1;
        double gFl[N];
        stageCotangent<N>(st, c - g.step[side], inRange(g, cl[0], cl[1], cl[2], 2, 2), gFl);
        if (side == 0)
            adjFluxFace<D, 0>(g, gm1, lim, ks[0], U, DQ, B, FT, gFc, gFl, ph.rdx[0], S, first, c);
        else if (side == 1)
            adjFluxFace<D, (D > 1 ? 1 : 0)>(g, gm1, lim, ks[1], U, DQ, B, FT, gFc, gFl, ph.rdx[1], S, first, c);
        else
            adjFluxFace<D, (D > 2 ? 2 : 0)>(g, gm1, lim, ks[2], U, DQ, B, FT, gFc, gFl, ph.rdx[2], S, first, c);
    }
}

template <int D, int SIDE>
__device__ __forceinline__ void adjDeltaQFace(const Grid& g, double gm1, const double* __restrict__ U,
                                              const double* __restrict__ B, const AdjScratch& S, long long c) {
    const int N = D + 2, P = D + 2;
    const long long V = g.V, st = g.step[SIDE];
    FaceParams<D> p;
    loadParams<D>(B, V, SIDE, c, p);
    const long long o = (long long)SIDE * N * V + c;
    double gq[N], x[N], gx[N], gp[P];
#pragma unroll
    for (int i = 0; i < N; ++i) {
        const long long oi = o + (long long)i * V;
        gq[i] = S.gdqSelf[oi] + S.gdqToP[oi - st] + S.gdqToM[oi + st];
    }
#pragma unroll
    for (int j = 0; j < N; ++j) {
        const int pj = perm<SIDE>(j);
        x[j] = U[N * c + pj] - U[N * (c - st) + pj];
    }
#pragma unroll
    for (int q = 0; q < P; ++q) gp[q] = 0.;
    leftVJP<D>(p, gm1, gq, x, gx, gp);
#pragma unroll
    for (int j = 0; j < N; ++j) S.gDelta[o + (long long)perm<SIDE>(j) * V] = gx[j];
    double* gP = S.gParam + (long long)SIDE * P * V + c;
#pragma unroll
    for (int q = 0; q < P; ++q) gP[q * V] += gp[q];
}

template <int D>
__global__ void __launch_bounds__(kT) adjDeltaQKernel(Grid g, Phys<double> ph, const double* __restrict__ U,
                                                      const double* __restrict__ B, AdjScratch S) {
    long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.V) return;
    int x, y, z;
    cellCoords(g, c, x, y, z);
    const double gm1 = ph.gamma - 1.;
    if (roeFace(g, 0, x, y, z, 2, 1)) adjDeltaQFace<D, 0>(g, gm1, U, B, S, c);
    if (D > 1 && roeFace(g, 1, x, y, z, 2, 1)) adjDeltaQFace<D, (D > 1 ? 1 : 0)>(g, gm1, U, B, S, c);
    if (D > 2 && roeFace(g, 2, x, y, z, 2, 1)) adjDeltaQFace<D, (D > 2 ? 2 : 0)>(g, gm1, U, B, S, c);
}

// lambda_k = sum_i alpha_i lam_i + face cotangents of this cell (right cell of face c,
// left cell of face c + step on every axis)
template <int D>
__global__ void __launch_bounds__(kT) adjCellsKernel(Grid g, AdjStage st, AdjScratch S, double* __restrict__ out) {
    const int N = D + 2;
    long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.V) return;
    int x, y, z;
    cellCoords(g, c, x, y, z);
    const int co[3] = {x, y, z};
    double acc[N];
#pragma unroll
    for (int j = 0; j < N; ++j) acc[j] = 0.;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        if (i >= st.nlam) break;
        const double a = st.alpha[i];
        if (isZeroBits(a)) continue;
        const double* l = st.lam[i] + (long long)N * c;
#pragma unroll
        for (int j = 0; j < N; ++j) acc[j] += a * l[j];
    }
    const long long V = g.V;
#pragma unroll
    for (int side = 0; side < D; ++side) {
        const long long o = (long long)side * N * V + c;
#pragma unroll
        for (int j = 0; j < N; ++j) acc[j] += S.gAvg[o + j * V] + S.gDelta[o + j * V];
        if (co[side] + 1 < g.S[side]) {
            const long long o2 = o + g.step[side];
#pragma unroll
            for (int j = 0; j < N; ++j) acc[j] += S.gAvg[o2 + j * V] - S.gDelta[o2 + j * V];
        }
    }
#pragma unroll
    for (int j = 0; j < N; ++j) out[(long long)N * c + j] = acc[j];
}

// eigenbasis parameters -> (v..., h, w) of both cells of the face (Roe averages)
template <int D, int SIDE>
__device__ __forceinline__ void adjBasisFace(const Grid& g, const Phys<double>& ph, const double* __restrict__ U,
                                             const AdjScratch& S, long long c) {
    const int N = D + 2, P = D + 2;
    const long long V = g.V, st = g.step[SIDE];
    const double gm1 = ph.gamma - 1.;
    double sL[N], sR[N];
#pragma unroll
    for (int j = 0; j < N; ++j) {
        sL[j] = U[N * (c - st) + j];
        sR[j] = U[N * c + j];
    }
    RoePrim<double, D> L, R;
    roePrim<double, D>(sL, ph.gamma, L);
    roePrim<double, D>(sR, ph.gamma, R);
    const double norm = divI(1., L.w + R.w);
    const double wL = L.w * norm, wR = R.w * norm;              // d(average) / d(side value)
    double v[3] = {0., 0., 0.}, vv = 0.;
#pragma unroll
    for (int k = 0; k < D; ++k) {
        v[k] = wL * L.v[k] + wR * R.v[k];
        vv += v[k] * v[k];
    }
    const double H = wL * L.h + wR * R.h;
    const double c0 = sqrt((H - halfOf(vv)) * gm1);
    const double* gP = S.gParam + (long long)SIDE * P * V + c;
    const double gc = gP[(D + 1) * V];
    const double gcs = divI(halfOf(gc * gm1), c0);     // dc/dH; dc/dv_k = -gcs v_k
    double gv[3] = {0., 0., 0.};
    gv[SIDE] = gP[0];
    if (D > 1) gv[SIDE == 1 ? 0 : 1] = gP[1 * V];
    if (D > 2) gv[SIDE == 2 ? 0 : 2] = gP[2 * V];
    const double gH = gP[D * V] + gcs;
    double gwL = gH * (L.h - H), gwR = gH * (R.h - H);
#pragma unroll
    for (int k = 0; k < D; ++k) {
        gv[k] -= gcs * v[k];
        gwL += gv[k] * (L.v[k] - v[k]);
        gwR += gv[k] * (R.v[k] - v[k]);
    }
    double* oL = S.gPrimL + (long long)SIDE * P * V + c;
    double* oR = S.gPrimR + (long long)SIDE * P * V + c;
#pragma unroll
    for (int k = 0; k < D; ++k) {
        oL[k * V] = gv[k] * wL;
        oR[k * V] = gv[k] * wR;
    }
    oL[D * V] = gH * wL;
    oR[D * V] = gH * wR;
    oL[(D + 1) * V] = gwL * norm;
    oR[(D + 1) * V] = gwR * norm;
}

template <int D>
__global__ void __launch_bounds__(kT) adjBasisKernel(Grid g, Phys<double> ph, const double* __restrict__ U,
                                                     AdjScratch S) {
    long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.V) return;
    int x, y, z;
    cellCoords(g, c, x, y, z);
    if (roeFace(g, 0, x, y, z, 2, 1)) adjBasisFace<D, 0>(g, ph, U, S, c);
    if (D > 1 && roeFace(g, 1, x, y, z, 2, 1)) adjBasisFace<D, (D > 1 ? 1 : 0)>(g, ph, U, S, c);
    if (D > 2 && roeFace(g, 2, x, y, z, 2, 1)) adjBasisFace<D, (D > 2 ? 2 : 0)>(g, ph, U, S, c);
}

// (v..., h, w) cotangents of a cell -> its conserved state, added to lam
//   v_k = m_k / rho,  h = gamma E / rho - (gamma - 1) .5 |v|^2,  w = sqrt(rho)
template <int D>
__global__ void __launch_bounds__(kT) adjPrimsKernel(Grid g, Phys<double> ph, const double* __restrict__ U,
                                                     AdjScratch S, double* __restrict__ lam) {
    const int N = D + 2, P = D + 2, E = N - 1;
    long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.V) return;
    int x, y, z;
    cellCoords(g, c, x, y, z);
    const int co[3] = {x, y, z};
    const long long V = g.V;
    double gp[P];
#pragma unroll
    for (int q = 0; q < P; ++q) gp[q] = 0.;
    bool any = false;
#pragma unroll
    for (int side = 0; side < D; ++side) {
        if (roeFace(g, side, x, y, z, 2, 1)) {
            any = true;
#pragma unroll
            for (int q = 0; q < P; ++q) gp[q] += S.gPrimR[((long long)side * P + q) * V + c];
        }
        if (co[side] + 1 < g.S[side]) {
            int cn[3] = {co[0], co[1], co[2]};
            cn[side] += 1;
            if (roeFace(g, side, cn[0], cn[1], cn[2], 2, 1)) {
                any = true;
#pragma unroll
                for (int q = 0; q < P; ++q) gp[q] += S.gPrimL[((long long)side * P + q) * V + c + g.step[side]];
            }
        }
    }
    if (!any) return;
    const double* s = U + (long long)N * c;
    const double rho = s[0], ir = divI(1., rho), gm1 = ph.gamma - 1.;
    double v[3], vv = 0.;
#pragma unroll
    for (int k = 0; k < D; ++k) {
        v[k] = s[1 + k] * ir;
        vv += v[k] * v[k];
    }
    const double eTot = s[E] * ir;
    const double gh = gp[D], gw = gp[D + 1];
    double* l = lam + (long long)N * c;
    double grho = gh * (gm1 * vv - ph.gamma * eTot);
#pragma unroll
    for (int k = 0; k < D; ++k) {
        grho -= gp[k] * v[k];
        l[1 + k] += (gp[k] - gh * gm1 * v[k]) * ir;
    }
    l[E] += gh * ph.gamma * ir;
    l[0] += grho * ir + divI(gw * .5, sqrt(rho));
}

// transposed ghost fill of one line along `axis` (boundaryLine run backwards)
__global__ void adjBoundaryKernel(Grid g, int axis, int N, int mMin, int mMax, double* __restrict__ lam) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int A = axis == 0 ? 1 : 0, B = axis == 2 ? 1 : 2;
    long long nA = g.S[A], nB = g.S[B];
    if (g.dim == 1) { nA = 1; nB = 1; }
    if (t >= nA * nB) return;
    int a = (int)(t % nA), b = (int)(t / nA);
    int cc[3];
    cc[A] = a; cc[B] = b; cc[axis] = 0;
    long long base = cc[0] + (long long)g.S[0] * (cc[1] + (long long)g.S[1] * cc[2]);
    long long stp = g.step[axis];
    int S = g.S[axis];
    for (int j = 0; j < N; ++j) {
        double* p = lam + j;
#define AT(k) p[(long long)N * (base + (long long)(k) * stp)]
#define MOVE(dst, src, sgn) { AT(src) += (sgn) * AT(dst); AT(dst) = 0.; }
        for (int side = 1; side >= 0; --side) {
            int m = side == 0 ? mMin : mMax;
            if (m < 0) continue;
            int kern = m == 0 ? 0 : (m == 1 ? ((axis + 1 == j) ? 2 : 1) : 3);
            if (kern == 0) {                                  // periodic
                if (side == 0) { MOVE(1, S - 3, 1.); MOVE(0, S - 4, 1.); }
                else { MOVE(S - 1, 3, 1.); MOVE(S - 2, 2, 1.); }
            } else if (kern == 1 || kern == 2) {              // mirror / reflect
                double sg = kern == 1 ? 1. : -1.;
                if (side == 0) { MOVE(1, 2, sg); MOVE(0, 3, sg); }
                else { MOVE(S - 2, S - 3, sg); MOVE(S - 1, S - 4, sg); }
            } else {                                          // free flow
                if (side == 0) { MOVE(0, 2, 1.); MOVE(1, 2, 1.); }
                else { MOVE(S - 1, S - 3, 1.); MOVE(S - 2, S - 3, 1.); }
            }
        }
#undef MOVE
#undef AT
    }
}

}  // namespace

void launchAdjFlux(const Grid& g, const Phys<double>& ph, int limiter, const double* dtdx, const double* stage,
                   const double* dq, const double* basis, const double* fluxTape, const AdjStage& st,
                   const AdjScratch& s, int first, cudaStream_t stream) {
#define L(DD) adjFluxKernel<DD><<<blocksFor(g.V), kT, 0, stream>>>(g, ph, limiter, dtdx[0], dtdx[1], dtdx[2], stage, dq, basis, fluxTape, st, s, first)
    if (g.dim == 1) { L(1); }
    else if (g.dim == 2) { L(2); }
    else { L(3); }
#undef L
}

void launchAdjDeltaQ(const Grid& g, const Phys<double>& ph, const double* stage, const double* basis,
                     const AdjScratch& s, cudaStream_t stream) {
#define L(DD) adjDeltaQKernel<DD><<<blocksFor(g.V), kT, 0, stream>>>(g, ph, stage, basis, s)
    if (g.dim == 1) L(1);
    else if (g.dim == 2) L(2);
    else L(3);
#undef L
}

void launchAdjCells(const Grid& g, const AdjStage& st, const AdjScratch& s, double* lamOut, cudaStream_t stream) {
#define L(DD) adjCellsKernel<DD><<<blocksFor(g.V), kT, 0, stream>>>(g, st, s, lamOut)
    if (g.dim == 1) L(1);
    else if (g.dim == 2) L(2);
    else L(3);
#undef L
}

void launchAdjBasis(const Grid& g, const Phys<double>& ph, const double* u0, const AdjScratch& s,
                    cudaStream_t stream) {
#define L(DD) adjBasisKernel<DD><<<blocksFor(g.V), kT, 0, stream>>>(g, ph, u0, s)
    if (g.dim == 1) L(1);
    else if (g.dim == 2) L(2);
    else L(3);
#undef L
}

void launchAdjPrims(const Grid& g, const Phys<double>& ph, const double* u0, const AdjScratch& s, double* lam,
                    cudaStream_t stream) {
#define L(DD) adjPrimsKernel<DD><<<blocksFor(g.V), kT, 0, stream>>>(g, ph, u0, s, lam)
    if (g.dim == 1) L(1);
    else if (g.dim == 2) L(2);
    else L(3);
#undef L
}

void launchAdjBoundary(const Grid& g, const int methods[3][2], double* lam, cudaStream_t stream) {
    for (int axis = g.dim - 1; axis >= 0; --axis) {
        int A = axis == 0 ? 1 : 0, B = axis == 2 ? 1 : 2;
        long long lines = g.dim == 1 ? 1 : (long long)g.S[A] * g.S[B];
        adjBoundaryKernel<<<blocksFor(lines), kT, 0, stream>>>(g, axis, g.dim + 2, methods[axis][0], methods[axis][1],
                                                               lam);
    }
}

}  // namespace hgpu
