// roe_cells.cuh -- per-cell and per-tile bodies of the EulerRoe kernels.
//
// Shared by the single-problem kernels (roe.cu) and the batched persistent kernels
// (batch.cu).  Each body works on one grid `g` whose buffers start at the given
// pointers; the batched kernels pass each problem's grid and offset pointers.
#pragma once
#include "kernels.h"
#include "roe.cuh"

namespace hgpu {

// faces along `side` in [loA, S-hiA), transverse in [2, S-3] (the faces the divergence reads)
__device__ __forceinline__ bool roeFace(const Grid& g, int side, int x, int y, int z, int loA, int hiA) {
    int c[3] = {x, y, z};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (a >= g.dim) break;
        int lo = a == side ? loA : 2, hi = a == side ? hiA : 2;
        if (c[a] < lo || c[a] >= g.S[a] - hi) return false;
    }
    return true;
}

template <typename real, int D>
__device__ __forceinline__ void loadState(const real* __restrict__ s, long long c, real* out) {
#pragma unroll
    for (int j = 0; j < D + 2; ++j) out[j] = s[(long long)(D + 2) * c + j];
}

template <typename real, int D, int SIDE, bool GRAV = false>
__device__ __forceinline__ void storeFace(const Grid& g, const RoePrim<real, D>& L, const RoePrim<real, D>& R,
                                          real gamma, real* __restrict__ basis, long long c) {
    const int NB = RoeRec<D>::NB;
    real rec[NB];
    roeBasisFromPrim<real, D, SIDE, GRAV>(L, R, gamma, rec);
#pragma unroll
    for (int k = 0; k < NB; ++k) basis[((long long)SIDE * NB + k) * g.V + c] = rec[k];
}

// Eigenbasis of the faces of one tile of cells [x0, x0+TX) x [y0, y0+TY) x [z0, z0+TZ)
// (res/EulerRoe.cl:261-271).  The per-cell primitives of the tile plus one cell below
// it on every axis go to shared memory `prim` ((TX+1)(TY+1)(TZ+1) entries for the
// active axes) once; then each thread builds the faces of its own cell.  All threads
// of the block must call this (it synchronises).  GRAV: with the potential `pot`.
template <typename real, int D, bool GRAV = false>
__device__ __forceinline__ void roeBasisTile(const Grid& g, const Phys<real>& ph, const real* __restrict__ state,
                                             real* __restrict__ basis, int loA, int hiA, int x0, int y0, int z0,
                                             int TX, int TY, int TZ, RoePrim<real, D>* prim,
                                             const real* __restrict__ pot = nullptr) {
    const int HX = TX + 1, HY = D > 1 ? TY + 1 : 1, HZ = D > 2 ? TZ + 1 : 1;
    const int ox = 1, oy = D > 1 ? 1 : 0, oz = D > 2 ? 1 : 0;
    for (int i = threadIdx.x; i < HX * HY * HZ; i += blockDim.x) {
        int hx = i % HX, hy = (i / HX) % HY, hz = i / (HX * HY);
        int gx = x0 - ox + hx, gy = y0 - oy + hy, gz = z0 - oz + hz;
        if (gx >= 0 && gx < g.S[0] && gy >= 0 && gy < g.S[1] && gz >= 0 && gz < g.S[2]) {
            long long c = gx + (long long)g.S[0] * (gy + (long long)g.S[1] * gz);
            real s[D + 2];
            loadState<real, D>(state, c, s);
            roePrim<real, D, GRAV>(s, ph.gamma, prim[i], GRAV ? pot[c] : (real)0);
        }
    }
    __syncthreads();
    const int tx = threadIdx.x % TX, ty = (threadIdx.x / TX) % TY, tz = threadIdx.x / (TX * TY);
    const int x = x0 + tx, y = y0 + ty, z = z0 + tz;
    const long long cc = x + (long long)g.S[0] * (y + (long long)g.S[1] * z);
    if (tz < TZ && x < g.S[0] && y < g.S[1] && z < g.S[2] && cellOk(g, cc)) {
        const long long c = cc;
        const int self = (tz + oz) * HY * HX + (ty + oy) * HX + (tx + ox);
        if (roeFace(g, 0, x, y, z, loA, hiA))
            storeFace<real, D, 0, GRAV>(g, prim[self - 1], prim[self], ph.gamma, basis, c);
        if (D > 1 && roeFace(g, 1, x, y, z, loA, hiA))
            storeFace<real, D, (D > 1 ? 1 : 0), GRAV>(g, prim[self - HX], prim[self], ph.gamma, basis, c);
        if (D > 2 && roeFace(g, 2, x, y, z, loA, hiA))
            storeFace<real, D, (D > 2 ? 2 : 0), GRAV>(g, prim[self - HX * HY], prim[self], ph.gamma, basis, c);
    }
    __syncthreads();
}

// Cell timestep of one cell, as its minimum over axes in IEEE bits (res/Roe.cl:4-65):
// interior cells dx / (|max(0, lambda_max(face c)) - min(0, lambda_min(face c+1))| + 1e-9),
// others INFINITY.
template <typename real, int D>
__device__ __forceinline__ unsigned long long roeDtCell(const Grid& g, const Phys<real>& ph,
                                                        const real* __restrict__ basis, long long c, int x, int y,
                                                        int z, bool& nan) {
    typedef RoeRec<D> R_;
    if (!inRange(g, x, y, z, 2, 2)) return realBits((real)INFINITY);
    unsigned long long best = ~0ULL;
#pragma unroll
    for (int side = 0; side < D; ++side) {
        if (!cellOk(g, c) || !cellOk(g, c + g.step[side])) continue;
        real lamMax = basis[((long long)side * R_::NB + R_::LAME) * g.V + c];
        real lamMin = basis[((long long)side * R_::NB + R_::LAM0) * g.V + c + g.step[side]];
        real maxLambda = fmaxLibm((real)0., lamMax);
        real minLambda = fminLibm((real)0., lamMin);
        real dum = (real)divI((double)ph.dx[side], (double)fabs(maxLambda - minLambda) + 1e-9);
        if (dum != dum) nan = true;
        unsigned long long b = realBits(dum);
        best = b < best ? b : best;
    }
    return best;
}

template <typename real, int D, int SIDE>
__device__ __forceinline__ void deltaQFace(const Grid& g, const real* __restrict__ stage, const real* __restrict__ basis,
                                           real* __restrict__ dq, long long c, const real* sR) {
    const int N = D + 2, NB = RoeRec<D>::NB;
    if (!cellOk(g, c - g.step[SIDE])) return;
    real sL[N], rec[NB], ds[N], y[N];
    loadState<real, D>(stage, c - g.step[SIDE], sL);
#pragma unroll
    for (int k = 0; k < NB; ++k) rec[k] = basis[((long long)SIDE * NB + k) * g.V + c];
#pragma unroll
    for (int j = 0; j < N; ++j) ds[j] = sR[j] - sL[j];
    leftTransform<real, D, SIDE, true>(rec, ds, y);
#pragma unroll
    for (int i = 0; i < N; ++i) dq[((long long)SIDE * N + i) * g.V + c] = y[i];
}

// Delta-q-tilde of the faces of one cell (res/Roe.cl:67-168)
template <typename real, int D>
__device__ __forceinline__ void roeDeltaQCell(const Grid& g, const real* __restrict__ stage,
                                              const real* __restrict__ basis, real* __restrict__ dq, long long c,
                                              int x, int y, int z, int loA, int hiA) {
    if (!cellOk(g, c)) return;
    real sR[D + 2];
    loadState<real, D>(stage, c, sR);
    if (roeFace(g, 0, x, y, z, loA, hiA)) deltaQFace<real, D, 0>(g, stage, basis, dq, c, sR);
    if (D > 1 && roeFace(g, 1, x, y, z, loA, hiA)) deltaQFace<real, D, (D > 1 ? 1 : 0)>(g, stage, basis, dq, c, sR);
    if (D > 2 && roeFace(g, 2, x, y, z, loA, hiA)) deltaQFace<real, D, (D > 2 ? 2 : 0)>(g, stage, basis, dq, c, sR);
}

template <typename real, int D, int SIDE, int LIM = -1, bool REC = false>
__device__ __forceinline__ void fluxFace(const Grid& g, int lim, real dt_dx, const real* __restrict__ stage,
                                         const real* __restrict__ basis, const real* __restrict__ dq,
                                         real* __restrict__ flux, long long c, const real* sR,
                                         real* __restrict__ tape = nullptr) {
    const int N = D + 2, NB = RoeRec<D>::NB;
    real sL[N], rec[NB], qL[N], q[N], qR[N], F[N];
    const long long st = g.step[SIDE];
    if (!cellOk(g, c - st) || !cellOk(g, c + st)) return;
    loadState<real, D>(stage, c - st, sL);
#pragma unroll
    for (int k = 0; k < NB; ++k) rec[k] = basis[((long long)SIDE * NB + k) * g.V + c];
#pragma unroll
    for (int i = 0; i < N; ++i) {
        const real* p = dq + ((long long)SIDE * N + i) * g.V + c;
        qL[i] = p[-st];
        q[i] = p[0];
        qR[i] = p[st];
    }
    roeFlux<real, D, SIDE, LIM, REC>(rec, sL, sR, qL, q, qR, dt_dx, lim, F,
                                     REC ? tape + (long long)SIDE * FT_PLANES * N * g.V + c : nullptr, g.V);
#pragma unroll
    for (int j = 0; j < N; ++j) flux[((long long)SIDE * N + j) * g.V + c] = F[j];
}

// Limited flux of the faces of one cell (res/Roe.cl:170-320), faces along [2, S-2]
template <typename real, int D, int LIM = -1, bool REC = false>
__device__ __forceinline__ void roeFluxCell(const Grid& g, int lim, const StepConst<real>& sc,
                                            const real* __restrict__ stage, const real* __restrict__ basis,
                                            const real* __restrict__ dq, real* __restrict__ flux, long long c, int x,
                                            int y, int z, real* __restrict__ tape = nullptr) {
    if (!cellOk(g, c)) return;
    real sR[D + 2];
    loadState<real, D>(stage, c, sR);
    if (roeFace(g, 0, x, y, z, 2, 1))
        fluxFace<real, D, 0, LIM, REC>(g, lim, sc.dt_dx[0], stage, basis, dq, flux, c, sR, tape);
    if (D > 1 && roeFace(g, 1, x, y, z, 2, 1))
        fluxFace<real, D, (D > 1 ? 1 : 0), LIM, REC>(g, lim, sc.dt_dx[1], stage, basis, dq, flux, c, sR, tape);
    if (D > 2 && roeFace(g, 2, x, y, z, 2, 1))
        fluxFace<real, D, (D > 2 ? 2 : 0), LIM, REC>(g, lim, sc.dt_dx[2], stage, basis, dq, flux, c, sR, tape);
}


// the two passes of the split FP64 flux (roe.cuh) over the faces of one cell
// (REC: tape planes per face as for roeFluxCell)
template <int D, int LIM, bool REC = false, bool FLATQ = false>
__device__ __forceinline__ void roeFluxCorrectionsCell(const Grid& g, int lim, const StepConst<double>& sc,
                                                       const double* __restrict__ basis,
                                                       const double* __restrict__ dq, double* __restrict__ flux,
                                                       long long c, int x, int y, int z,
                                                       double* __restrict__ tape = nullptr) {
    const int N = D + 2, NB = RoeRec<D>::NB;
#pragma unroll
    for (int side = 0; side < D; ++side) {
        if (!roeFace(g, side, x, y, z, 2, 1)) continue;
        const long long st = g.step[side];
        if (!cellOk(g, c) || !cellOk(g, c - st) || !cellOk(g, c + st)) continue;
        double rec[NB], qL[N], q[N], qR[N], corr[N];
#pragma unroll
        for (int k = 0; k < NB; ++k) rec[k] = basis[((long long)side * NB + k) * g.V + c];
#pragma unroll
        for (int i = 0; i < N; ++i) {
            const double* p = dq + ((long long)side * N + i) * g.V + c;
            qL[i] = p[-st];
            q[i] = p[0];
            qR[i] = p[st];
        }
        double* tf = REC ? tape + (long long)side * FT_PLANES * N * g.V + c : nullptr;
        if (side == 0) roeFluxCorrections<D, 0, LIM, REC, FLATQ>(rec, qL, q, qR, sc.dt_dx[0], lim, corr, tf, g.V);
        else if (side == 1)
            roeFluxCorrections<D, (D > 1 ? 1 : 0), LIM, REC, FLATQ>(rec, qL, q, qR, sc.dt_dx[1], lim, corr, tf, g.V);
        else roeFluxCorrections<D, (D > 2 ? 2 : 0), LIM, REC, FLATQ>(rec, qL, q, qR, sc.dt_dx[2], lim, corr, tf, g.V);
#pragma unroll
        for (int i = 0; i < N; ++i) flux[((long long)side * N + i) * g.V + c] = corr[i];
    }
}

template <int D, bool REC = false>
__device__ __forceinline__ void roeFluxTransformsCell(const Grid& g, const double* __restrict__ stage,
                                                      const double* __restrict__ basis, double* __restrict__ flux,
                                                      long long c, int x, int y, int z,
                                                      double* __restrict__ tape = nullptr) {
    const int N = D + 2, NB = RoeRec<D>::NB;
    if (!cellOk(g, c)) return;
    double sR[N];
    loadState<double, D>(stage, c, sR);
#pragma unroll
    for (int side = 0; side < D; ++side) {
        if (!roeFace(g, side, x, y, z, 2, 1)) continue;
        if (!cellOk(g, c - g.step[side])) continue;
        double sL[N], rec[NB], corr[N], F[N];
        loadState<double, D>(stage, c - g.step[side], sL);
#pragma unroll
        for (int k = 0; k < NB; ++k) rec[k] = basis[((long long)side * NB + k) * g.V + c];
#pragma unroll
        for (int i = 0; i < N; ++i) corr[i] = flux[((long long)side * N + i) * g.V + c];
        double* tf = REC ? tape + (long long)side * FT_PLANES * N * g.V + c : nullptr;
        if (side == 0) roeFluxTransforms<D, 0, REC>(rec, sL, sR, corr, F, tf, g.V);
        else if (side == 1) roeFluxTransforms<D, (D > 1 ? 1 : 0), REC>(rec, sL, sR, corr, F, tf, g.V);
        else roeFluxTransforms<D, (D > 2 ? 2 : 0), REC>(rec, sL, sR, corr, F, tf, g.V);
#pragma unroll
        for (int j = 0; j < N; ++j) flux[((long long)side * N + j) * g.V + c] = F[j];
    }
}

}  // namespace hgpu
