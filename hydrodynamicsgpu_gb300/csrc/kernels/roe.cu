// roe.cu -- EulerRoe kernels for sm_103a: eigenbasis + CFL timestep once per step,
// Delta-q-tilde and limited flux once per Runge-Kutta stage.
//
// Reference kernels replaced: calcEigenBasis (res/EulerRoe.cl:261-271),
// calcCellTimestep (res/Roe.cl:4-65), calcDeltaQTilde (res/Roe.cl:152-168),
// calcFlux (res/Roe.cl:301-320).  The eigenbasis is stored as a compact record of
// RoeRec<D>::NB distinct entries per face (structure-of-arrays, one plane per
// entry) instead of two dense N x N matrices, and it is computed once per step
// from u^n exactly as the reference does (Roe.cpp:82-92).
#include "kernels.h"
#include "roe.cuh"
#include "reduce.cuh"

namespace hgpu {

int roeRecordSize(int dim) {
    return dim == 1 ? RoeRec<1>::NB : dim == 2 ? RoeRec<2>::NB : RoeRec<3>::NB;
}

namespace {

constexpr int kThreads = 256;

inline unsigned blocksFor(long long n) { return (unsigned)((n + kThreads - 1) / kThreads); }

// faces along `side` in [loA, S-hiA), transverse in [2, S-2-1]
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

// Tile of cells per block for the eigenbasis kernel (256 threads).
template <int D> struct BasisTile;
template <> struct BasisTile<1> { enum { X = 256, Y = 1, Z = 1 }; };
template <> struct BasisTile<2> { enum { X = 32, Y = 8, Z = 1 }; };
template <> struct BasisTile<3> { enum { X = 32, Y = 4, Z = 2 }; };

template <typename real, int D, int SIDE>
__device__ __forceinline__ void storeFace(const Grid& g, const RoePrim<real, D>& L, const RoePrim<real, D>& R,
                                          real gamma, real* __restrict__ basis, long long c) {
    const int NB = RoeRec<D>::NB;
    real rec[NB];
    roeBasisFromPrim<real, D, SIDE>(L, R, gamma, rec);
#pragma unroll
    for (int k = 0; k < NB; ++k) basis[((long long)SIDE * NB + k) * g.V + c] = rec[k];
}

// Eigenbasis of every face (res/EulerRoe.cl:261-271).  A block covers a tile of cells;
// the per-cell primitives (RoePrim) of the tile plus one cell below it on every axis
// are computed once into shared memory, then each thread builds the faces of its cell.
template <typename real, int D>
__global__ void __launch_bounds__(256) roeBasisKernel(Grid g, Phys<real> ph, const real* __restrict__ state,
                                                     real* __restrict__ basis, int loA, int hiA) {
    typedef BasisTile<D> T;
    constexpr int HX = T::X + 1, HY = D > 1 ? T::Y + 1 : 1, HZ = D > 2 ? T::Z + 1 : 1;
    __shared__ RoePrim<real, D> prim[HZ * HY * HX];
    const int x0 = blockIdx.x * T::X, y0 = blockIdx.y * T::Y, z0 = blockIdx.z * T::Z;
    const int ox = 1, oy = D > 1 ? 1 : 0, oz = D > 2 ? 1 : 0;
    for (int i = threadIdx.x; i < HX * HY * HZ; i += blockDim.x) {
        int hx = i % HX, hy = (i / HX) % HY, hz = i / (HX * HY);
        int gx = x0 - ox + hx, gy = y0 - oy + hy, gz = z0 - oz + hz;
        if (gx >= 0 && gx < g.S[0] && gy >= 0 && gy < g.S[1] && gz >= 0 && gz < g.S[2]) {
            long long c = gx + (long long)g.S[0] * (gy + (long long)g.S[1] * gz);
            real s[D + 2];
#pragma unroll
            for (int j = 0; j < D + 2; ++j) s[j] = state[(long long)(D + 2) * c + j];
            roePrim<real, D>(s, ph.gamma, prim[i]);
        }
    }
    __syncthreads();
    const int tx = threadIdx.x % T::X, ty = (threadIdx.x / T::X) % T::Y, tz = threadIdx.x / (T::X * T::Y);
    const int x = x0 + tx, y = y0 + ty, z = z0 + tz;
    if (x >= g.S[0] || y >= g.S[1] || z >= g.S[2]) return;
    const long long c = x + (long long)g.S[0] * (y + (long long)g.S[1] * z);
    const int self = (tz + oz) * HY * HX + (ty + oy) * HX + (tx + ox);
    if (roeFace(g, 0, x, y, z, loA, hiA)) storeFace<real, D, 0>(g, prim[self - 1], prim[self], ph.gamma, basis, c);
    if (D > 1 && roeFace(g, 1, x, y, z, loA, hiA))
        storeFace<real, D, (D > 1 ? 1 : 0)>(g, prim[self - HX], prim[self], ph.gamma, basis, c);
    if (D > 2 && roeFace(g, 2, x, y, z, loA, hiA))
        storeFace<real, D, (D > 2 ? 2 : 0)>(g, prim[self - HX * HY], prim[self], ph.gamma, basis, c);
}

// per interior cell and side: dx / (|max(0, lambda_max(face c)) - min(0, lambda_min(face c+1))| + 1e-9)
template <typename real, int D>
__global__ void __launch_bounds__(kThreads) roeDtKernel(Grid g, Phys<real> ph, const real* __restrict__ basis,
                                                        unsigned long long* acc, unsigned* health) {
    typedef RoeRec<D> R_;
    long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long best = ~0ULL;
    bool nan = false;
    if (c < g.V) {
        int x, y, z;
        cellCoords(g, c, x, y, z);
        if (inRange(g, x, y, z, 2, 2)) {
#pragma unroll
            for (int side = 0; side < D; ++side) {
                real lamMax = basis[((long long)side * R_::NB + R_::LAME) * g.V + c];
                real lamMin = basis[((long long)side * R_::NB + R_::LAM0) * g.V + c + g.step[side]];
                real maxLambda = fmaxLibm((real)0., lamMax);
                real minLambda = fminLibm((real)0., lamMin);
                real dum = (real)((double)ph.dx[side] / ((double)fabs(maxLambda - minLambda) + 1e-9));
                if (dum != dum) nan = true;
                unsigned long long b = realBits(dum);
                best = b < best ? b : best;
            }
        } else if (c < g.V) {
            best = realBits((real)INFINITY);
        }
    }
    if (nan) atomicOr(health, HEALTH_NONFINITE_DT);
    blockMinToGlobal(best, acc);
}

template <typename real, int D, int SIDE>
__device__ __forceinline__ void deltaQFace(const Grid& g, const real* __restrict__ stage, const real* __restrict__ basis,
                                           real* __restrict__ dq, long long c, const real* sR) {
    const int N = D + 2, NB = RoeRec<D>::NB;
    real sL[N], rec[NB], ds[N], y[N];
    loadState<real, D>(stage, c - g.step[SIDE], sL);
#pragma unroll
    for (int k = 0; k < NB; ++k) rec[k] = basis[((long long)SIDE * NB + k) * g.V + c];
#pragma unroll
    for (int j = 0; j < N; ++j) ds[j] = sR[j] - sL[j];
    leftTransform<real, D, SIDE>(rec, ds, y);
#pragma unroll
    for (int i = 0; i < N; ++i) dq[((long long)SIDE * N + i) * g.V + c] = y[i];
}

template <typename real, int D>
__global__ void __launch_bounds__(kThreads) roeDeltaQKernel(Grid g, const real* __restrict__ stage,
                                                            const real* __restrict__ basis, real* __restrict__ dq,
                                                            int loA, int hiA) {
    long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.V) return;
    int x, y, z;
    cellCoords(g, c, x, y, z);
    real sR[D + 2];
    loadState<real, D>(stage, c, sR);
    if (roeFace(g, 0, x, y, z, loA, hiA)) deltaQFace<real, D, 0>(g, stage, basis, dq, c, sR);
    if (D > 1 && roeFace(g, 1, x, y, z, loA, hiA)) deltaQFace<real, D, (D > 1 ? 1 : 0)>(g, stage, basis, dq, c, sR);
    if (D > 2 && roeFace(g, 2, x, y, z, loA, hiA)) deltaQFace<real, D, (D > 2 ? 2 : 0)>(g, stage, basis, dq, c, sR);
}

template <typename real, int D, int SIDE>
__device__ __forceinline__ void fluxFace(const Grid& g, int lim, real dt_dx, const real* __restrict__ stage,
                                         const real* __restrict__ basis, const real* __restrict__ dq,
                                         real* __restrict__ flux, long long c, const real* sR) {
    const int N = D + 2, NB = RoeRec<D>::NB;
    real sL[N], rec[NB], qL[N], q[N], qR[N], F[N];
    const long long st = g.step[SIDE];
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
    roeFlux<real, D, SIDE>(rec, sL, sR, qL, q, qR, dt_dx, lim, F);
#pragma unroll
    for (int j = 0; j < N; ++j) flux[((long long)SIDE * N + j) * g.V + c] = F[j];
}

template <typename real, int D>
__global__ void __launch_bounds__(kThreads) roeFluxKernel(Grid g, int lim, const real* __restrict__ stage,
                                                          const real* __restrict__ basis, const real* __restrict__ dq,
                                                          const StepConst<real>* __restrict__ sc,
                                                          real* __restrict__ flux) {
    long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.V) return;
    int x, y, z;
    cellCoords(g, c, x, y, z);
    real sR[D + 2];
    loadState<real, D>(stage, c, sR);
    if (roeFace(g, 0, x, y, z, 2, 1)) fluxFace<real, D, 0>(g, lim, sc->dt_dx[0], stage, basis, dq, flux, c, sR);
    if (D > 1 && roeFace(g, 1, x, y, z, 2, 1))
        fluxFace<real, D, (D > 1 ? 1 : 0)>(g, lim, sc->dt_dx[1], stage, basis, dq, flux, c, sR);
    if (D > 2 && roeFace(g, 2, x, y, z, 2, 1))
        fluxFace<real, D, (D > 2 ? 2 : 0)>(g, lim, sc->dt_dx[2], stage, basis, dq, flux, c, sR);
}

}  // namespace

// REF: faces along [2, S-2] (res/EulerRoe.cl:27-34, res/Roe.cl:88-95); SEAM: [1, S-1].
template <typename real>
void launchRoeBasis(const Grid& g, const Phys<real>& ph, const real* state, real* basis, int seam, cudaStream_t st) {
    int loA = seam ? 1 : 2, hiA = seam ? 0 : 1;
    auto grid = [&](int tx, int ty, int tz) {
        return dim3((unsigned)((g.S[0] + tx - 1) / tx), (unsigned)((g.S[1] + ty - 1) / ty), (unsigned)((g.S[2] + tz - 1) / tz));
    };
    if (g.dim == 1)
        roeBasisKernel<real, 1><<<grid(BasisTile<1>::X, 1, 1), 256, 0, st>>>(g, ph, state, basis, loA, hiA);
    else if (g.dim == 2)
        roeBasisKernel<real, 2><<<grid(BasisTile<2>::X, BasisTile<2>::Y, 1), 256, 0, st>>>(g, ph, state, basis, loA, hiA);
    else
        roeBasisKernel<real, 3><<<grid(BasisTile<3>::X, BasisTile<3>::Y, BasisTile<3>::Z), 256, 0, st>>>(g, ph, state, basis,
                                                                                                      loA, hiA);
}

template <typename real>
void launchRoeDt(const Grid& g, const Phys<real>& ph, const real* basis, unsigned long long* acc, unsigned* health,
                 cudaStream_t st) {
    if (g.dim == 1) roeDtKernel<real, 1><<<blocksFor(g.V), kThreads, 0, st>>>(g, ph, basis, acc, health);
    else if (g.dim == 2) roeDtKernel<real, 2><<<blocksFor(g.V), kThreads, 0, st>>>(g, ph, basis, acc, health);
    else roeDtKernel<real, 3><<<blocksFor(g.V), kThreads, 0, st>>>(g, ph, basis, acc, health);
}

template <typename real>
void launchRoeDeltaQ(const Grid& g, const real* stage, const real* basis, real* dq, int seam, cudaStream_t st) {
    int loA = seam ? 1 : 2, hiA = seam ? 0 : 1;
    if (g.dim == 1) roeDeltaQKernel<real, 1><<<blocksFor(g.V), kThreads, 0, st>>>(g, stage, basis, dq, loA, hiA);
    else if (g.dim == 2) roeDeltaQKernel<real, 2><<<blocksFor(g.V), kThreads, 0, st>>>(g, stage, basis, dq, loA, hiA);
    else roeDeltaQKernel<real, 3><<<blocksFor(g.V), kThreads, 0, st>>>(g, stage, basis, dq, loA, hiA);
}

template <typename real>
void launchRoeFlux(const Grid& g, int limiter, const real* stage, const real* basis, const real* dq,
                   const StepConst<real>* sc, real* flux, int seam, cudaStream_t st) {
    (void)seam;
    if (g.dim == 1) roeFluxKernel<real, 1><<<blocksFor(g.V), kThreads, 0, st>>>(g, limiter, stage, basis, dq, sc, flux);
    else if (g.dim == 2) roeFluxKernel<real, 2><<<blocksFor(g.V), kThreads, 0, st>>>(g, limiter, stage, basis, dq, sc, flux);
    else roeFluxKernel<real, 3><<<blocksFor(g.V), kThreads, 0, st>>>(g, limiter, stage, basis, dq, sc, flux);
}

#define INST(real)                                                                                              \
    template void launchRoeBasis<real>(const Grid&, const Phys<real>&, const real*, real*, int, cudaStream_t);  \
    template void launchRoeDt<real>(const Grid&, const Phys<real>&, const real*, unsigned long long*, unsigned*, \
                                    cudaStream_t);                                                             \
    template void launchRoeDeltaQ<real>(const Grid&, const real*, const real*, real*, int, cudaStream_t);       \
    template void launchRoeFlux<real>(const Grid&, int, const real*, const real*, const real*,                   \
                                      const StepConst<real>*, real*, int, cudaStream_t);
INST(double)
INST(float)
#undef INST

}  // namespace hgpu
