// roe.cu -- EulerRoe kernels for sm_103a: eigenbasis + CFL timestep once per step,
// Delta-q-tilde and limited flux once per Runge-Kutta stage (one problem).
//
// Reference kernels replaced: calcEigenBasis (res/EulerRoe.cl:261-271),
// calcCellTimestep (res/Roe.cl:4-65), calcDeltaQTilde (res/Roe.cl:152-168),
// calcFlux (res/Roe.cl:301-320).  The eigenbasis is stored as a compact record of
// RoeRec<D>::NB distinct entries per face (structure-of-arrays, one plane per
// entry) instead of two dense N x N matrices, and it is computed once per step
// from u^n exactly as the reference does (Roe.cpp:82-92).  The bodies live in
// roe_cells.cuh (shared with the batched kernels).
#include "../../../include/hgpu/hgpu.h"
#include "kernels.h"
#include "reduce.cuh"
#include "roe_cells.cuh"

namespace hgpu {

int roeRecordSize(int dim) {
    return dim == 1 ? RoeRec<1>::NB : dim == 2 ? RoeRec<2>::NB : RoeRec<3>::NB;
}

namespace {

constexpr int kThreads = 256;

inline unsigned blocksFor(long long n) { return (unsigned)((n + kThreads - 1) / kThreads); }

// Tile of cells per block for the eigenbasis kernel (256 threads).
template <int D> struct BasisTile;
template <> struct BasisTile<1> { enum { X = 256, Y = 1, Z = 1 }; };
template <> struct BasisTile<2> { enum { X = 32, Y = 8, Z = 1 }; };
template <> struct BasisTile<3> { enum { X = 32, Y = 4, Z = 2 }; };

// slowOff: tiles skipped along the slowest axis (y in 2D, z in 3D), for a band of it
template <typename real, int D, bool GRAV>
__global__ void __launch_bounds__(256) roeBasisKernel(Grid g, Phys<real> ph, const real* __restrict__ state,
                                                     real* __restrict__ basis, int loA, int hiA,
                                                     const real* __restrict__ pot, int slowOff) {
    typedef BasisTile<D> T;
    constexpr int HX = T::X + 1, HY = D > 1 ? T::Y + 1 : 1, HZ = D > 2 ? T::Z + 1 : 1;
    __shared__ RoePrim<real, D> prim[HZ * HY * HX];
    const int ty = blockIdx.y + (D == 2 ? slowOff : 0), tz = blockIdx.z + (D == 3 ? slowOff : 0);
    roeBasisTile<real, D, GRAV>(g, ph, state, basis, loA, hiA, blockIdx.x * T::X, ty * T::Y, tz * T::Z, T::X, T::Y,
                                T::Z, prim, pot);
}

template <typename real, int D>
__global__ void __launch_bounds__(kThreads) roeDtKernel(Grid g, Phys<real> ph, const real* __restrict__ basis,
                                                        unsigned long long* acc, unsigned* health) {
    long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long best = ~0ULL;
    bool nan = false;
    if (c < g.V) {
        int x, y, z;
        cellCoords(g, c, x, y, z);
        best = roeDtCell<real, D>(g, ph, basis, c, x, y, z, nan);
    }
    if (nan) atomicOr(health, HEALTH_NONFINITE_DT);
    blockMinToGlobal(best, acc);
}

template <typename real, int D>
__global__ void __launch_bounds__(kThreads) roeDeltaQKernel(Grid g, const real* __restrict__ stage,
                                                            const real* __restrict__ basis, real* __restrict__ dq,
                                                            int loA, int hiA, long long c0, long long c1) {
    long long c = c0 + (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= c1) return;
    int x, y, z;
    cellCoords(g, c, x, y, z);
    roeDeltaQCell<real, D>(g, stage, basis, dq, c, x, y, z, loA, hiA);
}

template <typename real, int D, int LIM>
__global__ void __launch_bounds__(kThreads) roeFluxKernel(Grid g, int lim, const real* __restrict__ stage,
                                                          const real* __restrict__ basis, const real* __restrict__ dq,
                                                          const StepConst<real>* __restrict__ sc,
                                                          real* __restrict__ flux, long long c0, long long c1) {
    long long c = c0 + (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= c1) return;
    int x, y, z;
    cellCoords(g, c, x, y, z);
    roeFluxCell<real, D, LIM>(g, lim, *sc, stage, basis, dq, flux, c, x, y, z);
}

template <int D, int LIM>
__global__ void __launch_bounds__(kThreads) roeFluxCorrKernel(Grid g, int lim, const double* __restrict__ basis,
                                                              const double* __restrict__ dq,
                                                              const StepConst<double>* __restrict__ sc,
                                                              double* __restrict__ flux, long long c0, long long c1) {
    long long c = c0 + (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= c1) return;
    int x, y, z;
    cellCoords(g, c, x, y, z);
    roeFluxCorrectionsCell<D, LIM>(g, lim, *sc, basis, dq, flux, c, x, y, z);
}

template <int D>
__global__ void __launch_bounds__(kThreads) roeFluxXformKernel(Grid g, const double* __restrict__ stage,
                                                               const double* __restrict__ basis,
                                                               double* __restrict__ flux, long long c0, long long c1) {
    long long c = c0 + (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= c1) return;
    int x, y, z;
    cellCoords(g, c, x, y, z);
    roeFluxTransformsCell<D>(g, stage, basis, flux, c, x, y, z);
}

}  // namespace

template <typename real, bool GRAV>
void launchRoeBasisG(const Grid& g, const Phys<real>& ph, const real* state, real* basis, int loA, int hiA,
                     const real* pot, cudaStream_t st, int slow0, int slowTiles) {
    auto grid = [&](int tx, int ty, int tz) {
        return dim3((unsigned)((g.S[0] + tx - 1) / tx), (unsigned)((g.S[1] + ty - 1) / ty),
                    (unsigned)((g.S[2] + tz - 1) / tz));
    };
    if (g.dim == 1) {
        roeBasisKernel<real, 1, GRAV><<<grid(BasisTile<1>::X, 1, 1), 256, 0, st>>>(g, ph, state, basis, loA, hiA, pot,
                                                                                   0);
        return;
    }
    dim3 gr = g.dim == 2 ? grid(BasisTile<2>::X, BasisTile<2>::Y, 1)
                         : grid(BasisTile<3>::X, BasisTile<3>::Y, BasisTile<3>::Z);
    unsigned& slow = g.dim == 2 ? gr.y : gr.z;
    if (slow0 < 0) slow0 = 0;
    if (slowTiles < 0 || slow0 + slowTiles > (int)slow) slowTiles = (int)slow - slow0;
    if (slowTiles <= 0) return;
    slow = (unsigned)slowTiles;
    if (g.dim == 2)
        roeBasisKernel<real, 2, GRAV><<<gr, 256, 0, st>>>(g, ph, state, basis, loA, hiA, pot, slow0);
    else
        roeBasisKernel<real, 3, GRAV><<<gr, 256, 0, st>>>(g, ph, state, basis, loA, hiA, pot, slow0);
}

// REF: faces along [2, S-2] (res/EulerRoe.cl:27-34, res/Roe.cl:88-95); SEAM: [1, S-1].
// pot: the gravitational potential, or null for a zero potential.
template <typename real>
void launchRoeBasis(const Grid& g, const Phys<real>& ph, const real* state, real* basis, int seam, cudaStream_t st,
                    const real* pot, int slow0, int slowTiles) {
    int loA = seam ? 1 : 2, hiA = seam ? 0 : 1;
    if (pot) launchRoeBasisG<real, true>(g, ph, state, basis, loA, hiA, pot, st, slow0, slowTiles);
    else launchRoeBasisG<real, false>(g, ph, state, basis, loA, hiA, nullptr, st, slow0, slowTiles);
}

int roeBasisSlowTile(int dim) { return dim == 2 ? BasisTile<2>::Y : dim == 3 ? BasisTile<3>::Z : 1; }

template <typename real>
void launchRoeDt(const Grid& g, const Phys<real>& ph, const real* basis, unsigned long long* acc, unsigned* health,
                 cudaStream_t st) {
    if (g.dim == 1) roeDtKernel<real, 1><<<blocksFor(g.V), kThreads, 0, st>>>(g, ph, basis, acc, health);
    else if (g.dim == 2) roeDtKernel<real, 2><<<blocksFor(g.V), kThreads, 0, st>>>(g, ph, basis, acc, health);
    else roeDtKernel<real, 3><<<blocksFor(g.V), kThreads, 0, st>>>(g, ph, basis, acc, health);
}

// cells [c0, c1) (c1 < 0: to the end of the grid); whole-grid launches take every cell
static inline long long rangeEnd(const Grid& g, long long c1) { return c1 < 0 ? g.V : c1; }

template <typename real>
void launchRoeDeltaQ(const Grid& g, const real* stage, const real* basis, real* dq, int seam, cudaStream_t st,
                     long long c0, long long c1) {
    int loA = seam ? 1 : 2, hiA = seam ? 0 : 1;
    c1 = rangeEnd(g, c1);
    if (c1 <= c0) return;
    const unsigned b = blocksFor(c1 - c0);
    if (g.dim == 1) roeDeltaQKernel<real, 1><<<b, kThreads, 0, st>>>(g, stage, basis, dq, loA, hiA, c0, c1);
    else if (g.dim == 2) roeDeltaQKernel<real, 2><<<b, kThreads, 0, st>>>(g, stage, basis, dq, loA, hiA, c0, c1);
    else roeDeltaQKernel<real, 3><<<b, kThreads, 0, st>>>(g, stage, basis, dq, loA, hiA, c0, c1);
}

template <int LIM>
void launchRoeFluxSplit(const Grid& g, int limiter, const double* stage, const double* basis, const double* dq,
                        const StepConst<double>* sc, double* flux, cudaStream_t st, long long c0, long long c1) {
    const unsigned b = blocksFor(c1 - c0);
    if (g.dim == 1) {
        roeFluxCorrKernel<1, LIM><<<b, kThreads, 0, st>>>(g, limiter, basis, dq, sc, flux, c0, c1);
        roeFluxXformKernel<1><<<b, kThreads, 0, st>>>(g, stage, basis, flux, c0, c1);
    } else if (g.dim == 2) {
        roeFluxCorrKernel<2, LIM><<<b, kThreads, 0, st>>>(g, limiter, basis, dq, sc, flux, c0, c1);
        roeFluxXformKernel<2><<<b, kThreads, 0, st>>>(g, stage, basis, flux, c0, c1);
    } else {
        roeFluxCorrKernel<3, LIM><<<b, kThreads, 0, st>>>(g, limiter, basis, dq, sc, flux, c0, c1);
        roeFluxXformKernel<3><<<b, kThreads, 0, st>>>(g, stage, basis, flux, c0, c1);
    }
}

template <typename real, int LIM>
void launchRoeFluxLim(const Grid& g, int limiter, const real* stage, const real* basis, const real* dq,
                      const StepConst<real>* sc, real* flux, cudaStream_t st, long long c0, long long c1) {
    // FP64 runs the flux as two lighter passes (more resident warps, same bits)
    if (sizeof(real) == 8) {
        launchRoeFluxSplit<LIM>(g, limiter, (const double*)stage, (const double*)basis, (const double*)dq,
                                (const StepConst<double>*)sc, (double*)flux, st, c0, c1);
        return;
    }
    const unsigned b = blocksFor(c1 - c0);
    if (g.dim == 1) roeFluxKernel<real, 1, LIM><<<b, kThreads, 0, st>>>(g, limiter, stage, basis, dq, sc, flux, c0, c1);
    else if (g.dim == 2) roeFluxKernel<real, 2, LIM><<<b, kThreads, 0, st>>>(g, limiter, stage, basis, dq, sc, flux, c0, c1);
    else roeFluxKernel<real, 3, LIM><<<b, kThreads, 0, st>>>(g, limiter, stage, basis, dq, sc, flux, c0, c1);
}

// the benchmark limiters and the common ones get kernels of their own; the others
// share one kernel that dispatches on the limiter at run time
template <typename real>
void launchRoeFlux(const Grid& g, int limiter, const real* stage, const real* basis, const real* dq,
                   const StepConst<real>* sc, real* flux, int seam, cudaStream_t st, long long c0, long long c1) {
    (void)seam;
    c1 = rangeEnd(g, c1);
    if (c1 <= c0) return;
#define F(LL) launchRoeFluxLim<real, LL>(g, limiter, stage, basis, dq, sc, flux, st, c0, c1)
    switch (limiter) {
    case HGPU_LIMITER_DONORCELL: F(HGPU_LIMITER_DONORCELL); break;
    case HGPU_LIMITER_LAXWENDROFF: F(HGPU_LIMITER_LAXWENDROFF); break;
    case HGPU_LIMITER_MINMOD: F(HGPU_LIMITER_MINMOD); break;
    case HGPU_LIMITER_VANLEER: F(HGPU_LIMITER_VANLEER); break;
    case HGPU_LIMITER_MONOTIZEDCENTRAL: F(HGPU_LIMITER_MONOTIZEDCENTRAL); break;
    case HGPU_LIMITER_SUPERBEE: F(HGPU_LIMITER_SUPERBEE); break;
    default: F(-1); break;
    }
#undef F
}

#define INST(real)                                                                                              \
    template void launchRoeBasis<real>(const Grid&, const Phys<real>&, const real*, real*, int, cudaStream_t,    \
                                       const real*, int, int);                                                  \
    template void launchRoeDt<real>(const Grid&, const Phys<real>&, const real*, unsigned long long*, unsigned*, \
                                    cudaStream_t);                                                             \
    template void launchRoeDeltaQ<real>(const Grid&, const real*, const real*, real*, int, cudaStream_t,        \
                                        long long, long long);                                                  \
    template void launchRoeFlux<real>(const Grid&, int, const real*, const real*, const real*,                   \
                                      const StepConst<real>*, real*, int, cudaStream_t, long long, long long);
INST(double)
INST(float)
#undef INST

}  // namespace hgpu
