// hllc.cu -- EulerHLLC kernels for sm_103a: wave speeds + CFL timestep once per
// step, HLLC interface flux once per Runge-Kutta stage.
//
// Reference kernels replaced (res/EulerHLLC.cl): calcEigenvalues (:15-131),
// calcCellTimestep (:135-168), calcFlux with HLLC_METHOD 2 (:170-445).  Only the
// outer wave speeds sl and sr are kept per face: the middle eigenvalues (the Roe
// velocity) are never read by the timestep or the flux.  The reference's slope
// limiter for HLLC is compiled out (:393-411), so the flux is first order.
// A face where no HLLC branch applies keeps the flux of its previous evaluation,
// momentum components swapped back once more, exactly as the reference buffer does.
// With `hll` the same launches run EulerHLL (res/EulerHLL.cl): Davis-bounded wave
// speeds and the two-state HLL flux; its timestep kernel is HLLC's.
#include "hllc_cells.cuh"
#include "kernels.h"
#include "reduce.cuh"

namespace hgpu {
namespace {

constexpr int kThreads = 256;
inline unsigned blocksFor(long long n) { return (unsigned)((n + kThreads - 1) / kThreads); }

template <typename real, int D, bool HLL, bool GRAV>
__global__ void __launch_bounds__(kThreads) hllcWaveKernel(Grid g, Phys<real> ph, double gq,
                                                           const real* __restrict__ state, real* __restrict__ waves,
                                                           const real* __restrict__ pot, long long c0, long long c1) {
    long long c = c0 + (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= c1) return;
    int x, y, z;
    cellCoords(g, c, x, y, z);
    hllcWaveCell<real, D, HLL, GRAV>(g, ph, gq, state, waves, c, x, y, z, pot);
}

template <typename real, int D>
__global__ void __launch_bounds__(kThreads) hllcDtKernel(Grid g, Phys<real> ph, const real* __restrict__ waves,
                                                         unsigned long long* acc, unsigned* health) {
    long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long best = ~0ULL;
    bool nan = false;
    if (c < g.V) {
        int x, y, z;
        cellCoords(g, c, x, y, z);
        best = hllcDtCell<real, D>(g, ph, waves, c, x, y, z, nan);
    }
    if (nan) atomicOr(health, HEALTH_NONFINITE_DT);
    blockMinToGlobal(best, acc);
}

template <typename real, int D, bool HLL, bool GRAV>
__global__ void __launch_bounds__(kThreads) hllcFluxKernel(Grid g, Phys<real> ph, const real* __restrict__ stage,
                                                           const real* __restrict__ waves, real* __restrict__ flux,
                                                           unsigned* health, const real* __restrict__ pot,
                                                           long long c0, long long c1) {
    long long c = c0 + (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= c1) return;
    int x, y, z;
    cellCoords(g, c, x, y, z);
    if (!hllcFluxCell<real, D, HLL, GRAV>(g, ph, stage, waves, flux, c, x, y, z, pot))
        atomicOr(health, HEALTH_HLLC_NOBRANCH);
}

// the flux with each cell's primitives staged once per tile (hllc_cells.cuh
// hllcFluxTile), for slow-axis planes [s0, s1) (y in 2D, z in 3D)
template <int D> struct FluxTile;
template <> struct FluxTile<2> { enum { X = 32, Y = 8, Z = 1 }; };
template <> struct FluxTile<3> { enum { X = 32, Y = 4, Z = 2 }; };

template <typename real, int D, bool HLL, bool GRAV>
__global__ void __launch_bounds__(kThreads) hllcFluxTileKernel(Grid g, Phys<real> ph, const real* __restrict__ stage,
                                                               const real* __restrict__ waves,
                                                               real* __restrict__ flux, unsigned* health,
                                                               const real* __restrict__ pot, int s0, int s1) {
    typedef FluxTile<D> T;
    constexpr int HX = T::X + 1, HY = T::Y + 1, HZ = D > 2 ? T::Z + 1 : 1;
    __shared__ Prim<real, D> prim[HX * HY * HZ];
    const int x0 = blockIdx.x * T::X;
    const int y0 = D == 2 ? s0 + (int)blockIdx.y * T::Y : (int)blockIdx.y * T::Y;
    const int z0 = D == 2 ? 0 : s0 + (int)blockIdx.z * T::Z;
    const bool ok = hllcFluxTile<real, D, HLL, GRAV>(g, ph, stage, waves, flux, x0, y0, z0, T::X, T::Y, T::Z, s0, s1,
                                                     prim, pot);
    if (!ok) atomicOr(health, HEALTH_HLLC_NOBRANCH);
}

// The same for 2D EulerHLLC with the register budget of one block per SM: ptxas then
// keeps 102 registers (2 blocks per SM) instead of its default 80 (3 blocks), which
// measured faster (KH 2048^2 RK4 8.32 -> 7.71 ms a step); EulerHLL and 3D measured
// slower that way and keep the kernel above.
template <typename real, bool GRAV>
__global__ void __launch_bounds__(kThreads, 1) hllcFluxTileKernelWide(Grid g, Phys<real> ph,
                                                                      const real* __restrict__ stage,
                                                                      const real* __restrict__ waves,
                                                                      real* __restrict__ flux, unsigned* health,
                                                                      const real* __restrict__ pot, int s0, int s1) {
    typedef FluxTile<2> T;
    constexpr int HX = T::X + 1, HY = T::Y + 1;
    __shared__ Prim<real, 2> prim[HX * HY];
    const int x0 = blockIdx.x * T::X, y0 = s0 + (int)blockIdx.y * T::Y;
    const bool ok = hllcFluxTile<real, 2, false, GRAV>(g, ph, stage, waves, flux, x0, y0, 0, T::X, T::Y, 1, s0, s1,
                                                       prim, pot);
    if (!ok) atomicOr(health, HEALTH_HLLC_NOBRANCH);
}

template <typename real, int D, bool HLL, bool GRAV>
__global__ void __launch_bounds__(kThreads) hllcWaveTileKernel(Grid g, Phys<real> ph, double gq,
                                                               const real* __restrict__ state,
                                                               real* __restrict__ waves, const real* __restrict__ pot,
                                                               int s0, int s1) {
    typedef FluxTile<D> T;
    constexpr int HX = T::X + 1, HY = T::Y + 1, HZ = D > 2 ? T::Z + 1 : 1;
    __shared__ Prim<real, D> prim[HX * HY * HZ];
    const int x0 = blockIdx.x * T::X;
    const int y0 = D == 2 ? s0 + (int)blockIdx.y * T::Y : (int)blockIdx.y * T::Y;
    const int z0 = D == 2 ? 0 : s0 + (int)blockIdx.z * T::Z;
    hllcWaveTile<real, D, HLL, GRAV>(g, ph, gq, state, waves, x0, y0, z0, T::X, T::Y, T::Z, s0, s1, prim, pot);
}

}  // namespace

// the grid of a tile kernel over slow-axis planes [s0, s1)
template <int D>
static dim3 tileGrid(const Grid& g, int s0, int s1) {
    typedef FluxTile<D> FT;
    return dim3((unsigned)((g.S[0] + FT::X - 1) / FT::X),
                (unsigned)(D == 2 ? (s1 - s0 + FT::Y - 1) / FT::Y : (g.S[1] + FT::Y - 1) / FT::Y),
                (unsigned)(D == 2 ? 1 : (s1 - s0 + FT::Z - 1) / FT::Z));
}

// pot: the gravitational potential, or null for a zero potential
template <typename real, bool GRAV>
void launchHllcWavesG(const Grid& g, const Phys<real>& ph, const real* state, real* waves, int hll, cudaStream_t st,
                      const real* pot, long long c0, long long c1) {
    if (c1 < 0 || c1 > g.V) c1 = g.V;
    if (c0 < 0) c0 = 0;
    if (c0 >= c1) return;
    // (gamma + 1.) / (2. * gamma) is a per-program constant (double literals); computed once, identically
    double gq = ((double)ph.gamma + 1.) / (2. * (double)ph.gamma);
    // 2D and 3D: the staged tile kernel over whole slow-axis planes
    const long long plane = g.dim > 1 ? (long long)g.V / g.S[g.dim - 1] : 0;
    if (g.dim > 1 && c0 % plane == 0 && c1 % plane == 0) {
        const int s0 = (int)(c0 / plane), s1 = (int)(c1 / plane);
#define T(DD, H) \
    hllcWaveTileKernel<real, DD, H, GRAV><<<tileGrid<DD>(g, s0, s1), kThreads, 0, st>>>(g, ph, gq, state, waves, pot, s0, s1)
        if (hll) {
            if (g.dim == 2) T(2, true);
            else T(3, true);
        } else {
            if (g.dim == 2) T(2, false);
            else T(3, false);
        }
#undef T
        return;
    }
#define L(DD, H) \
    hllcWaveKernel<real, DD, H, GRAV><<<blocksFor(c1 - c0), kThreads, 0, st>>>(g, ph, gq, state, waves, pot, c0, c1)
    if (hll) {
        if (g.dim == 1) L(1, true);
        else if (g.dim == 2) L(2, true);
        else L(3, true);
    } else {
        if (g.dim == 1) L(1, false);
        else if (g.dim == 2) L(2, false);
        else L(3, false);
    }
#undef L
}

template <typename real>
void launchHllcWaves(const Grid& g, const Phys<real>& ph, const real* state, real* waves, int hll, cudaStream_t st,
                     const real* pot, long long c0, long long c1) {
    if (pot) launchHllcWavesG<real, true>(g, ph, state, waves, hll, st, pot, c0, c1);
    else launchHllcWavesG<real, false>(g, ph, state, waves, hll, st, nullptr, c0, c1);
}

template <typename real>
void launchHllcDt(const Grid& g, const Phys<real>& ph, const real* waves, unsigned long long* acc, unsigned* health,
                  cudaStream_t st) {
    if (g.dim == 1) hllcDtKernel<real, 1><<<blocksFor(g.V), kThreads, 0, st>>>(g, ph, waves, acc, health);
    else if (g.dim == 2) hllcDtKernel<real, 2><<<blocksFor(g.V), kThreads, 0, st>>>(g, ph, waves, acc, health);
    else hllcDtKernel<real, 3><<<blocksFor(g.V), kThreads, 0, st>>>(g, ph, waves, acc, health);
}

template <typename real, bool GRAV>
void launchHllcFluxG(const Grid& g, const Phys<real>& ph, const real* stage, const real* waves, real* flux,
                     unsigned* health, int hll, cudaStream_t st, const real* pot, long long c0, long long c1) {
    if (c1 < 0) c1 = g.V;
    if (c1 <= c0) return;
    // 2D and 3D: the tile kernel over whole slow-axis planes
    const long long plane = g.dim > 1 ? (long long)g.V / g.S[g.dim - 1] : 0;
    if (g.dim > 1 && c0 % plane == 0 && c1 % plane == 0) {
        const int s0 = (int)(c0 / plane), s1 = (int)(c1 / plane);
#define T(DD, H)                                                                                                  \
    {                                                                                                             \
        typedef FluxTile<DD> FT;                                                                                  \
        dim3 grid((unsigned)((g.S[0] + FT::X - 1) / FT::X),                                                       \
                  (unsigned)(DD == 2 ? (s1 - s0 + FT::Y - 1) / FT::Y : (g.S[1] + FT::Y - 1) / FT::Y),             \
                  (unsigned)(DD == 2 ? 1 : (s1 - s0 + FT::Z - 1) / FT::Z));                                        \
        hllcFluxTileKernel<real, DD, H, GRAV><<<grid, kThreads, 0, st>>>(g, ph, stage, waves, flux, health, pot,  \
                                                                          s0, s1);                                \
    }
        if (hll) {
            if (g.dim == 2) T(2, true)
            else T(3, true)
        } else {
            if (g.dim == 2)
                hllcFluxTileKernelWide<real, GRAV><<<tileGrid<2>(g, s0, s1), kThreads, 0, st>>>(g, ph, stage, waves,
                                                                                                flux, health, pot, s0,
                                                                                                s1);
            else T(3, false)
        }
#undef T
        return;
    }
#define L(DD, H)                                                                                                  \
    hllcFluxKernel<real, DD, H, GRAV><<<blocksFor(c1 - c0), kThreads, 0, st>>>(g, ph, stage, waves, flux, health, pot, \
                                                                             c0, c1)
    if (hll) {
        if (g.dim == 1) L(1, true);
        else if (g.dim == 2) L(2, true);
        else L(3, true);
    } else {
        if (g.dim == 1) L(1, false);
        else if (g.dim == 2) L(2, false);
        else L(3, false);
    }
#undef L
}

template <typename real>
void launchHllcFlux(const Grid& g, const Phys<real>& ph, const real* stage, const real* waves, real* flux,
                    unsigned* health, int hll, cudaStream_t st, const real* pot, long long c0, long long c1) {
    if (pot) launchHllcFluxG<real, true>(g, ph, stage, waves, flux, health, hll, st, pot, c0, c1);
    else launchHllcFluxG<real, false>(g, ph, stage, waves, flux, health, hll, st, nullptr, c0, c1);
}

#define INST(real)                                                                                                \
    template void launchHllcWaves<real>(const Grid&, const Phys<real>&, const real*, real*, int, cudaStream_t,    \
                                        const real*, long long, long long);                                       \
    template void launchHllcDt<real>(const Grid&, const Phys<real>&, const real*, unsigned long long*, unsigned*, \
                                     cudaStream_t);                                                               \
    template void launchHllcFlux<real>(const Grid&, const Phys<real>&, const real*, const real*, real*, unsigned*, \
                                       int, cudaStream_t, const real*, long long, long long);
INST(double)
INST(float)
#undef INST

}  // namespace hgpu
