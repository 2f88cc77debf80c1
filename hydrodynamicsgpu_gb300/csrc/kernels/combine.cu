// combine.cu -- ghost fill, flux divergence + Runge-Kutta stage combine, dt finalisation.
//
// Reference pieces replaced:
//  * Solver::boundary + stateBoundary* kernels (src/Solver/Solver.cpp:448-464,
//    res/Common.cl:49-194): one launch per axis handles every state and both sides;
//  * calcFluxDeriv (res/CalcFluxDeriv.cl:7-44) fused with the integrator's multAdd
//    chain (res/Common.cl:201-210, include/HydroGPU/Integrator/RungeKutta.h:59-125):
//    instead of zero-filling a deriv buffer per stage and re-summing every stage
//    state from buffers, each stage adds its column of the tableau to the running
//    sums of all later rows.  Row m's additions still happen in column order, alpha
//    term before beta term, starting from +0, so every sum is bit-identical;
//  * findMinTimestep's host read and `dt * cfl` (Solver.cpp:466-516): dt is
//    finalised on the device, with dt/dx and beta*dt, for the whole step.
#include "combine_cells.cuh"
#include "kernels.h"

namespace hgpu {

namespace {
const double kA[12][4][4] = HGPU_TABLE_A;
const double kB[12][4][4] = HGPU_TABLE_B;
const int kOrder[12] = HGPU_TABLE_ORDER;
}  // namespace

int tableauOrder(int integ) { return kOrder[integ]; }
double tableauAlpha(int integ, int m, int k) { return kA[integ][m][k]; }
double tableauBeta(int integ, int m, int k) { return kB[integ][m][k]; }

namespace {

constexpr int kThreads = 256;
inline unsigned blocksFor(long long n) { return (unsigned)((n + kThreads - 1) / kThreads); }

// ---------------- ghost fill ----------------
template <typename real>
__global__ void __launch_bounds__(kThreads) boundaryKernel(Grid g, int axis, int N, int mMin, int mMax,
                                                           real* __restrict__ state, long long t0, long long t1) {
    const long long t = t0 + (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= t1) return;
    boundaryLine<real>(g, axis, N, mMin, mMax, state, t);
}

// ---------------- flux divergence + stage combine ----------------
// 5 blocks per SM (46 registers, no spills; 52 registers gave 4): KH 2048^2 step -1.1 %
template <typename real, int D>
__global__ void __launch_bounds__(kThreads, 5) derivCombineKernel(Grid g, Phys<real> ph, const real* __restrict__ flux,
                                                               CombinePlan<real> plan,
                                                               const StepConst<real>* __restrict__ sc, long long c0,
                                                               long long c1) {
    long long c = c0 + (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= c1) return;
    int x, y, z;
    cellCoords(g, c, x, y, z);
    derivCombineCell<real, D>(g, ph, flux, plan, *sc, c, x, y, z, 0);
}

template <typename real>
__global__ void __launch_bounds__(kThreads) alphaOnlyKernel(long long n, int integ, real* __restrict__ state,
                                                            const StepConst<real>* __restrict__ sc) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    state[i] = alphaOnlyElem<real>(integ, state[i], *sc);
}

template <typename real>
__global__ void finalizeDtKernel(Phys<real> ph, int integ, int useFixed, double fixedDt, unsigned long long* acc,
                                 unsigned long long accInit, StepConst<real>* sc) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    finalizeOne<real>(ph, integ, useFixed, fixedDt, acc, accInit, sc);
}

__global__ void resetAccKernel(unsigned long long* acc, unsigned long long v) { *acc = v; }

// Self-gravity pass with ForwardEuler and a zero potential: the (ghost-refreshed)
// state gets `state + deriv * dt` with deriv == +0 (ForwardEuler.cpp:20-32).
template <typename real>
__global__ void __launch_bounds__(kThreads) zeroAddKernel(long long n, real* __restrict__ state,
                                                          const StepConst<real>* __restrict__ sc) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    state[i] = state[i] + (real)0. * sc->dt;
}

}  // namespace

long long boundaryLines(const Grid& g, int axis) {
    return g.dim == 1 ? 1 : (long long)g.S[axis == 0 ? 1 : 0] * g.S[axis == 2 ? 1 : 2];
}

template <typename real>
void launchBoundaryAxis(const Grid& g, const int methods[3][2], real* state, cudaStream_t st, int axis, long long t0,
                        long long t1) {
    const long long n = boundaryLines(g, axis);
    if (t1 < 0 || t1 > n) t1 = n;
    if (t0 < 0) t0 = 0;
    if (t0 >= t1) return;
    boundaryKernel<real><<<blocksFor(t1 - t0), kThreads, 0, st>>>(g, axis, g.dim + 2, methods[axis][0],
                                                                   methods[axis][1], state, t0, t1);
}

template <typename real>
void launchBoundary(const Grid& g, const int methods[3][2], real* state, cudaStream_t st) {
    for (int axis = 0; axis < g.dim; ++axis) launchBoundaryAxis<real>(g, methods, state, st, axis, 0, -1);
}

template <typename real>
void launchDerivCombine(const Grid& g, const Phys<real>& ph, const real* flux, const CombinePlan<real>& plan,
                        const StepConst<real>* sc, cudaStream_t st, long long c0, long long c1) {
    if (c1 < 0 || c1 > g.V) c1 = g.V;
    if (c0 < 0) c0 = 0;
    if (c0 >= c1) return;
    const unsigned b = blocksFor(c1 - c0);
    if (g.dim == 1) derivCombineKernel<real, 1><<<b, kThreads, 0, st>>>(g, ph, flux, plan, sc, c0, c1);
    else if (g.dim == 2) derivCombineKernel<real, 2><<<b, kThreads, 0, st>>>(g, ph, flux, plan, sc, c0, c1);
    else derivCombineKernel<real, 3><<<b, kThreads, 0, st>>>(g, ph, flux, plan, sc, c0, c1);
}

template <typename real>
void launchAlphaOnly(const Grid& g, int integrator, real* state, const StepConst<real>* sc, cudaStream_t st) {
    long long n = g.V * (g.dim + 2);
    alphaOnlyKernel<real><<<blocksFor(n), kThreads, 0, st>>>(n, integrator, state, sc);
}

template <typename real>
void launchZeroAdd(const Grid& g, real* state, const StepConst<real>* sc, cudaStream_t st) {
    long long n = g.V * (g.dim + 2);
    zeroAddKernel<real><<<blocksFor(n), kThreads, 0, st>>>(n, state, sc);
}

template <typename real>
void launchFinalizeDt(const Phys<real>& ph, int integrator, int useFixed, double fixedDt, unsigned long long* acc,
                      unsigned long long accInit, StepConst<real>* sc, unsigned* health, cudaStream_t st) {
    (void)health;
    finalizeDtKernel<real><<<1, 32, 0, st>>>(ph, integrator, useFixed, fixedDt, acc, accInit, sc);
}

template <typename real>
void launchResetAcc(unsigned long long* acc, unsigned long long accInit, cudaStream_t st) {
    resetAccKernel<<<1, 1, 0, st>>>(acc, accInit);
}

#define INST(real)                                                                                              \
    template void launchBoundary<real>(const Grid&, const int[3][2], real*, cudaStream_t);                      \
    template void launchBoundaryAxis<real>(const Grid&, const int[3][2], real*, cudaStream_t, int, long long,   \
                                           long long);                                                          \
    template void launchDerivCombine<real>(const Grid&, const Phys<real>&, const real*, const CombinePlan<real>&, \
                                           const StepConst<real>*, cudaStream_t, long long, long long);         \
    template void launchAlphaOnly<real>(const Grid&, int, real*, const StepConst<real>*, cudaStream_t);         \
    template void launchZeroAdd<real>(const Grid&, real*, const StepConst<real>*, cudaStream_t);                \
    template void launchFinalizeDt<real>(const Phys<real>&, int, int, double, unsigned long long*,              \
                                         unsigned long long, StepConst<real>*, unsigned*, cudaStream_t);        \
    template void launchResetAcc<real>(unsigned long long*, unsigned long long, cudaStream_t);
INST(double)
INST(float)
#undef INST

}  // namespace hgpu
