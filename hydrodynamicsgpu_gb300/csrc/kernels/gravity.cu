// gravity.cu -- self-gravity with a live potential for sm_103a: the potential's
// starting guess, its ghost fill, the Poisson relaxation sweeps and the gravity
// source term fused with the integrator's combine.
//
// Reference pieces replaced (KennethYeah/HydrodynamicsGPU):
//  * SelfGravitation::resetState (src/Solver/SelfGravitation.cpp:35-98): with
//    useGravity the potential starts as -density, is relaxed, and the starting guess
//    (the host vector, not the relaxed buffer) is added to the total energy;
//  * SelfGravitation::potentialBoundary (:126-140) with the potential's boundary
//    kernels (include/HydroGPU/Equation/SelfGravitationBehavior.h:22-34: PERIODIC ->
//    periodic, MIRROR and FREEFLOW -> free flow) on a stride-1 buffer;
//  * gravityPotentialPoissonRelax (res/SelfGravitation.cl:20-63).  The reference
//    kernel updates the potential in place while its neighbours read it, so a launch
//    has no single result: each order in which a device runs the work-items gives its
//    own.  Here a launch is the red-black order, one of those the reference permits:
//    every interior cell with x + y + z even first (their neighbours are all odd, so
//    these updates do not see each other), then every odd cell (reading the new even
//    values).  It is deterministic and each half is one parallel sweep;
//  * calcGravityDeriv (res/SelfGravitation.cl:65-102) into a deriv that goes straight
//    into the integrator's combine (combinePlanCell), as the flux divergence does.
// Per-cell expressions follow the reference's operation order and types: in FP32 the
// double literals of `4. * M_PI * G * density`, `-2. * (1. / (DX * DX) ...)` and
// `/ (2. * dx[side])` promote those expressions to double.
#include "../../../include/hgpu/hgpu.h"
#include "combine_cells.cuh"
#include "gravity.h"

namespace hgpu {
namespace {

constexpr int kThreads = 256;
inline unsigned blocksFor(long long n) { return (unsigned)((n + kThreads - 1) / kThreads); }

// potential = -density (useGravity) or the given channel; total energy += that potential
template <typename real, int D>
__global__ void __launch_bounds__(kThreads) potentialInitKernel(Grid g, int fromDensity, real* __restrict__ state,
                                                                real* __restrict__ pot, long long c0, long long c1) {
    const long long c = c0 + (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= c1) return;
    real* s = state + (long long)(D + 2) * c;
    const real p = fromDensity ? -s[0] : pot[c];
    pot[c] = p;
    s[D + 1] = s[D + 1] + p;
}

// the potential's ghost fill along one axis: boundaryLine on a one-component buffer
template <typename real>
__global__ void __launch_bounds__(kThreads) potentialBoundaryKernel(Grid g, int axis, int mMin, int mMax,
                                                                    real* __restrict__ pot) {
    boundaryLine<real>(g, axis, 1, mMin, mMax, pot, (long long)blockIdx.x * blockDim.x + threadIdx.x);
}

// rhs = 4. * M_PI * G * density (double) of every cell, from the stage state: fixed
// while a callback's sweeps run, so it is formed once and the sweeps read 8 bytes a
// cell instead of the state's record
template <typename real, int D>
__global__ void __launch_bounds__(kThreads) relaxRhsKernel(Grid g, GravityConst<real> gc,
                                                           const real* __restrict__ state, double* __restrict__ rhs) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.V) return;
    rhs[c] = mulI(gc.fourPiG, (double)state[(long long)(D + 2) * c]);
}

// x / dx^2 of the relaxation, exact: FP64 by the quotient correction on RN(1 / dx^2)
// (fp64ops.cuh divByRecip: two FMAs on the FP64 unit) or on the integer pipes (divI);
// FP32 the float division.  Measured on GB300 (2048^2 sweep): the x neighbours by the
// correction and the rest on the integer pipes balance the two units best (0.134 ms a
// sweep; all on the integer pipes 0.168, every neighbour by the correction 0.154).
template <bool RECIP>
__device__ __forceinline__ double overDxSq(double x, double d, double rd) {
    return RECIP ? divByRecip(x, d, rd) : divI(x, d);
}
template <bool RECIP>
__device__ __forceinline__ float overDxSq(float x, float d, double) { return x / d; }

// one colour of a relaxation sweep: blockIdx.y (+ gridDim.y * blockIdx.z) = the interior
// row (y, z), thread x = the k-th cell of that colour along the row
template <typename real, int D>
__global__ void __launch_bounds__(kThreads) relaxKernel(Grid g, GravityConst<real> gc, int colour,
                                                        const double* __restrict__ rhs, real* __restrict__ pot) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = D > 1 ? (int)blockIdx.y + 2 : 0, z = D > 2 ? (int)blockIdx.z + 2 : 0;
    // x = 2 + 2k + shift, with shift chosen so that x + y + z has the colour's parity
    const int x = 2 + 2 * k + (((y + z) & 1) ^ colour);
    if (x >= g.S[0] - 2) return;
    const long long c = x + (long long)g.S[0] * (y + (long long)g.S[1] * z);
    // skewSum: +x, -x, +y, -y, +z, -z neighbours inside [2, S-3] (SelfGravitation.cl:39-51)
    real skewSum = (real)0;
    if (x < g.S[0] - 3) skewSum = skewSum + overDxSq<true>(pot[c + 1], gc.dxSq[0], gc.rdxSq[0]);
    if (x > 2) skewSum = skewSum + overDxSq<true>(pot[c - 1], gc.dxSq[0], gc.rdxSq[0]);
    if (D > 1) {
        const long long sy = g.step[1];
        if (y < g.S[1] - 3) skewSum = skewSum + overDxSq<false>(pot[c + sy], gc.dxSq[1], gc.rdxSq[1]);
        if (y > 2) skewSum = skewSum + overDxSq<false>(pot[c - sy], gc.dxSq[1], gc.rdxSq[1]);
    }
    if (D > 2) {
        const long long sz = g.step[2];
        if (z < g.S[2] - 3) skewSum = skewSum + overDxSq<false>(pot[c + sz], gc.dxSq[2], gc.rdxSq[2]);
        if (z > 2) skewSum = skewSum + overDxSq<false>(pot[c - sz], gc.dxSq[2], gc.rdxSq[2]);
    }
    // (4. * M_PI * G * density - skewSum) / diag, in double for both precisions
    pot[c] = (real)divI(rhs[c] - (double)skewSum, gc.diag);
}

// calcGravityDeriv of one cell into d (zero outside the interior), then the combine
template <typename real, int D>
__global__ void __launch_bounds__(kThreads) gravityCombineKernel(Grid g, GravityConst<real> gc,
                                                                 const real* __restrict__ stage,
                                                                 const real* __restrict__ pot, CombinePlan<real> plan,
                                                                 const StepConst<real>* __restrict__ sc) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.V) return;
    int x, y, z;
    cellCoords(g, c, x, y, z);
    const int N = D + 2, E = D + 1;
    real d[N];
#pragma unroll
    for (int j = 0; j < N; ++j) d[j] = (real)0;
    if (inRange(g, x, y, z, 2, 2)) {
        const real* st = stage + (long long)N * c;
        const real density = st[0];
        real derivEnergyTotal = (real)0;
#pragma unroll
        for (int side = 0; side < D; ++side) {
            const long long sp = g.step[side];
            const real dphi = pot[c + sp] - pot[c - sp];
            // (phi[next] - phi[prev]) / (2. * dx[side]): a double quotient, stored as real
            const real gradient = (real)divI((double)dphi, gc.twoDx[side]);
            const real gravity = -gradient;
            const real f = mulI(density, gravity);
            d[1 + side] = zfix(-f);                                  // deriv (+0) -= density * gravity
            const real e = mulI(f, st[1 + side]);
            derivEnergyTotal = side == 0 ? zfix(-e) : derivEnergyTotal - e;
        }
        d[E] = zfix(derivEnergyTotal);                               // deriv[E] (+0) += derivEnergyTotal
    }
    combinePlanCell<real, D>(d, plan, *sc, c, 0);
}

}  // namespace

template <typename real>
GravityConst<real> gravityConst(const double dx[3], double G, int dim) {
    GravityConst<real> gc;
    // ((real)G) as the program's define makes it; 4. * M_PI * G in double, left to right
    gc.fourPiG = (4. * 3.14159265358979323846) * (double)(real)G;
    double invSum = 0.;
    for (int i = 0; i < dim; ++i) {
        const real dxr = (real)dx[i];
        const real sq = dxr * dxr;                                  // DX * DX in the program's type
        gc.dxSq[i] = sq;
        gc.rdxSq[i] = 1. / (double)sq;                                // RN(1 / dx^2) for the exact quotient
        invSum = i == 0 ? 1. / (double)sq : invSum + 1. / (double)sq;
        gc.twoDx[i] = 2. * (double)dxr;
    }
    for (int i = dim; i < 3; ++i) { gc.dxSq[i] = (real)1; gc.rdxSq[i] = 1.; gc.twoDx[i] = 2.; }
    gc.diag = (double)(real)(-2. * invSum);                          // `const real diag`
    return gc;
}

template <typename real>
void launchPotentialInit(const Grid& g, int fromDensity, real* state, real* pot, cudaStream_t st, long long c0,
                         long long c1) {
    if (c1 < 0 || c1 > g.V) c1 = g.V;
    if (c0 < 0) c0 = 0;
    if (c0 >= c1) return;
    const unsigned b = blocksFor(c1 - c0);
    if (g.dim == 1) potentialInitKernel<real, 1><<<b, kThreads, 0, st>>>(g, fromDensity, state, pot, c0, c1);
    else if (g.dim == 2) potentialInitKernel<real, 2><<<b, kThreads, 0, st>>>(g, fromDensity, state, pot, c0, c1);
    else potentialInitKernel<real, 3><<<b, kThreads, 0, st>>>(g, fromDensity, state, pot, c0, c1);
}

template <typename real>
void launchPotentialBoundary(const Grid& g, const int methods[3][2], real* pot, cudaStream_t st) {
    for (int axis = 0; axis < g.dim; ++axis) {
        int m[2];
        for (int k = 0; k < 2; ++k)
            m[k] = methods[axis][k] == HGPU_BOUNDARY_MIRROR ? HGPU_BOUNDARY_FREEFLOW : methods[axis][k];
        const long long n = g.dim == 1 ? 1 : (long long)g.S[axis == 0 ? 1 : 0] * g.S[axis == 2 ? 1 : 2];
        potentialBoundaryKernel<real><<<blocksFor(n), kThreads, 0, st>>>(g, axis, m[0], m[1], pot);
    }
}

template <typename real>
void launchRelaxRhs(const Grid& g, const GravityConst<real>& gc, const real* state, double* rhs, cudaStream_t st) {
    if (g.dim == 1) relaxRhsKernel<real, 1><<<blocksFor(g.V), kThreads, 0, st>>>(g, gc, state, rhs);
    else if (g.dim == 2) relaxRhsKernel<real, 2><<<blocksFor(g.V), kThreads, 0, st>>>(g, gc, state, rhs);
    else relaxRhsKernel<real, 3><<<blocksFor(g.V), kThreads, 0, st>>>(g, gc, state, rhs);
}

template <typename real>
void launchRelaxSweep(const Grid& g, const GravityConst<real>& gc, const double* rhs, real* pot, cudaStream_t st) {
    const int nx = g.S[0] - 4, ny = g.dim > 1 ? g.S[1] - 4 : 1, nz = g.dim > 2 ? g.S[2] - 4 : 1;
    if (nx <= 0 || ny <= 0 || nz <= 0) return;
    const dim3 grid((unsigned)((nx + 1) / 2 + kThreads - 1) / kThreads, (unsigned)ny, (unsigned)nz);
    for (int colour = 0; colour < 2; ++colour) {
        if (g.dim == 1) relaxKernel<real, 1><<<grid, kThreads, 0, st>>>(g, gc, colour, rhs, pot);
        else if (g.dim == 2) relaxKernel<real, 2><<<grid, kThreads, 0, st>>>(g, gc, colour, rhs, pot);
        else relaxKernel<real, 3><<<grid, kThreads, 0, st>>>(g, gc, colour, rhs, pot);
    }
}

template <typename real>
void launchGravityCombine(const Grid& g, const GravityConst<real>& gc, const real* stage, const real* pot,
                          const CombinePlan<real>& plan, const StepConst<real>* sc, cudaStream_t st) {
    if (g.dim == 1) gravityCombineKernel<real, 1><<<blocksFor(g.V), kThreads, 0, st>>>(g, gc, stage, pot, plan, sc);
    else if (g.dim == 2) gravityCombineKernel<real, 2><<<blocksFor(g.V), kThreads, 0, st>>>(g, gc, stage, pot, plan, sc);
    else gravityCombineKernel<real, 3><<<blocksFor(g.V), kThreads, 0, st>>>(g, gc, stage, pot, plan, sc);
}

#define INST(real)                                                                                              \
    template GravityConst<real> gravityConst<real>(const double[3], double, int);                              \
    template void launchPotentialInit<real>(const Grid&, int, real*, real*, cudaStream_t, long long, long long);                      \
    template void launchPotentialBoundary<real>(const Grid&, const int[3][2], real*, cudaStream_t);            \
    template void launchRelaxRhs<real>(const Grid&, const GravityConst<real>&, const real*, double*, cudaStream_t); \
    template void launchRelaxSweep<real>(const Grid&, const GravityConst<real>&, const double*, real*, cudaStream_t); \
    template void launchGravityCombine<real>(const Grid&, const GravityConst<real>&, const real*, const real*,    \
                                             const CombinePlan<real>&, const StepConst<real>*, cudaStream_t);
INST(double)
INST(float)
#undef INST

}  // namespace hgpu
