// combine_cells.cuh -- per-cell bodies of the ghost fill, flux divergence + RK combine
// and timestep finalisation, shared by combine.cu and the batched kernels (batch.cu).
#pragma once
#include "kernels.h"

namespace hgpu {

// ---------------- tableaus: include/HydroGPU/Integrator/RungeKutta.h:129-294 ----------------
#define HGPU_TABLE_A                                                                                         \
    {{{1}},                                                                                                  \
     {{1, 0}, {1, 0}},                                                                                       \
     {{1, 0}, {1, 0}},                                                                                       \
     {{1, 0}, {1, 0}},                                                                                       \
     {{1, 0, 0}, {1, 0, 0}, {1, 0, 0}},                                                                      \
     {{1, 0, 0, 0}, {1, 0, 0, 0}, {1, 0, 0, 0}, {1, 0, 0, 0}},                                               \
     {{1, 0, 0, 0}, {1, 0, 0, 0}, {1, 0, 0, 0}, {1, 0, 0, 0}},                                               \
     {{1, 0}, {.5, .5}},                                                                                     \
     {{1, 0}, {1, 0}},                                                                                       \
     {{1, 0, 0}, {3. / 4., 1. / 4., 0}, {1. / 3., 2. / 3., 0}},                                              \
     {{1, 0, 0, 0}, {649. / 1600., 951. / 1600., 0, 0},                                                      \
      {53989. / 2500000., 4806213. / 20000000., 23619. / 32000., 0},                                         \
      {1. / 5., 6127. / 30000., 7873. / 30000., 1. / 3.}},                                                   \
     {{1, 0, 0, 0}, {1, 0, 0, 0}, {1, 0, 0, 0}, {-1. / 3., 1. / 3., 2. / 3., 1. / 3.}}}
#define HGPU_TABLE_B                                                                                         \
    {{{1}},                                                                                                  \
     {{.5, 0}, {0, 1}},                                                                                      \
     {{1, 0}, {.5, .5}},                                                                                     \
     {{2. / 3., 0}, {1. / 4., 3. / 4.}},                                                                     \
     {{.5, 0, 0}, {-1, 2, 0}, {1. / 6., 2. / 6., 1. / 6.}},                                                  \
     {{.5, 0, 0, 0}, {0, .5, 0, 0}, {0, 0, 1, 0}, {1. / 6., 2. / 6., 2. / 6., 1. / 6.}},                     \
     {{1. / 3., 0, 0, 0}, {-1. / 3., 0, 0, 0}, {1, -1, 1, 0}, {1. / 8., 3. / 8., 3. / 8., 1. / 8.}},         \
     {{1, 0}, {0, .5}},                                                                                      \
     {{-20, 0}, {41. / 40., -1. / 40.}},                                                                     \
     {{1, 0, 0}, {0, 1. / 4., 0}, {0, 0, 2. / 3.}},                                                          \
     {{.5, 0, 0, 0}, {-10890423. / 25193600., 5000. / 7873, 0, 0},                                           \
      {-102261. / 5000000., -5121. / 20000., 7873. / 10000., 0}, {1. / 10., 1. / 6., 0, 1. / 6.}},          \
     {{.5, 0, 0, 0}, {0, .5, 0, 0}, {0, 0, 1, 0}, {0, 0, 0, 1. / 6.}}}
#define HGPU_TABLE_ORDER {1, 2, 2, 2, 3, 4, 4, 2, 2, 3, 4, 4}

namespace {
__constant__ double cA[12][4][4] = HGPU_TABLE_A;
__constant__ double cB[12][4][4] = HGPU_TABLE_B;
__constant__ int cOrder[12] = HGPU_TABLE_ORDER;
__device__ __forceinline__ int kOrderDev(int i) { return cOrder[i]; }
__device__ __forceinline__ double kAlphaDev(int i, int m, int k) { return cA[i][m][k]; }
__device__ __forceinline__ double kBetaDev(int i, int m, int k) { return cB[i][m][k]; }
}  // namespace

// One ghost line of the boundary pass along `axis` (thread = transverse line t):
// every state, min side then max side.  In 1D the reference's Mirror/Reflect/FreeFlow
// kernels have no range guard and only work-item 0 addresses the buffer; that
// work-item is what runs here.
template <typename real>
__device__ __forceinline__ void boundaryLine(const Grid& g, int axis, int N, int mMin, int mMax,
                                             real* __restrict__ state, long long t) {
    int A = axis == 0 ? 1 : 0, B = axis == 2 ? 1 : 2;   // transverse axes
    long long nA = g.S[A], nB = g.S[B];
    if (g.dim == 1) { nA = 1; nB = 1; }
    if (t >= nA * nB) return;
    int a = (int)(t % nA), b = (int)(t / nA);
    int c[3];
    c[A] = a; c[B] = b; c[axis] = 0;
    long long base = c[0] + (long long)g.S[0] * (c[1] + (long long)g.S[1] * c[2]);
    long long st = g.step[axis];
    int S = g.S[axis];
    if (!cellOk(g, base) || !cellOk(g, base + (long long)(S - 1) * st)) return;
    for (int j = 0; j < N; ++j) {
        real* p = state + j;
#define AT(k) p[(long long)N * (base + (long long)(k) * st)]
        for (int side = 0; side < 2; ++side) {
            int m = side == 0 ? mMin : mMax;
            if (m < 0) continue;
            // Euler::stateGetBoundaryKernelForBoundaryMethod: MIRROR reflects the normal momentum
            int kern = m == 0 ? 0 : (m == 1 ? ((axis + 1 == j) ? 2 : 1) : 3);
            if (kern == 0) {                                  // periodic
                if (side == 0) { AT(0) = AT(S - 4); AT(1) = AT(S - 3); }
                else { AT(S - 2) = AT(2); AT(S - 1) = AT(3); }
            } else if (kern == 1) {                           // mirror
                if (side == 0) { AT(0) = AT(3); AT(1) = AT(2); }
                else { AT(S - 1) = AT(S - 4); AT(S - 2) = AT(S - 3); }
            } else if (kern == 2) {                           // reflect
                if (side == 0) { AT(0) = -AT(3); AT(1) = -AT(2); }
                else { AT(S - 1) = -AT(S - 4); AT(S - 2) = -AT(S - 3); }
            } else {                                          // free flow
                if (side == 0) { real v = AT(2); AT(1) = v; AT(0) = v; }
                else { real v = AT(S - 3); AT(S - 2) = v; AT(S - 1) = v; }
            }
        }
#undef AT
    }
}

// x * y for an x that is often +-0 (flux differences of piecewise-constant states):
// the signed zero from the bit patterns when x is zero and y finite (what the product
// gives), otherwise mulI, whose zero operands take an out-of-line FP64 call
__device__ __forceinline__ double mulZ(double x, double y) {
    if (isZeroBits(x) && finiteD(y)) return fromBits((bitsOf(x) ^ bitsOf(y)) & (long long)0x8000000000000000ULL);
    return mulI(x, y);
}
__device__ __forceinline__ float mulZ(float x, float y) { return x * y; }

// FLATD: the deriv's products by mulZ (the batched kernels, whose states are mostly flat)
template <typename real, int D, bool FLATD = false>
__device__ __forceinline__ void combinePlanCell(const real* d, const CombinePlan<real>& plan,
                                                const StepConst<real>& sc, long long c, long long off);

// Flux divergence and Runge-Kutta combine of one cell (res/CalcFluxDeriv.cl:7-44 and
// the multAdd chain).  `off` is the cell offset of this grid inside the slot arrays
// (0 for a single problem; the problem's first cell in a batch).
// RECIP_SIDES: deltaFlux / dx by the exact quotient correction on RN(1/dx) (divByRecip,
// two FMAs) for the first RECIP_SIDES axes, on the integer pipes (divI) for the rest.
// Measured: the single-problem kernel is fastest with 1 (0.357 ms a launch at 2048^2,
// 0.390 with 0, 0.408 with every axis), the batched persistent one with every axis.
template <typename real, int D, int RECIP_SIDES = 1, bool FLATD = false>
__device__ __forceinline__ void derivCombineCell(const Grid& g, const Phys<real>& ph, const real* __restrict__ flux,
                                                 const CombinePlan<real>& plan, const StepConst<real>& sc,
                                                 long long c, int x, int y, int z, long long off) {
    const int N = D + 2;
    real d[N];
    if (!cellOk(g, c)) return;
    // calcFluxDeriv: interior cells only, deriv[j] -= (F[i+1] - F[i]) / dx, sides ascending, from 0
    if (inRange(g, x, y, z, 2, 2)) {
#pragma unroll
        for (int side = 0; side < D; ++side)
            if (!cellOk(g, c + g.step[side])) return;
#pragma unroll
        for (int side = 0; side < D; ++side) {
#pragma unroll
            for (int j = 0; j < N; ++j) {
                const real* f = flux + ((long long)side * N + j) * g.V + c;
                const real df = f[g.step[side]] - f[0];                 // deltaFlux / dx[side]
                real t = side < RECIP_SIDES ? divByRecip(df, ph.dx[side], ph.rdx[side]) : divI(df, ph.dx[side]);
                d[j] = side == 0 ? zfix(-t) : d[j] - t;
            }
        }
    } else {
#pragma unroll
        for (int j = 0; j < N; ++j) d[j] = (real)0.;
    }
    combinePlanCell<real, D, FLATD>(d, plan, sc, c, off);
}

// The integrator's use of one cell's deriv d: ForwardEuler's state += deriv * dt, or
// this stage's column of the Runge-Kutta rows (see combine.cu).
template <typename real, int D, bool FLATD>
__device__ __forceinline__ void combinePlanCell(const real* d, const CombinePlan<real>& plan,
                                                const StepConst<real>& sc, long long c, long long off) {
    const int N = D + 2;
    if (plan.fe) {                                            // ForwardEuler::integrate: state += deriv * dt
        real dt = sc.dt;
        real* s = plan.slot[0] + (long long)N * (off + c);
#pragma unroll
        for (int j = 0; j < N; ++j) s[j] = s[j] + (FLATD ? mulZ(d[j], dt) : mulI(d[j], dt));
        return;
    }
    real u[N];
    const real* in = plan.slot[plan.in] + (long long)N * (off + c);
#pragma unroll
    for (int j = 0; j < N; ++j) u[j] = in[j];
    for (int o = 0; o < plan.nops; ++o) {
        const CombineOp<real>& op = plan.ops[o];
        real v[N];
        bool empty = op.prior < 0;
        if (!empty) {
            const real* p = plan.slot[op.prior] + (long long)N * (off + c);
#pragma unroll
            for (int j = 0; j < N; ++j) v[j] = op.priorAlias ? zfix(p[j]) : p[j];
        }
        if (op.hasAlpha) {
#pragma unroll
            for (int j = 0; j < N; ++j) {
                real t = op.alphaIsOne ? u[j] : mulI(u[j], op.alpha);
                v[j] = empty ? zfix(t) : v[j] + t;
            }
            empty = false;
        }
        if (op.hasBeta) {
            real cf = sc.coef[op.brow][op.bcol];
#pragma unroll
            for (int j = 0; j < N; ++j) {
                real t = FLATD ? mulZ(d[j], cf) : mulI(d[j], cf);
                v[j] = empty ? zfix(t) : v[j] + t;
            }
        }
        real* o_ = plan.slot[op.out] + (long long)N * (off + c);
#pragma unroll
        for (int j = 0; j < N; ++j) o_[j] = v[j];
    }
}

// dt of one problem from its reduced minimum: `dt * app->cfl` (Solver.cpp:515) or the
// fixed dt; then dt/dx and beta*dt for the step; re-arms the accumulator.
template <typename real>
__device__ __forceinline__ void finalizeOne(const Phys<real>& ph, int integ, int useFixed, double fixedDt,
                                            unsigned long long* acc, unsigned long long accInit, StepConst<real>* sc) {
    real dt;
    if (useFixed) dt = (real)fixedDt;
    else {
        real mn = (real)bitsToDouble(*acc, sizeof(real) == 4);
        dt = (real)(mn * (real)ph.cfl);
        *acc = accInit;
    }
    sc->dt = dt;
    sc->dt_f64 = (double)dt;
    for (int s = 0; s < 3; ++s) sc->dt_dx[s] = dt / ph.dx[s];
    for (int m = 0; m < 4; ++m)
        for (int k = 0; k < 4; ++k) sc->coef[m][k] = (real)kBetaDev(integ, m, k) * dt;
}

// self-gravity pass with a zero potential and a Runge-Kutta integrator, one element
template <typename real>
__device__ __forceinline__ real alphaOnlyElem(int integ, real u0, const StepConst<real>& sc) {
    const int order = kOrderDev(integ);
    real u[5];
    u[0] = u0;
    for (int s = 1; s <= order; ++s) {
        real r = 0;
        bool empty = true;
        for (int k = 0; k < s; ++k) {
            double a = kAlphaDev(integ, s - 1, k), b = kBetaDev(integ, s - 1, k);
            if (a != 0) { real t = u[k] * (real)a; r = empty ? zfix(t) : r + t; empty = false; }
            if (b != 0) { real t = (real)0. * sc.coef[s - 1][k]; r = empty ? zfix(t) : r + t; empty = false; }
        }
        u[s] = r;
    }
    return u[order];
}

}  // namespace hgpu
