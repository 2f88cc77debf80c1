// batch_flux.cu -- the batched interface-flux kernels (one translation unit of their
// own: they are instantiated per solver and slope limiter).  See batch.cu.
#include "../../../include/hgpu/hgpu.h"
#include "batch.h"
#include "batch_common.cuh"
#include "hllc_cells.cuh"
#include "roe_cells.cuh"

namespace hgpu {
namespace {

// HLLC (0 EulerRoe, 1 EulerHLLC, 2 EulerHLL) and LIM >= 0 fix the solver and the
// slope limiter at compile time (the kernel then carries one flux body and one
// limiter); -1 dispatches at run time
template <typename real, int D, int HLLC, int LIM>
__global__ void __launch_bounds__(256) batchFluxKernel(const BatchProblem<real>* __restrict__ P,
                                                       const BatchTile* __restrict__ tiles, int nT, BatchTuning tu,
                                                       int hllc, int lim, const StepConst<real>* __restrict__ sc,
                                                       const real* __restrict__ stage, const real* __restrict__ faces,
                                                       const real* __restrict__ dq, real* __restrict__ flux,
                                                       unsigned* health, unsigned* q) {
    for (int t = firstItem(q, tu); t < nT; t = nextItemAfter(q, tu)) {
        const BatchTile tl = tiles[t];
        const BatchProblem<real>& pr = P[tl.p];
        const real* st = stage + (long long)(D + 2) * pr.stateOff;
        for (int r = 0; r < tu.cpt; ++r) {
            int x, y, z;
            long long c;
            if (!tileCell(pr.g, tl, tu, threadIdx.x + r * blockDim.x, x, y, z, c)) continue;
            if (HLLC == 2 || (HLLC < 0 && hllc == 2)) {
                if (!hllcFluxCell<real, D, true>(pr.g, pr.ph, st, faces + pr.faceOff, flux + pr.dqOff, c, x, y, z))
                    atomicOr(health, HEALTH_HLLC_NOBRANCH);
            } else if (HLLC == 1 || (HLLC < 0 && hllc == 1)) {
                if (!hllcFluxCell<real, D>(pr.g, pr.ph, st, faces + pr.faceOff, flux + pr.dqOff, c, x, y, z))
                    atomicOr(health, HEALTH_HLLC_NOBRANCH);
            } else {
                roeFluxCell<real, D, LIM>(pr.g, lim, sc[tl.p], st, faces + pr.faceOff, dq + pr.dqOff,
                                          flux + pr.dqOff, c, x, y, z);
            }
        }
    }
}

// The FP64 EulerRoe flux in the single-problem kernels' two passes (roe_cells.cuh):
// per-wave corrections into the flux buffer, then the transforms over them.  Fewer
// live registers than the one-pass body, the same bits.
template <int D, int LIM, bool PLAIN>
__global__ void __launch_bounds__(256) batchFluxCorrKernel(const BatchProblem<double>* __restrict__ P,
                                                           const BatchTile* __restrict__ tiles, int nT, BatchTuning tu,
                                                           int lim, const StepConst<double>* __restrict__ sc,
                                                           const double* __restrict__ faces,
                                                           const double* __restrict__ dq, double* __restrict__ flux,
                                                           unsigned* q) {
    for (int t = firstTile<PLAIN>(q); t < nT; t = nextTile<PLAIN>(q, nT)) {
        const BatchTile tl = tiles[t];
        const BatchProblem<double>& pr = P[tl.p];
        const Grid g = pr.g;
        for (int r = 0; r < (PLAIN ? 1 : tu.cpt); ++r) {
            int x, y, z;
            long long c;
            if (!tileCell(g, tl, tu, threadIdx.x + r * blockDim.x, x, y, z, c)) continue;
            roeFluxCorrectionsCell<D, LIM, false, true>(g, lim, sc[tl.p], faces + pr.faceOff, dq + pr.dqOff,
                                                        flux + pr.dqOff, c, x, y, z);
        }
    }
}

// (2D plain: capped at 3 blocks per SM, 80 registers with a few spilled, as measured faster)
template <int D, bool PLAIN>
__global__ void __launch_bounds__(256, PLAIN && D <= 2 ? 3 : 1) batchFluxXformKernel(const BatchProblem<double>* __restrict__ P,
                                                            const BatchTile* __restrict__ tiles, int nT, BatchTuning tu,
                                                            const double* __restrict__ stage,
                                                            const double* __restrict__ faces,
                                                            double* __restrict__ flux, unsigned* q) {
    for (int t = firstTile<PLAIN>(q); t < nT; t = nextTile<PLAIN>(q, nT)) {
        const BatchTile tl = tiles[t];
        const BatchProblem<double>& pr = P[tl.p];
        const Grid g = pr.g;
        for (int r = 0; r < (PLAIN ? 1 : tu.cpt); ++r) {
            int x, y, z;
            long long c;
            if (!tileCell(g, tl, tu, threadIdx.x + r * blockDim.x, x, y, z, c)) continue;
            roeFluxTransformsCell<D>(g, stage + (long long)(D + 2) * pr.stateOff, faces + pr.faceOff, flux + pr.dqOff,
                                     c, x, y, z);
        }
    }
}

}  // namespace

template <typename real, int HLLC, int LIM>
static void batchFluxLaunch(const BatchLaunch<real>& b, int hllc, int lim, const StepConst<real>* sc,
                            const real* stage, const real* dq, real* fluxBuf, unsigned* health, unsigned* q) {
#define L(DD)                                                                                                       \
    batchFluxKernel<real, DD, HLLC, LIM><<<persistentBlocks(batchFluxKernel<real, DD, HLLC, LIM>, 0, b.tu.blocksPerSM, b.nT), \
                                           256, 0, b.st>>>(b.P, b.tiles, b.nT, b.tu, hllc, lim, sc, stage, b.faces, dq, \
                                                           fluxBuf, health, q)
    if (b.dim == 1) L(1);
    else if (b.dim == 2) L(2);
    else L(3);
#undef L
}

template <typename real>
void BatchLaunch<real>::flux(int hllc, int lim, const StepConst<real>* sc, const real* stage, const real* dq,
                             real* fluxBuf, unsigned* health, unsigned* q) const {
    if (hllc == 1) { batchFluxLaunch<real, 1, -1>(*this, hllc, lim, sc, stage, dq, fluxBuf, health, q); return; }
    if (hllc == 2) { batchFluxLaunch<real, 2, -1>(*this, hllc, lim, sc, stage, dq, fluxBuf, health, q); return; }
    switch (lim) {
    case HGPU_LIMITER_MINMOD: batchFluxLaunch<real, 0, HGPU_LIMITER_MINMOD>(*this, hllc, lim, sc, stage, dq, fluxBuf, health, q); break;
    case HGPU_LIMITER_SUPERBEE: batchFluxLaunch<real, 0, HGPU_LIMITER_SUPERBEE>(*this, hllc, lim, sc, stage, dq, fluxBuf, health, q); break;
    case HGPU_LIMITER_VANLEER: batchFluxLaunch<real, 0, HGPU_LIMITER_VANLEER>(*this, hllc, lim, sc, stage, dq, fluxBuf, health, q); break;
    case HGPU_LIMITER_MONOTIZEDCENTRAL: batchFluxLaunch<real, 0, HGPU_LIMITER_MONOTIZEDCENTRAL>(*this, hllc, lim, sc, stage, dq, fluxBuf, health, q); break;
    default: batchFluxLaunch<real, 0, -1>(*this, hllc, lim, sc, stage, dq, fluxBuf, health, q); break;
    }
}

template <int LIM>
static void batchFluxSplitLaunch(const BatchProblem<double>* P, const BatchTile* tiles, int nT, const BatchTuning& tu,
                                 int dim, cudaStream_t st, const double* faces, int lim, const StepConst<double>* sc,
                                 const double* stage, const double* dq, double* fluxBuf, unsigned* q0, unsigned* q1) {
#define L(DD)                                                                                                       \
    if (tu.blocksPerSM < 0 && tu.cpt == 1) {                                                                                       \
        batchFluxCorrKernel<DD, LIM, true><<<nT, 256, 0, st>>>(P, tiles, nT, tu, lim, sc, faces, dq, fluxBuf, q0);   \
        batchFluxXformKernel<DD, true><<<nT, 256, 0, st>>>(P, tiles, nT, tu, stage, faces, fluxBuf, q1);             \
    } else {                                                                                                        \
        batchFluxCorrKernel<DD, LIM, false><<<persistentBlocks(batchFluxCorrKernel<DD, LIM, false>, 0,               \
                                                               tu.blocksPerSM, nT), 256, 0, st>>>(                  \
            P, tiles, nT, tu, lim, sc, faces, dq, fluxBuf, q0);                                                     \
        batchFluxXformKernel<DD, false><<<persistentBlocks(batchFluxXformKernel<DD, false>, 0, tu.blocksPerSM, nT),  \
                                          256, 0, st>>>(P, tiles, nT, tu, stage, faces, fluxBuf, q1);               \
    }
    if (dim == 1) { L(1); }
    else if (dim == 2) { L(2); }
    else { L(3); }
#undef L
}

// FP64 only (the FP32 flux is not FP64-issue-bound and keeps the one-pass kernel)
template <typename real>
void BatchLaunch<real>::fluxSplit(int lim, const StepConst<real>* sc, const real* stage, const real* dq,
                                  real* fluxBuf, unsigned* q0, unsigned* q1) const {
    if (sizeof(real) != 8) return;
    const auto* P8 = reinterpret_cast<const BatchProblem<double>*>(P);
    const auto* sc8 = reinterpret_cast<const StepConst<double>*>(sc);
    const auto* st8 = reinterpret_cast<const double*>(stage);
    const auto* dq8 = reinterpret_cast<const double*>(dq);
    const auto* f8 = reinterpret_cast<const double*>(faces);
    auto* out8 = reinterpret_cast<double*>(fluxBuf);
#define S(LL) batchFluxSplitLaunch<LL>(P8, tiles, nT, tu, dim, st, f8, lim, sc8, st8, dq8, out8, q0, q1)
    switch (lim) {
    case HGPU_LIMITER_MINMOD: S(HGPU_LIMITER_MINMOD); break;
    case HGPU_LIMITER_SUPERBEE: S(HGPU_LIMITER_SUPERBEE); break;
    case HGPU_LIMITER_VANLEER: S(HGPU_LIMITER_VANLEER); break;
    case HGPU_LIMITER_MONOTIZEDCENTRAL: S(HGPU_LIMITER_MONOTIZEDCENTRAL); break;
    default: S(-1); break;
    }
#undef S
}

template void BatchLaunch<double>::fluxSplit(int, const StepConst<double>*, const double*, const double*, double*,
                                             unsigned*, unsigned*) const;
template void BatchLaunch<float>::fluxSplit(int, const StepConst<float>*, const float*, const float*, float*,
                                            unsigned*, unsigned*) const;

template void BatchLaunch<double>::flux(int, int, const StepConst<double>*, const double*, const double*, double*,
                                         unsigned*, unsigned*) const;
template void BatchLaunch<float>::flux(int, int, const StepConst<float>*, const float*, const float*, float*,
                                        unsigned*, unsigned*) const;

}  // namespace hgpu
