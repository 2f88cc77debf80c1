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
    for (;;) {
        int t = nextItem(q);
        if (t >= nT) break;
        const BatchTile tl = tiles[t];
        const BatchProblem<real>& pr = P[tl.p];
        int x, y, z;
        long long c;
        if (!tileCell(pr.g, tl, tu, x, y, z, c)) continue;
        const real* st = stage + (long long)(D + 2) * pr.stateOff;
        if (HLLC == 2 || (HLLC < 0 && hllc == 2)) {
            if (!hllcFluxCell<real, D, true>(pr.g, pr.ph, st, faces + pr.faceOff, flux + pr.dqOff, c, x, y, z))
                atomicOr(health, HEALTH_HLLC_NOBRANCH);
        } else if (HLLC == 1 || (HLLC < 0 && hllc == 1)) {
            if (!hllcFluxCell<real, D>(pr.g, pr.ph, st, faces + pr.faceOff, flux + pr.dqOff, c, x, y, z))
                atomicOr(health, HEALTH_HLLC_NOBRANCH);
        } else {
            roeFluxCell<real, D, LIM>(pr.g, lim, sc[tl.p], st, faces + pr.faceOff, dq + pr.dqOff, flux + pr.dqOff, c,
                                      x, y, z);
        }
    }
}

}  // namespace

template <typename real, int HLLC, int LIM>
static void batchFluxLaunch(const BatchLaunch<real>& b, int hllc, int lim, const StepConst<real>* sc,
                            const real* stage, const real* dq, real* fluxBuf, unsigned* health, unsigned* q) {
#define L(DD)                                                                                                       \
    batchFluxKernel<real, DD, HLLC, LIM><<<persistentBlocks(batchFluxKernel<real, DD, HLLC, LIM>, 0, b.tu.blocksPerSM), \
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

template void BatchLaunch<double>::flux(int, int, const StepConst<double>*, const double*, const double*, double*,
                                         unsigned*, unsigned*) const;
template void BatchLaunch<float>::flux(int, int, const StepConst<float>*, const float*, const float*, float*,
                                        unsigned*, unsigned*) const;

}  // namespace hgpu
