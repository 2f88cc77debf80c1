// roe_record.cu -- the Roe flux kernel that also records, per face and wave, the
// values the adjoint's flux VJP reads back (roe.cuh FT_* planes).  The flux it writes
// is bit-identical to roeFluxKernel's (same code, extra stores).  FP64 only.
#include "../../../include/hgpu/hgpu.h"
#include "kernels.h"
#include "roe_cells.cuh"

namespace hgpu {
namespace {

constexpr int kThreads = 256;

template <int D, int LIM>
__global__ void __launch_bounds__(kThreads) roeFluxRecordKernel(Grid g, int lim, const double* __restrict__ stage,
                                                                const double* __restrict__ basis,
                                                                const double* __restrict__ dq,
                                                                const StepConst<double>* __restrict__ sc,
                                                                double* __restrict__ flux, double* __restrict__ tape) {
    long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.V) return;
    int x, y, z;
    cellCoords(g, c, x, y, z);
    roeFluxCell<double, D, LIM, true>(g, lim, *sc, stage, basis, dq, flux, c, x, y, z, tape);
}

template <int LIM>
void launchLim(const Grid& g, int lim, const double* stage, const double* basis, const double* dq,
               const StepConst<double>* sc, double* flux, double* tape, cudaStream_t st) {
    const unsigned blocks = (unsigned)((g.V + kThreads - 1) / kThreads);
    if (g.dim == 1) roeFluxRecordKernel<1, LIM><<<blocks, kThreads, 0, st>>>(g, lim, stage, basis, dq, sc, flux, tape);
    else if (g.dim == 2) roeFluxRecordKernel<2, LIM><<<blocks, kThreads, 0, st>>>(g, lim, stage, basis, dq, sc, flux, tape);
    else roeFluxRecordKernel<3, LIM><<<blocks, kThreads, 0, st>>>(g, lim, stage, basis, dq, sc, flux, tape);
}
}  // namespace

int roeFluxTapePlanes(int dim) { return FT_PLANES * (dim + 2) * dim; }

void launchRoeFluxRecord(const Grid& g, int limiter, const double* stage, const double* basis, const double* dq,
                         const StepConst<double>* sc, double* flux, double* tape, cudaStream_t st) {
    switch (limiter) {
    case HGPU_LIMITER_MINMOD: launchLim<HGPU_LIMITER_MINMOD>(g, limiter, stage, basis, dq, sc, flux, tape, st); break;
    case HGPU_LIMITER_SUPERBEE: launchLim<HGPU_LIMITER_SUPERBEE>(g, limiter, stage, basis, dq, sc, flux, tape, st); break;
    case HGPU_LIMITER_VANLEER: launchLim<HGPU_LIMITER_VANLEER>(g, limiter, stage, basis, dq, sc, flux, tape, st); break;
    case HGPU_LIMITER_MONOTIZEDCENTRAL:
        launchLim<HGPU_LIMITER_MONOTIZEDCENTRAL>(g, limiter, stage, basis, dq, sc, flux, tape, st);
        break;
    default: launchLim<-1>(g, limiter, stage, basis, dq, sc, flux, tape, st); break;
    }
}

}  // namespace hgpu
