// roe_record.cu -- the Roe flux kernels that also record, per face and wave, the
// values the adjoint's flux VJP reads back (roe.cuh FT_* planes).  The flux they
// write is bit-identical to the production FP64 flux's (same code, extra stores).
#include "../../../include/hgpu/hgpu.h"
#include "kernels.h"
#include "roe_cells.cuh"

namespace hgpu {
namespace {

constexpr int kThreads = 256;

// two passes, as the production FP64 flux runs (roe.cu): the per-wave corrections
// (recording A, phi, phi', r), then the transforms (recording L avg and ft)
template <int D, int LIM>
__global__ void __launch_bounds__(kThreads) roeFluxCorrRecordKernel(Grid g, int lim,
                                                                    const double* __restrict__ basis,
                                                                    const double* __restrict__ dq,
                                                                    const StepConst<double>* __restrict__ sc,
                                                                    double* __restrict__ flux,
                                                                    double* __restrict__ tape) {
    long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.V) return;
    int x, y, z;
    cellCoords(g, c, x, y, z);
    roeFluxCorrectionsCell<D, LIM, true>(g, lim, *sc, basis, dq, flux, c, x, y, z, tape);
}

template <int D>
__global__ void __launch_bounds__(kThreads) roeFluxXformRecordKernel(Grid g, const double* __restrict__ stage,
                                                                     const double* __restrict__ basis,
                                                                     double* __restrict__ flux,
                                                                     double* __restrict__ tape) {
    long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.V) return;
    int x, y, z;
    cellCoords(g, c, x, y, z);
    roeFluxTransformsCell<D, true>(g, stage, basis, flux, c, x, y, z, tape);
}

template <int LIM>
void launchLim(const Grid& g, int lim, const double* stage, const double* basis, const double* dq,
               const StepConst<double>* sc, double* flux, double* tape, cudaStream_t st) {
    const unsigned blocks = (unsigned)((g.V + kThreads - 1) / kThreads);
#define L(DD)                                                                                            \
    roeFluxCorrRecordKernel<DD, LIM><<<blocks, kThreads, 0, st>>>(g, lim, basis, dq, sc, flux, tape);      \
    roeFluxXformRecordKernel<DD><<<blocks, kThreads, 0, st>>>(g, stage, basis, flux, tape)
    if (g.dim == 1) { L(1); }
    else if (g.dim == 2) { L(2); }
    else { L(3); }
#undef L
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
