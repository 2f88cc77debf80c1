// adjoint.h -- reverse-mode kernels of one EulerRoe step (FP64), launched by host/adjoint.cu.
//
// The step being differentiated is the forward step with its dt frozen:
//   u_0 = G(u^n)                       (ghost fill, a linear map)
//   B   = eigenbasis(u_0)              (frozen for the step, res/Roe.cl via Roe.cpp:82-92)
//   u_m = sum_k alpha[m][k] u_k + beta[m][k] dt F(u_k; B),   m = 1..s
// with F the limited-flux divergence.  Its vector-Jacobian product runs the stages
// backwards: the flux kernel turns the divergence cotangent of stage k into face
// cotangents (cells, Delta-q-tilde of three faces, and the four eigenbasis
// parameters vx, vt, H, c), the Delta-q kernel folds the Delta-q cotangents back to
// cells, the cell kernel gathers them plus the alpha terms into lambda_k; after the
// last stage the eigenbasis cotangents go back through the Roe averages to u_0 and
// the transposed ghost fill gives lambda^n.
#pragma once
#include "kernels.h"

namespace hgpu {

// cotangents of the later stages that feed stage k:
// dL/dF_k = sum_i coefF[i] lam[i],   lambda_k += sum_i alpha[i] lam[i]
struct AdjStage {
    const double* lam[4];
    double coefF[4];
    double alpha[4];
    int nlam;
};

// per-face scratch (planes of V values; face planes indexed [(side*W + j)*V + cell])
struct AdjScratch {
    double* gAvg;     // N per face: d/d(state of either cell) through the face average (half of it)
    double* gdqSelf;  // N per face: Delta-q-tilde cotangent of this face from its own flux
    double* gdqToM;   // N per face: ... of face f - step (the upwind face of a right-going wave)
    double* gdqToP;   // N per face: ... of face f + step
    double* gDelta;   // N per face: L^T gdq, added to the right cell and taken from the left cell
    double* gParam;   // D+2 per face: (vx, vt..., H, c) in the face's normal frame, summed over stages
    double* gPrimL;   // D+2 per face: (v..., h, w) of the left cell
    double* gPrimR;   // D+2 per face: (v..., h, w) of the right cell
};

// the forward flux that also records the per-wave values the flux VJP reads
// (roe_record.cu); roeFluxTapePlanes(dim) planes of V values
int roeFluxTapePlanes(int dim);
void launchRoeFluxRecord(const Grid& g, int limiter, const double* stage, const double* basis, const double* dq,
                         const StepConst<double>* sc, double* flux, double* tape, cudaStream_t st);

void launchAdjFlux(const Grid& g, const Phys<double>& ph, int limiter, const double* dtdx, const double* stage,
                   const double* dq, const double* basis, const double* fluxTape, const AdjStage& st,
                   const AdjScratch& s, int first, cudaStream_t stream);
void launchAdjDeltaQ(const Grid& g, const Phys<double>& ph, const double* stage, const double* basis,
                     const AdjScratch& s, cudaStream_t stream);
void launchAdjCells(const Grid& g, const AdjStage& st, const AdjScratch& s, double* lamOut, cudaStream_t stream);
void launchAdjBasis(const Grid& g, const Phys<double>& ph, const double* u0, const AdjScratch& s,
                    cudaStream_t stream);
void launchAdjPrims(const Grid& g, const Phys<double>& ph, const double* u0, const AdjScratch& s, double* lam,
                    cudaStream_t stream);
// lambda <- G^T lambda for the ghost fill of every axis (axes in reverse order)
void launchAdjBoundary(const Grid& g, const int methods[3][2], double* lam, cudaStream_t stream);

}  // namespace hgpu
