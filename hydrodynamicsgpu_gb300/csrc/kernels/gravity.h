// gravity.h -- launchers of the self-gravity kernels (gravity.cu).
#pragma once
#include "kernels.h"

namespace hgpu {

// Constants of the relaxation and the gravity source, as the program bakes them.
template <typename real>
struct GravityConst {
    double fourPiG;   // 4. * M_PI * ((real)G), double
    double diag;      // (double)(real)(-2. * (1. / (DX * DX) + ...)), `const real diag`
    real dxSq[3];     // DX * DX in the program's type
    double rdxSq[3];  // RN(1 / (DX * DX)), FP64 quotient correction
    double twoDx[3];  // 2. * dx[side], double
};

template <typename real>
GravityConst<real> gravityConst(const double dx[3], double G, int dim);

// potential = -density (fromDensity) or its current contents; total energy += potential;
// cells [c0, c1) (default: every cell)
template <typename real>
void launchPotentialInit(const Grid& g, int fromDensity, real* state, real* pot, cudaStream_t st, long long c0 = 0,
                         long long c1 = -1);
// SelfGravitation::potentialBoundary: every axis, min then max side
template <typename real>
void launchPotentialBoundary(const Grid& g, const int methods[3][2], real* pot, cudaStream_t st);
// rhs = 4. * M_PI * G * density of every cell (double), from the state the sweeps relax against
template <typename real>
void launchRelaxRhs(const Grid& g, const GravityConst<real>& gc, const real* state, double* rhs, cudaStream_t st);
// one gravityPotentialPoissonRelax launch in the red-black order (two kernels)
template <typename real>
void launchRelaxSweep(const Grid& g, const GravityConst<real>& gc, const double* rhs, real* pot, cudaStream_t st);
// calcGravityDeriv of the stage state, fused with the integrator's combine
template <typename real>
void launchGravityCombine(const Grid& g, const GravityConst<real>& gc, const real* stage, const real* pot,
                          const CombinePlan<real>& plan, const StepConst<real>* sc, cudaStream_t st);

}  // namespace hgpu
