// kernels.h -- host-side launchers of the sm_103a Euler kernels (plain C++ types).
#pragma once
#include <cuda_runtime.h>
#include <string>
#include "common.cuh"

namespace hgpu {

template <typename real>
struct Phys {
    real dx[3];      // DX/DY/DZ as the program bakes them
    real rdx[3];     // RN(1 / dx), for the exact division by dx (fp64ops.cuh divByRecip)
    real gamma;      // ((real)<defs value>)
    float cfl;
};

// One output row of the Runge-Kutta combine at a stage (see combine.cu).
template <typename real>
struct CombineOp {
    int out;         // slot written
    int prior;       // slot holding the partial sum so far, or -1 (sum starts at +0)
    int priorAlias;  // the prior is u^n itself (sum == +0 + u^n): read it through zfix
    int hasAlpha;    // add alpha * u^(k)
    int alphaIsOne;
    real alpha;
    int hasBeta;     // add (beta * dt) * d^(k), coefficient from StepConst::coef[brow][bcol]
    int brow, bcol;
};

template <typename real>
struct CombinePlan {
    int fe;                   // forward Euler: slot[0] = slot[0] + d * dt
    int in;                   // slot of the stage input u^(k)
    int nops;
    CombineOp<real> ops[4];
    real* slot[8];
};

// ---- boundary.cu ----
template <typename real>
void launchBoundary(const Grid& g, const int methods[3][2], real* state, cudaStream_t st);
// the ghost fill along one axis over its transverse lines [t0, t1) (line t of axis a
// addresses the cell with c[A] + S[A] * c[B] = t, A < B the other two axes)
long long boundaryLines(const Grid& g, int axis);
template <typename real>
void launchBoundaryAxis(const Grid& g, const int methods[3][2], real* state, cudaStream_t st, int axis,
                        long long t0 = 0, long long t1 = -1);
// cells [c0, c1) (default: every cell)
template <typename real>
void launchDerivCombine(const Grid& g, const Phys<real>& ph, const real* flux, const CombinePlan<real>& plan,
                        const StepConst<real>* sc, cudaStream_t st, long long c0 = 0, long long c1 = -1);
template <typename real>
void launchAlphaOnly(const Grid& g, int integrator, real* state, const StepConst<real>* sc, cudaStream_t st);
template <typename real>
void launchZeroAdd(const Grid& g, real* state, const StepConst<real>* sc, cudaStream_t st);
template <typename real>
void launchFinalizeDt(const Phys<real>& ph, int integrator, int useFixed, double fixedDt, unsigned long long* acc,
                      unsigned long long accInit, StepConst<real>* sc, unsigned* health, cudaStream_t st);
template <typename real>
void launchResetAcc(unsigned long long* acc, unsigned long long accInit, cudaStream_t st);

// ---- roe.cu ----
// pot: the gravitational potential (V values), or null for a zero potential.  In 2D
// and 3D, only the tiles [slow0, slow0 + slowTiles) along the slowest axis (y, z) of
// roeBasisSlowTile(dim) cells each (default: all of them).
template <typename real>
void launchRoeBasis(const Grid& g, const Phys<real>& ph, const real* state, real* basis, int seam, cudaStream_t st,
                    const real* pot = nullptr, int slow0 = 0, int slowTiles = -1);
int roeBasisSlowTile(int dim);
template <typename real>
void launchRoeDt(const Grid& g, const Phys<real>& ph, const real* basis, unsigned long long* acc, unsigned* health,
                 cudaStream_t st);
template <typename real>
// cells [c0, c1) only (c1 < 0: to the end of the grid)
void launchRoeDeltaQ(const Grid& g, const real* stage, const real* basis, real* dq, int seam, cudaStream_t st,
                     long long c0 = 0, long long c1 = -1);
template <typename real>
void launchRoeFlux(const Grid& g, int limiter, const real* stage, const real* basis, const real* dq,
                   const StepConst<real>* sc, real* flux, int seam, cudaStream_t st, long long c0 = 0,
                   long long c1 = -1);
int roeRecordSize(int dim);

// ---- hllc.cu ----
// the wave speeds of the faces of cells [c0, c1) (default: every cell)
template <typename real>
void launchHllcWaves(const Grid& g, const Phys<real>& ph, const real* state, real* waves, int hll, cudaStream_t st,
                     const real* pot = nullptr, long long c0 = 0, long long c1 = -1);
template <typename real>
void launchHllcDt(const Grid& g, const Phys<real>& ph, const real* waves, unsigned long long* acc, unsigned* health,
                  cudaStream_t st);
template <typename real>
void launchHllcFlux(const Grid& g, const Phys<real>& ph, const real* stage, const real* waves, real* flux,
                    unsigned* health, int hll, cudaStream_t st, const real* pot = nullptr, long long c0 = 0,
                    long long c1 = -1);

// ---- display scalar (display.cu, convertToTex): method = the reference's DISPLAY_* index ----
int displayCount(int dim);
template <typename real>
void launchDisplay(const Grid& g, real gamma, int method, const real* state, float* out, cudaStream_t st,
                   const real* pot = nullptr);

// ---- health.cu: the state check (health.cuh) of every interior cell into *health;
// pot: the potential, or null for a zero potential ----
template <typename real>
void launchStateCheck(const Grid& g, const real* state, const real* pot, unsigned* health, cudaStream_t st);

// ---- roe_fused.cu: the 2D FP64 EulerRoe stage as two fused per-direction kernels
// (x pass, then y pass with the divergence and the integrator's combine), FP64 2D only.
// tensorMap: from makeRoeFusedTensorMap for `stage` (roeFusedTensorMapSize() bytes,
// 64-byte aligned); dX: V x 4 doubles of scratch for the x part of the divergence.
// The plan must not write the stage buffer (Runge-Kutta stages; not ForwardEuler). ----
size_t roeFusedTensorMapSize();
bool makeRoeFusedTensorMap(const Grid& g, const double* stage, void* out, std::string& err);
void roeFusedPrepare();
void launchRoeStageFused(const Grid& g, const Phys<double>& ph, int limiter, const StepConst<double>* sc,
                         const double* stage, const double* basis, double* dX, const CombinePlan<double>& plan,
                         int seam, const void* tensorMap, unsigned* health, cudaStream_t st);

// ---- tableaus (combine.cu): alpha/beta in double, order ----
int tableauOrder(int integrator);
double tableauAlpha(int integrator, int m, int k);
double tableauBeta(int integrator, int m, int k);

}  // namespace hgpu
