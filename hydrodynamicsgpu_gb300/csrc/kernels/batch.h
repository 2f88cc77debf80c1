// batch.h -- descriptors and launchers of the batched persistent kernels (batch.cu).
#pragma once
#include "kernels.h"

namespace hgpu {

// One problem of a batch: its own grid, constants and boundary methods, and where
// its data start inside the concatenated arrays.
template <typename real>
struct BatchProblem {
    Grid g;
    Phys<real> ph;
    int methods[3][2];
    long long stateOff;   // first cell in the state and Runge-Kutta slot arrays (N values per cell)
    long long faceOff;    // first element in the per-face array (Roe record planes / HLLC wave speeds)
    long long dqOff;      // first element in the Delta-q-tilde and flux arrays
    unsigned long long accInit;
    int useFixed;
    double fixedDt;
};

// A work tile: cells [x0, x0+tx) x [y0, y0+ty) x [z0, z0+tz) of problem p.
struct BatchTile {
    int p, x0, y0, z0;
};

// Launch shape chosen by the autotuner.
struct BatchTuning {
    int tx, ty, tz;      // tile shape (tx*ty*tz <= 256 * cpt cells)
    int staged;          // eigenbasis: per-cell primitives staged in shared memory (1) or recomputed per face (0)
    int blocksPerSM;     // persistent blocks per SM (0 = as many as fit)
    int split;           // FP64 EulerRoe flux in two passes (corrections, then transforms) instead of one
    int cpt;             // cells per thread: each of a block's 256 threads takes cpt cells of the tile
};

template <typename real>
struct BatchLaunch {
    const BatchProblem<real>* P;
    int nP;
    const BatchTile* tiles;
    int nT;
    BatchTuning tu;
    int dim;
    cudaStream_t st;
    real* state;
    real* faces;
    void boundary(unsigned* q) const;
    void roeBasis(int loA, int hiA, unsigned* q) const;
    void waves(int hll, unsigned* q) const;
    void dt(int hllc, unsigned long long* acc, unsigned* health, unsigned* q) const;
    void finalize(int integ, unsigned long long* acc, StepConst<real>* sc) const;
    void deltaQ(int loA, int hiA, const real* stage, real* dq, unsigned* q) const;
    // kind: 0 EulerRoe, 1 EulerHLLC, 2 EulerHLL
    void flux(int kind, int lim, const StepConst<real>* sc, const real* stage, const real* dq, real* fluxBuf,
              unsigned* health, unsigned* q) const;
    // the FP64 EulerRoe flux as two passes (q0: corrections, q1: transforms); real = double only
    void fluxSplit(int lim, const StepConst<real>* sc, const real* stage, const real* dq, real* fluxBuf, unsigned* q0,
                   unsigned* q1) const;
    void combine(const real* fluxBuf, const CombinePlan<real>& plan, const StepConst<real>* sc, unsigned* q) const;
    void gravity(int integ, const StepConst<real>* sc, unsigned* q) const;
    // the state check (health.cuh) of every problem: bits into healthP[p] and *health
    void stateCheck(unsigned* health, unsigned* healthP, unsigned* q) const;
};

}  // namespace hgpu
