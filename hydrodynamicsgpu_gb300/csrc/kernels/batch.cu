// batch.cu -- many independent Euler problems of uneven sizes in persistent launches.
//
// Every kernel of the step has a batched form here.  A launch is persistent (a fixed
// number of blocks per SM) and pulls work tiles (problem, x0, y0, z0) from an atomic
// queue until the tile list is exhausted, so the uneven problems of a sweep share
// every SM without one launch per problem.  Each problem keeps its own grid,
// constants, boundary methods, dt and RK step constants (BatchProblem).  The per-cell
// arithmetic is the single-problem code (roe_cells.cuh, hllc_cells.cuh,
// combine_cells.cuh), so a batched problem is bit-identical to the same problem run alone.
#include "../../../include/hgpu/hgpu.h"
#include "batch.h"
#include "combine_cells.cuh"
#include "hllc_cells.cuh"
#include "reduce.cuh"
#include "roe_cells.cuh"
#include "batch_common.cuh"
#include "health.cuh"

namespace hgpu {
namespace {

// ghost fill of one problem per work item: every axis in order, lines in parallel
template <typename real, int D>
__global__ void __launch_bounds__(256) batchBoundaryKernel(const BatchProblem<real>* __restrict__ P, int nP,
                                                           real* __restrict__ state, unsigned* q) {
    for (;;) {
        int p = nextItem(q);
        if (p >= nP) break;
        const BatchProblem<real>& pr = P[p];
        real* s = state + (long long)(D + 2) * pr.stateOff;
        for (int axis = 0; axis < D; ++axis) {
            int A = axis == 0 ? 1 : 0, B = axis == 2 ? 1 : 2;
            long long nLines = D == 1 ? 1 : (long long)pr.g.S[A] * pr.g.S[B];
            for (long long t = threadIdx.x; t < nLines; t += blockDim.x)
                boundaryLine<real>(pr.g, axis, D + 2, pr.methods[axis][0], pr.methods[axis][1], s, t);
            __syncthreads();   // the next axis reads ghost lines this one wrote
        }
    }
}

template <typename real, int D, bool PLAIN>
__global__ void __launch_bounds__(256) batchRoeBasisKernel(const BatchProblem<real>* __restrict__ P,
                                                           const BatchTile* __restrict__ tiles, int nT, BatchTuning tu,
                                                           int loA, int hiA, const real* __restrict__ state,
                                                           real* __restrict__ basis, unsigned* q) {
    extern __shared__ unsigned char smem[];
    RoePrim<real, D>* prim = reinterpret_cast<RoePrim<real, D>*>(smem);
    for (int t = firstTile<PLAIN>(q); t < nT; t = nextTile<PLAIN>(q, nT)) {
        const BatchTile tl = tiles[t];
        const BatchProblem<real>& pr = P[tl.p];
        const Grid g = pr.g;
        const real* s = state + (long long)(D + 2) * pr.stateOff;
        real* b = basis + pr.faceOff;
        if (tu.staged) {
            roeBasisTile<real, D>(g, pr.ph, s, b, loA, hiA, tl.x0, tl.y0, tl.z0, tu.tx, tu.ty, tu.tz, prim);
        } else {
            for (int r = 0; r < (PLAIN ? 1 : tu.cpt); ++r) {
            int x, y, z;
            long long c;
            if (tileCell(g, tl, tu, threadIdx.x + r * blockDim.x, x, y, z, c)) {
                const int NB = RoeRec<D>::NB;
                real sR[D + 2], sL[D + 2], rec[NB];
                loadState<real, D>(s, c, sR);
#pragma unroll
                for (int side = 0; side < D; ++side) {
                    if (!roeFace(g, side, x, y, z, loA, hiA)) continue;
                    loadState<real, D>(s, c - g.step[side], sL);
                    if (side == 0) roeBasis<real, D, 0>(sL, sR, pr.ph.gamma, rec);
                    else if (side == 1) roeBasis<real, D, (D > 1 ? 1 : 0)>(sL, sR, pr.ph.gamma, rec);
                    else roeBasis<real, D, (D > 2 ? 2 : 0)>(sL, sR, pr.ph.gamma, rec);
#pragma unroll
                    for (int k = 0; k < NB; ++k) b[((long long)side * NB + k) * g.V + c] = rec[k];
                }
            }
            }
        }
    }
}

template <typename real, int D, bool PLAIN>
__global__ void __launch_bounds__(256) batchDtKernel(const BatchProblem<real>* __restrict__ P,
                                                     const BatchTile* __restrict__ tiles, int nT, BatchTuning tu, int hllc,
                                                     const real* __restrict__ faces, unsigned long long* acc,
                                                     unsigned* health, unsigned* q) {
    for (int t = firstTile<PLAIN>(q); t < nT; t = nextTile<PLAIN>(q, nT)) {
        const BatchTile tl = tiles[t];
        const BatchProblem<real>& pr = P[tl.p];
        const Grid g = pr.g;
        int x, y, z;
        long long c;
        unsigned long long best = ~0ULL;
        bool nan = false;
        for (int r = 0; r < (PLAIN ? 1 : tu.cpt); ++r)
            if (tileCell(g, tl, tu, threadIdx.x + r * blockDim.x, x, y, z, c)) {
                unsigned long long b = hllc ? hllcDtCell<real, D>(g, pr.ph, faces + pr.faceOff, c, x, y, z, nan)
                                            : roeDtCell<real, D>(g, pr.ph, faces + pr.faceOff, c, x, y, z, nan);
                best = b < best ? b : best;
            }
        if (nan) atomicOr(health, HEALTH_NONFINITE_DT);
        blockMinToGlobal(best, acc + tl.p);
    }
}

template <typename real>
__global__ void batchFinalizeKernel(const BatchProblem<real>* __restrict__ P, int nP, int integ,
                                    unsigned long long* acc, StepConst<real>* sc) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nP) return;
    const BatchProblem<real>& pr = P[p];
    finalizeOne<real>(pr.ph, integ, pr.useFixed, pr.fixedDt, acc + p, pr.accInit, sc + p);
}

template <typename real, int D, bool PLAIN>
__global__ void __launch_bounds__(256) batchDeltaQKernel(const BatchProblem<real>* __restrict__ P,
                                                         const BatchTile* __restrict__ tiles, int nT, BatchTuning tu,
                                                         int loA, int hiA, const real* __restrict__ stage,
                                                         const real* __restrict__ basis, real* __restrict__ dq,
                                                         unsigned* q) {
    for (int t = firstTile<PLAIN>(q); t < nT; t = nextTile<PLAIN>(q, nT)) {
        const BatchTile tl = tiles[t];
        const BatchProblem<real>& pr = P[tl.p];
        const Grid g = pr.g;
        int x, y, z;
        long long c;
        for (int r = 0; r < (PLAIN ? 1 : tu.cpt); ++r)
        if (tileCell(g, tl, tu, threadIdx.x + r * blockDim.x, x, y, z, c))
            roeDeltaQCell<real, D>(g, stage + (long long)(D + 2) * pr.stateOff, basis + pr.faceOff, dq + pr.dqOff, c,
                                   x, y, z, loA, hiA);
    }
}

// (plain: 5 blocks per SM, 48 registers, measured faster than 56 and 4)
template <typename real, int D, bool PLAIN>
__global__ void __launch_bounds__(256, PLAIN ? 5 : 1) batchCombineKernel(const BatchProblem<real>* __restrict__ P,
                                                          const BatchTile* __restrict__ tiles, int nT, BatchTuning tu,
                                                          const real* __restrict__ flux, CombinePlan<real> plan,
                                                          const StepConst<real>* __restrict__ sc, unsigned* q) {
    for (int t = firstTile<PLAIN>(q); t < nT; t = nextTile<PLAIN>(q, nT)) {
        const BatchTile tl = tiles[t];
        const BatchProblem<real>& pr = P[tl.p];
        const Grid g = pr.g;
        int x, y, z;
        long long c;
        for (int r = 0; r < (PLAIN ? 1 : tu.cpt); ++r)
        if (tileCell(g, tl, tu, threadIdx.x + r * blockDim.x, x, y, z, c))
            derivCombineCell<real, D, D, true>(g, pr.ph, flux + pr.dqOff, plan, sc[tl.p], c, x, y, z, pr.stateOff);
    }
}

// the self-gravity pass with a zero potential: ForwardEuler adds deriv*dt == +0*dt to
// every element (after its ghost refresh); Runge-Kutta forms the alpha-combination.
template <typename real, int D>
__global__ void __launch_bounds__(256) batchGravityKernel(const BatchProblem<real>* __restrict__ P,
                                                          const BatchTile* __restrict__ tiles, int nT, BatchTuning tu,
                                                          int integ, const StepConst<real>* __restrict__ sc,
                                                          real* __restrict__ state, unsigned* q) {
    for (int t = firstItem(q, tu); t < nT; t = nextItemAfter(q, tu)) {
        const BatchTile tl = tiles[t];
        const BatchProblem<real>& pr = P[tl.p];
        for (int r = 0; r < tu.cpt; ++r) {
            int x, y, z;
            long long c;
            if (!tileCell(pr.g, tl, tu, threadIdx.x + r * blockDim.x, x, y, z, c)) continue;
            real* s = state + (long long)(D + 2) * (pr.stateOff + c);
            const StepConst<real>& k = sc[tl.p];
#pragma unroll
            for (int j = 0; j < D + 2; ++j)
                s[j] = integ == HGPU_INTEGRATOR_FORWARD_EULER ? s[j] + (real)0. * k.dt
                                                               : alphaOnlyElem<real>(integ, s[j], k);
        }
    }
}

// the state check (health.cuh) of every problem: bits into the problem's word and the batch's
template <typename real, int D, bool PLAIN>
__global__ void __launch_bounds__(256) batchStateCheckKernel(const BatchProblem<real>* __restrict__ P,
                                                             const BatchTile* __restrict__ tiles, int nT,
                                                             BatchTuning tu, const real* __restrict__ state,
                                                             unsigned* health, unsigned* healthP, unsigned* q) {
    for (int t = firstTile<PLAIN>(q); t < nT; t = nextTile<PLAIN>(q, nT)) {
        const BatchTile tl = tiles[t];
        const BatchProblem<real>& pr = P[tl.p];
        const Grid g = pr.g;
        int x, y, z;
        long long c;
        unsigned bits = 0;
        for (int r = 0; r < (PLAIN ? 1 : tu.cpt); ++r)
        if (tileCell(g, tl, tu, threadIdx.x + r * blockDim.x, x, y, z, c))
            bits |= stateCheckCell<real, D>(g, state + (long long)(D + 2) * pr.stateOff, nullptr, c, x, y, z);
        warpHealthOr(bits, healthP + tl.p, health);
    }
}

template <typename real, int D, bool HLL>
__global__ void __launch_bounds__(256) batchWaveKernel(const BatchProblem<real>* __restrict__ P,
                                                       const BatchTile* __restrict__ tiles, int nT, BatchTuning tu,
                                                       const real* __restrict__ state, real* __restrict__ waves,
                                                       unsigned* q) {
    for (int t = firstItem(q, tu); t < nT; t = nextItemAfter(q, tu)) {
        const BatchTile tl = tiles[t];
        const BatchProblem<real>& pr = P[tl.p];
        double gq = ((double)pr.ph.gamma + 1.) / (2. * (double)pr.ph.gamma);
        for (int r = 0; r < tu.cpt; ++r) {
            int x, y, z;
            long long c;
            if (!tileCell(pr.g, tl, tu, threadIdx.x + r * blockDim.x, x, y, z, c)) continue;
            hllcWaveCell<real, D, HLL>(pr.g, pr.ph, gq, state + (long long)(D + 2) * pr.stateOff, waves + pr.faceOff, c,
                                       x, y, z);
        }
    }
}

}  // namespace

template <typename real>
void BatchLaunch<real>::boundary(unsigned* q) const {
    if (dim == 1) batchBoundaryKernel<real, 1><<<persistentBlocks(batchBoundaryKernel<real, 1>, 0, tu.blocksPerSM, nP), 256, 0, st>>>(P, nP, state, q);
    else if (dim == 2) batchBoundaryKernel<real, 2><<<persistentBlocks(batchBoundaryKernel<real, 2>, 0, tu.blocksPerSM, nP), 256, 0, st>>>(P, nP, state, q);
    else batchBoundaryKernel<real, 3><<<persistentBlocks(batchBoundaryKernel<real, 3>, 0, tu.blocksPerSM, nP), 256, 0, st>>>(P, nP, state, q);
}

template <typename real>
static int primSmem(int dim, const BatchTuning& tu) {
    int hx = tu.tx + 1, hy = dim > 1 ? tu.ty + 1 : 1, hz = dim > 2 ? tu.tz + 1 : 1;
    size_t one = dim == 1 ? sizeof(RoePrim<real, 1>) : dim == 2 ? sizeof(RoePrim<real, 2>) : sizeof(RoePrim<real, 3>);
    return (int)(one * hx * hy * hz);
}

template <typename real>
void BatchLaunch<real>::roeBasis(int loA, int hiA, unsigned* q) const {
    int smem = tu.staged ? primSmem<real>(dim, tu) : 0;
#define L(DD)                                                                                                      \
    if (tu.blocksPerSM < 0 && tu.cpt == 1)                                                                                        \
        batchRoeBasisKernel<real, DD, true><<<nT, 256, smem, st>>>(P, tiles, nT, tu, loA, hiA, state, faces, q);    \
    else                                                                                                           \
        batchRoeBasisKernel<real, DD, false><<<persistentBlocks(batchRoeBasisKernel<real, DD, false>, smem,         \
                                                                tu.blocksPerSM, nT), 256, smem, st>>>(              \
            P, tiles, nT, tu, loA, hiA, state, faces, q)
    if (dim == 1) { L(1); }
    else if (dim == 2) { L(2); }
    else { L(3); }
#undef L
}

template <typename real>
void BatchLaunch<real>::waves(int hll, unsigned* q) const {
#define L(DD, H) batchWaveKernel<real, DD, H><<<persistentBlocks(batchWaveKernel<real, DD, H>, 0, tu.blocksPerSM, nT), 256, 0, st>>>(P, tiles, nT, tu, state, faces, q)
    if (hll) {
        if (dim == 1) L(1, true);
        else if (dim == 2) L(2, true);
        else L(3, true);
    } else {
        if (dim == 1) L(1, false);
        else if (dim == 2) L(2, false);
        else L(3, false);
    }
#undef L
}

template <typename real>
void BatchLaunch<real>::dt(int hllc, unsigned long long* acc, unsigned* health, unsigned* q) const {
#define L(DD)                                                                                                      \
    if (tu.blocksPerSM < 0 && tu.cpt == 1)                                                                         \
        batchDtKernel<real, DD, true><<<nT, 256, 0, st>>>(P, tiles, nT, tu, hllc, faces, acc, health, q);           \
    else                                                                                                           \
        batchDtKernel<real, DD, false><<<persistentBlocks(batchDtKernel<real, DD, false>, 0, tu.blocksPerSM, nT),   \
                                         256, 0, st>>>(P, tiles, nT, tu, hllc, faces, acc, health, q)
    if (dim == 1) { L(1); }
    else if (dim == 2) { L(2); }
    else { L(3); }
#undef L
}

template <typename real>
void BatchLaunch<real>::finalize(int integ, unsigned long long* acc, StepConst<real>* sc) const {
    batchFinalizeKernel<real><<<(nP + 127) / 128, 128, 0, st>>>(P, nP, integ, acc, sc);
}

template <typename real>
void BatchLaunch<real>::deltaQ(int loA, int hiA, const real* stage, real* dq, unsigned* q) const {
#define L(DD)                                                                                                      \
    if (tu.blocksPerSM < 0 && tu.cpt == 1)                                                                                        \
        batchDeltaQKernel<real, DD, true><<<nT, 256, 0, st>>>(P, tiles, nT, tu, loA, hiA, stage, faces, dq, q);     \
    else                                                                                                           \
        batchDeltaQKernel<real, DD, false><<<persistentBlocks(batchDeltaQKernel<real, DD, false>, 0, tu.blocksPerSM, \
                                                              nT), 256, 0, st>>>(P, tiles, nT, tu, loA, hiA, stage,  \
                                                                                 faces, dq, q)
    if (dim == 1) { L(1); }
    else if (dim == 2) { L(2); }
    else { L(3); }
#undef L
}

template <typename real>
void BatchLaunch<real>::combine(const real* fluxBuf, const CombinePlan<real>& plan, const StepConst<real>* sc,
                                unsigned* q) const {
#define L(DD)                                                                                                      \
    if (tu.blocksPerSM < 0 && tu.cpt == 1)                                                                                        \
        batchCombineKernel<real, DD, true><<<nT, 256, 0, st>>>(P, tiles, nT, tu, fluxBuf, plan, sc, q);             \
    else                                                                                                           \
        batchCombineKernel<real, DD, false><<<persistentBlocks(batchCombineKernel<real, DD, false>, 0,              \
                                                               tu.blocksPerSM, nT), 256, 0, st>>>(P, tiles, nT, tu,  \
                                                                                                  fluxBuf, plan, sc, q)
    if (dim == 1) { L(1); }
    else if (dim == 2) { L(2); }
    else { L(3); }
#undef L
}

template <typename real>
void BatchLaunch<real>::gravity(int integ, const StepConst<real>* sc, unsigned* q) const {
#define L(DD) batchGravityKernel<real, DD><<<persistentBlocks(batchGravityKernel<real, DD>, 0, tu.blocksPerSM, nT), 256, 0, st>>>(P, tiles, nT, tu, integ, sc, state, q)
    if (dim == 1) L(1);
    else if (dim == 2) L(2);
    else L(3);
#undef L
}

template <typename real>
void BatchLaunch<real>::stateCheck(unsigned* health, unsigned* healthP, unsigned* q) const {
#define L(DD)                                                                                                      \
    if (tu.blocksPerSM < 0 && tu.cpt == 1)                                                                         \
        batchStateCheckKernel<real, DD, true><<<nT, 256, 0, st>>>(P, tiles, nT, tu, state, health, healthP, q);     \
    else                                                                                                           \
        batchStateCheckKernel<real, DD, false><<<persistentBlocks(batchStateCheckKernel<real, DD, false>, 0,        \
                                                                  tu.blocksPerSM, nT), 256, 0, st>>>(               \
            P, tiles, nT, tu, state, health, healthP, q)
    if (dim == 1) { L(1); }
    else if (dim == 2) { L(2); }
    else { L(3); }
#undef L
}

template struct BatchLaunch<double>;
template struct BatchLaunch<float>;

}  // namespace hgpu
