// roe_fused.cu -- the 2D FP64 EulerRoe Runge-Kutta stage in two fused per-direction
// kernels (an alternative to roeDeltaQKernel + roeFluxCorrKernel + roeFluxXformKernel
// + derivCombineKernel; the same operations in the same order, so the same bits).
//
// The reference runs a stage as calcDeltaQTilde -> calcFlux -> calcFluxDeriv ->
// multAdd with every intermediate in global memory (src/Solver/Roe.cpp:101-112,
// res/Roe.cl:152-320, res/CalcFluxDeriv.cl:7-44, res/Common.cl:201-210).  Here:
//
//  * x pass (roeStageXKernel): one block per row segment of kSegX interior cells.  The
//    segment's stage cells plus a two-cell halo land in shared memory by one bulk
//    copy (TMA); Delta-q-tilde of its kSegX + 3 x faces, then the limited flux of its
//    kSegX + 1 faces (corrections and transforms), stay in shared memory; it writes
//    only the x part of each cell's flux divergence, zfix(-(F[i+1] - F[i]) / dx).
//  * y pass (roeStageYKernel): one block per strip of 32 columns x kStrip rows, marching
//    down the strip 8 rows at a time.  Stage rows arrive by 2D tensor copies (TMA), two
//    steps ahead in a ring of three slots; each y face's Delta-q-tilde and flux are
//    formed once (two rings of two slots), so a strip repeats only its first rows'
//    halo.  Each cell then adds the y part of its divergence to the x part and runs
//    the integrator's combine (combinePlanCell) for its row of the tableau.
//
// Every bulk copy is waited for with a bounded poll; a wait that gives up sets
// HEALTH_COPY_TIMEOUT and the block stops (its cells keep their old values).
#include <cuda.h>

#include <mutex>
#include <string>

#include "../../../include/hgpu/hgpu.h"
#include "combine_cells.cuh"
#include "kernels.h"
#include "roe_cells.cuh"
#include "tma.cuh"

namespace hgpu {

namespace {

constexpr int kThreads = 256;         // y pass: threads per block
constexpr int kThreadsX = 256;        // x pass: threads per block
constexpr int kBlocksX = 3;           // x pass: blocks per SM the register budget is sized for
constexpr int kSegX = kThreadsX - 3;  // x pass: cells per segment (kSegX + 3 Delta-q-tilde faces)
constexpr int kCols = 32;             // y pass: columns per strip (one warp across)
constexpr int kRows = kThreads / kCols;   // y pass: rows per marching step
constexpr int kStrip = 128;           // y pass: rows per strip
constexpr int kRow = kCols * 4;       // doubles per strip row (4 conserved values per cell)
static_assert(kRows == 8, "the y pass's ring indexing assumes 8 rows per step");

// ---------------- x pass ----------------
template <int LIM>
__global__ void __launch_bounds__(kThreadsX, kBlocksX)
    roeStageXKernel(Grid g, Phys<double> ph, int lim, const StepConst<double>* __restrict__ sc,
                    const double* __restrict__ stage, const double* __restrict__ basis, double* __restrict__ dX,
                    int loA, int hiA, unsigned* health) {
    constexpr int N = 4, NB = RoeRec<2>::NB;
    __shared__ __align__(128) double sS[(kSegX + 4) * N];   // cells [x0 - 2, xEnd + 1]
    __shared__ __align__(16) double sQ[(kSegX + 3) * N];    // Delta-q-tilde, faces [x0 - 1, xEnd + 1]
    __shared__ __align__(16) double sF[(kSegX + 1) * N];    // flux, faces [x0, xEnd]
    __shared__ __align__(8) unsigned long long bar;
    const int y = 2 + blockIdx.y;                           // interior rows only
    const int x0 = 2 + blockIdx.x * kSegX;
    const int xEnd = min(x0 + kSegX, g.S[0] - 2);          // cells [x0, xEnd)
    const int nc = xEnd - x0;
    const int t = threadIdx.x;
    const long long row = (long long)g.S[0] * y;
    if (t == 0) {
        mbarInit(&bar, 1);
        fenceBarrierInit();
    }
    __syncthreads();
    if (t == 0) {
        const unsigned bytes = (unsigned)((nc + 4) * N * sizeof(double));
        mbarExpectTx(&bar, bytes);
        bulkLoad(sS, stage + (long long)N * (row + x0 - 2), bytes, &bar);
    }
    const bool landed = __syncthreads_and(mbarWait(&bar, 0));
    if (!landed) {
        if (t == 0) atomicOr(health, HEALTH_COPY_TIMEOUT);
        return;
    }
    // Delta-q-tilde = L (q_R - q_L) of face f = x0 - 1 + t (res/Roe.cl:67-168); faces
    // the reference never writes are zero
    if (t < nc + 3) {
        const int f = x0 - 1 + t;
        double q[N] = {0, 0, 0, 0};
        if (roeFace(g, 0, f, y, 0, loA, hiA)) {
            const long long c = row + f;
            double rec[NB], ds[N];
#pragma unroll
            for (int k = 0; k < NB; ++k) rec[k] = basis[(long long)k * g.V + c];
#pragma unroll
            for (int j = 0; j < N; ++j) ds[j] = sS[(t + 1) * N + j] - sS[t * N + j];
            leftTransform<double, 2, 0, true>(rec, ds, q);
        }
#pragma unroll
        for (int j = 0; j < N; ++j) sQ[t * N + j] = q[j];
    }
    __syncthreads();
    // limited flux of face f = x0 + t (res/Roe.cl:170-320): every face here is one the
    // reference computes (along [2, S-2], row interior)
    if (t < nc + 1) {
        const long long c = row + x0 + t;
        double rec[NB], qL[N], q[N], qR[N], corr[N], sL[N], sR[N], F[N];
#pragma unroll
        for (int k = 0; k < NB; ++k) rec[k] = basis[(long long)k * g.V + c];
#pragma unroll
        for (int j = 0; j < N; ++j) {
            qL[j] = sQ[t * N + j];
            q[j] = sQ[(t + 1) * N + j];
            qR[j] = sQ[(t + 2) * N + j];
        }
        roeFluxCorrections<2, 0, LIM>(rec, qL, q, qR, sc->dt_dx[0], lim, corr);
#pragma unroll
        for (int j = 0; j < N; ++j) {
            sL[j] = sS[(t + 1) * N + j];
            sR[j] = sS[(t + 2) * N + j];
        }
        roeFluxTransforms<2, 0>(rec, sL, sR, corr, F);
#pragma unroll
        for (int j = 0; j < N; ++j) sF[t * N + j] = F[j];
    }
    __syncthreads();
    // x part of calcFluxDeriv (res/CalcFluxDeriv.cl:7-44): -(F[i+1] - F[i]) / dx
    if (t < nc) {
        double* out = dX + (long long)N * (row + x0 + t);
#pragma unroll
        for (int j = 0; j < N; ++j) {
            const double df = sF[(t + 1) * N + j] - sF[t * N + j];
            out[j] = zfix(-divByRecip(df, ph.dx[0], ph.rdx[0]));
        }
    }
}

// ---------------- y pass ----------------
struct YShared {
    double s[3][kRows][kRow];   // stage rows: batch b = rows [r0 + 8b - 6, r0 + 8b + 1] in slot b % 3
    double q[2][kRows][kRow];   // Delta-q-tilde, y faces: batch b as the stage rows, slot b % 2
    double f[2][kRows][kRow];   // flux, y faces: batch b = rows [r0 + 8b - 7, r0 + 8b], slot b % 2
    unsigned long long bar[3];
};

__device__ __forceinline__ const double* yRow(const YShared& sm, int y, int r0) {
    const int k = y - r0 + 6;
    return sm.s[(k >> 3) % 3][k & 7];
}
__device__ __forceinline__ double* qRow(YShared& sm, int f, int r0) {
    const int k = f - r0 + 6;
    return sm.q[(k >> 3) & 1][k & 7];
}
__device__ __forceinline__ double* fRow(YShared& sm, int f, int r0) {
    const int k = f - r0 + 7;
    return sm.f[(k >> 3) & 1][k & 7];
}

template <int LIM>
__global__ void __launch_bounds__(kThreads, 3)
    roeStageYKernel(Grid g, Phys<double> ph, int lim, const StepConst<double>* __restrict__ sc,
                    const double* __restrict__ basis, const double* __restrict__ dX, CombinePlan<double> plan,
                    const __grid_constant__ CUtensorMap tm, int loA, int hiA, unsigned* health) {
    constexpr int N = 4, NB = RoeRec<2>::NB;
    constexpr unsigned kBox = kRows * kRow * sizeof(double);
    extern __shared__ __align__(128) unsigned char smemRaw[];
    YShared& sm = *reinterpret_cast<YShared*>(smemRaw);
    const int tx = threadIdx.x & (kCols - 1), ty = threadIdx.x / kCols;
    const int x0 = blockIdx.x * kCols, x = x0 + tx;
    const int r0 = blockIdx.y * kStrip, r1 = min(r0 + kStrip, g.S[1]);
    const bool col = x < g.S[0];
    const StepConst<double>& k = *sc;
    auto issue = [&](int b) {   // stage rows of batch b into slot b % 3 (thread 0)
        fenceProxyAsync();
        mbarExpectTx(&sm.bar[b % 3], kBox);
        tensorLoad2D(sm.s[b % 3], &tm, x0 * N, r0 + 8 * b - 6, &sm.bar[b % 3]);
    };
    if (threadIdx.x == 0) {
        for (int i = 0; i < 3; ++i) mbarInit(&sm.bar[i], 1);
        fenceBarrierInit();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        issue(0);
        if (r0 < r1) issue(1);
    }
    // Delta-q-tilde of y face f into its ring row (zero where the reference writes none)
    auto deltaQ = [&](int f) {
        double q[N] = {0, 0, 0, 0};
        if (col && roeFace(g, 1, x, f, 0, loA, hiA)) {
            const long long c = x + (long long)g.S[0] * f;
            double rec[NB], ds[N];
#pragma unroll
            for (int kk = 0; kk < NB; ++kk) rec[kk] = basis[(long long)(NB + kk) * g.V + c];
            const double* sR = yRow(sm, f, r0) + tx * N;
            const double* sL = yRow(sm, f - 1, r0) + tx * N;
#pragma unroll
            for (int j = 0; j < N; ++j) ds[j] = sR[j] - sL[j];
            leftTransform<double, 2, 1, true>(rec, ds, q);
        }
        double* o = qRow(sm, f, r0) + tx * N;
#pragma unroll
        for (int j = 0; j < N; ++j) o[j] = q[j];
    };
    // limited flux of y face f into its ring row (faces the divergence never reads are skipped)
    auto flux = [&](int f) {
        if (!(col && roeFace(g, 1, x, f, 0, 2, 1))) return;
        const long long c = x + (long long)g.S[0] * f;
        double rec[NB], qL[N], q[N], qR[N], corr[N], sL[N], sR[N], F[N];
#pragma unroll
        for (int kk = 0; kk < NB; ++kk) rec[kk] = basis[(long long)(NB + kk) * g.V + c];
        const double* a = qRow(sm, f - 1, r0) + tx * N;
        const double* b = qRow(sm, f, r0) + tx * N;
        const double* d = qRow(sm, f + 1, r0) + tx * N;
#pragma unroll
        for (int j = 0; j < N; ++j) {
            qL[j] = a[j];
            q[j] = b[j];
            qR[j] = d[j];
        }
        roeFluxCorrections<2, 1, LIM>(rec, qL, q, qR, k.dt_dx[1], lim, corr);
        const double* pl = yRow(sm, f - 1, r0) + tx * N;
        const double* pr = yRow(sm, f, r0) + tx * N;
#pragma unroll
        for (int j = 0; j < N; ++j) {
            sL[j] = pl[j];
            sR[j] = pr[j];
        }
        roeFluxTransforms<2, 1>(rec, sL, sR, corr, F);
        double* o = fRow(sm, f, r0) + tx * N;
#pragma unroll
        for (int j = 0; j < N; ++j) o[j] = F[j];
    };
    auto fail = [&]() {
        if (threadIdx.x == 0) atomicOr(health, HEALTH_COPY_TIMEOUT);
    };
    // prologue: the Delta-q-tilde of faces r0-1 .. r0+1 and the flux of face r0
    if (!__syncthreads_and(mbarWait(&sm.bar[0], 0))) { fail(); return; }
    if (ty < 3) deltaQ(r0 - 1 + ty);
    __syncthreads();
    if (ty == 0) flux(r0);
    __syncthreads();
    for (int it = 0; r0 + 8 * it < r1; ++it) {
        const int ya = r0 + 8 * it;
        const int b1 = it + 1;
        if (!__syncthreads_and(mbarWait(&sm.bar[b1 % 3], (b1 / 3) & 1))) { fail(); return; }
        if (threadIdx.x == 0 && ya + 8 < r1) issue(it + 2);   // its slot held batch it - 1, now read
        deltaQ(ya + 2 + ty);                                  // faces ya+2 .. ya+9
        __syncthreads();
        flux(ya + 1 + ty);                                    // faces ya+1 .. ya+8
        __syncthreads();
        const int y = ya + ty;
        if (col && y < r1) {
            const long long c = x + (long long)g.S[0] * y;
            double dv[N];
            if (inRange(g, x, y, 0, 2, 2)) {
                const double* lo = fRow(sm, y, r0) + tx * N;
                const double* hi = fRow(sm, y + 1, r0) + tx * N;
                const double* dx = dX + (long long)N * c;
#pragma unroll
                for (int j = 0; j < N; ++j) dv[j] = dx[j] - divI(hi[j] - lo[j], ph.dx[1]);
            } else {
#pragma unroll
                for (int j = 0; j < N; ++j) dv[j] = 0.;
            }
            combinePlanCell<double, 2>(dv, plan, k, c, 0);
        }
        __syncthreads();
    }
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encodeTiled(std::string& err) {
    static std::mutex mu;
    static EncodeTiledFn fn = nullptr;
    std::lock_guard<std::mutex> lock(mu);
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q);
        if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !p) {
            err = "cuTensorMapEncodeTiled unavailable";
            return nullptr;
        }
        fn = reinterpret_cast<EncodeTiledFn>(p);
    }
    return fn;
}

template <int LIM>
void launchFusedLim(const Grid& g, const Phys<double>& ph, int limiter, const StepConst<double>* sc,
                    const double* stage, const double* basis, double* dX, const CombinePlan<double>& plan, int loA,
                    int hiA, const CUtensorMap& tm, unsigned* health, cudaStream_t st) {
    const int rows = g.S[1] - 4;
    const int segs = (g.S[0] - 4 + kSegX - 1) / kSegX;
    if (rows > 0 && segs > 0)
        roeStageXKernel<LIM><<<dim3(segs, rows), kThreadsX, 0, st>>>(g, ph, limiter, sc, stage, basis, dX, loA, hiA,
                                                                   health);
    dim3 grid((g.S[0] + kCols - 1) / kCols, (g.S[1] + kStrip - 1) / kStrip);
    roeStageYKernel<LIM><<<grid, kThreads, sizeof(YShared), st>>>(g, ph, limiter, sc, basis, dX, plan, tm, loA, hiA,
                                                                   health);
}

}  // namespace

size_t roeFusedTensorMapSize() { return sizeof(CUtensorMap); }

// the y pass's dynamic shared memory (above the 48 KB default), for the current device
void roeFusedPrepare() {
    const int bytes = (int)sizeof(YShared);
    cudaFuncSetAttribute(roeStageYKernel<HGPU_LIMITER_MINMOD>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    cudaFuncSetAttribute(roeStageYKernel<HGPU_LIMITER_SUPERBEE>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    cudaFuncSetAttribute(roeStageYKernel<HGPU_LIMITER_VANLEER>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    cudaFuncSetAttribute(roeStageYKernel<-1>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

// The 2D tensor map of a stage buffer for the y pass: rows of S0 x 4 doubles, boxes of
// 32 cells x 8 rows (the row pitch S0 x 32 bytes is a multiple of 16, as required).
bool makeRoeFusedTensorMap(const Grid& g, const double* stage, void* out, std::string& err) {
    EncodeTiledFn fn = encodeTiled(err);
    if (!fn) return false;
    cuuint64_t dims[2] = {(cuuint64_t)g.S[0] * 4, (cuuint64_t)g.S[1]};
    cuuint64_t strides[1] = {(cuuint64_t)g.S[0] * 4 * sizeof(double)};
    cuuint32_t box[2] = {(cuuint32_t)kRow, (cuuint32_t)kRows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = fn(static_cast<CUtensorMap*>(out), CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, const_cast<double*>(stage),
                    dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        err = "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")";
        return false;
    }
    return true;
}

void launchRoeStageFused(const Grid& g, const Phys<double>& ph, int limiter, const StepConst<double>* sc,
                         const double* stage, const double* basis, double* dX, const CombinePlan<double>& plan,
                         int seam, const void* tensorMap, unsigned* health, cudaStream_t st) {
    const int loA = seam ? 1 : 2, hiA = seam ? 0 : 1;
    const CUtensorMap& tm = *static_cast<const CUtensorMap*>(tensorMap);
    switch (limiter) {
    case HGPU_LIMITER_MINMOD: launchFusedLim<HGPU_LIMITER_MINMOD>(g, ph, limiter, sc, stage, basis, dX, plan, loA, hiA, tm, health, st); break;
    case HGPU_LIMITER_SUPERBEE: launchFusedLim<HGPU_LIMITER_SUPERBEE>(g, ph, limiter, sc, stage, basis, dX, plan, loA, hiA, tm, health, st); break;
    case HGPU_LIMITER_VANLEER: launchFusedLim<HGPU_LIMITER_VANLEER>(g, ph, limiter, sc, stage, basis, dX, plan, loA, hiA, tm, health, st); break;
    default: launchFusedLim<-1>(g, ph, limiter, sc, stage, basis, dX, plan, loA, hiA, tm, health, st); break;
    }
}

}  // namespace hgpu
