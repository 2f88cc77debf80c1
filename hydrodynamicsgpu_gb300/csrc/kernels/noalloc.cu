// noalloc.cu -- a CFL timestep entry point that allocates no device memory.
//
// Some callers cannot call cudaMalloc: a host application that already owns the
// whole device-memory budget through its own pool, code running where allocation
// is forbidden or would deadlock (inside a custom allocator's callback, a
// real-time loop with a fixed memory footprint), or plug-in hosts that hand us
// their device buffers and nothing else.  For them, hgpu_cfl_timestep_noalloc
// computes what Solver::calcTimestep returns for a ghost-filled device state
// (dt = cfl * the minimum over interior cells and axes of the cell timestep) using
// only the caller's input and output plus one fixed scratch array that lives in
// this file and is part of the library image.
//
// The scratch is `g_cflScratch`: kMaxBlocks per-block partial minima, a block
// counter and a flag word.  Every GPU that loads the library holds it (about
// 512 KiB) until the process exits.  Its size bounds the grid: at most
// kMaxBlocks * kThreads = 16,777,216 cells (e.g. 4096 x 4096, or 256^3).
#include <cfloat>
#include <cstring>
#include <mutex>
#include <string>

#include "../../../include/hgpu/hgpu.h"
#include "../host/solver.h"
#include "kernels.h"
#include "reduce.cuh"
#include "roe.cuh"

namespace hgpu {
namespace {

constexpr int kThreads = 256;
constexpr long long kMaxBlocks = 65536;
constexpr int kMaxDevices = 64;

struct CflScratch {
    unsigned long long partial[kMaxBlocks];  // per-block minimum (IEEE bit pattern)
    unsigned long long done;                 // blocks finished; must be 0 when a launch starts
    unsigned long long flags;                // bit 0: a NaN cell timestep was seen
    unsigned long long result;               // dt bit pattern written by the last block
};

static __device__ __align__(256) CflScratch g_cflScratch;

// Host-side device address of g_cflScratch, one per device, looked up once.
std::mutex g_setupMutex;
CflScratch* g_scratchPtr[kMaxDevices] = {};

// Roe: interior cells, per axis dx / (|max(0, lambda_max(face c)) - min(0, lambda_min(face c+1))| + 1e-9)
// (res/Roe.cl:4-65) with both faces' Roe eigenvalues computed here.
template <typename real, int D, int SIDE>
__device__ __forceinline__ real roeCellDt(const Grid& g, const Phys<real>& ph, const real* __restrict__ st,
                                          long long c) {
    const int N = D + 2, NB = RoeRec<D>::NB;
    real a[N], b[N], e[N], rec0[NB], rec1[NB];
    const long long s = g.step[SIDE];
#pragma unroll
    for (int j = 0; j < N; ++j) {
        a[j] = st[(long long)N * (c - s) + j];
        b[j] = st[(long long)N * c + j];
        e[j] = st[(long long)N * (c + s) + j];
    }
    roeBasis<real, D, SIDE>(a, b, ph.gamma, rec0);   // face c
    roeBasis<real, D, SIDE>(b, e, ph.gamma, rec1);   // face c + 1
    real maxLambda = fmax((real)0., rec0[RoeRec<D>::LAME]);
    real minLambda = fmin((real)0., rec1[RoeRec<D>::LAM0]);
    return (real)((double)ph.dx[SIDE] / ((double)fabs(maxLambda - minLambda) + 1e-9));
}

template <typename real, int D>
__device__ __forceinline__ void hllcSpeeds(const real* sL, const real* sR, real gamma, double gq, real& sl,
                                           real& sr) {
    // EulerHLLC.cl:54-97 in the rotated frame (sL, sR already rotated)
    const int E = D + 1;
    real rho[2] = {sL[0], sR[0]}, v0[2], p[2], cc[2];
    const real* ss[2] = {sL, sR};
#pragma unroll
    for (int q = 0; q < 2; ++q) {
        const real* x = ss[q];
        real invDensity = (real)(1. / (double)rho[q]);
        real v[3];
#pragma unroll
        for (int k = 0; k < D; ++k) v[k] = x[1 + k] / rho[q];
        real vv = v[0] * v[0];
#pragma unroll
        for (int k = 1; k < D; ++k) vv = vv + v[k] * v[k];
        real eT = x[E] * invDensity;
        real eI = eT - .5f * vv;
        p[q] = (real)(((double)gamma - 1.) * (double)rho[q] * (double)eI);
        real hT = eT + p[q] * invDensity;
        cc[q] = (real)sqrt(((double)gamma - 1.) * (double)(hT - .5f * vv));
        v0[q] = v[0];
    }
    real pStar = (real)fmax(0., (double)(.5f * (p[0] + p[1]) -
                                         .5f * (v0[1] - v0[0]) * .5f * (rho[0] + rho[1]) * .5f * (cc[0] + cc[1])));
    real qL = pStar <= p[0] ? (real)1. : (real)sqrt(1. + gq * ((double)(pStar / p[0]) - 1.));
    real qR = pStar <= p[1] ? (real)1. : (real)sqrt(1. + gq * ((double)(pStar / p[1]) - 1.));
    sl = v0[0] - cc[0] * qL;
    sr = v0[1] + cc[1] * qR;
}

template <typename real, int D>
__device__ __forceinline__ void hllSpeeds(const real* sL, const real* sR, real gamma, real& sl, real& sr) {
    // EulerHLL.cl:54-113 in the rotated frame: Davis bounded with the Roe averages;
    // `.5 * velocitySq` and `(gamma - 1.)` are double literals there
    const int E = D + 1;
    real rho[2] = {sL[0], sR[0]}, v[2][3], hT[2], cc[2], w[2];
    const real* ss[2] = {sL, sR};
#pragma unroll
    for (int q = 0; q < 2; ++q) {
        const real* x = ss[q];
        real invDensity = (real)(1. / (double)rho[q]);
#pragma unroll
        for (int k = 0; k < D; ++k) v[q][k] = x[1 + k] / rho[q];
        real vv = v[q][0] * v[q][0];
#pragma unroll
        for (int k = 1; k < D; ++k) vv = vv + v[q][k] * v[q][k];
        real eT = x[E] * invDensity;
        real eI = eT - (real)(.5 * (double)vv);
        real p = (real)(((double)gamma - 1.) * (double)rho[q] * (double)eI);
        hT[q] = eT + p * invDensity;
        cc[q] = (real)sqrt(((double)gamma - 1.) * ((double)hT[q] - .5 * (double)vv));
        w[q] = sqrt(rho[q]);
    }
    real norm = (real)(1. / (double)(w[0] + w[1]));
    real vr[3], vvr;
#pragma unroll
    for (int k = 0; k < D; ++k) vr[k] = (w[0] * v[0][k] + w[1] * v[1][k]) * norm;
    real H = (w[0] * hT[0] + w[1] * hT[1]) * norm;
    vvr = vr[0] * vr[0];
#pragma unroll
    for (int k = 1; k < D; ++k) vvr = vvr + vr[k] * vr[k];
    real cs = (real)sqrt(((double)gamma - 1.) * ((double)H - .5 * (double)vvr));
    sl = fminLibm(v[0][0] - cc[0], vr[0] - cs);
    sr = fmaxLibm(v[1][0] + cc[1], vr[0] + cs);
}

template <typename real, int D>
__device__ __forceinline__ void familySpeeds(int hll, const real* sL, const real* sR, real gamma, double gq, real& sl,
                                             real& sr) {
    if (hll) hllSpeeds<real, D>(sL, sR, gamma, sl, sr);
    else hllcSpeeds<real, D>(sL, sR, gamma, gq, sl, sr);
}

template <typename real, int D, int SIDE>
__device__ __forceinline__ real hllcSideDt(const Grid& g, const Phys<real>& ph, double gq, int hll,
                                           const real* __restrict__ st, long long c, int coordAlong) {
    const int N = D + 2;
    const long long s = g.step[SIDE];
    real a[N], b[N];
    auto load = [&](long long cell, real* out) {
#pragma unroll
        for (int j = 0; j < N; ++j) out[j] = st[(long long)N * cell + j];
        if (SIDE > 0) { real t = out[1]; out[1] = out[1 + SIDE]; out[1 + SIDE] = t; }
    };
    real sl, sr, slNext = (real)0., srHere;
    load(c - s, a);
    load(c, b);
    familySpeeds<real, D>(hll, a, b, ph.gamma, gq, sl, srHere);
    if (coordAlong + 1 <= g.S[SIDE] - 2) {        // face c+1 is computed only up to S-2
        load(c + s, a);
        familySpeeds<real, D>(hll, b, a, ph.gamma, gq, slNext, sr);
    }
    real minLambda = (real)fmin(0., (double)slNext);
    real maxLambda = (real)fmax(0., (double)srHere);
    return ph.dx[SIDE] / (maxLambda - minLambda);
}

template <typename real, int D>
__global__ void __launch_bounds__(kThreads) cflNoAllocKernel(Grid g, Phys<real> ph, int hllc, double gq,
                                                             const real* __restrict__ st, unsigned long long init) {
    CflScratch& sc = g_cflScratch;
    long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long best = ~0ULL;
    bool nan = false;
    if (c < g.V) {
        int xyz[3];
        cellCoords(g, c, xyz[0], xyz[1], xyz[2]);
        real r = (real)INFINITY;
        if (!hllc) {
            if (inRange(g, xyz[0], xyz[1], xyz[2], 2, 2)) {
                real d0 = roeCellDt<real, D, 0>(g, ph, st, c);
                best = realBits(d0) < best ? realBits(d0) : best;
                nan |= d0 != d0;
                if (D > 1) {
                    real d1 = roeCellDt<real, D, (D > 1 ? 1 : 0)>(g, ph, st, c);
                    best = realBits(d1) < best ? realBits(d1) : best;
                    nan |= d1 != d1;
                }
                if (D > 2) {
                    real d2 = roeCellDt<real, D, (D > 2 ? 2 : 0)>(g, ph, st, c);
                    best = realBits(d2) < best ? realBits(d2) : best;
                    nan |= d2 != d2;
                }
            } else {
                best = realBits(r);
            }
        } else {
            if (inRange(g, xyz[0], xyz[1], xyz[2], 2, 1)) {
                real d = hllcSideDt<real, D, 0>(g, ph, gq, hllc == 2, st, c, xyz[0]);
                nan |= d != d;
                r = fmin(r, d);
                if (D > 1) {
                    d = hllcSideDt<real, D, (D > 1 ? 1 : 0)>(g, ph, gq, hllc == 2, st, c, xyz[1]);
                    nan |= d != d;
                    r = fmin(r, d);
                }
                if (D > 2) {
                    d = hllcSideDt<real, D, (D > 2 ? 2 : 0)>(g, ph, gq, hllc == 2, st, c, xyz[2]);
                    nan |= d != d;
                    r = fmin(r, d);
                }
            }
            best = realBits(r);
        }
    }
    if (nan) atomicOr(&sc.flags, 1ULL);
    // block minimum into this block's partial slot
    __shared__ unsigned long long warpMins[kThreads / 32];
    best = warpMinU64(best);
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) warpMins[warp] = best;
    __syncthreads();
    __shared__ bool last;
    if (threadIdx.x == 0) {
        unsigned long long m = warpMins[0];
        for (int w = 1; w < kThreads / 32; ++w) m = warpMins[w] < m ? warpMins[w] : m;
        sc.partial[blockIdx.x] = m;
        __threadfence();
        last = atomicAdd(&sc.done, 1ULL) == (unsigned long long)gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    // the last block reduces every partial, applies cfl and re-arms the counter
    __threadfence();
    unsigned long long m = init;
    for (long long i = threadIdx.x; i < gridDim.x; i += kThreads) {
        unsigned long long v = ((volatile unsigned long long*)sc.partial)[i];
        m = v < m ? v : m;
    }
    m = warpMinU64(m);
    if (lane == 0) warpMins[warp] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long mm = warpMins[0];
        for (int w = 1; w < kThreads / 32; ++w) mm = warpMins[w] < mm ? warpMins[w] : mm;
        real mn = (real)bitsToDouble(mm, sizeof(real) == 4);
        real dt = (real)(mn * (real)ph.cfl);
        sc.result = realBits(dt);
        sc.done = 0;
    }
}

template <typename real>
unsigned long long initBits(int solver, int dim) {
    // Roe writes every dtBuffer entry; HLLC leaves entries V..V*dim-1 at max() (Solver.cpp:217-222)
    bool maxInit = solver != HGPU_SOLVER_ROE && dim > 1;
    real v = maxInit ? (sizeof(real) == 8 ? (real)DBL_MAX : (real)FLT_MAX) : (real)INFINITY;
    unsigned long long b = 0;
    memcpy(&b, &v, sizeof(real));
    return b;
}

template <typename real>
void launchCfl(const ResolvedConfig& rc, int hllc, const void* state, long long blocks, cudaStream_t st) {
    Phys<real> ph;
    for (int i = 0; i < 3; ++i) {
        ph.dx[i] = (real)rc.dx[i];
        ph.rdx[i] = (real)1 / ph.dx[i];
    }
    ph.gamma = (real)rc.gamma;
    ph.cfl = rc.cfg.cfl;
    double gq = ((double)ph.gamma + 1.) / (2. * (double)ph.gamma);
    unsigned long long init = initBits<real>(rc.cfg.solver, rc.dim);
    const real* s = static_cast<const real*>(state);
    if (rc.dim == 1) cflNoAllocKernel<real, 1><<<(unsigned)blocks, kThreads, 0, st>>>(rc.grid, ph, hllc, gq, s, init);
    else if (rc.dim == 2) cflNoAllocKernel<real, 2><<<(unsigned)blocks, kThreads, 0, st>>>(rc.grid, ph, hllc, gq, s, init);
    else cflNoAllocKernel<real, 3><<<(unsigned)blocks, kThreads, 0, st>>>(rc.grid, ph, hllc, gq, s, init);
}

// Looks up the device address of g_cflScratch for the current device the first time
// that device is used (host code cannot pass the symbol itself to a kernel).
CflScratch* scratchForCurrentDevice(std::string& err) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        err = "no usable CUDA device";
        return nullptr;
    }
    std::lock_guard<std::mutex> lock(g_setupMutex);
    if (!g_scratchPtr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_cflScratch);
        if (e != cudaSuccess || !p) {
            err = std::string("cudaGetSymbolAddress(g_cflScratch) failed: ") + cudaGetErrorString(e);
            return nullptr;
        }
        g_scratchPtr[dev] = static_cast<CflScratch*>(p);
    }
    return g_scratchPtr[dev];
}

}  // namespace

void setLastError(const std::string& msg);

}  // namespace hgpu

extern "C" int hgpu_cfl_timestep_noalloc(const hgpu_config* cfg, const void* d_state, double* dt_out, void* stream) {
    using namespace hgpu;
    if (!cfg || !d_state || !dt_out) {
        setLastError("hgpu_cfl_timestep_noalloc: null argument");
        return HGPU_ERR_ARG;
    }
    ResolvedConfig rc;
    try {
        rc = resolveConfig(*cfg);
    } catch (const ConfigError& e) {
        setLastError(e.what());
        return e.status;
    }
    if (cfg->use_gravity) {              // the timestep would need the solver's potential
        setLastError("hgpu_cfl_timestep_noalloc: a zero gravitational potential only");
        return HGPU_ERR_UNSUPPORTED;
    }
    long long blocks = (rc.grid.V + kThreads - 1) / kThreads;
    if (blocks > kMaxBlocks) {
        setLastError("hgpu_cfl_timestep_noalloc: grid of " + std::to_string(rc.grid.V) +
                     " cells exceeds the fixed scratch limit of " + std::to_string(kMaxBlocks * kThreads) + " cells");
        return HGPU_ERR_OOB;
    }
    std::string err;
    CflScratch* sc = scratchForCurrentDevice(err);
    if (!sc) {
        setLastError(err);
        return HGPU_ERR_CUDA;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e = cudaMemsetAsync(&sc->done, 0, sizeof(sc->done), st);      // must start at zero
    if (e == cudaSuccess) e = cudaMemsetAsync(&sc->flags, 0, sizeof(sc->flags), st);
    if (e != cudaSuccess) {
        setLastError(std::string("scratch clear failed: ") + cudaGetErrorString(e));
        return HGPU_ERR_CUDA;
    }
    int hllc = rc.cfg.solver == HGPU_SOLVER_ROE ? 0 : (rc.cfg.solver == HGPU_SOLVER_HLL ? 2 : 1);   // 2: EulerHLL
    if (rc.cfg.precision == HGPU_FP32) launchCfl<float>(rc, hllc, d_state, blocks, st);
    else launchCfl<double>(rc, hllc, d_state, blocks, st);
    unsigned long long bits = 0, flags = 0;
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(&bits, &sc->result, sizeof bits, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&flags, &sc->flags, sizeof flags, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        setLastError(std::string("hgpu_cfl_timestep_noalloc: ") + cudaGetErrorString(e));
        return HGPU_ERR_CUDA;
    }
    *dt_out = bitsToDouble(bits, rc.cfg.precision == HGPU_FP32);
    if (flags & 1ULL) {
        setLastError("hgpu_cfl_timestep_noalloc: a cell timestep was NaN");
        return HGPU_ERR_NONFINITE;
    }
    return HGPU_OK;
}
