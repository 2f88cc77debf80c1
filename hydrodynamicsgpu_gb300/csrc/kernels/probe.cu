// probe.cu -- FP64 fused multiply-add issue-rate probe (the FP64 roofline denominator),
// a self-test of the integer-pipe product and quotient (fp64ops.cuh) against the
// FP64 unit, and one of the bit-pattern MinMod and Superbee (common.cuh) against their
// fmin/fmax expressions.  Eight independent dependency chains per thread keep the FP64 pipe busy;
// every thread writes one result, so nothing is optimised away and every store is in bounds.
#include <cuda_runtime.h>

#include "common.cuh"

namespace hgpu {
namespace {
constexpr int kIter = 4096;
__global__ void __launch_bounds__(256) dfmaProbe(double* out, double a, double b) {
    double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < kIter; ++i) {
        x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
        x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
    out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
}
__device__ __forceinline__ unsigned long long splitmix(unsigned long long z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// operand classes: any exponent (zeros, subnormals, Inf/NaN included), moderate
// exponents, short significands (exact products/quotients, powers of two), extremes,
// exact zeros / infinities / NaNs
__device__ double operand(unsigned long long s, int cls) {
    const unsigned long long r = splitmix(s), m = r & 0xFFFFFFFFFFFFFull, sg = (r >> 63) << 63;
    const unsigned long long t = splitmix(s ^ 0x5bd1e995ull);
    unsigned e;
    unsigned long long mm = m;
    if (cls == 0) e = (unsigned)(t % 2048);
    else if (cls == 1) e = 1023 - 60 + (unsigned)(t % 120);
    else if (cls == 2) { e = 1023 - 4 + (unsigned)(t % 8); mm = m & ~((1ull << (t >> 32) % 53) - 1); }
    else if (cls == 3) e = (t & 1) ? (unsigned)(t % 40) : 2047 - (unsigned)(t % 40);
    else { e = (t & 2) ? 0 : 2047; mm = (t & 4) ? 0 : (t & 8) ? mm : 1; }      // zeros, infinities, NaNs
    return fromBits((long long)(sg | ((unsigned long long)e << 52) | mm));
}

__global__ void selftestKernel(unsigned long long seed, long long cases, unsigned long long* bad) {
    unsigned long long nm = 0, nd = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < cases;
         i += (long long)gridDim.x * blockDim.x) {
        const unsigned long long s = splitmix(seed + (unsigned long long)i);
        const double x = operand(s, (int)(s % 5)), y = operand(s ^ 0xabcdefull, (int)((s >> 8) % 5));
        const double pm = x * y, qm = mulI(x, y), pd = x / y, qd = divI(x, y);
        if (bitsOf(pm) != bitsOf(qm) && !(pm != pm && qm != qm)) ++nm;
        if (bitsOf(pd) != bitsOf(qd) && !(pd != pd && qd != qd)) ++nd;
    }
    if (nm) atomicAdd(&bad[0], nm);
    if (nd) atomicAdd(&bad[1], nd);
}
// the limiters' res/SlopeLimiter.cl expressions with C-library fmin/fmax semantics
__device__ double minmodExpr(double r) { return fmaxLibm(0., fminLibm(r, 1.)); }
__device__ double superbeeExpr(double r) { return fmaxLibm(0., fmaxLibm(fminLibm(1., 2. * r), fminLibm(2., r))); }

// r: a seeded operand of any class, or a quotient of two (the ratios the flux forms)
__global__ void limiterSelftestKernel(unsigned long long seed, long long cases, unsigned long long* bad) {
    unsigned long long n = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < cases;
         i += (long long)gridDim.x * blockDim.x) {
        const unsigned long long s = splitmix(seed + (unsigned long long)i);
        double r = operand(s, (int)(s % 5));
        if ((s >> 40) & 1) r = r / operand(s ^ 0x1234567ull, (int)((s >> 8) % 5));
        if (bitsOf(minmodBits(r)) != bitsOf(minmodExpr(r))) ++n;
        if (bitsOf(superbeeBits(r)) != bitsOf(superbeeExpr(r))) ++n;
    }
    if (n) atomicAdd(bad, n);
}
}  // namespace

// mismatches (bit patterns, signs of zero included) of the bit-pattern MinMod and
// Superbee against their expressions over `cases` seeded ratios
int selftestLimiters(unsigned long long seed, long long cases, long long* bad) {
    unsigned long long* d = nullptr;
    if (cudaMalloc(&d, sizeof(unsigned long long)) != cudaSuccess) return -1;
    cudaMemset(d, 0, sizeof(unsigned long long));
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    limiterSelftestKernel<<<sms * 8, 256>>>(seed, cases, d);
    unsigned long long h = 0;
    cudaError_t e = cudaMemcpy(&h, d, sizeof h, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return -1;
    *bad = (long long)h;
    return 0;
}

// mismatches of mulI / divI against the FP64 unit over `cases` seeded operand pairs
int selftestFp64Ops(unsigned long long seed, long long cases, long long* mulBad, long long* divBad) {
    unsigned long long* bad = nullptr;
    if (cudaMalloc(&bad, 2 * sizeof(unsigned long long)) != cudaSuccess) return -1;
    cudaMemset(bad, 0, 2 * sizeof(unsigned long long));
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    selftestKernel<<<sms * 8, 256>>>(seed, cases, bad);
    unsigned long long h[2] = {0, 0};
    cudaError_t e = cudaMemcpy(h, bad, sizeof h, cudaMemcpyDeviceToHost);
    cudaFree(bad);
    if (e != cudaSuccess) return -1;
    *mulBad = (long long)h[0];
    *divBad = (long long)h[1];
    return 0;
}

// returns fma instructions per second over the whole device, or a negative value on error
double measureFp64FmaRate() {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return -1;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return -1;
    int blocks = sms * 8, threads = 256;
    double* out = nullptr;
    if (cudaMalloc(&out, sizeof(double) * (size_t)blocks * threads) != cudaSuccess) return -1;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    dfmaProbe<<<blocks, threads>>>(out, 0.999999, 1e-7);
    cudaEventRecord(e0);
    const int reps = 5;
    for (int r = 0; r < reps; ++r) dfmaProbe<<<blocks, threads>>>(out, 0.999999, 1e-7);
    cudaEventRecord(e1);
    cudaError_t err = cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (err != cudaSuccess || ms <= 0) return -1;
    double fmas = 8.0 * kIter * (double)blocks * threads * reps;
    return fmas / (ms * 1e-3);
}
}  // namespace hgpu
