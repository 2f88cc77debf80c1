// probe.cu -- FP64 fused multiply-add issue-rate probe (the FP64 roofline denominator).
// Eight independent dependency chains per thread keep the FP64 pipe busy; every
// thread writes one result, so nothing is optimised away and every store is in bounds.
#include <cuda_runtime.h>

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
}  // namespace

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
