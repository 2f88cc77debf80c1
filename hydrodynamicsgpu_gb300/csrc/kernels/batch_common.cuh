// batch_common.cuh -- work-queue helpers shared by the batched kernels (batch.cu,
// batch_flux.cu).
#pragma once
#include "batch.h"

namespace hgpu {
namespace {

// next work index for the whole block (all threads must call)
__device__ __forceinline__ int nextItem(unsigned* q) {
    __shared__ int item;
    __syncthreads();
    if (threadIdx.x == 0) item = (int)atomicAdd(q, 1u);
    __syncthreads();
    return item;
}

// the cell of this thread inside a tile, or false if outside the tile/grid
__device__ __forceinline__ bool tileCell(const Grid& g, const BatchTile& t, const BatchTuning& tu, int& x, int& y, int& z,
                                         long long& c) {
    int tx = threadIdx.x % tu.tx, ty = (threadIdx.x / tu.tx) % tu.ty, tz = threadIdx.x / (tu.tx * tu.ty);
    x = t.x0 + tx;
    y = t.y0 + ty;
    z = t.z0 + tz;
    if (tz >= tu.tz || x >= g.S[0] || y >= g.S[1] || z >= g.S[2]) return false;
    c = x + (long long)g.S[0] * (y + (long long)g.S[1] * z);
    return true;
}

template <typename K>
int persistentBlocks(K kernel, int smem, int perSM) {
    int dev = 0, sms = 0, occ = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, 256, smem);
    if (occ < 1) occ = 1;
    if (perSM > 0 && perSM < occ) occ = perSM;
    return sms * occ;
}


}  // namespace
}  // namespace hgpu
