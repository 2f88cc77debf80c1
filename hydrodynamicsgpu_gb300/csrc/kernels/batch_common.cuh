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

// cell `i` of a tile (i = threadIdx.x + r * blockDim.x for the thread's r-th cell,
// r < tu.cpt), or false if outside the tile/grid
__device__ __forceinline__ bool tileCell(const Grid& g, const BatchTile& t, const BatchTuning& tu, int i, int& x,
                                         int& y, int& z, long long& c) {
    int tx = i % tu.tx, ty = (i / tu.tx) % tu.ty, tz = i / (tu.tx * tu.ty);
    x = t.x0 + tx;
    y = t.y0 + ty;
    z = t.z0 + tz;
    if (tz >= tu.tz || x >= g.S[0] || y >= g.S[1] || z >= g.S[2]) return false;
    c = x + (long long)g.S[0] * (y + (long long)g.S[1] * z);
    return true;
}
__device__ __forceinline__ bool tileCell(const Grid& g, const BatchTile& t, const BatchTuning& tu, int& x, int& y, int& z,
                                         long long& c) {
    return tileCell(g, t, tu, (int)threadIdx.x, x, y, z, c);
}

// The tile kernels run either persistent (perSM >= 0: SMs x blocks per SM blocks pull
// tiles from the queue) or one block per work item (perSM < 0: `items` blocks, block b
// takes item b, no queue).
__device__ __forceinline__ int firstItem(unsigned* q, const BatchTuning& tu) {
    return tu.blocksPerSM < 0 ? (int)blockIdx.x : nextItem(q);
}
__device__ __forceinline__ int nextItemAfter(unsigned* q, const BatchTuning& tu) {
    return tu.blocksPerSM < 0 ? 0x7fffffff : nextItem(q);
}

// The hot kernels come in two forms: the general one (either launch form, any cells
// per thread) and PLAIN, one block per tile and one cell per thread fixed at compile
// time.  Without the two loops, and with the problem's grid copied by value, a plain
// body keeps 15-40 fewer registers live, which buys one or two more blocks per SM.
template <bool PLAIN>
__device__ __forceinline__ int firstTile(unsigned* q) {
    return PLAIN ? (int)blockIdx.x : nextItem(q);
}
template <bool PLAIN>
__device__ __forceinline__ int nextTile(unsigned* q, int nT) {
    return PLAIN ? nT : nextItem(q);
}

template <typename K>
int persistentBlocks(K kernel, int smem, int perSM, int items) {
    if (perSM < 0) return items;
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
