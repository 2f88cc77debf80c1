// reduce.cuh -- single-pass minimum of non-negative reals (the CFL timestep).
//
// Replaces findMinTimestep's multi-pass 16-wide tree with a host read after every
// pass (res/Common.cl:9-40, src/Solver/Solver.cpp:466-516): each thread's minimum
// goes through a warp shuffle and a shared-memory block minimum, and one thread
// per block merges it into a 64-bit accumulator with atomicMin on the IEEE bit
// pattern (order-preserving for non-negative values).  dt never leaves the GPU.
#pragma once
#include "common.cuh"

namespace hgpu {

__device__ __forceinline__ unsigned long long warpMinU64(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w < v ? w : v;
    }
    return v;
}

// Block-wide min of `v` (all threads of the block must call), merged into *acc.
__device__ __forceinline__ void blockMinToGlobal(unsigned long long v, unsigned long long* acc) {
    __shared__ unsigned long long warpMins[32];
    v = warpMinU64(v);
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int nwarps = (blockDim.x + 31) >> 5;
    if (lane == 0) warpMins[warp] = v;
    __syncthreads();
    if (warp == 0) {
        v = lane < nwarps ? warpMins[lane] : ~0ULL;
        v = warpMinU64(v);
        if (lane == 0 && v != ~0ULL) atomicMin(acc, v);
    }
}

}  // namespace hgpu
