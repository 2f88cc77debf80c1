// health.cu -- the state check of one problem (health.cuh): after every step and
// after every upload, over the interior cells, into the solver's health word.
#include "health.cuh"

namespace hgpu {

namespace {

constexpr int kThreads = 256;

template <typename real, int D>
__global__ void __launch_bounds__(kThreads) stateCheckKernel(Grid g, const real* __restrict__ state,
                                                             const real* __restrict__ pot, unsigned* health) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned bits = 0;
    if (c < g.V) {
        int x, y, z;
        cellCoords(g, c, x, y, z);
        bits = stateCheckCell<real, D>(g, state, pot, c, x, y, z);
    }
    warpHealthOr(bits, health);
}

}  // namespace

template <typename real>
void launchStateCheck(const Grid& g, const real* state, const real* pot, unsigned* health, cudaStream_t st) {
    const unsigned b = (unsigned)((g.V + kThreads - 1) / kThreads);
    if (g.dim == 1) stateCheckKernel<real, 1><<<b, kThreads, 0, st>>>(g, state, pot, health);
    else if (g.dim == 2) stateCheckKernel<real, 2><<<b, kThreads, 0, st>>>(g, state, pot, health);
    else stateCheckKernel<real, 3><<<b, kThreads, 0, st>>>(g, state, pot, health);
}

template void launchStateCheck<double>(const Grid&, const double*, const double*, unsigned*, cudaStream_t);
template void launchStateCheck<float>(const Grid&, const float*, const float*, unsigned*, cudaStream_t);

}  // namespace hgpu
