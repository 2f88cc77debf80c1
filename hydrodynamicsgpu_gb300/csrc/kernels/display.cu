// display.cu -- the display scalar of every cell into a headless device buffer.
//
// Reference kernel replaced: convertToTex (res/EulerMHDCommon.cl:4-116), its non-GL
// path, which writes float4(value, 0, 0, 0) per cell; here one float per cell.  The
// display index is the reference's DISPLAY_* enum, whose numbering depends on dim
// (src/Equation/Euler.cpp:18-27): DENSITY, VELOCITY, VELOCITY_X, [VELOCITY_Y],
// [VELOCITY_Z], PRESSURE, ENERGY_INTERNAL, ENERGY_KINETIC, ENERGY_TOTAL, POTENTIAL.
// energyPotential = density * potential, with the solver's potential buffer (zero
// unless self-gravity or a static potential is in use).
#include "kernels.h"

namespace hgpu {
namespace {

constexpr int kThreads = 256;

template <typename real, int D>
__global__ void __launch_bounds__(kThreads) displayKernel(Grid g, real gamma, int kind,
                                                          const real* __restrict__ state, float* __restrict__ out,
                                                          const real* __restrict__ pot) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.V) return;
    const int E = D + 1;
    const real* st = state + (long long)(D + 2) * c;
    const real density = st[0];
    real v[3] = {0, 0, 0};
#pragma unroll
    for (int k = 0; k < D; ++k) v[k] = st[1 + k] / density;       // VELOCITY(state)
    real velocitySq = v[0] * v[0];                                 // dot over four components
#pragma unroll
    for (int k = 1; k < D; ++k) velocitySq = velocitySq + v[k] * v[k];
    const real energyTotal = st[E];
    const real energyKinetic = (real)(.5 * (double)density * (double)velocitySq);   // `.5 * density * velocitySq`
    const real potential = pot ? pot[c] : (real)0;
    const real energyPotential = density * potential;
    const real energyInternal = energyTotal - energyKinetic - energyPotential;
    real value = 0;
    switch (kind) {
    case 0: value = density; break;
    case 1: value = sqrt(velocitySq); break;
    case 2: value = v[0]; break;
    case 3: value = v[1]; break;
    case 4: value = v[2]; break;
    case 5: value = (real)(((double)gamma - 1.) * (double)energyInternal); break;
    case 6: value = energyInternal; break;
    case 7: value = energyKinetic; break;
    case 8: value = energyTotal; break;
    case 9: value = potential; break;                               // gravityPotentialBuffer
    }
    out[c] = (float)value;
}

}  // namespace

int displayCount(int dim) { return 7 + dim; }

template <typename real>
void launchDisplay(const Grid& g, real gamma, int method, const real* state, float* out, cudaStream_t st,
                   const real* pot) {
    const int kind = method >= 2 + g.dim ? method + (3 - g.dim) : method;   // the dim-3 numbering
    const unsigned blocks = (unsigned)((g.V + kThreads - 1) / kThreads);
    if (g.dim == 1) displayKernel<real, 1><<<blocks, kThreads, 0, st>>>(g, gamma, kind, state, out, pot);
    else if (g.dim == 2) displayKernel<real, 2><<<blocks, kThreads, 0, st>>>(g, gamma, kind, state, out, pot);
    else displayKernel<real, 3><<<blocks, kThreads, 0, st>>>(g, gamma, kind, state, out, pot);
}

template void launchDisplay<double>(const Grid&, double, int, const double*, float*, cudaStream_t, const double*);
template void launchDisplay<float>(const Grid&, float, int, const float*, float*, cudaStream_t, const float*);

}  // namespace hgpu
