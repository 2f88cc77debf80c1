// solver.h -- C++ host classes of the GB300 Euler update, mirroring HydroGPU's
// Solver / Equation / Integrator hierarchy (include/HydroGPU/Solver/*.h,
// include/HydroGPU/Equation/*.h, include/HydroGPU/Integrator/*.h).
//
// Differences from the reference that the GB300 design introduces:
//  * buffers are CUDA device allocations owned by the solver (DeviceBuffer);
//  * the timestep is reduced and kept on the device; update() never blocks;
//  * Integrator::integrate's callback receives the stage state and produces the
//    interface fluxes of that stage; the integrator's fused kernel turns them into
//    the flux divergence and folds it into every Runge-Kutta row that needs it.
#pragma once
#include <cuda_runtime.h>
#include <functional>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../../include/hgpu/hgpu.h"
#include "../kernels/kernels.h"
#include "../kernels/gravity.h"

namespace hgpu {

struct CudaError : std::runtime_error {
    cudaError_t code;
    CudaError(cudaError_t c, const std::string& what) : std::runtime_error(what), code(c) {}
};
void cudaCheck(cudaError_t e, const char* what);

struct ConfigError : std::runtime_error {
    int status;
    ConfigError(int s, const std::string& what) : std::runtime_error(what), status(s) {}
};

// owning device allocation (replaces cl::Buffer, Solver::CL::alloc/zero: Solver.cpp:17-38)
class DeviceBuffer {
public:
    DeviceBuffer() = default;
    explicit DeviceBuffer(size_t bytes, bool zero = true);
    ~DeviceBuffer();
    DeviceBuffer(const DeviceBuffer&) = delete;
    DeviceBuffer& operator=(const DeviceBuffer&) = delete;
    DeviceBuffer(DeviceBuffer&& o) noexcept : ptr_(o.ptr_), bytes_(o.bytes_) { o.ptr_ = nullptr; o.bytes_ = 0; }
    DeviceBuffer& operator=(DeviceBuffer&& o) noexcept;
    void* get() const { return ptr_; }
    template <typename T> T* as() const { return static_cast<T*>(ptr_); }
    size_t bytes() const { return bytes_; }
private:
    void* ptr_ = nullptr;
    size_t bytes_ = 0;
    void release();
};

// ---- checked build (HGPU_CHECKED) ----
// Every DeviceBuffer then carries guard bands of a fixed byte pattern on both sides,
// and kernel bodies test their cell indices (common.cuh cellOk) into one device word.
// checkWord(): that word's device address for the current device (null in the normal
// build).  takeChecks(): waits for the device, then returns and clears the word's
// CHECK_INDEX bit and adds CHECK_GUARD if any live buffer's guard band changed
// (`where` names the first); throws ConfigError(HGPU_ERR_UNSUPPORTED) in the normal build.
unsigned* checkWord();
unsigned takeChecks(std::string& where);

// Validated configuration with the program-preamble constants resolved
// (src/Solver/Solver.cpp:260-315, src/HydroGPUApp.cpp:164-226).
struct ResolvedConfig {
    hgpu_config cfg;
    int dim = 0;
    int numStates = 0;
    double dx[3] = {1, 1, 1};   // as baked (6 significant digits in REF mode)
    double gamma = 1.4;         // as baked (%.14g in REF mode)
    double gravityG = 1.;       // defs.selfGrav_gravitationalConstant as baked (%.14g)
    Grid grid;
};
ResolvedConfig resolveConfig(const hgpu_config& cfg);

// ---------------- Equation (src/Equation/Equation.cpp, Euler.cpp) ----------------
class Equation {
public:
    virtual ~Equation() = default;
    std::vector<std::string> states;
    std::vector<std::string> boundaryMethods;
    virtual std::string name() const = 0;
    // kernel chosen for (axis, state, min/max): 0 periodic, 1 mirror, 2 reflect, 3 freeflow, -1 none
    virtual int stateGetBoundaryKernelForBoundaryMethod(int dim, int state, int minmax) const = 0;
};

class Euler : public Equation {
public:
    Euler(const hgpu_config& cfg, int dim);
    std::string name() const override { return "Euler"; }
    int stateGetBoundaryKernelForBoundaryMethod(int dim, int state, int minmax) const override;
private:
    hgpu_config cfg_;
};

template <typename real> class Solver;

// Runge-Kutta stage plans of a tableau (see buildStagePlans in solver.cu)
template <typename real>
struct StagePlans {
    std::vector<CombinePlan<real>> plans;   // one per stage, slot pointers unset
    std::vector<int> inputSlot;             // stage k reads u^(k) from this slot
    int nslots = 0;                         // work buffers needed besides the state
};
template <typename real> StagePlans<real> buildStagePlans(int tableau);
bool tableauAlphaIsBinary(int tableau);

// ---------------- Integrator (include/HydroGPU/Integrator/Integrator.h:13-17) ----------------
template <typename real>
class Integrator {
public:
    explicit Integrator(Solver<real>* s) : solver(s) {}
    virtual ~Integrator() = default;
    // computeFlux(stage) must leave the interface fluxes of `stage` in the solver's flux buffer
    virtual void integrate(const std::function<void(real* stage)>& computeFlux) = 0;
    // the same stages, each done by stageKernel(stage, plan): a kernel that forms the
    // stage's flux divergence itself and applies the combine `plan` of this stage
    virtual void integrateFused(const std::function<void(real* stage, const CombinePlan<real>& plan)>& stageKernel) = 0;
    // the self-gravity pass with a zero potential (SelfGravitation::applyPotential)
    virtual void integrateZeroDeriv() = 0;
    // the self-gravity pass with a live potential: per callback the relaxation sweeps
    // (useGravity) and calcGravityDeriv of the stage state (SelfGravitation.cpp:100-124)
    virtual void integrateGravity() = 0;
    virtual int order() const = 0;
    virtual int extraBuffers() const = 0;
    // true when the last stage's combine writes the new state and nothing after it in
    // the step (the self-gravity pass with a zero potential) touches the state again
    virtual bool lastCombineWritesState() const { return false; }
    // when set, the last stage (its fluxes and its combine) is handed to this instead
    // of launched whole
    std::function<void(real* stage, const CombinePlan<real>&)> lastStage;
protected:
    Solver<real>* solver;
};

template <typename real>
class ForwardEuler : public Integrator<real> {        // src/Integrator/ForwardEuler.cpp
public:
    using Integrator<real>::Integrator;
    void integrate(const std::function<void(real* stage)>& computeFlux) override;
    void integrateFused(const std::function<void(real* stage, const CombinePlan<real>& plan)>& stageKernel) override;
    void integrateZeroDeriv() override;
    void integrateGravity() override;
    int order() const override { return 1; }
    int extraBuffers() const override { return 0; }
};

template <typename real>
class RungeKutta : public Integrator<real> {          // include/HydroGPU/Integrator/RungeKutta.h
public:
    RungeKutta(Solver<real>* s, int tableau);
    void integrate(const std::function<void(real* stage)>& computeFlux) override;
    void integrateFused(const std::function<void(real* stage, const CombinePlan<real>& plan)>& stageKernel) override;
    void integrateZeroDeriv() override;
    void integrateGravity() override;
    int order() const override { return order_; }
    int extraBuffers() const override { return nslots_; }
    bool lastCombineWritesState() const override { return alphaIsBinary_; }
private:
    int tableau_, order_, nslots_ = 0;
    bool alphaIsBinary_ = true;
    std::vector<CombinePlan<real>> plans_;   // one per stage
    std::vector<int> inputSlot_;             // stage k reads u^(k) from this slot
    std::vector<bool> callbackK_;            // the reference calls back at stage k (a nonzero beta in column k)
    std::vector<DeviceBuffer> work_;
    void buildPlans();
};

// ---------------- Solver (include/HydroGPU/Solver/Solver.h, ISolver.h) ----------------
class ISolver {
public:
    virtual ~ISolver() = default;
    virtual void init() = 0;
    // Converter::toGPU + SelfGravitation::resetState; potential: the initial conditions'
    // potential channel (V values) or null for zero
    virtual void resetState(const void* host, size_t count, const void* potential = nullptr) = 0;
    virtual std::string name() const = 0;
    virtual const Equation& getEquation() const = 0;
};

// per-launch event pair recorded while profiling (hgpu_profile_update)
struct LaunchRecord {
    const char* kind;
    cudaEvent_t start, stop;
};

class SolverBase : public ISolver {
public:
    virtual ~SolverBase();
    // launch wrapper: counts kernels and, while profiling, brackets them with events
    template <class F>
    void launch(const char* kind, int nkernels, F&& f) {
        cudaEvent_t a = nullptr, b = nullptr;
        if (profiling) { a = eventFromPool(); cudaEventRecord(a, stream); }
        f();
        launches_ += nkernels;
        if (profiling) { b = eventFromPool(); cudaEventRecord(b, stream); records.push_back({kind, a, b}); }
    }
    bool profiling = false;
    std::vector<LaunchRecord> records;
    std::vector<cudaEvent_t> eventPool;
    size_t eventNext = 0;
    cudaEvent_t eventFromPool();
    int launches_ = 0;                     // kernels launched by the last update()
    virtual void update() = 0;
    virtual void readState(void* host, size_t count) = 0;
    virtual void readPotential(void* host, size_t count) = 0;
    virtual bool potentialLive() const = 0;
    virtual double lastDt() = 0;
    virtual void* stateDevicePtr() = 0;
    virtual int kernelsPerStep() const = 0;
    // update_host's overlapped form (see Solver<real>::hostStep): supported for this
    // configuration?  hostStep(in, out, upload, download) is one update() that first
    // uploads the state from `in` (upload) and/or ends by downloading it into `out`
    // (download), the copies in bands on a second stream; nothing is synchronised.
    virtual bool hostPipelined() const = 0;
    virtual void hostStep(const void* in, void* out, bool upload, bool download) = 0;
    virtual size_t volume() const = 0;
    // run each Runge-Kutta stage as fused kernels (2D FP64 EulerRoe; HGPU_ERR_UNSUPPORTED otherwise)
    virtual int setFusedStages(bool on) { return on ? HGPU_ERR_UNSUPPORTED : HGPU_OK; }
    virtual int dim() const = 0;
    virtual int numStates() const = 0;
    cudaStream_t stream = nullptr;
    unsigned* health = nullptr;       // device word
    // state check after every step and upload (health.cuh): 0 off, 1 on (default)
    int stateChecks = 1;
};

template <typename real>
class Solver : public SolverBase {
public:
    explicit Solver(const ResolvedConfig& rc);
    ~Solver() override;
    void init() override;
    void resetState(const void* host, size_t count, const void* potential = nullptr) override;
    void readState(void* host, size_t count) override;
    void readPotential(void* host, size_t count) override;
    bool potentialLive() const override { return potentialLive_; }
    const Equation& getEquation() const override { return *equation; }
    void update() override;                 // Solver::update (Solver.cpp:521-546)
    void boundary();                        // Solver::boundary (Solver.cpp:448-464)
    void checkState();                      // the state check into the health word (health.cuh)
    void boundaryOn(real* buf);
    double lastDt() override;
    void* stateDevicePtr() override { return state.get(); }
    size_t volume() const override { return (size_t)rc.grid.V; }
    int dim() const override { return rc.dim; }
    int numStates() const override { return rc.numStates; }
    int kernelsPerStep() const override { return this->launches_; }
    bool hostPipelined() const override;
    void hostStep(const void* in, void* out, bool upload, bool download) override;

    // accessors used by integrators
    ResolvedConfig rc;
    Phys<real> ph;
    DeviceBuffer state, flux, stepConst, dtAcc, healthBuf;
    DeviceBuffer potential;                 // SelfGravitation::potentialBuffer (V values)
    DeviceBuffer relaxRhs;                  // 4 pi G density of the state being relaxed against (double)
    GravityConst<real> gc;                  // relaxation / gravity-source constants
    // the potential the flux kernels see: null while it is zero (its terms change no bit)
    const real* livePotential() const { return potentialLive_ ? potential.as<real>() : nullptr; }
    void relaxPotential(const real* densitySource, int sweeps);   // sweeps x (ghost fill, relax)
    std::unique_ptr<Equation> equation;
    std::unique_ptr<Integrator<real>> integrator;
    StepConst<real>* sc() const { return stepConst.as<StepConst<real>>(); }
    unsigned long long accInit() const;
    int methods[3][2];

protected:
    virtual void initBuffers();
    virtual void initStep() {}
    virtual void calcTimestep() = 0;        // device-side; leaves the minimum in dtAcc
    virtual void step() = 0;
    void finalizeDt(bool fixed);
    void applyPotential();                  // SelfGravitation::applyPotential (SelfGravitation.cpp:100-124)
    bool potentialLive_ = false;            // useGravity, or a nonzero static potential was given

    // The step's work before the stages, split in bands along the slowest axis so that
    // it can start while later bands are still being uploaded.  A solver that supports
    // it does, for the band of slow-axis tiles [tile0, tile0 + tiles) of slowTile()
    // planes each, the part of initStep() + calcTimestep() that reads only the planes
    // of the band and the one below it (bandedPrologueWork), then the rest once every
    // band is done (bandedPrologueEnd).
    virtual bool bandedPrologue() const { return false; }
    virtual int slowTile() const { return 1; }
    virtual void bandedPrologueWork(int tile0, int tiles, cudaStream_t st) { (void)tile0; (void)tiles; (void)st; }
    virtual void bandedPrologueEnd() {}
    // the stages run as fused kernels (no separate combine to cut in bands)
    virtual bool fusedActive() const { return false; }
    // calcFlux in two parts, so that hostStep can run the last stage band by band:
    // fluxPrepare (on the solver's stream) does what precedes the fluxes for the whole
    // grid (EulerRoe: the ghost refresh of SEAM, Delta-q-tilde), then fluxPlanes the
    // interface fluxes of the faces of slow-axis planes [from, to) on stream `st`; the
    // ranges' union gives the same values as calcFlux.
    virtual bool fluxByPlanes() const { return false; }
    virtual void fluxPrepare(real* stage) { (void)stage; }
    virtual void fluxPlanes(real* stage, long long from, long long to, cudaStream_t st) {
        (void)stage; (void)from; (void)to; (void)st;
    }

private:
    cudaStream_t copyStream_ = nullptr;     // update_host's uploads and downloads
    cudaStream_t prepStream_ = nullptr;     // update_host, high priority: the bands' preparation as they
                                            // land, the last stage's band combines
    cudaStream_t sideStream_ = nullptr;     // update_host: every other band's eigenbasis and last-stage fluxes
    std::vector<cudaEvent_t> pipeEvents_;
    cudaEvent_t pipeEvent(size_t i);
};

template <typename real>
class FiniteVolumeSolver : public Solver<real> {   // src/Solver/FiniteVolumeSolver.cpp
public:
    using Solver<real>::Solver;
protected:
    void initBuffers() override;
};

template <typename real>
class Roe : public FiniteVolumeSolver<real> {      // src/Solver/Roe.cpp
public:
    using FiniteVolumeSolver<real>::FiniteVolumeSolver;
protected:
    DeviceBuffer basis, deltaQTilde;
    bool fused_ = false;
    struct alignas(64) TensorMap { unsigned char bytes[128]; };
    std::map<const void*, TensorMap> tensorMaps_;     // per stage buffer, for the fused y pass
    const void* tensorMapFor(const real* stage);
    void fusedStage(real* stage, const CombinePlan<real>& plan);
    bool fusedActive() const override { return fused_; }
    void initBuffers() override;
    void initFlux();                              // calcEigenBasis once per step
    void cflReduce();                             // calcCellTimestep + the min-reduction
    void calcTimestep() override;
    void step() override;
    void calcFlux(real* stage);                   // calcDeltaQTilde + calcFlux
    bool bandedPrologue() const override { return !this->livePotential(); }
    int slowTile() const override { return roeBasisSlowTile(this->rc.dim); }
    void bandedPrologueWork(int tile0, int tiles, cudaStream_t st) override;
    void bandedPrologueEnd() override { cflReduce(); }
    bool fluxByPlanes() const override { return true; }
    void fluxPrepare(real* stage) override;
    void fluxPlanes(real* stage, long long from, long long to, cudaStream_t st) override;
public:
    int setFusedStages(bool on) override;
};

template <typename real>
class EulerRoe : public Roe<real> {               // src/Solver/EulerRoe.cpp
public:
    using Roe<real>::Roe;
    std::string name() const override { return "EulerRoe"; }
protected:
    void step() override;
};

template <typename real>
class HLL : public FiniteVolumeSolver<real> {     // src/Solver/HLL.cpp
public:
    using FiniteVolumeSolver<real>::FiniteVolumeSolver;
protected:
    DeviceBuffer waves;
    void initBuffers() override;
    void initStep() override;                     // calcEigenvalues (frozen for the step)
    void calcTimestep() override;
    void step() override;
    // bands of the wave speeds: the same plane granularity as the Roe eigenbasis bands
    bool bandedPrologue() const override { return !this->livePotential(); }
    int slowTile() const override { return roeBasisSlowTile(this->rc.dim); }
    void bandedPrologueWork(int tile0, int tiles, cudaStream_t st) override;
    void bandedPrologueEnd() override { calcTimestep(); }
    bool fluxByPlanes() const override { return true; }
    void fluxPrepare(real* stage) override;
    void fluxPlanes(real* stage, long long from, long long to, cudaStream_t st) override;
};

template <typename real>
class EulerHLL : public HLL<real> {               // src/Solver/EulerHLL.cpp
public:
    using HLL<real>::HLL;
    std::string name() const override { return "EulerHLL"; }
protected:
    void step() override;
};

template <typename real>
class EulerHLLC : public EulerHLL<real> {         // src/Solver/EulerHLLC.cpp
public:
    using EulerHLL<real>::EulerHLL;
    std::string name() const override { return "EulerHLLC"; }
};

std::unique_ptr<SolverBase> createSolver(const hgpu_config& cfg);

}  // namespace hgpu
