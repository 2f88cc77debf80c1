// solver.cu -- host side of the GB300 Euler update: configuration, buffers, the
// step sequence and the Runge-Kutta stage plans.  Host code only (built by nvcc
// so the launchers' CUDA types resolve); the kernels live in ../kernels/.
#include <type_traits>

#include "solver.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <map>
#include <mutex>

namespace hgpu {

#ifdef HGPU_CHECKED
namespace {
__device__ unsigned g_checkWord;               // CHECK_INDEX bits of the kernels' index tests
constexpr size_t kGuard = 4096;                 // bytes of each guard band
constexpr int kGuardByte = 0xA5;
std::mutex g_guardMu;
std::map<void*, size_t> g_guarded;              // user pointer -> bytes of every live buffer
}  // namespace
#endif

unsigned* checkWord() {
#ifdef HGPU_CHECKED
    static std::mutex mu;
    static unsigned* ptrs[64] = {};
    int dev = 0;
    cudaCheck(cudaGetDevice(&dev), "cudaGetDevice");
    std::lock_guard<std::mutex> lock(mu);
    if (dev < 0 || dev >= 64) return nullptr;
    if (!ptrs[dev]) {
        void* p = nullptr;
        cudaCheck(cudaGetSymbolAddress(&p, g_checkWord), "check word address");
        ptrs[dev] = static_cast<unsigned*>(p);
    }
    return ptrs[dev];
#else
    return nullptr;
#endif
}

unsigned takeChecks(std::string& where) {
#ifdef HGPU_CHECKED
    cudaCheck(cudaDeviceSynchronize(), "synchronize");
    unsigned f = 0, zero = 0;
    cudaCheck(cudaMemcpyFromSymbol(&f, g_checkWord, sizeof f), "check word read");
    cudaCheck(cudaMemcpyToSymbol(g_checkWord, &zero, sizeof zero), "check word clear");
    if (f) where = "a kernel computed a cell index outside its grid";
    std::vector<unsigned char> band(kGuard);
    std::lock_guard<std::mutex> lock(g_guardMu);
    for (const auto& kv : g_guarded) {
        const unsigned char* p = static_cast<const unsigned char*>(kv.first);
        for (const unsigned char* b : {p - kGuard, p + kv.second}) {
            cudaCheck(cudaMemcpy(band.data(), b, kGuard, cudaMemcpyDeviceToHost), "guard band read");
            for (unsigned char v : band)
                if (v != (unsigned char)kGuardByte) {
                    if (!(f & CHECK_GUARD))
                        where = "a write landed in the guard band " + std::string(b < p ? "before" : "after") +
                                " a buffer of " + std::to_string(kv.second) + " bytes";
                    f |= CHECK_GUARD;
                    break;
                }
        }
    }
    return f;
#else
    (void)where;
    throw ConfigError(HGPU_ERR_UNSUPPORTED, "this library was built without HGPU_CHECKED");
#endif
}

void cudaCheck(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw CudaError(e, std::string(what) + ": " + cudaGetErrorString(e));
}

DeviceBuffer::DeviceBuffer(size_t bytes, bool zero) : bytes_(bytes) {
    if (bytes == 0) return;
#ifdef HGPU_CHECKED
    void* base = nullptr;
    cudaError_t e = cudaMalloc(&base, bytes + 2 * kGuard);
    if (e == cudaSuccess) {
        ptr_ = static_cast<unsigned char*>(base) + kGuard;
        cudaCheck(cudaMemset(base, kGuardByte, kGuard), "guard band");
        cudaCheck(cudaMemset(static_cast<unsigned char*>(ptr_) + bytes, kGuardByte, kGuard), "guard band");
        cudaCheck(cudaStreamSynchronize(nullptr), "guard band sync");
        std::lock_guard<std::mutex> lock(g_guardMu);
        g_guarded[ptr_] = bytes;
    }
#else
    cudaError_t e = cudaMalloc(&ptr_, bytes);
#endif
    if (e != cudaSuccess) {
        ptr_ = nullptr;
        (void)cudaGetLastError();
        throw CudaError(e, "cudaMalloc of " + std::to_string(bytes) + " bytes");
    }
    if (zero) {
        // the memset runs on the legacy stream, which the solvers' non-blocking streams
        // do not wait for: finish it before any kernel can read the buffer
        cudaCheck(cudaMemset(ptr_, 0, bytes), "cudaMemset");
        cudaCheck(cudaStreamSynchronize(nullptr), "cudaMemset sync");
    }
}

void DeviceBuffer::release() {
    if (!ptr_) return;
#ifdef HGPU_CHECKED
    {
        std::lock_guard<std::mutex> lock(g_guardMu);
        g_guarded.erase(ptr_);
    }
    cudaFree(static_cast<unsigned char*>(ptr_) - kGuard);
#else
    cudaFree(ptr_);
#endif
    ptr_ = nullptr;
}

DeviceBuffer::~DeviceBuffer() { release(); }

DeviceBuffer& DeviceBuffer::operator=(DeviceBuffer&& o) noexcept {
    if (this != &o) {
        release();
        ptr_ = o.ptr_; bytes_ = o.bytes_;
        o.ptr_ = nullptr; o.bytes_ = 0;
    }
    return *this;
}

SolverBase::~SolverBase() {
    for (cudaEvent_t e : eventPool) cudaEventDestroy(e);
}

cudaEvent_t SolverBase::eventFromPool() {
    if (eventNext == eventPool.size()) {
        cudaEvent_t e;
        cudaCheck(cudaEventCreate(&e), "cudaEventCreate");
        eventPool.push_back(e);
    }
    return eventPool[eventNext++];
}

// ---------------- configuration ----------------
// toNumericString<double> (include/HydroGPU/toNumericString.h:12-22): ostream default
// formatting, i.e. 6 significant digits.
static double bakedDx(double v) {
    char buf[64];
    std::snprintf(buf, sizeof buf, "%g", v);
    return std::strtod(buf, nullptr);
}

ResolvedConfig resolveConfig(const hgpu_config& cfg) {
    ResolvedConfig rc;
    rc.cfg = cfg;
    int dim = cfg.dim;
    if (dim == 0) {                                   // HydroGPUApp.cpp:214-221
        for (dim = 3; dim > 0; --dim)
            if (cfg.size[dim - 1] > 1) break;
    }
    if (dim < 1 || dim > 3) throw ConfigError(HGPU_ERR_CONFIG, "could not determine the dimension from size");
    for (int i = 0; i < 3; ++i) {
        if (i < dim && cfg.size[i] < 5) throw ConfigError(HGPU_ERR_CONFIG, "size must be >= 5 on every active axis");
        if (i >= dim && cfg.size[i] != 1) throw ConfigError(HGPU_ERR_CONFIG, "size must be 1 beyond dim");
    }
    if (cfg.solver != HGPU_SOLVER_ROE && cfg.solver != HGPU_SOLVER_HLLC && cfg.solver != HGPU_SOLVER_HLL)
        throw ConfigError(HGPU_ERR_CONFIG, "unknown solver");
    if (cfg.limiter < 0 || cfg.limiter >= HGPU_NUM_LIMITERS) throw ConfigError(HGPU_ERR_CONFIG, "unknown slope limiter");
    if (cfg.integrator < 0 || cfg.integrator >= HGPU_NUM_INTEGRATORS)
        throw ConfigError(HGPU_ERR_CONFIG, "unknown integrator");
    if (cfg.precision != HGPU_FP64 && cfg.precision != HGPU_FP32) throw ConfigError(HGPU_ERR_CONFIG, "unknown precision");
    if (cfg.compat != HGPU_COMPAT_REF && cfg.compat != HGPU_COMPAT_SEAM)
        throw ConfigError(HGPU_ERR_CONFIG, "unknown compat mode");
    for (int i = 0; i < dim; ++i)
        for (int m = 0; m < 2; ++m) {
            int b = cfg.boundary[i][m];
            if (b < HGPU_BOUNDARY_NONE || b > HGPU_BOUNDARY_FREEFLOW)
                throw ConfigError(HGPU_ERR_CONFIG, "unknown boundary method");
        }
    if (!(cfg.gamma > 1.0)) throw ConfigError(HGPU_ERR_CONFIG, "gamma must be > 1");
    if (!(cfg.cfl > 0.f)) throw ConfigError(HGPU_ERR_CONFIG, "cfl must be > 0");
    if (cfg.use_fixed_dt && !(cfg.fixed_dt > 0)) throw ConfigError(HGPU_ERR_CONFIG, "fixed_dt must be > 0");
    // dx = (xmax - xmin) / (float)size, in the program's real type (HydroGPUApp.cpp:224-226)
    for (int i = 0; i < 3; ++i) {
        double d;
        if (cfg.precision == HGPU_FP32)
            d = (double)(((float)cfg.xmax[i] - (float)cfg.xmin[i]) / (float)cfg.size[i]);
        else
            d = (cfg.xmax[i] - cfg.xmin[i]) / (double)(float)cfg.size[i];
        rc.dx[i] = cfg.compat == HGPU_COMPAT_REF ? bakedDx(d) : d;
        if (i < dim && !(rc.dx[i] > 0)) throw ConfigError(HGPU_ERR_CONFIG, "xmax must exceed xmin");
    }
    if (cfg.gauss_seidel_max_iter < 0) throw ConfigError(HGPU_ERR_CONFIG, "gauss_seidel_max_iter must be >= 0");
    if (cfg.use_gravity && cfg.compat != HGPU_COMPAT_REF)
        throw ConfigError(HGPU_ERR_UNSUPPORTED, "self-gravity is provided with the REF scheme only");
    // `defs` values reach the program through Lua's number formatting (%.14g)
    if (cfg.compat == HGPU_COMPAT_REF) {
        char buf[64];
        std::snprintf(buf, sizeof buf, "%.14g", cfg.gamma);
        rc.gamma = std::strtod(buf, nullptr);
        std::snprintf(buf, sizeof buf, "%.14g", cfg.gravitational_constant);
        rc.gravityG = std::strtod(buf, nullptr);
    } else {
        rc.gamma = cfg.gamma;
        rc.gravityG = cfg.gravitational_constant;
    }
    rc.dim = dim;
    rc.numStates = dim + 2;
    Grid& g = rc.grid;
    for (int i = 0; i < 3; ++i) g.S[i] = cfg.size[i];
    g.dim = dim;
    g.step[0] = 1;
    g.step[1] = cfg.size[0];
    g.step[2] = (long long)cfg.size[0] * cfg.size[1];
    g.V = (long long)cfg.size[0] * cfg.size[1] * cfg.size[2];
    return rc;
}

// ---------------- Equation ----------------
Euler::Euler(const hgpu_config& cfg, int dim) : cfg_(cfg) {      // src/Equation/Euler.cpp:12-49
    boundaryMethods = {"PERIODIC", "MIRROR", "FREEFLOW"};
    states.push_back("DENSITY");
    states.push_back("MOMENTUM_X");
    if (dim > 1) states.push_back("MOMENTUM_Y");
    if (dim > 2) states.push_back("MOMENTUM_Z");
    states.push_back("ENERGY_TOTAL");
}

int Euler::stateGetBoundaryKernelForBoundaryMethod(int dim, int state, int minmax) const {   // Euler.cpp:63-75
    switch (cfg_.boundary[dim][minmax]) {
    case HGPU_BOUNDARY_NONE: return -1;
    case HGPU_BOUNDARY_PERIODIC: return 0;
    case HGPU_BOUNDARY_MIRROR: return dim + 1 == state ? 2 : 1;
    case HGPU_BOUNDARY_FREEFLOW: return 3;
    }
    throw ConfigError(HGPU_ERR_CONFIG, "unknown boundary method");
}

// ---------------- Integrators ----------------
template <typename real>
void ForwardEuler<real>::integrate(const std::function<void(real* stage)>& computeFlux) {
    Solver<real>* s = this->solver;
    computeFlux(s->state.template as<real>());
    CombinePlan<real> plan{};
    plan.fe = 1;
    plan.slot[0] = s->state.template as<real>();
    s->launch("flux_divergence_combine", 1, [&] {
        launchDerivCombine<real>(s->rc.grid, s->ph, s->flux.template as<real>(), plan, s->sc(), s->stream);
    });
}

// ForwardEuler updates its stage buffer (the state) in place, which a kernel that also
// reads its neighbours' stage values cannot do; solvers keep it on the unfused path.
template <typename real>
void ForwardEuler<real>::integrateFused(const std::function<void(real*, const CombinePlan<real>&)>&) {
    throw ConfigError(HGPU_ERR_UNSUPPORTED, "fused stages need a Runge-Kutta integrator");
}

template <typename real>
void ForwardEuler<real>::integrateZeroDeriv() {
    Solver<real>* s = this->solver;
    s->boundary();                                            // the callback's solver->boundary()
    s->launch("gravity_pass", 1, [&] { launchZeroAdd<real>(s->rc.grid, s->state.template as<real>(), s->sc(), s->stream); });
}

// FE: the callback's relaxation and calcGravityDeriv read the state, its boundary()
// refreshes the ghosts, then state += deriv * dt (the deriv reads interior cells only,
// so it is formed after the ghost fill, fused with the update)
template <typename real>
void ForwardEuler<real>::integrateGravity() {
    Solver<real>* s = this->solver;
    if (s->rc.cfg.use_gravity) s->relaxPotential(s->state.template as<real>(), s->rc.cfg.gauss_seidel_max_iter);
    s->boundary();
    CombinePlan<real> plan{};
    plan.fe = 1;
    plan.slot[0] = s->state.template as<real>();
    s->launch("gravity_source_combine", 1, [&] {
        launchGravityCombine<real>(s->rc.grid, s->gc, s->state.template as<real>(), s->potential.template as<real>(),
                                   plan, s->sc(), s->stream);
    });
}

template <typename real>
RungeKutta<real>::RungeKutta(Solver<real>* s, int tableau) : Integrator<real>(s), tableau_(tableau) {
    order_ = tableauOrder(tableau);
    alphaIsBinary_ = tableauAlphaIsBinary(tableau);
    buildPlans();
}

// Build the per-stage combine plans.  Row m of the tableau (the input of stage m+1,
// or the new state for m = order-1) is accumulated column by column: at stage k
// its alpha(m,k) u^(k) and beta(m,k) dt d^(k) terms are added, in that order, to its
// partial sum.  A row whose sum is still exactly u^n (alpha = 1, nothing else) is
// not materialised: it aliases the state buffer, which holds u^n until the last
// stage writes the new state into it.  Slot 0 is the state; slots 1..nslots are work
// buffers of the state's size.  Pointers are filled in by the caller.
template <typename real>
StagePlans<real> buildStagePlans(int tableau) {
    StagePlans<real> out;
    const int order = tableauOrder(tableau);
    struct Row { int slot = -1; bool alias0 = false; };
    std::vector<Row> rows(order);
    std::vector<bool> slotBusy(8, false);
    slotBusy[0] = true;
    int maxSlot = 0;
    auto alloc = [&]() {
        for (int i = 1; i < 8; ++i)
            if (!slotBusy[i]) { slotBusy[i] = true; maxSlot = std::max(maxSlot, i); return i; }
        throw std::logic_error("out of Runge-Kutta work slots");
    };
    int inSlot = 0;
    for (int k = 0; k < order; ++k) {
        CombinePlan<real> plan{};
        plan.fe = 0;
        plan.in = inSlot;
        for (int m = k; m < order; ++m) {
            double a = tableauAlpha(tableau, m, k), b = tableauBeta(tableau, m, k);
            if (a == 0.0 && b == 0.0) continue;
            Row& r = rows[m];
            bool fresh = r.slot < 0 && !r.alias0;
            if (fresh && a == 1.0 && b == 0.0 && inSlot == 0 && !(m == order - 1 && k == order - 1)) {
                r.alias0 = true;           // sum so far == +0 + u^n * 1
                continue;
            }
            CombineOp<real> op{};
            op.prior = r.alias0 ? 0 : r.slot;
            op.priorAlias = r.alias0 ? 1 : 0;
            op.hasAlpha = a != 0.0;
            op.alpha = (real)a;
            op.alphaIsOne = a == 1.0;
            op.hasBeta = b != 0.0;
            op.brow = m;
            op.bcol = k;
            if (m == order - 1 && k == order - 1) op.out = 0;
            else if (r.slot >= 0) op.out = r.slot;
            else op.out = alloc();
            r.slot = op.out;
            r.alias0 = false;
            if (plan.nops >= 4) throw std::logic_error("too many rows in a stage");
            plan.ops[plan.nops++] = op;
        }
        out.plans.push_back(plan);
        out.inputSlot.push_back(inSlot);
        if (k < order - 1) {
            if (inSlot != 0) slotBusy[inSlot] = false;   // u^(k) is consumed by stage k
            inSlot = rows[k].alias0 ? 0 : rows[k].slot;
        }
    }
    out.nslots = maxSlot;
    return out;
}

bool tableauAlphaIsBinary(int tableau) {
    int order = tableauOrder(tableau);
    for (int m = 0; m < order; ++m)
        for (int k = 0; k <= m; ++k) {
            double a = tableauAlpha(tableau, m, k);
            if (a != 0.0 && a != 1.0) return false;
        }
    return true;
}

template <typename real>
void RungeKutta<real>::buildPlans() {
    StagePlans<real> sp = buildStagePlans<real>(tableau_);
    plans_ = sp.plans;
    inputSlot_ = sp.inputSlot;
    nslots_ = sp.nslots;
    callbackK_.assign(order_, false);
    for (int k = 0; k < order_; ++k)
        for (int m = k; m < order_; ++m) callbackK_[k] = callbackK_[k] || tableauBeta(tableau_, m, k) != 0.0;
    work_.clear();
    size_t bytes = sizeof(real) * (size_t)this->solver->rc.grid.V * this->solver->rc.numStates;
    for (int i = 0; i < nslots_; ++i) work_.emplace_back(bytes, true);
    for (auto& p : plans_) {
        p.slot[0] = this->solver->state.template as<real>();
        for (int i = 0; i < nslots_; ++i) p.slot[1 + i] = work_[i].template as<real>();
    }
}

template <typename real>
void RungeKutta<real>::integrate(const std::function<void(real* stage)>& computeFlux) {
    Solver<real>* s = this->solver;
    for (int k = 0; k < order_; ++k) {
        real* in = plans_[k].slot[inputSlot_[k]];
        if (k == order_ - 1 && this->lastStage) {
            this->lastStage(in, plans_[k]);
            continue;
        }
        computeFlux(in);
        s->launch("flux_divergence_combine", 1, [&] {
            launchDerivCombine<real>(s->rc.grid, s->ph, s->flux.template as<real>(), plans_[k], s->sc(), s->stream);
        });
    }
}

// the same stages; plans_[k] never writes the slot stage k reads (buildStagePlans)
template <typename real>
void RungeKutta<real>::integrateFused(const std::function<void(real*, const CombinePlan<real>&)>& stageKernel) {
    for (int k = 0; k < order_; ++k) stageKernel(plans_[k].slot[inputSlot_[k]], plans_[k]);
}

template <typename real>
void RungeKutta<real>::integrateZeroDeriv() {
    // With every deriv +0 the stage states are alpha-combinations of u^n.  For
    // tableaus whose alphas are all 0 or 1 that is u^n itself (the step leaves no -0
    // in the state), so nothing runs.
    if (alphaIsBinary_) return;
    Solver<real>* s = this->solver;
    s->launch("gravity_pass", 1, [&] {
        launchAlphaOnly<real>(s->rc.grid, tableau_, s->state.template as<real>(), s->sc(), s->stream);
    });
}

// RK: the callback of stage k (RungeKutta.h:76-123) relaxes the potential against the
// stage state's density and forms calcGravityDeriv from it; the deriv goes into this
// stage's column of the combine.  Its boundary() only touches the stage buffer, which
// the next stage rebuilds from the saved stage states, so it changes nothing.
template <typename real>
void RungeKutta<real>::integrateGravity() {
    Solver<real>* s = this->solver;
    for (int k = 0; k < order_; ++k) {
        real* in = plans_[k].slot[inputSlot_[k]];
        if (callbackK_[k] && s->rc.cfg.use_gravity) s->relaxPotential(in, s->rc.cfg.gauss_seidel_max_iter);
        s->launch("gravity_source_combine", 1, [&] {
            launchGravityCombine<real>(s->rc.grid, s->gc, in, s->potential.template as<real>(), plans_[k], s->sc(),
                                       s->stream);
        });
    }
}

// ---------------- Solver ----------------
template <typename real>
Solver<real>::Solver(const ResolvedConfig& rc_) : rc(rc_) {
    rc.grid.check = checkWord();
    for (int i = 0; i < 3; ++i) {
        ph.dx[i] = (real)rc.dx[i];
        ph.rdx[i] = (real)1 / ph.dx[i];
    }
    ph.gamma = (real)rc.gamma;
    ph.cfl = rc.cfg.cfl;
    gc = gravityConst<real>(rc.dx, rc.gravityG, rc.dim);
}

template <typename real>
Solver<real>::~Solver() {
    integrator.reset();
    for (cudaEvent_t e : pipeEvents_) cudaEventDestroy(e);
    if (copyStream_) cudaStreamDestroy(copyStream_);
    if (prepStream_) cudaStreamDestroy(prepStream_);
    if (sideStream_) cudaStreamDestroy(sideStream_);
    if (stream) cudaStreamDestroy(stream);
}

template <typename real>
unsigned long long Solver<real>::accInit() const {
    // Roe writes every dtBuffer entry (INFINITY outside the interior); HLLC writes only
    // the first volume entries, the rest keep their initial max() (Solver.cpp:217-222,
    // EulerHLLC.cl:135-168), which joins the minimum when dim > 1.
    bool maxInit = rc.cfg.solver != HGPU_SOLVER_ROE && rc.dim > 1;   // the HLL driver (HLLC and HLL)
    if (sizeof(real) == 8) {
        double v = maxInit ? DBL_MAX : std::numeric_limits<double>::infinity();
        unsigned long long b;
        std::memcpy(&b, &v, 8);
        return b;
    }
    float v = maxInit ? FLT_MAX : std::numeric_limits<float>::infinity();
    unsigned int b;
    std::memcpy(&b, &v, 4);
    return b;
}

template <typename real>
void Solver<real>::init() {                                  // Solver::init (Solver.cpp:48-205)
    equation.reset(new Euler(rc.cfg, rc.dim));
    cudaCheck(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "cudaStreamCreate");
    for (int i = 0; i < 3; ++i)
        for (int m = 0; m < 2; ++m) methods[i][m] = i < rc.dim ? rc.cfg.boundary[i][m] : -1;
    initBuffers();
    if (rc.cfg.integrator == HGPU_INTEGRATOR_FORWARD_EULER) integrator.reset(new ForwardEuler<real>(this));
    else integrator.reset(new RungeKutta<real>(this, rc.cfg.integrator));
    unsigned long long init = accInit();
    cudaCheck(cudaMemcpy(dtAcc.get(), &init, sizeof init, cudaMemcpyHostToDevice), "dt accumulator init");
    cudaCheck(cudaDeviceSynchronize(), "init");
}

template <typename real>
void Solver<real>::initBuffers() {                           // Solver::initBuffers (Solver.cpp:208-223)
    size_t n = (size_t)rc.grid.V * rc.numStates;
    state = DeviceBuffer(sizeof(real) * n, true);
    stepConst = DeviceBuffer(sizeof(StepConst<real>), true);
    dtAcc = DeviceBuffer(sizeof(unsigned long long), true);
    healthBuf = DeviceBuffer(sizeof(unsigned), true);
    health = healthBuf.as<unsigned>();
    potential = DeviceBuffer(sizeof(real) * (size_t)rc.grid.V, true);
    if (rc.cfg.use_gravity) relaxRhs = DeviceBuffer(sizeof(double) * (size_t)rc.grid.V, true);
}

// Converter::toGPU (Solver.cpp:333-337) then SelfGravitation::resetState
// (SelfGravitation.cpp:35-98): the potential is -density with useGravity (relaxed
// 100 x gaussSeidelMaxIter times), else the initial conditions' channel; the total
// energy gets the potential as it was before relaxing (the host vector) added.
template <typename real>
void Solver<real>::resetState(const void* host, size_t count, const void* pot) {
    if (count != (size_t)rc.grid.V * rc.numStates) throw ConfigError(HGPU_ERR_ARG, "state element count mismatch");
    const size_t V = (size_t)rc.grid.V;
    cudaCheck(cudaMemcpyAsync(state.get(), host, sizeof(real) * count, cudaMemcpyHostToDevice, stream), "set_state");
    bool nonzero = false;
    if (!rc.cfg.use_gravity && pot) {
        const unsigned char* b = static_cast<const unsigned char*>(pot);
        for (size_t i = 0; i < sizeof(real) * V && !nonzero; ++i) nonzero = b[i] != 0;
    }
    if (!rc.cfg.use_gravity && nonzero)
        cudaCheck(cudaMemcpyAsync(potential.get(), pot, sizeof(real) * V, cudaMemcpyHostToDevice, stream),
                  "set_potential");
    else
        cudaCheck(cudaMemsetAsync(potential.get(), 0, sizeof(real) * V, stream), "zero potential");
    launchPotentialInit<real>(rc.grid, rc.cfg.use_gravity ? 1 : 0, state.as<real>(), potential.as<real>(), stream);
    potentialLive_ = rc.cfg.use_gravity || nonzero;
    // 100 x gaussSeidelMaxIter relaxations; they read the density, which the energy
    // update above does not touch
    if (rc.cfg.use_gravity) relaxPotential(state.as<real>(), 100 * rc.cfg.gauss_seidel_max_iter);
    checkState();
    cudaCheck(cudaGetLastError(), "reset kernels");
    cudaCheck(cudaStreamSynchronize(stream), "set_state sync");
}

// `sweeps` x (potentialBoundary, relax) (SelfGravitation.cpp:81-86, 112-117).  The
// relaxation reads and writes interior cells only and the ghost fill writes ghosts only,
// so the ghosts end up as the last fill leaves them and the interior as the sweeps do:
// sweeps-1 relaxations, one fill, one relaxation give the same bits.
template <typename real>
void Solver<real>::relaxPotential(const real* densitySource, int sweeps) {
    if (sweeps <= 0) return;
    launch("poisson_relax_rhs", 1, [&] {
        launchRelaxRhs<real>(rc.grid, gc, densitySource, relaxRhs.template as<double>(), stream);
    });
    auto sweep = [&] {
        launch("poisson_relax", 2, [&] {
            launchRelaxSweep<real>(rc.grid, gc, relaxRhs.template as<double>(), potential.as<real>(), stream);
        });
    };
    for (int i = 0; i < sweeps - 1; ++i) sweep();
    launch("potential_boundary", rc.dim, [&] {
        launchPotentialBoundary<real>(rc.grid, methods, potential.as<real>(), stream);
    });
    sweep();
}

template <typename real>
void Solver<real>::readPotential(void* host, size_t count) {
    if (count != (size_t)rc.grid.V) throw ConfigError(HGPU_ERR_ARG, "potential element count mismatch");
    cudaCheck(cudaMemcpyAsync(host, potential.get(), sizeof(real) * count, cudaMemcpyDeviceToHost, stream),
              "get_potential");
    cudaCheck(cudaStreamSynchronize(stream), "get_potential sync");
}

template <typename real>
void Solver<real>::readState(void* host, size_t count) {
    if (count != (size_t)rc.grid.V * rc.numStates) throw ConfigError(HGPU_ERR_ARG, "state element count mismatch");
    cudaCheck(cudaMemcpyAsync(host, state.get(), sizeof(real) * count, cudaMemcpyDeviceToHost, stream), "get_state");
    cudaCheck(cudaStreamSynchronize(stream), "get_state sync");
}

template <typename real>
double Solver<real>::lastDt() {
    double dt = 0;
    cudaCheck(cudaMemcpyAsync(&dt, &sc()->dt_f64, sizeof dt, cudaMemcpyDeviceToHost, stream), "last dt");
    cudaCheck(cudaStreamSynchronize(stream), "last dt sync");
    return dt;
}

template <typename real>
void Solver<real>::boundaryOn(real* buf) {
    launch("boundary", rc.dim, [&] { launchBoundary<real>(rc.grid, methods, buf, stream); });
}

template <typename real>
void Solver<real>::boundary() { boundaryOn(state.as<real>()); }

template <typename real>
cudaEvent_t Solver<real>::pipeEvent(size_t i) {
    while (pipeEvents_.size() <= i) {
        cudaEvent_t e;
        cudaCheck(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event create");
        pipeEvents_.push_back(e);
    }
    return pipeEvents_[i];
}

template <typename real>
bool Solver<real>::hostPipelined() const {
    return rc.dim >= 2 && !rc.cfg.use_fixed_dt && !rc.cfg.use_gravity && bandedPrologue();
}

// One update() whose state comes from host memory `in` (upload) and/or goes back to
// host memory `out` (download), with the copies overlapped with the step's own work
// (EulerRoe: the eigenbasis; EulerHLLC / EulerHLL: the wave speeds).
// The slowest axis (y in 2D, z in 3D) is cut into bands of slow-axis tiles.  Upload:
// band after band goes up on the copy stream, the last band first (it holds the planes
// the periodic / mirror / free-flow fill of the first ghost planes reads), then band
// 0, 1, ...; a preparation stream takes each band as it lands: E += 0 (the zero
// potential's resetState pass) and the ghost fill of the other axes on the band's
// planes; the slow axis's own ghost fill runs once the first and last bands are in.
// Each band's share of the eigenbasis (or wave speeds), which reads the band's planes
// and the one below, follows its preparation on one of two streams (alternate bands),
// so consecutive bands overlap.  Download: the last stage runs band by band, its
// fluxes on the solver's stream and each band's combine on the side stream as soon as
// the fluxes it reads are there, and each band goes down as soon as it is written.
// Every cell sees the same operations as in set_state + update + get_state, so the
// results are the same bits.
template <typename real>
void Solver<real>::hostStep(const void* in, void* out, bool upload, bool download) {
    this->launches_ = 0;
    if (!copyStream_) {
        int lowest = 0, highest = 0;
        cudaCheck(cudaDeviceGetStreamPriorityRange(&lowest, &highest), "stream priorities");
        cudaCheck(cudaStreamCreateWithFlags(&copyStream_, cudaStreamNonBlocking), "update_host stream");
        // the bands' preparations and last combines gate the next band's work and
        // its download: their blocks go ahead of the eigenbasis and flux blocks queued
        cudaCheck(cudaStreamCreateWithPriority(&prepStream_, cudaStreamNonBlocking, highest), "update_host stream");
        cudaCheck(cudaStreamCreateWithFlags(&sideStream_, cudaStreamNonBlocking), "update_host stream");
    }
    const Grid& g = rc.grid;
    const int A = rc.dim - 1;                                       // slowest axis
    const long long S_A = g.S[A];
    const long long plane = (long long)g.V / S_A;                   // cells per slow-axis plane
    const long long N = rc.numStates;
    const int T_A = slowTile();
    const long long tilesA = (S_A + T_A - 1) / T_A;
    // tiles a band: 128 rows in 2D (measured at 2048^2, ms per update_host step: 4 tiles
    // 9.99, 8 9.15, 16 8.74, 32 8.71, 64 8.78, 128 9.09; smaller bands cost launches
    // and partial waves), 16 planes in 3D; at least 4 planes in the first and last band
    const long long per = std::max<long long>(rc.dim == 2 ? 16 : 8, (4 + T_A - 1) / T_A + 1);
    const int K = (int)std::max<long long>(1, tilesA / per);
    auto tile0 = [&](int j) { return (long long)j * per; };
    auto tile1 = [&](int j) { return j == K - 1 ? tilesA : (long long)(j + 1) * per; };
    auto plane0 = [&](int j) { return tile0(j) * T_A; };
    auto plane1 = [&](int j) { return std::min<long long>(tile1(j) * T_A, S_A); };
    auto bytesOf = [&](long long planes) { return (size_t)(planes * plane * N) * sizeof(real); };
    auto offOf = [&](long long p) { return (size_t)(p * plane * N) * sizeof(real); };
    size_t ev = 0;
    cudaEvent_t start = pipeEvent(ev++);
    cudaCheck(cudaEventRecord(start, stream), "event record");
    cudaCheck(cudaStreamWaitEvent(copyStream_, start, 0), "stream wait");   // the state is free to overwrite

    if (upload) {
        cudaCheck(cudaMemsetAsync(potential.get(), 0, sizeof(real) * (size_t)g.V, stream), "zero potential");
        potentialLive_ = false;
        std::vector<cudaEvent_t> landed(K);
        std::vector<int> order;
        order.push_back(K - 1);
        for (int j = 0; j < K - 1; ++j) order.push_back(j);
        for (int j : order) {
            cudaCheck(cudaMemcpyAsync(static_cast<char*>(state.get()) + offOf(plane0(j)),
                                      static_cast<const char*>(in) + offOf(plane0(j)),
                                      bytesOf(plane1(j) - plane0(j)), cudaMemcpyHostToDevice, copyStream_),
                      "update_host upload");
            landed[j] = pipeEvent(ev++);
            cudaCheck(cudaEventRecord(landed[j], copyStream_), "event record");
        }
        // the preparation of each band as it lands, on its own stream (after the zeroing
        // of the potential); prepped[j]: band j is ready, and so is every band prepared
        // before it (prep order K-1, 0, then the slow axis's fill, then 1 .. K-2)
        cudaEvent_t zeroed = pipeEvent(ev++);
        cudaCheck(cudaEventRecord(zeroed, stream), "event record");
        cudaCheck(cudaStreamWaitEvent(prepStream_, zeroed, 0), "stream wait");
        std::vector<cudaEvent_t> prepped(K);
        auto prep = [&](int j) {
            cudaCheck(cudaStreamWaitEvent(prepStream_, landed[j], 0), "stream wait");
            launch("potential_init", 1, [&] {
                launchPotentialInit<real>(g, 0, state.as<real>(), potential.as<real>(), prepStream_,
                                          plane0(j) * plane, plane1(j) * plane);
            });
            for (int a = 0; a < A; ++a) {
                // lines of axis a through the band: t = c[T] + S[T] c[U] with U the slow axis
                // in 3D (S[T] lines a plane), T the slow axis in 2D (one line a plane)
                const long long perPlane = rc.dim == 2 ? 1 : g.S[a == 0 ? 1 : 0];
                launch("boundary", 1, [&] {
                    launchBoundaryAxis<real>(g, methods, state.as<real>(), prepStream_, a, plane0(j) * perPlane,
                                             plane1(j) * perPlane);
                });
            }
        };
        auto mark = [&](int j) {
            prepped[j] = pipeEvent(ev++);
            cudaCheck(cudaEventRecord(prepped[j], prepStream_), "event record");
        };
        prep(K - 1);
        if (K > 1) prep(0);
        launch("boundary", 1, [&] { launchBoundaryAxis<real>(g, methods, state.as<real>(), prepStream_, A); });
        mark(0);
        if (K > 1) prepped[K - 1] = prepped[0];
        for (int j = 1; j < K - 1; ++j) {
            prep(j);
            mark(j);
        }
        // each band's eigenbasis (wave speeds) once its planes and the plane below are
        // ready, bands alternating between two streams: a band's kernel reads no other
        // band's output, so consecutive bands overlap (and fill each other's tail wave)
        cudaEvent_t sideLast = nullptr;
        for (int j = 0; j < K; ++j) {
            cudaStream_t bs = (j & 1) ? sideStream_ : stream;
            const int need = (j == K - 1 && K > 2) ? K - 2 : j;     // band K-1 reads band K-2's top plane
            cudaCheck(cudaStreamWaitEvent(bs, prepped[need], 0), "stream wait");
            bandedPrologueWork((int)tile0(j), (int)(tile1(j) - tile0(j)), bs);
            if (bs == sideStream_) {
                sideLast = pipeEvent(ev++);
                cudaCheck(cudaEventRecord(sideLast, sideStream_), "event record");
            }
        }
        if (sideLast) cudaCheck(cudaStreamWaitEvent(stream, sideLast, 0), "stream wait");
        bandedPrologueEnd();
    } else {
        boundary();
        initStep();
        calcTimestep();
    }
    finalizeDt(false);

    const bool banded = download && integrator->lastCombineWritesState() && !fusedActive() && fluxByPlanes();
    struct Unhook {
        Integrator<real>* i;
        ~Unhook() { i->lastStage = nullptr; }
    } unhook{integrator.get()};
    if (banded) {
        // The last stage band by band: on the solver's stream the fluxes the band's
        // combine reads (planes [p0, p1], continuing from the previous band's); on the
        // side stream the band's combine once they are there, then its download.  The
        // fluxes of band j+1 overlap the combine of band j: they write flux planes past
        // p1(j) and read the stage input, which the last combine (it writes the state,
        // never its own stage's input) does not touch.
        integrator->lastStage = [&](real* stageIn, const CombinePlan<real>& plan) {
            fluxPrepare(stageIn);
            cudaEvent_t prepared = pipeEvent(ev++);
            cudaCheck(cudaEventRecord(prepared, stream), "event record");
            cudaCheck(cudaStreamWaitEvent(sideStream_, prepared, 0), "stream wait");
            long long fluxDone = 0;
            cudaEvent_t prevFluxed = nullptr;
            for (int j = 0; j < K; ++j) {
                // band j's fluxes on alternating streams (they read only what fluxPrepare
                // wrote and the stage input); its combine reads flux planes up to p1(j),
                // written by this band's call and the previous one
                cudaStream_t fs = (j & 1) ? sideStream_ : stream;
                const long long fEnd = std::min<long long>(plane1(j) + 1, S_A);
                fluxPlanes(stageIn, fluxDone, fEnd, fs);
                fluxDone = fEnd;
                cudaEvent_t fluxed = pipeEvent(ev++);
                cudaCheck(cudaEventRecord(fluxed, fs), "event record");
                cudaCheck(cudaStreamWaitEvent(prepStream_, fluxed, 0), "stream wait");
                if (prevFluxed) cudaCheck(cudaStreamWaitEvent(prepStream_, prevFluxed, 0), "stream wait");
                prevFluxed = fluxed;
                launch("flux_divergence_combine", 1, [&] {
                    launchDerivCombine<real>(g, ph, flux.template as<real>(), plan, sc(), prepStream_,
                                             plane0(j) * plane, plane1(j) * plane);
                });
                cudaEvent_t written = pipeEvent(ev++);
                cudaCheck(cudaEventRecord(written, prepStream_), "event record");
                cudaCheck(cudaStreamWaitEvent(copyStream_, written, 0), "stream wait");
                cudaCheck(cudaMemcpyAsync(static_cast<char*>(out) + offOf(plane0(j)),
                                          static_cast<const char*>(state.get()) + offOf(plane0(j)),
                                          bytesOf(plane1(j) - plane0(j)), cudaMemcpyDeviceToHost, copyStream_),
                          "update_host download");
            }
            cudaEvent_t combined = pipeEvent(ev++);
            cudaCheck(cudaEventRecord(combined, prepStream_), "event record");
            cudaCheck(cudaStreamWaitEvent(stream, combined, 0), "stream wait");
        };
    }
    step();
    checkState();
    if (download && !banded) {
        cudaEvent_t stepped = pipeEvent(ev++);
        cudaCheck(cudaEventRecord(stepped, stream), "event record");
        cudaCheck(cudaStreamWaitEvent(copyStream_, stepped, 0), "stream wait");
        cudaCheck(cudaMemcpyAsync(out, state.get(), bytesOf(S_A), cudaMemcpyDeviceToHost, copyStream_),
                  "update_host download");
    }
    cudaEvent_t copied = pipeEvent(ev++);
    cudaCheck(cudaEventRecord(copied, copyStream_), "event record");
    cudaCheck(cudaStreamWaitEvent(stream, copied, 0), "stream wait");   // later work may overwrite the state
    cudaCheck(cudaGetLastError(), "update_host launches");
}

template <typename real>
void Solver<real>::finalizeDt(bool fixed) {
    launch("finalize_dt", 1, [&] {
        launchFinalizeDt<real>(ph, rc.cfg.integrator, fixed ? 1 : 0, rc.cfg.fixed_dt, dtAcc.as<unsigned long long>(),
                               accInit(), sc(), health, stream);
    });
}

template <typename real>
void Solver<real>::update() {                                // Solver::update (Solver.cpp:521-546)
    this->launches_ = 0;
    boundary();
    initStep();
    if (rc.cfg.use_fixed_dt) finalizeDt(true);
    else {
        calcTimestep();
        finalizeDt(false);
    }
    step();
    checkState();
}

template <typename real>
void Solver<real>::checkState() {
    if (!this->stateChecks) return;
    launch("state_check", 1, [&] {
        launchStateCheck<real>(rc.grid, state.as<real>(), livePotential(), health, stream);
    });
}

template <typename real>
void Solver<real>::applyPotential() {
    if (potentialLive_) integrator->integrateGravity();
    else integrator->integrateZeroDeriv();
}

template <typename real>
void FiniteVolumeSolver<real>::initBuffers() {               // FiniteVolumeSolver.cpp:10-15
    Solver<real>::initBuffers();
    this->flux = DeviceBuffer(sizeof(real) * (size_t)this->rc.grid.V * this->rc.numStates * this->rc.dim, true);
}

template <typename real>
void Roe<real>::initBuffers() {                              // Roe.cpp:11-16 (compact basis record)
    FiniteVolumeSolver<real>::initBuffers();
    const auto& rc = this->rc;
    basis = DeviceBuffer(sizeof(real) * (size_t)rc.grid.V * rc.dim * roeRecordSize(rc.dim), true);
    deltaQTilde = DeviceBuffer(sizeof(real) * (size_t)rc.grid.V * rc.dim * rc.numStates, true);
}

template <typename real>
void Roe<real>::initFlux() {                                 // Roe::initFlux (Roe.cpp:82-86)
    this->launch("roe_eigenbasis", 1, [&] {
        launchRoeBasis<real>(this->rc.grid, this->ph, this->state.template as<real>(), basis.template as<real>(),
                             this->rc.cfg.compat == HGPU_COMPAT_SEAM, this->stream, this->livePotential());
    });
}

template <typename real>
void Roe<real>::cflReduce() {
    this->launch("cfl_min_reduce", 1, [&] {
        launchRoeDt<real>(this->rc.grid, this->ph, basis.template as<real>(),
                          this->dtAcc.template as<unsigned long long>(), this->health, this->stream);
    });
}

template <typename real>
void Roe<real>::calcTimestep() {                             // Roe::calcTimestep (Roe.cpp:88-92)
    initFlux();
    cflReduce();
}

// the eigenbasis of the faces of the band's cells (it reads the band's planes and the
// plane below the band)
template <typename real>
void Roe<real>::bandedPrologueWork(int tile0, int tiles, cudaStream_t st) {
    this->launch("roe_eigenbasis", 1, [&] {
        launchRoeBasis<real>(this->rc.grid, this->ph, this->state.template as<real>(), basis.template as<real>(),
                             this->rc.cfg.compat == HGPU_COMPAT_SEAM, st, nullptr, tile0, tiles);
    });
}

template <typename real>
void Roe<real>::calcFlux(real* stage) {                      // Roe::calcDeriv (Roe.cpp:101-112)
    bool seam = this->rc.cfg.compat == HGPU_COMPAT_SEAM;
    if (seam && stage != this->state.template as<real>()) this->boundaryOn(stage);
    this->launch("roe_delta_q_tilde", 1, [&] {
        launchRoeDeltaQ<real>(this->rc.grid, stage, basis.template as<real>(), deltaQTilde.template as<real>(), seam,
                              this->stream);
    });
    // FP64: per-wave corrections, then the transforms (two kernels, roe.cu)
    this->launch("roe_flux", sizeof(real) == 8 ? 2 : 1, [&] {
        launchRoeFlux<real>(this->rc.grid, this->rc.cfg.limiter, stage, basis.template as<real>(),
                            deltaQTilde.template as<real>(), this->sc(), this->flux.template as<real>(), seam,
                            this->stream);
    });
}

// calcFlux in two parts: the ghost refresh (SEAM) and Delta-q-tilde of the whole grid,
// then the flux of the faces of slow-axis planes [from, to) on stream st
template <typename real>
void Roe<real>::fluxPrepare(real* stage) {
    const bool seam = this->rc.cfg.compat == HGPU_COMPAT_SEAM;
    if (seam && stage != this->state.template as<real>()) this->boundaryOn(stage);
    this->launch("roe_delta_q_tilde", 1, [&] {
        launchRoeDeltaQ<real>(this->rc.grid, stage, basis.template as<real>(), deltaQTilde.template as<real>(), seam,
                              this->stream);
    });
}

template <typename real>
void Roe<real>::fluxPlanes(real* stage, long long from, long long to, cudaStream_t st) {
    const Grid& g = this->rc.grid;
    const long long plane = (long long)g.V / g.S[this->rc.dim - 1];
    if (to <= from) return;
    this->launch("roe_flux", sizeof(real) == 8 ? 2 : 1, [&] {
        launchRoeFlux<real>(g, this->rc.cfg.limiter, stage, basis.template as<real>(), deltaQTilde.template as<real>(),
                            this->sc(), this->flux.template as<real>(), this->rc.cfg.compat == HGPU_COMPAT_SEAM, st,
                            from * plane, to * plane);
    });
}

template <typename real>
void Roe<real>::step() {                                     // Roe::step (Roe.cpp:94-99)
    if (fused_) {
        this->integrator->integrateFused([this](real* stage, const CombinePlan<real>& plan) { fusedStage(stage, plan); });
        return;
    }
    this->integrator->integrate([this](real* stage) { calcFlux(stage); });
}

// The fused form of Roe::calcDeriv + the integrator's combine for one stage (2D FP64;
// kernels/roe_fused.cu): x pass, then y pass with the divergence and the combine.  The
// flux buffer holds the x part of the divergence between them.
template <typename real>
void Roe<real>::fusedStage(real* stage, const CombinePlan<real>& plan) {
    if constexpr (std::is_same<real, double>::value) {
        const bool seam = this->rc.cfg.compat == HGPU_COMPAT_SEAM;
        if (seam && stage != this->state.template as<real>()) this->boundaryOn(stage);
        const void* tm = tensorMapFor(stage);
        this->launch("roe_stage_fused", 2, [&] {
            launchRoeStageFused(this->rc.grid, this->ph, this->rc.cfg.limiter, this->sc(), stage,
                                basis.template as<double>(), this->flux.template as<double>(), plan, seam, tm,
                                this->health, this->stream);
        });
    } else {
        (void)stage;
        (void)plan;
        throw ConfigError(HGPU_ERR_UNSUPPORTED, "fused stages are FP64 only");
    }
}

template <typename real>
const void* Roe<real>::tensorMapFor(const real* stage) {
    auto it = tensorMaps_.find(stage);
    if (it != tensorMaps_.end()) return it->second.bytes;
    TensorMap m{};
    std::string err;
    if (roeFusedTensorMapSize() > sizeof m.bytes ||
        !makeRoeFusedTensorMap(this->rc.grid, reinterpret_cast<const double*>(stage), m.bytes, err))
        throw ConfigError(HGPU_ERR_CUDA, "fused stage tensor map: " + err);
    return tensorMaps_.emplace(stage, m).first->second.bytes;
}

template <typename real>
int Roe<real>::setFusedStages(bool on) {
    if (!on) {
        fused_ = false;
        return HGPU_OK;
    }
    if (sizeof(real) != 8 || this->rc.dim != 2 || this->integrator->order() < 2) return HGPU_ERR_UNSUPPORTED;
    roeFusedPrepare();
    fused_ = true;
    return HGPU_OK;
}

template <typename real>
void EulerRoe<real>::step() {                                // EulerRoe::step (EulerRoe.cpp:31-34)
    Roe<real>::step();
    this->applyPotential();
}

template <typename real>
void HLL<real>::initBuffers() {                              // HLL.cpp:7-11 (sl, sr per face)
    FiniteVolumeSolver<real>::initBuffers();
    waves = DeviceBuffer(sizeof(real) * (size_t)this->rc.grid.V * this->rc.dim * 2, true);
}

template <typename real>
void HLL<real>::initStep() {                                 // HLL::initStep (HLL.cpp:31-33)
    this->launch("hllc_wave_speeds", 1, [&] {
        launchHllcWaves<real>(this->rc.grid, this->ph, this->state.template as<real>(), waves.template as<real>(),
                              this->rc.cfg.solver == HGPU_SOLVER_HLL, this->stream, this->livePotential());
    });
}

// the wave speeds of the faces of the band's cells (they read the band's planes and
// the plane below the band)
template <typename real>
void HLL<real>::bandedPrologueWork(int tile0, int tiles, cudaStream_t st) {
    const Grid& g = this->rc.grid;
    const int T_A = this->slowTile();
    const long long S_A = g.S[this->rc.dim - 1], plane = (long long)g.V / S_A;
    const long long p0 = (long long)tile0 * T_A, p1 = std::min<long long>((long long)(tile0 + tiles) * T_A, S_A);
    this->launch("hllc_wave_speeds", 1, [&] {
        launchHllcWaves<real>(g, this->ph, this->state.template as<real>(), waves.template as<real>(),
                              this->rc.cfg.solver == HGPU_SOLVER_HLL, st, nullptr, p0 * plane, p1 * plane);
    });
}

template <typename real>
void HLL<real>::calcTimestep() {                             // HLL::calcTimestep (HLL.cpp:35-38)
    this->launch("cfl_min_reduce", 1, [&] {
        launchHllcDt<real>(this->rc.grid, this->ph, waves.template as<real>(),
                           this->dtAcc.template as<unsigned long long>(), this->health, this->stream);
    });
}

template <typename real>
void HLL<real>::step() {                                     // HLL::step (HLL.cpp:40-47)
    this->integrator->integrate([this](real* stage) {
        // SEAM: the stage's ghosts are refreshed, so both periodic seam faces see the same cells
        if (this->rc.cfg.compat == HGPU_COMPAT_SEAM && stage != this->state.template as<real>()) this->boundaryOn(stage);
        this->launch("hllc_flux", 1, [&] {
            launchHllcFlux<real>(this->rc.grid, this->ph, stage, waves.template as<real>(),
                                 this->flux.template as<real>(), this->health, this->rc.cfg.solver == HGPU_SOLVER_HLL,
                                 this->stream, this->livePotential());
        });
    });
}

// calcFlux in two parts: the ghost refresh (SEAM), then the flux of the faces of
// slow-axis planes [from, to) on stream st (each reads the stage's planes q-1, q and the
// wave speeds of plane q)
template <typename real>
void HLL<real>::fluxPrepare(real* stage) {
    if (this->rc.cfg.compat == HGPU_COMPAT_SEAM && stage != this->state.template as<real>()) this->boundaryOn(stage);
}

template <typename real>
void HLL<real>::fluxPlanes(real* stage, long long from, long long to, cudaStream_t st) {
    const Grid& g = this->rc.grid;
    const long long plane = (long long)g.V / g.S[this->rc.dim - 1];
    if (to <= from) return;
    this->launch("hllc_flux", 1, [&] {
        launchHllcFlux<real>(g, this->ph, stage, waves.template as<real>(), this->flux.template as<real>(),
                             this->health, this->rc.cfg.solver == HGPU_SOLVER_HLL, st, this->livePotential(),
                             from * plane, to * plane);
    });
}

template <typename real>
void EulerHLL<real>::step() {                                // EulerHLL::step (EulerHLL.cpp:25-28)
    HLL<real>::step();
    this->applyPotential();
}

template <typename real>
static std::unique_ptr<SolverBase> makeSolver(const ResolvedConfig& rc) {
    std::unique_ptr<SolverBase> s;
    if (rc.cfg.solver == HGPU_SOLVER_ROE) s.reset(new EulerRoe<real>(rc));
    else if (rc.cfg.solver == HGPU_SOLVER_HLL) s.reset(new EulerHLL<real>(rc));
    else s.reset(new EulerHLLC<real>(rc));
    s->init();
    return s;
}

std::unique_ptr<SolverBase> createSolver(const hgpu_config& cfg) {
    ResolvedConfig rc = resolveConfig(cfg);
    if (cfg.precision == HGPU_FP32) return makeSolver<float>(rc);
    return makeSolver<double>(rc);
}

template StagePlans<double> buildStagePlans<double>(int);
template StagePlans<float> buildStagePlans<float>(int);
template class Solver<double>;
template class Solver<float>;
template class ForwardEuler<double>;
template class ForwardEuler<float>;
template class RungeKutta<double>;
template class RungeKutta<float>;

}  // namespace hgpu
