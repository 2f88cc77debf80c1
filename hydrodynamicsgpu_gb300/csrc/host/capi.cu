// capi.cu -- the extern "C" boundary declared in include/hgpu/hgpu.h.
// No C++ exception crosses it: every entry point maps failures to an hgpu_status
// and keeps a per-thread message for hgpu_last_error().
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "adjoint.h"
#include "batch_solver.h"
#include "fits.h"
#include "solver.h"

namespace hgpu {
double measureFp64FmaRate();
int selftestFp64Ops(unsigned long long seed, long long cases, long long* mulBad, long long* divBad);
int selftestLimiters(unsigned long long seed, long long cases, long long* bad);
void setLastError(const std::string& msg);
}

struct hgpu_solver {
    std::unique_ptr<hgpu::SolverBase> s;
    bool graphs = true;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    int kernelsPerStep = 0;
    std::unique_ptr<hgpu::RoeAdjoint> adjoint;   // created on first use
    std::vector<hgpu_checkpoint*> checkpoints;   // live trajectories of this solver
    hgpu::DeviceBuffer display;                   // one float per cell, created on first use
    int healthMode = HGPU_HEALTH_RECORD;
};

struct hgpu_checkpoint {
    hgpu_solver* h;
    std::unique_ptr<hgpu::Checkpoints> c;
};

namespace {
thread_local std::string g_lastError;

int fail(int status, const std::string& msg) {
    g_lastError = msg;
    return status;
}

template <class F>
int guarded(F f) {
    try {
        return f();
    } catch (const hgpu::ConfigError& e) {
        return fail(e.status, e.what());
    } catch (const hgpu::CudaError& e) {
        return fail(e.code == cudaErrorMemoryAllocation ? HGPU_ERR_NOMEM : HGPU_ERR_CUDA, e.what());
    } catch (const std::bad_alloc&) {
        return fail(HGPU_ERR_NOMEM, "host allocation failed");
    } catch (const std::exception& e) {
        return fail(HGPU_ERR_CUDA, e.what());
    }
}

void runSteps(hgpu_solver* h, int nsteps);

// Strict health mode: wait for the solver's stream, then map the health word's bits
// (left set) to a status.
int healthStatus(hgpu_solver* h) {
    if (h->healthMode != HGPU_HEALTH_STRICT) return HGPU_OK;
    hgpu::cudaCheck(cudaStreamSynchronize(h->s->stream), "synchronize");
    unsigned f = 0;
    hgpu::cudaCheck(cudaMemcpy(&f, h->s->health, sizeof f, cudaMemcpyDeviceToHost), "health read");
    if (f & hgpu::HEALTH_COPY_TIMEOUT)
        return fail(HGPU_ERR_TIMEOUT, "health " + std::to_string(f) + ": a bounded wait for a bulk copy gave up");
    if (f & (hgpu::HEALTH_NONFINITE_DT | hgpu::HEALTH_STATE_NONFINITE))
        return fail(HGPU_ERR_NONFINITE, "health " + std::to_string(f) + ": a non-finite value in the state or the CFL reduction");
    if (f & (hgpu::HEALTH_STATE_DENSITY | hgpu::HEALTH_STATE_PRESSURE))
        return fail(HGPU_ERR_UNPHYSICAL, "health " + std::to_string(f) + ": density or pressure <= 0 in the state");
    return HGPU_OK;
}

void destroyGraph(hgpu_solver* h) {
    if (h->exec) cudaGraphExecDestroy(h->exec);
    if (h->graph) cudaGraphDestroy(h->graph);
    h->exec = nullptr;
    h->graph = nullptr;
}

void captureStep(hgpu_solver* h) {
    cudaStream_t st = h->s->stream;
    hgpu::cudaCheck(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "begin capture");
    try {
        h->s->update();
    } catch (...) {
        cudaGraph_t g = nullptr;
        cudaStreamEndCapture(st, &g);
        if (g) cudaGraphDestroy(g);
        throw;
    }
    hgpu::cudaCheck(cudaStreamEndCapture(st, &h->graph), "end capture");
    hgpu::cudaCheck(cudaGraphInstantiate(&h->exec, h->graph, 0), "graph instantiate");
    h->kernelsPerStep = h->s->kernelsPerStep();
}
void runSteps(hgpu_solver* h, int nsteps) {
    for (int i = 0; i < nsteps; ++i) {
        if (h->graphs) {
            if (!h->exec) captureStep(h);
            hgpu::cudaCheck(cudaGraphLaunch(h->exec, h->s->stream), "graph launch");
        } else {
            h->s->update();
            h->kernelsPerStep = h->s->kernelsPerStep();
            hgpu::cudaCheck(cudaGetLastError(), "kernel launch");
        }
    }
}
}  // namespace

void hgpu::setLastError(const std::string& msg) { g_lastError = msg; }

extern "C" {

const char* hgpu_last_error(void) { return g_lastError.c_str(); }

const char* hgpu_status_string(int status) {
    switch (status) {
    case HGPU_OK: return "HGPU_OK";
    case HGPU_ERR_CONFIG: return "HGPU_ERR_CONFIG";
    case HGPU_ERR_CUDA: return "HGPU_ERR_CUDA";
    case HGPU_ERR_NONFINITE: return "HGPU_ERR_NONFINITE";
    case HGPU_ERR_TIMEOUT: return "HGPU_ERR_TIMEOUT";
    case HGPU_ERR_OOB: return "HGPU_ERR_OOB";
    case HGPU_ERR_ARG: return "HGPU_ERR_ARG";
    case HGPU_ERR_UNSUPPORTED: return "HGPU_ERR_UNSUPPORTED";
    case HGPU_ERR_NOMEM: return "HGPU_ERR_NOMEM";
    case HGPU_ERR_UNPHYSICAL: return "HGPU_ERR_UNPHYSICAL";
    }
    return "HGPU_ERR_UNKNOWN";
}

int hgpu_config_default(hgpu_config* cfg) {
    if (!cfg) return fail(HGPU_ERR_ARG, "null config");
    std::memset(cfg, 0, sizeof *cfg);
    cfg->solver = HGPU_SOLVER_ROE;
    cfg->dim = 0;
    cfg->size[0] = 256; cfg->size[1] = 256; cfg->size[2] = 1;
    for (int i = 0; i < 3; ++i) { cfg->xmin[i] = -.5; cfg->xmax[i] = .5; }
    cfg->gamma = 1.4;
    cfg->cfl = .5f;
    cfg->use_fixed_dt = 0;
    cfg->fixed_dt = .001;
    for (int i = 0; i < 3; ++i) { cfg->boundary[i][0] = HGPU_BOUNDARY_FREEFLOW; cfg->boundary[i][1] = HGPU_BOUNDARY_FREEFLOW; }
    cfg->limiter = HGPU_LIMITER_SUPERBEE;
    cfg->integrator = HGPU_INTEGRATOR_FORWARD_EULER;
    cfg->precision = HGPU_FP64;
    cfg->compat = HGPU_COMPAT_REF;
    cfg->use_gravity = 0;                      // config.lua:65
    cfg->gauss_seidel_max_iter = 20;           // config.lua:68
    cfg->gravitational_constant = 1.;          // config.lua:74
    return HGPU_OK;
}

int hgpu_create(const hgpu_config* cfg, hgpu_solver** out) {
    if (!cfg || !out) return fail(HGPU_ERR_ARG, "null argument");
    *out = nullptr;
    return guarded([&]() {
        std::unique_ptr<hgpu_solver> h(new hgpu_solver());
        h->s = hgpu::createSolver(*cfg);
        *out = h.release();
        return (int)HGPU_OK;
    });
}

int hgpu_destroy(hgpu_solver* h) {
    if (!h) return HGPU_OK;
    return guarded([&]() {
        if (h->s && h->s->stream) cudaStreamSynchronize(h->s->stream);
        for (hgpu_checkpoint* c : h->checkpoints) {   // they keep pointers into this solver
            c->c.reset();
            c->h = nullptr;
        }
        destroyGraph(h);
        if (h->t0) cudaEventDestroy(h->t0);
        if (h->t1) cudaEventDestroy(h->t1);
        delete h;
        return (int)HGPU_OK;
    });
}

int hgpu_get_shape(const hgpu_solver* h, int* dim, int* num_states, size_t* volume) {
    if (!h) return fail(HGPU_ERR_ARG, "null handle");
    if (dim) *dim = h->s->dim();
    if (num_states) *num_states = h->s->numStates();
    if (volume) *volume = h->s->volume();
    return HGPU_OK;
}

int hgpu_set_state(hgpu_solver* h, const void* host_state, size_t count) {
    return hgpu_set_state_potential(h, host_state, count, nullptr, 0);
}

int hgpu_set_state_potential(hgpu_solver* h, const void* host_state, size_t count, const void* host_potential,
                             size_t potential_count) {
    if (!h || !host_state) return fail(HGPU_ERR_ARG, "null argument");
    if (host_potential && potential_count != h->s->volume())
        return fail(HGPU_ERR_ARG, "potential element count mismatch");
    return guarded([&]() {
        const bool wasLive = h->s->potentialLive();
        h->s->resetState(host_state, count, host_potential);
        if (h->s->potentialLive() != wasLive) destroyGraph(h);   // the step's kernels differ
        return healthStatus(h);
    });
}

int hgpu_get_potential(hgpu_solver* h, void* host_potential, size_t count) {
    if (!h || !host_potential) return fail(HGPU_ERR_ARG, "null argument");
    return guarded([&]() { h->s->readPotential(host_potential, count); return (int)HGPU_OK; });
}

int hgpu_get_state(hgpu_solver* h, void* host_state, size_t count) {
    if (!h || !host_state) return fail(HGPU_ERR_ARG, "null argument");
    return guarded([&]() { h->s->readState(host_state, count); return (int)HGPU_OK; });
}

int hgpu_update(hgpu_solver* h, int nsteps, double* last_dt) {
    if (!h || nsteps < 0) return fail(HGPU_ERR_ARG, "bad argument");
    return guarded([&]() {
        runSteps(h, nsteps);
        if (last_dt) *last_dt = h->s->lastDt();
        return healthStatus(h);
    });
}

int hgpu_step(hgpu_solver* h, int nsteps, double* last_dt) { return hgpu_update(h, nsteps, last_dt); }

int hgpu_update_host(hgpu_solver* h, const void* host_in, size_t in_count, int nsteps, void* host_out,
                     size_t out_count, double* last_dt) {
    if (!h || !host_in || !host_out || nsteps < 1) return fail(HGPU_ERR_ARG, "bad argument");
    const size_t n = h->s->volume() * (size_t)h->s->numStates();
    if (in_count != n || out_count != n) return fail(HGPU_ERR_ARG, "state element count mismatch");
    return guarded([&]() {
        const bool wasLive = h->s->potentialLive();
        if (!h->s->hostPipelined()) {
            h->s->resetState(host_in, in_count, nullptr);
            if (h->s->potentialLive() != wasLive) destroyGraph(h);
            runSteps(h, nsteps);
            h->s->readState(host_out, out_count);
        } else {
            h->s->hostStep(host_in, host_out, true, nsteps == 1);
            if (h->s->potentialLive() != wasLive) destroyGraph(h);   // the step's kernels differ
            if (nsteps > 1) {
                runSteps(h, nsteps - 2);
                h->s->hostStep(nullptr, host_out, false, true);
            }
        }
        const double dt = h->s->lastDt();   // waits for the stream, which waited for the copies
        if (last_dt) *last_dt = dt;
        return healthStatus(h);
    });
}

int hgpu_last_dt(hgpu_solver* h, double* dt) {
    if (!h || !dt) return fail(HGPU_ERR_ARG, "null argument");
    return guarded([&]() { *dt = h->s->lastDt(); return (int)HGPU_OK; });
}

int hgpu_synchronize(hgpu_solver* h) {
    if (!h) return fail(HGPU_ERR_ARG, "null handle");
    return guarded([&]() {
        hgpu::cudaCheck(cudaStreamSynchronize(h->s->stream), "synchronize");
        unsigned flags = 0;
        hgpu::cudaCheck(cudaMemcpy(&flags, h->s->health, sizeof flags, cudaMemcpyDeviceToHost), "health read");
        if (flags & hgpu::HEALTH_COPY_TIMEOUT) return fail(HGPU_ERR_TIMEOUT, "a bounded wait for a bulk copy gave up");
        if (flags & hgpu::HEALTH_NONFINITE_DT) return fail(HGPU_ERR_NONFINITE, "non-finite value in the CFL reduction");
        return (int)HGPU_OK;
    });
}

int hgpu_health(hgpu_solver* h, uint32_t* flags) {
    if (!h || !flags) return fail(HGPU_ERR_ARG, "null argument");
    return guarded([&]() {
        unsigned f = 0;
        hgpu::cudaCheck(cudaStreamSynchronize(h->s->stream), "synchronize");
        hgpu::cudaCheck(cudaMemcpy(&f, h->s->health, sizeof f, cudaMemcpyDeviceToHost), "health read");
        hgpu::cudaCheck(cudaMemset(h->s->health, 0, sizeof f), "health clear");
        *flags = f;
        return (int)HGPU_OK;
    });
}

int hgpu_set_health_mode(hgpu_solver* h, int mode) {
    if (!h) return fail(HGPU_ERR_ARG, "null handle");
    if (mode < HGPU_HEALTH_OFF || mode > HGPU_HEALTH_STRICT) return fail(HGPU_ERR_ARG, "unknown health mode");
    return guarded([&]() {
        const int checks = mode == HGPU_HEALTH_OFF ? 0 : 1;
        if (checks != h->s->stateChecks) destroyGraph(h);   // the step's kernels differ
        h->s->stateChecks = checks;
        h->healthMode = mode;
        return (int)HGPU_OK;
    });
}

int hgpu_checked_status(uint32_t* flags) {
    if (!flags) return fail(HGPU_ERR_ARG, "null argument");
    return guarded([&]() {
        std::string where;
        *flags = hgpu::takeChecks(where);
        if (*flags) hgpu::setLastError(where);
        return (int)HGPU_OK;
    });
}

int hgpu_set_fused_stages(hgpu_solver* h, int enabled) {
    if (!h) return fail(HGPU_ERR_ARG, "null handle");
    return guarded([&]() {
        const int st = h->s->setFusedStages(enabled != 0);
        if (st != HGPU_OK) return fail(st, "fused stages: 2D FP64 EulerRoe with a Runge-Kutta integrator only");
        destroyGraph(h);                                     // the step's kernels differ
        return (int)HGPU_OK;
    });
}

int hgpu_state_device_ptr(hgpu_solver* h, void** dptr) {
    if (!h || !dptr) return fail(HGPU_ERR_ARG, "null argument");
    *dptr = h->s->stateDevicePtr();
    return HGPU_OK;
}

int hgpu_stream(hgpu_solver* h, void** stream) {
    if (!h || !stream) return fail(HGPU_ERR_ARG, "null argument");
    *stream = (void*)h->s->stream;
    return HGPU_OK;
}

int hgpu_set_graphs(hgpu_solver* h, int enabled) {
    if (!h) return fail(HGPU_ERR_ARG, "null handle");
    return guarded([&]() {
        h->graphs = enabled != 0;
        if (!h->graphs) destroyGraph(h);
        return (int)HGPU_OK;
    });
}

int hgpu_kernels_per_step(const hgpu_solver* h, int* count) {
    if (!h || !count) return fail(HGPU_ERR_ARG, "null argument");
    *count = h->kernelsPerStep;
    return HGPU_OK;
}

int hgpu_select_device(int device) {
    return guarded([&]() {
        hgpu::cudaCheck(cudaSetDevice(device), "cudaSetDevice");
        return (int)HGPU_OK;
    });
}

int hgpu_timed_update(hgpu_solver* h, int nsteps, float* ms) {
    if (!h || !ms || nsteps < 0) return fail(HGPU_ERR_ARG, "bad argument");
    return guarded([&]() {
        if (!h->t0) {
            hgpu::cudaCheck(cudaEventCreate(&h->t0), "event create");
            hgpu::cudaCheck(cudaEventCreate(&h->t1), "event create");
        }
        if (h->graphs && !h->exec) captureStep(h);
        hgpu::cudaCheck(cudaEventRecord(h->t0, h->s->stream), "event record");
        runSteps(h, nsteps);
        hgpu::cudaCheck(cudaEventRecord(h->t1, h->s->stream), "event record");
        hgpu::cudaCheck(cudaEventSynchronize(h->t1), "event sync");
        hgpu::cudaCheck(cudaEventElapsedTime(ms, h->t0, h->t1), "elapsed");
        return (int)HGPU_OK;
    });
}

int hgpu_profile_update(hgpu_solver* h, int nsteps, hgpu_kernel_time* out, int cap, int* count) {
    if (!h || nsteps < 0 || (cap > 0 && !out)) return fail(HGPU_ERR_ARG, "bad argument");
    return guarded([&]() {
        hgpu::SolverBase* s = h->s.get();
        s->records.clear();
        s->eventNext = 0;
        s->profiling = true;
        try {
            for (int i = 0; i < nsteps; ++i) s->update();
        } catch (...) {
            s->profiling = false;
            throw;
        }
        s->profiling = false;
        hgpu::cudaCheck(cudaStreamSynchronize(s->stream), "profile sync");
        std::vector<hgpu_kernel_time> agg;
        for (const auto& r : s->records) {
            float ms = 0;
            hgpu::cudaCheck(cudaEventElapsedTime(&ms, r.start, r.stop), "elapsed");
            size_t k = 0;
            for (; k < agg.size(); ++k)
                if (!std::strncmp(agg[k].name, r.kind, sizeof agg[k].name)) break;
            if (k == agg.size()) {
                hgpu_kernel_time t{};
                std::strncpy(t.name, r.kind, sizeof t.name - 1);
                agg.push_back(t);
            }
            agg[k].launches += 1;
            agg[k].total_ms += ms;
        }
        int n = (int)agg.size();
        for (int i = 0; i < n && i < cap; ++i) out[i] = agg[i];
        if (count) *count = n;
        return (int)HGPU_OK;
    });
}

int hgpu_host_alloc(size_t bytes, void** ptr) {
    if (!ptr) return fail(HGPU_ERR_ARG, "null argument");
    return guarded([&]() {
        hgpu::cudaCheck(cudaHostAlloc(ptr, bytes, cudaHostAllocPortable), "cudaHostAlloc");
        return (int)HGPU_OK;
    });
}

int hgpu_host_free(void* ptr) {
    return guarded([&]() {
        if (ptr) hgpu::cudaCheck(cudaFreeHost(ptr), "cudaFreeHost");
        return (int)HGPU_OK;
    });
}

namespace {
hgpu::RoeAdjoint& adjointOf(hgpu_solver* h) {
    if (h->s->potentialLive())
        throw hgpu::ConfigError(HGPU_ERR_UNSUPPORTED, "the adjoint covers a zero gravitational potential");
    if (!h->adjoint) {
        auto* s = dynamic_cast<hgpu::Solver<double>*>(h->s.get());
        if (!s) throw hgpu::ConfigError(HGPU_ERR_UNSUPPORTED, "the adjoint covers EulerRoe in FP64");
        h->adjoint.reset(new hgpu::RoeAdjoint(s->rc, s->stream));
    }
    return *h->adjoint;
}
}  // namespace

int hgpu_update_frozen_dt(hgpu_solver* h, int nsteps, const double* dts) {
    if (!h || nsteps < 0 || (nsteps > 0 && !dts)) return fail(HGPU_ERR_ARG, "bad argument");
    return guarded([&]() {
        hgpu::RoeAdjoint& a = adjointOf(h);
        double* st = static_cast<double*>(h->s->stateDevicePtr());
        for (int i = 0; i < nsteps; ++i) a.advance(st, dts[i]);
        return (int)HGPU_OK;
    });
}

int hgpu_adjoint_step(hgpu_solver* h, const void* d_u_n, const void* d_lambda_next, void* d_lambda_n, double dt) {
    if (!h || !d_u_n || !d_lambda_next || !d_lambda_n) return fail(HGPU_ERR_ARG, "null argument");
    return guarded([&]() {
        adjointOf(h).step(static_cast<const double*>(d_u_n), static_cast<const double*>(d_lambda_next),
                          static_cast<double*>(d_lambda_n), dt);
        return (int)HGPU_OK;
    });
}

static int createCheckpoints(hgpu_solver* h, int nsteps, int every, bool taped, hgpu_checkpoint** out) {
    if (!h || !out || nsteps < 1 || every < 1) return fail(HGPU_ERR_ARG, "bad argument");
    *out = nullptr;
    return guarded([&]() {
        hgpu::RoeAdjoint& a = adjointOf(h);
        auto* s = dynamic_cast<hgpu::Solver<double>*>(h->s.get());
        std::unique_ptr<hgpu_checkpoint> c(new hgpu_checkpoint());
        c->h = h;
        c->c.reset(new hgpu::Checkpoints(&a, s->state.as<double>(), s->stream, nsteps, every,
                                         [h]() { runSteps(h, 1); }, &s->sc()->dt_f64, taped));
        h->checkpoints.push_back(c.get());
        *out = c.release();
        return (int)HGPU_OK;
    });
}

int hgpu_checkpoint_create(hgpu_solver* h, int nsteps, int every, hgpu_checkpoint** out) {
    return createCheckpoints(h, nsteps, every, false, out);
}

int hgpu_checkpoint_create_taped(hgpu_solver* h, int nsteps, hgpu_checkpoint** out) {
    return createCheckpoints(h, nsteps, nsteps, true, out);
}

int hgpu_checkpoint_forward(hgpu_checkpoint* c, const double* dts) {
    if (!c) return fail(HGPU_ERR_ARG, "null handle");
    if (!c->c) return fail(HGPU_ERR_ARG, "the solver of this checkpoint was destroyed");
    return guarded([&]() { c->c->forward(dts); return (int)HGPU_OK; });
}

int hgpu_checkpoint_dts(hgpu_checkpoint* c, double* dts, int n) {
    if (!c || !dts) return fail(HGPU_ERR_ARG, "null argument");
    if (!c->c) return fail(HGPU_ERR_ARG, "the solver of this checkpoint was destroyed");
    if (n != (int)c->c->dts.size()) return fail(HGPU_ERR_ARG, "dt array size mismatch");
    std::copy(c->c->dts.begin(), c->c->dts.end(), dts);
    return HGPU_OK;
}

int hgpu_checkpoint_backward(hgpu_checkpoint* c, const void* d_lambda_T, void* d_lambda_0) {
    if (!c || !d_lambda_T || !d_lambda_0) return fail(HGPU_ERR_ARG, "null argument");
    if (!c->c) return fail(HGPU_ERR_ARG, "the solver of this checkpoint was destroyed");
    return guarded([&]() {
        c->c->backward(static_cast<const double*>(d_lambda_T), static_cast<double*>(d_lambda_0));
        return (int)HGPU_OK;
    });
}

int hgpu_checkpoint_times(hgpu_checkpoint* c, float* forward_ms, float* backward_ms) {
    if (!c) return fail(HGPU_ERR_ARG, "null handle");
    if (!c->c) return fail(HGPU_ERR_ARG, "the solver of this checkpoint was destroyed");
    if (forward_ms) *forward_ms = c->c->forwardMs;
    if (backward_ms) *backward_ms = c->c->backwardMs;
    return HGPU_OK;
}

int hgpu_checkpoint_destroy(hgpu_checkpoint* c) {
    if (!c) return HGPU_OK;
    return guarded([&]() {
        if (c->h) {
            cudaStreamSynchronize(c->h->s->stream);
            auto& v = c->h->checkpoints;
            v.erase(std::remove(v.begin(), v.end(), c), v.end());
        }
        delete c;
        return (int)HGPU_OK;
    });
}

struct hgpu_batch {
    std::unique_ptr<hgpu::BatchBase> b;
};

int hgpu_batch_create(const hgpu_config* cfgs, int nproblems, hgpu_batch** out) {
    if (!cfgs || !out || nproblems <= 0) return fail(HGPU_ERR_ARG, "bad argument");
    *out = nullptr;
    for (int p = 0; p < nproblems; ++p)
        if (cfgs[p].use_gravity) return fail(HGPU_ERR_UNSUPPORTED, "batched problems run with a zero potential");
    return guarded([&]() {
        std::unique_ptr<hgpu_batch> h(new hgpu_batch());
        h->b = hgpu::createBatch(std::vector<hgpu_config>(cfgs, cfgs + nproblems));
        *out = h.release();
        return (int)HGPU_OK;
    });
}

int hgpu_batch_destroy(hgpu_batch* b) {
    if (!b) return HGPU_OK;
    return guarded([&]() {
        if (b->b && b->b->stream) cudaStreamSynchronize(b->b->stream);
        delete b;
        return (int)HGPU_OK;
    });
}

int hgpu_batch_info(const hgpu_batch* b, int* nproblems, long long* total_cells, int* kernels_per_step) {
    if (!b) return fail(HGPU_ERR_ARG, "null handle");
    if (nproblems) *nproblems = b->b->problems();
    if (total_cells) *total_cells = b->b->totalCells();
    if (kernels_per_step) *kernels_per_step = b->b->kernelsPerStep();
    return HGPU_OK;
}

int hgpu_batch_set_state(hgpu_batch* b, int problem, const void* host_state, size_t count) {
    if (!b || !host_state) return fail(HGPU_ERR_ARG, "null argument");
    return guarded([&]() { b->b->setState(problem, host_state, count); return (int)HGPU_OK; });
}

int hgpu_batch_get_state(hgpu_batch* b, int problem, void* host_state, size_t count) {
    if (!b || !host_state) return fail(HGPU_ERR_ARG, "null argument");
    return guarded([&]() { b->b->getState(problem, host_state, count); return (int)HGPU_OK; });
}

int hgpu_batch_update(hgpu_batch* b, int nsteps) {
    if (!b || nsteps < 0) return fail(HGPU_ERR_ARG, "bad argument");
    return guarded([&]() { b->b->run(nsteps); return (int)HGPU_OK; });
}

int hgpu_batch_step(hgpu_batch* b, int nsteps) { return hgpu_batch_update(b, nsteps); }

int hgpu_batch_timed_update(hgpu_batch* b, int nsteps, float* ms) {
    if (!b || !ms || nsteps < 0) return fail(HGPU_ERR_ARG, "bad argument");
    return guarded([&]() { *ms = b->b->timedRun(nsteps); return (int)HGPU_OK; });
}

int hgpu_batch_dts(hgpu_batch* b, double* dts, int n) {
    if (!b || !dts) return fail(HGPU_ERR_ARG, "null argument");
    return guarded([&]() { b->b->dts(dts, n); return (int)HGPU_OK; });
}

int hgpu_batch_health(hgpu_batch* b, uint32_t* flags) {
    if (!b || !flags) return fail(HGPU_ERR_ARG, "null argument");
    return guarded([&]() { *flags = b->b->readHealth(); return (int)HGPU_OK; });
}

int hgpu_batch_problem_health(hgpu_batch* b, uint32_t* flags, int n) {
    if (!b || !flags) return fail(HGPU_ERR_ARG, "null argument");
    return guarded([&]() {
        b->b->readProblemHealth(reinterpret_cast<unsigned*>(flags), n);
        return (int)HGPU_OK;
    });
}

int hgpu_batch_get_tuning(const hgpu_batch* b, hgpu_batch_tuning* t) {
    if (!b || !t) return fail(HGPU_ERR_ARG, "null argument");
    hgpu::BatchTuning tu = b->b->tuning();
    *t = {tu.tx, tu.ty, tu.tz, tu.staged, tu.blocksPerSM, tu.split, tu.cpt};
    return HGPU_OK;
}

int hgpu_batch_set_tuning(hgpu_batch* b, const hgpu_batch_tuning* t) {
    if (!b || !t) return fail(HGPU_ERR_ARG, "null argument");
    return guarded([&]() {
        b->b->setTuning({t->tile_x, t->tile_y, t->tile_z, t->staged, t->blocks_per_sm, t->split_flux,
                         t->cells_per_thread});
        return (int)HGPU_OK;
    });
}

int hgpu_batch_autotune(hgpu_batch* b, const char* cache_path, int steps) {
    if (!b || steps <= 0) return fail(HGPU_ERR_ARG, "bad argument");
    return guarded([&]() {
        b->b->autotune(cache_path ? std::string(cache_path) : std::string(), steps);
        return (int)HGPU_OK;
    });
}

extern "C++" {
namespace {
template <typename real>
bool displayAs(hgpu::SolverBase* b, int method, float* d_out) {
    auto* s = dynamic_cast<hgpu::Solver<real>*>(b);
    if (!s) return false;
    hgpu::launchDisplay<real>(s->rc.grid, s->ph.gamma, method, s->state.template as<real>(), d_out, s->stream,
                              s->potential.template as<real>());
    return true;
}

void displayInto(hgpu_solver* h, int method, float* d_out) {
    if (method < 0 || method >= hgpu::displayCount(h->s->dim()))
        throw hgpu::ConfigError(HGPU_ERR_ARG, "display method out of range for this dimension");
    if (!displayAs<double>(h->s.get(), method, d_out)) displayAs<float>(h->s.get(), method, d_out);
    hgpu::cudaCheck(cudaGetLastError(), "display launch");
}
}  // namespace
}  // extern "C++"

int hgpu_display_device(hgpu_solver* h, int method, void* d_out) {
    if (!h || !d_out) return fail(HGPU_ERR_ARG, "null argument");
    return guarded([&]() {
        displayInto(h, method, static_cast<float*>(d_out));
        return (int)HGPU_OK;
    });
}

int hgpu_display(hgpu_solver* h, int method, float* host_out, size_t count) {
    if (!h || !host_out) return fail(HGPU_ERR_ARG, "null argument");
    return guarded([&]() {
        const size_t V = h->s->volume();
        if (count != V) throw hgpu::ConfigError(HGPU_ERR_ARG, "display needs one float per cell");
        if (!h->display.get()) h->display = hgpu::DeviceBuffer(sizeof(float) * V, false);
        displayInto(h, method, h->display.as<float>());
        hgpu::cudaCheck(cudaMemcpyAsync(host_out, h->display.get(), sizeof(float) * V, cudaMemcpyDeviceToHost,
                                        h->s->stream),
                        "display download");
        hgpu::cudaCheck(cudaStreamSynchronize(h->s->stream), "display sync");
        return (int)HGPU_OK;
    });
}

int hgpu_save_fits(hgpu_solver* h, const char* directory, int* save_index) {
    if (!h || !directory) return fail(HGPU_ERR_ARG, "null argument");
    return guarded([&]() {
        const int dim = h->s->dim(), N = h->s->numStates();
        const size_t V = h->s->volume();
        std::vector<std::string> names = {"DENSITY", "MOMENTUM_X"};
        if (dim > 1) names.push_back("MOMENTUM_Y");
        if (dim > 2) names.push_back("MOMENTUM_Z");
        names.push_back("ENERGY_TOTAL");
        names.push_back("potential");                   // SelfGravitationBehavior::getSaveChannelNames
        std::string dir(directory);
        if (!dir.empty() && dir.back() != '/') dir += '/';
        int index = -1;
        for (int i = 0; i < 1000000 && index < 0; ++i)   // Solver::getSaveIndex
            if (!hgpu::fileExists(dir + names[0] + std::to_string(i) + ".fits")) index = i;
        if (index < 0) throw hgpu::ConfigError(HGPU_ERR_ARG, "no free save index");
        const bool f32 = dynamic_cast<hgpu::Solver<float>*>(h->s.get()) != nullptr;
        std::vector<double> d(f32 ? 0 : V * N);
        std::vector<float> f(f32 ? V * N : 0), plane(V);
        std::vector<double> potD(f32 ? 0 : V);
        std::vector<float> potF(f32 ? V : 0);
        if (f32) { h->s->readState(f.data(), V * N); h->s->readPotential(potF.data(), V); }
        else { h->s->readState(d.data(), V * N); h->s->readPotential(potD.data(), V); }
        int S[3] = {1, 1, 1};
        if (auto* s = dynamic_cast<hgpu::Solver<double>*>(h->s.get())) for (int i = 0; i < 3; ++i) S[i] = s->rc.grid.S[i];
        if (auto* s = dynamic_cast<hgpu::Solver<float>*>(h->s.get())) for (int i = 0; i < 3; ++i) S[i] = s->rc.grid.S[i];
        for (int ch = 0; ch < (int)names.size(); ++ch) {
            for (size_t c = 0; c < V; ++c)
                plane[c] = ch < N ? (f32 ? f[c * N + ch] : (float)d[c * N + ch]) : (f32 ? potF[c] : (float)potD[c]);
            hgpu::writeFitsFloat(dir + names[ch] + std::to_string(index) + ".fits", plane.data(), S[0], S[1], S[2]);
        }
        if (save_index) *save_index = index;
        return (int)HGPU_OK;
    });
}

int hgpu_fp64_selftest(unsigned long long seed, long long cases, long long* mul_mismatches,
                       long long* div_mismatches) {
    if (!mul_mismatches || !div_mismatches || cases < 0) return fail(HGPU_ERR_ARG, "bad argument");
    return guarded([&]() {
        if (hgpu::selftestFp64Ops(seed, cases, mul_mismatches, div_mismatches) != 0)
            throw hgpu::CudaError(cudaGetLastError(), "fp64 self-test");
        return (int)HGPU_OK;
    });
}

int hgpu_limiter_selftest(unsigned long long seed, long long cases, long long* mismatches) {
    if (!mismatches || cases < 0) return fail(HGPU_ERR_ARG, "bad argument");
    return guarded([&]() {
        if (hgpu::selftestLimiters(seed, cases, mismatches) != 0)
            throw hgpu::CudaError(cudaGetLastError(), "limiter self-test");
        return (int)HGPU_OK;
    });
}

int hgpu_fp64_peak(double* fma_per_second) {
    if (!fma_per_second) return fail(HGPU_ERR_ARG, "null argument");
    double r = hgpu::measureFp64FmaRate();
    if (r <= 0) return fail(HGPU_ERR_CUDA, "fp64 probe failed");
    *fma_per_second = r;
    return HGPU_OK;
}

}  // extern "C"
