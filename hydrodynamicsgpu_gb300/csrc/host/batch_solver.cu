// batch_solver.cu -- many independent Euler problems advanced together.
//
// The reference runs one problem per process (src/HydroGPUApp.cpp:330-349).  A batch
// holds P problems of the same solver, dimension, integrator, limiter and precision
// but their own grid sizes, domains, gamma, cfl, boundary methods and dt, and runs
// each Solver::update step of all of them as one CUDA graph of persistent,
// queue-driven launches (kernels/batch.cu).  Results per problem are bit-identical to
// the single-problem path.  The tile shape, eigenbasis staging and persistent grid
// size come from an autotuner that times candidates on the batch itself and caches
// the winner per batch shape in a text file.
#include <algorithm>
#include <array>
#include <limits>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../kernels/batch.h"
#include "batch_solver.h"

namespace hgpu {

template <typename real>
BatchSolver<real>::BatchSolver(const std::vector<hgpu_config>& cfgs) {
    if (cfgs.empty()) throw ConfigError(HGPU_ERR_ARG, "empty batch");
    for (const auto& c : cfgs) rcs_.push_back(resolveConfig(c));
    const ResolvedConfig& r0 = rcs_[0];
    for (const auto& r : rcs_) {
        if (r.cfg.solver != r0.cfg.solver || r.dim != r0.dim || r.cfg.integrator != r0.cfg.integrator ||
            r.cfg.limiter != r0.cfg.limiter || r.cfg.precision != r0.cfg.precision ||
            r.cfg.use_fixed_dt != r0.cfg.use_fixed_dt)
            throw ConfigError(HGPU_ERR_CONFIG, "batch problems must share solver, dim, integrator, limiter, precision "
                                               "and use_fixed_dt");
        if (r.cfg.compat != HGPU_COMPAT_REF) throw ConfigError(HGPU_ERR_UNSUPPORTED, "batches run the REF scheme");
    }
    dim_ = r0.dim;
    N_ = r0.numStates;
    hllc_ = r0.cfg.solver != HGPU_SOLVER_ROE;        // the HLL driver: EulerHLLC or EulerHLL
    kind_ = r0.cfg.solver;
    integ_ = r0.cfg.integrator;
    cudaCheck(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "cudaStreamCreate");
    // offsets: each problem's cells start on a multiple of 32
    const int NB = hllc_ ? 2 : roeRecordSize(dim_);
    long long cell = 0, face = 0, dqe = 0;
    for (const auto& r : rcs_) {
        BatchProblem<real> p{};
        p.g = r.grid;
        p.g.check = checkWord();
        for (int i = 0; i < 3; ++i) {
            p.ph.dx[i] = (real)r.dx[i];
            p.ph.rdx[i] = (real)1 / p.ph.dx[i];
        }
        p.ph.gamma = (real)r.gamma;
        p.ph.cfl = r.cfg.cfl;
        for (int i = 0; i < 3; ++i)
            for (int m = 0; m < 2; ++m) p.methods[i][m] = i < dim_ ? r.cfg.boundary[i][m] : -1;
        p.stateOff = cell;
        p.faceOff = face;
        p.dqOff = dqe;
        p.useFixed = r.cfg.use_fixed_dt;
        p.fixedDt = r.cfg.fixed_dt;
        bool maxInit = hllc_ && dim_ > 1;
        real iv = maxInit ? std::numeric_limits<real>::max() : std::numeric_limits<real>::infinity();
        p.accInit = 0;
        std::memcpy(&p.accInit, &iv, sizeof(real));
        host_.push_back(p);
        cell += (r.grid.V + 31) / 32 * 32;
        face += r.grid.V * dim_ * NB;
        dqe += r.grid.V * dim_ * N_;
    }
    totalCells_ = cell;
    state_ = DeviceBuffer(sizeof(real) * cell * N_, true);
    faces_ = DeviceBuffer(sizeof(real) * face, true);
    if (!hllc_) dq_ = DeviceBuffer(sizeof(real) * dqe, true);
    flux_ = DeviceBuffer(sizeof(real) * dqe, true);
    probs_ = DeviceBuffer(sizeof(BatchProblem<real>) * host_.size(), false);
    cudaCheck(cudaMemcpy(probs_.get(), host_.data(), sizeof(BatchProblem<real>) * host_.size(), cudaMemcpyHostToDevice),
              "batch problems upload");
    sc_ = DeviceBuffer(sizeof(StepConst<real>) * host_.size(), true);
    acc_ = DeviceBuffer(sizeof(unsigned long long) * host_.size(), false);
    {
        std::vector<unsigned long long> init(host_.size());
        for (size_t i = 0; i < host_.size(); ++i) init[i] = host_[i].accInit;
        cudaCheck(cudaMemcpy(acc_.get(), init.data(), sizeof(unsigned long long) * init.size(), cudaMemcpyHostToDevice),
                  "dt accumulators");
    }
    health_ = DeviceBuffer(sizeof(unsigned), true);
    healthP_ = DeviceBuffer(sizeof(unsigned) * host_.size(), true);
    queues_ = DeviceBuffer(sizeof(unsigned) * kQueues, true);
    if (integ_ != HGPU_INTEGRATOR_FORWARD_EULER) {
        plans_ = buildStagePlans<real>(integ_);
        for (int i = 0; i < plans_.nslots; ++i) work_.emplace_back(sizeof(real) * cell * N_, true);
        for (auto& pl : plans_.plans) {
            pl.slot[0] = state_.as<real>();
            for (int i = 0; i < plans_.nslots; ++i) pl.slot[1 + i] = work_[i].template as<real>();
        }
        alphaBinary_ = tableauAlphaIsBinary(integ_);
    }
    BatchTuning def{};
    const int split = splitAvailable() ? 1 : 0;
    if (dim_ == 1) def = {256, 1, 1, 1, 0, split, 1};
    else if (dim_ == 2) def = {32, 8, 1, 1, 0, split, 1};
    else def = {32, 4, 2, 1, 0, split, 1};
    setTuning(def);
    cudaCheck(cudaDeviceSynchronize(), "batch init");
}

template <typename real>
BatchSolver<real>::~BatchSolver() {
    dropGraph();
    if (t0_) cudaEventDestroy(t0_);
    if (t1_) cudaEventDestroy(t1_);
    if (stream) cudaStreamDestroy(stream);
}

template <typename real>
void BatchSolver<real>::dropGraph() {
    if (exec_) cudaGraphExecDestroy(exec_);
    if (graph_) cudaGraphDestroy(graph_);
    exec_ = nullptr;
    graph_ = nullptr;
}

template <typename real>
bool BatchSolver<real>::splitAvailable() const {
    return sizeof(real) == 8 && kind_ == HGPU_SOLVER_ROE;
}

template <typename real>
void BatchSolver<real>::setTuning(const BatchTuning& tu) {
    if (tu.cpt < 1 || tu.cpt > 8) throw ConfigError(HGPU_ERR_CONFIG, "cells per thread must be 1 to 8");
    if (tu.blocksPerSM < -1) throw ConfigError(HGPU_ERR_CONFIG, "blocks per SM must be >= -1");
    if (tu.tx < 1 || tu.ty < 1 || tu.tz < 1 || tu.tx * tu.ty * tu.tz > 256 * tu.cpt)
        throw ConfigError(HGPU_ERR_CONFIG, "tile must have between 1 and 256 x (cells per thread) cells");
    if (tu.staged && tu.tx * tu.ty * tu.tz > 256)
        throw ConfigError(HGPU_ERR_CONFIG, "a staged eigenbasis tile has at most 256 cells");
    if (tu.split && !splitAvailable()) throw ConfigError(HGPU_ERR_UNSUPPORTED, "the two-pass flux is FP64 EulerRoe only");
    tuning_ = tu;
    std::vector<BatchTile> tiles;
    for (size_t p = 0; p < host_.size(); ++p) {
        const Grid& g = host_[p].g;
        for (int z0 = 0; z0 < g.S[2]; z0 += tu.tz)
            for (int y0 = 0; y0 < g.S[1]; y0 += tu.ty)
                for (int x0 = 0; x0 < g.S[0]; x0 += tu.tx) tiles.push_back({(int)p, x0, y0, z0});
    }
    nTiles_ = (int)tiles.size();
    tiles_ = DeviceBuffer(sizeof(BatchTile) * tiles.size(), false);
    cudaCheck(cudaMemcpy(tiles_.get(), tiles.data(), sizeof(BatchTile) * tiles.size(), cudaMemcpyHostToDevice),
              "tiles upload");
    dropGraph();
}

template <typename real>
void BatchSolver<real>::update() {                       // Solver::update for every problem
    BatchLaunch<real> L{probs_.as<BatchProblem<real>>(), (int)host_.size(), tiles_.as<BatchTile>(), nTiles_,
                        tuning_, dim_, stream, state_.as<real>(), faces_.as<real>()};
    unsigned* q = queues_.as<unsigned>();
    int qi = 0;
    auto nextQ = [&]() {
        if (qi >= kQueues) throw std::logic_error("out of batch queue counters");
        return q + qi++;
    };
    launches_ = 0;
    cudaCheck(cudaMemsetAsync(q, 0, sizeof(unsigned) * kQueues, stream), "queue reset");
    const bool fixed = rcs_[0].cfg.use_fixed_dt != 0;
    StepConst<real>* sc = sc_.as<StepConst<real>>();
    unsigned long long* acc = acc_.as<unsigned long long>();
    unsigned* health = health_.as<unsigned>();
    L.boundary(nextQ());
    ++launches_;
    if (hllc_) {
        L.waves(kind_ == HGPU_SOLVER_HLL, nextQ());       // HLL::initStep
        ++launches_;
    }
    if (!fixed) {
        if (!hllc_) {
            L.roeBasis(2, 1, nextQ());                    // Roe::initFlux
            ++launches_;
        }
        L.dt(hllc_, acc, health, nextQ());
        ++launches_;
    }
    L.finalize(integ_, acc, sc);
    ++launches_;
    const int lim = rcs_[0].cfg.limiter;
    auto stage = [&](const real* in, const CombinePlan<real>& plan) {
        if (!hllc_) {
            L.deltaQ(2, 1, in, dq_.as<real>(), nextQ());
            ++launches_;
        }
        if (tuning_.split) {
            unsigned* q0 = nextQ();
            L.fluxSplit(lim, sc, in, dq_.as<real>(), flux_.as<real>(), q0, nextQ());
            ++launches_;
        } else {
            L.flux(kind_ == HGPU_SOLVER_ROE ? 0 : (kind_ == HGPU_SOLVER_HLL ? 2 : 1), lim, sc, in,
                   hllc_ ? nullptr : dq_.as<real>(), flux_.as<real>(), health, nextQ());
        }
        L.combine(flux_.as<real>(), plan, sc, nextQ());
        launches_ += 2;
    };
    if (integ_ == HGPU_INTEGRATOR_FORWARD_EULER) {
        CombinePlan<real> plan{};
        plan.fe = 1;
        plan.slot[0] = state_.as<real>();
        stage(state_.as<real>(), plan);
        L.boundary(nextQ());                              // self-gravity pass: ghost refresh, then + 0 * dt
        L.gravity(integ_, sc, nextQ());
        launches_ += 2;
    } else {
        for (size_t k = 0; k < plans_.plans.size(); ++k)
            stage(plans_.plans[k].slot[plans_.inputSlot[k]], plans_.plans[k]);
        if (!alphaBinary_) {
            L.gravity(integ_, sc, nextQ());
            ++launches_;
        }
    }
    L.stateCheck(health, healthP_.as<unsigned>(), nextQ());
    ++launches_;
}

// capture one step into a CUDA graph (capture records the launches, it runs nothing)
template <typename real>
void BatchSolver<real>::ensureGraph() {
    if (exec_) return;
    cudaCheck(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal), "begin capture");
    try {
        update();
    } catch (...) {
        cudaGraph_t g = nullptr;
        cudaStreamEndCapture(stream, &g);
        if (g) cudaGraphDestroy(g);
        throw;
    }
    cudaCheck(cudaStreamEndCapture(stream, &graph_), "end capture");
    cudaCheck(cudaGraphInstantiate(&exec_, graph_, 0), "instantiate");
}

template <typename real>
void BatchSolver<real>::run(int nsteps) {
    if (nsteps <= 0) return;
    ensureGraph();
    for (int i = 0; i < nsteps; ++i) cudaCheck(cudaGraphLaunch(exec_, stream), "graph launch");
}

template <typename real>
float BatchSolver<real>::timedRun(int nsteps) {
    if (!t0_) {
        cudaCheck(cudaEventCreate(&t0_), "event");
        cudaCheck(cudaEventCreate(&t1_), "event");
    }
    ensureGraph();
    cudaCheck(cudaEventRecord(t0_, stream), "record");
    run(nsteps);
    cudaCheck(cudaEventRecord(t1_, stream), "record");
    cudaCheck(cudaEventSynchronize(t1_), "sync");
    float ms = 0;
    cudaCheck(cudaEventElapsedTime(&ms, t0_, t1_), "elapsed");
    return ms;
}

template <typename real>
void BatchSolver<real>::setState(int p, const void* host, size_t count) {
    checkProblem(p, count);
    cudaCheck(cudaMemcpyAsync(state_.as<real>() + (size_t)N_ * host_[p].stateOff, host, sizeof(real) * count,
                              cudaMemcpyHostToDevice, stream),
              "batch set_state");
    cudaCheck(cudaStreamSynchronize(stream), "sync");
}

template <typename real>
void BatchSolver<real>::getState(int p, void* host, size_t count) {
    checkProblem(p, count);
    cudaCheck(cudaMemcpyAsync(host, state_.as<real>() + (size_t)N_ * host_[p].stateOff, sizeof(real) * count,
                              cudaMemcpyDeviceToHost, stream),
              "batch get_state");
    cudaCheck(cudaStreamSynchronize(stream), "sync");
}

template <typename real>
void BatchSolver<real>::checkProblem(int p, size_t count) const {
    if (p < 0 || p >= (int)host_.size()) throw ConfigError(HGPU_ERR_OOB, "problem index out of range");
    if (count != (size_t)host_[p].g.V * N_) throw ConfigError(HGPU_ERR_ARG, "state element count mismatch");
}

template <typename real>
void BatchSolver<real>::dts(double* out, int n) {
    if (n != (int)host_.size()) throw ConfigError(HGPU_ERR_ARG, "dt array size mismatch");
    std::vector<StepConst<real>> sc(host_.size());
    cudaCheck(cudaMemcpyAsync(sc.data(), sc_.get(), sizeof(StepConst<real>) * sc.size(), cudaMemcpyDeviceToHost, stream),
              "dts");
    cudaCheck(cudaStreamSynchronize(stream), "sync");
    for (int i = 0; i < n; ++i) out[i] = sc[i].dt_f64;
}

template <typename real>
unsigned BatchSolver<real>::readHealth() {
    unsigned f = 0;
    cudaCheck(cudaStreamSynchronize(stream), "sync");
    cudaCheck(cudaMemcpy(&f, health_.get(), sizeof f, cudaMemcpyDeviceToHost), "health");
    cudaCheck(cudaMemset(health_.get(), 0, sizeof f), "health clear");
    return f;
}

template <typename real>
void BatchSolver<real>::readProblemHealth(unsigned* out, int n) {
    if (n != (int)host_.size()) throw ConfigError(HGPU_ERR_ARG, "health array size mismatch");
    cudaCheck(cudaStreamSynchronize(stream), "sync");
    cudaCheck(cudaMemcpy(out, healthP_.get(), sizeof(unsigned) * host_.size(), cudaMemcpyDeviceToHost), "health");
    cudaCheck(cudaMemset(healthP_.get(), 0, sizeof(unsigned) * host_.size()), "health clear");
}

// "hllc-2d-rk2-f64-p512-<fnv1a of the sizes>"
template <typename real>
std::string BatchSolver<real>::signature() const {
    unsigned long long h = 1469598103934665603ULL;
    for (const auto& r : rcs_)
        for (int i = 0; i < 3; ++i) {
            h ^= (unsigned long long)r.cfg.size[i];
            h *= 1099511628211ULL;
        }
    std::ostringstream s;
    s << "v2-" << (kind_ == HGPU_SOLVER_ROE ? "roe" : kind_ == HGPU_SOLVER_HLL ? "hll" : "hllc") << "-" << dim_ << "d-i" << integ_ << "-" << (sizeof(real) == 8 ? "f64" : "f32")
      << "-p" << host_.size() << "-" << std::hex << h;
    return s.str();
}

template <typename real>
bool BatchSolver<real>::loadTuning(const std::string& path) {
    std::ifstream f(path);
    if (!f) return false;
    std::string line, sig = signature();
    while (std::getline(f, line)) {
        std::istringstream ls(line);
        std::string key;
        BatchTuning tu{};
        double ms = 0;
        if (ls >> key >> tu.tx >> tu.ty >> tu.tz >> tu.staged >> tu.blocksPerSM >> tu.split >> tu.cpt >> ms &&
            key == sig) {
            setTuning(tu);
            tunedMs_ = ms;
            return true;
        }
    }
    return false;
}

template <typename real>
void BatchSolver<real>::autotune(const std::string& cachePath, int steps) {
    if (!cachePath.empty() && loadTuning(cachePath)) return;
    // the candidates run real steps: keep the user's state and restore it afterwards
    size_t bytes = sizeof(real) * (size_t)totalCells_ * N_;
    DeviceBuffer saved(bytes, false);
    cudaCheck(cudaMemcpyAsync(saved.get(), state_.get(), bytes, cudaMemcpyDeviceToDevice, stream), "save state");
    auto timeOf = [&](const BatchTuning& c) {
        setTuning(c);
        cudaCheck(cudaMemcpyAsync(state_.get(), saved.get(), bytes, cudaMemcpyDeviceToDevice, stream), "restore");
        run(1);                                              // capture + warm
        float ms = timedRun(steps);
        return ms / std::max(1, steps);
    };
    // 1) tile shape x eigenbasis staging x blocks per SM, one cell per thread, with the
    //    two-pass flux where it exists
    const int split = splitAvailable() ? 1 : 0;
    std::vector<BatchTuning> cands;
    std::vector<std::array<int, 3>> shapes;
    if (dim_ == 1) shapes = {{256, 1, 1}, {128, 1, 1}};
    else if (dim_ == 2) shapes = {{32, 8, 1}, {16, 16, 1}, {64, 4, 1}, {16, 8, 1}, {32, 4, 1}};
    else shapes = {{32, 4, 2}, {16, 4, 4}, {8, 8, 4}, {32, 2, 2}};
    for (auto& s : shapes)
        for (int staged = 0; staged < 2; ++staged)
            for (int bps : {0, 2, -1}) {
                if (hllc_ && staged == 0) continue;           // staging only changes the Roe eigenbasis
                cands.push_back({s[0], s[1], s[2], hllc_ ? 1 : staged, bps, split, 1});
            }
    BatchTuning best = tuning_;
    double bestMs = 1e30;
    for (const auto& c : cands) {
        double per = timeOf(c);
        if (per < bestMs) { bestMs = per; best = c; }
    }
    // 2) threads per cell: 1, 1/2 or 1/4 (each thread takes 1, 2 or 4 cells of a tile
    //    that many times larger along its slowest axis; unstaged eigenbasis), and the
    //    one-pass flux against the two-pass one
    std::vector<BatchTuning> second;
    for (int cpt : {1, 2, 4})
        for (int sp = 0; sp <= split; ++sp) {
            BatchTuning c = best;
            c.cpt = cpt;
            c.split = sp;
            if (cpt > 1) {
                c.staged = 0;
                if (dim_ == 1) c.tx *= cpt;
                else if (dim_ == 2) c.ty *= cpt;
                else c.tz *= cpt;
            }
            if (c.cpt == best.cpt && c.split == best.split) continue;
            second.push_back(c);
        }
    for (const auto& c : second) {
        double per = timeOf(c);
        if (per < bestMs) { bestMs = per; best = c; }
    }
    setTuning(best);
    tunedMs_ = bestMs;
    cudaCheck(cudaMemcpyAsync(state_.get(), saved.get(), bytes, cudaMemcpyDeviceToDevice, stream), "restore");
    cudaCheck(cudaStreamSynchronize(stream), "sync");
    if (!cachePath.empty()) {
        std::ofstream f(cachePath, std::ios::app);
        f << signature() << " " << best.tx << " " << best.ty << " " << best.tz << " " << best.staged << " "
          << best.blocksPerSM << " " << best.split << " " << best.cpt << " " << bestMs << "\n";
    }
}

std::unique_ptr<BatchBase> createBatch(const std::vector<hgpu_config>& cfgs) {
    if (cfgs.empty()) throw ConfigError(HGPU_ERR_ARG, "empty batch");
    if (cfgs[0].precision == HGPU_FP32) return std::unique_ptr<BatchBase>(new BatchSolver<float>(cfgs));
    return std::unique_ptr<BatchBase>(new BatchSolver<double>(cfgs));
}

template class BatchSolver<double>;
template class BatchSolver<float>;

}  // namespace hgpu
