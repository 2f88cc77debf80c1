// adjoint.h -- reverse-mode step and checkpointed trajectories of EulerRoe (FP64).
#pragma once
#include <functional>
#include <memory>
#include <vector>

#include "../kernels/adjoint.h"
#include "solver.h"

namespace hgpu {

// One EulerRoe step with a given (frozen) dt and its vector-Jacobian product.
// The forward uses the solver's own kernels and combine plans, so with the dt the
// CFL condition chose it reproduces Solver::update bit for bit, and it records the
// values the reverse pass needs (a Tape).
class RoeAdjoint {
public:
    struct Tape {
        DeviceBuffer basis;                  // eigenbasis of u_0 (compact records)
        std::vector<DeviceBuffer> U, DQ;     // stage inputs u_k (u_0 = ghost-filled u^n) and their Delta-q-tilde
        std::vector<DeviceBuffer> FT;        // per stage: the flux's per-wave values (roe_record.cu)
    };
    RoeAdjoint(const ResolvedConfig& rc, cudaStream_t stream);
    Tape makeTape() const;
    // u_next = step(u_n; dt) (u_next may be u_n or null); records `t`.  The step runs
    // on the working state (work()): u_n == work() and u_next == null skip both copies.
    // With dtOut (a device double) the step takes the CFL dt of u_n, as Solver::update
    // does, and writes it there; `dt` is then unused.
    void forward(const double* u_n, double dt, Tape& t, double* u_next, double* dtOut = nullptr);
    const double* work() const { return cur_.as<double>(); }
    // lamOut = (d u^{n+1} / d u^n)^T lamNext for the step recorded in `t` (lamOut != lamNext)
    void reverse(const Tape& t, double dt, const double* lamNext, double* lamOut);
    // state <- step(state; dt) (no tape kept beyond this call)
    void advance(double* state, double dt) { forward(state, dt, *one_, state); }
    // forward + reverse of one step
    void step(const double* u_n, const double* lamNext, double* lamOut, double dt);
    size_t tapeBytes() const;
    const ResolvedConfig& config() const { return rc_; }

private:
    ResolvedConfig rc_;
    Phys<double> ph_;
    cudaStream_t stream_;
    int methods_[3][2];
    int integ_, stages_;
    bool fe_, alphaBinary_ = true;
    StagePlans<double> plans_;
    DeviceBuffer cur_, flux_, sc_, acc_, health_, lamTmp_;
    std::vector<DeviceBuffer> slots_, lams_;
    std::vector<DeviceBuffer> scratch_;
    AdjScratch S_{};
    std::unique_ptr<Tape> one_;
};

// Checkpointed trajectory: the forward keeps the state every `every` steps and the dt
// of every step; the backward recomputes one segment at a time (recording its tapes)
// and runs the reverse steps, so memory is (nsteps/every) states + `every` tapes.
// Taped: the forward records every step's tape as it goes (the adjoint's recording
// step, the same kernels as Solver::update), and the backward runs the reverse steps
// only; memory is nsteps tapes (tapeBytes() each).
class Checkpoints {
public:
    Checkpoints(RoeAdjoint* adj, double* state, cudaStream_t stream, int nsteps, int every,
                std::function<void()> cflStep, const double* cflDt, bool taped = false);
    void forward(const double* dts);                         // host dts or null (CFL)
    void backward(const double* lamT, double* lam0);        // device arrays
    std::vector<double> dts;
    float forwardMs = 0, backwardMs = 0;

private:
    RoeAdjoint* adj_;
    double* state_;
    cudaStream_t stream_;
    int nsteps_, every_;
    bool taped_;
    std::function<void()> cflStep_;
    const double* cflDt_;
    std::vector<DeviceBuffer> ckpt_;
    std::vector<RoeAdjoint::Tape> tapes_;
    DeviceBuffer dtDev_, lamA_, lamB_;
    cudaEvent_t e0_ = nullptr, e1_ = nullptr;
    bool forwardDone_ = false;
public:
    ~Checkpoints();
};

}  // namespace hgpu
