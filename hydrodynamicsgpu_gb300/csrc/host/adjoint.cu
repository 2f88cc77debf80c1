// adjoint.cu -- host side of the EulerRoe vector-Jacobian product (kernels/adjoint.cu).
//
// No reference counterpart: the reference only runs the forward scheme
// (src/Solver/Roe.cpp:82-112, src/Integrator/RungeKutta.cpp).  The step being
// differentiated is Solver::update with its dt held at the value the forward chose.
#include <algorithm>
#include <cstring>

#include "adjoint.h"

namespace hgpu {

static const unsigned long long kAccInf = 0x7FF0000000000000ULL;   // the bits of +Inf

RoeAdjoint::RoeAdjoint(const ResolvedConfig& rc, cudaStream_t stream) : rc_(rc), stream_(stream) {
    rc_.grid.check = checkWord();
    if (rc.cfg.solver != HGPU_SOLVER_ROE || rc.cfg.precision != HGPU_FP64 || rc.cfg.compat != HGPU_COMPAT_REF)
        throw ConfigError(HGPU_ERR_UNSUPPORTED, "the adjoint covers EulerRoe in FP64 with the REF scheme");
    // with useFixedDT, Solver::update never calls calcTimestep, so EulerRoe steps with the
    // eigenbasis buffer as the last CFL step (or the allocation) left it
    // (src/Solver/Solver.cpp:521-535, src/Solver/Roe.cpp:82-92): not the step differentiated here
    if (rc.cfg.use_fixed_dt)
        throw ConfigError(HGPU_ERR_UNSUPPORTED, "the adjoint differentiates the CFL-dt step (use_fixed_dt = 0)");
    for (int i = 0; i < 3; ++i) {
        ph_.dx[i] = rc.dx[i];
        ph_.rdx[i] = 1. / ph_.dx[i];
        for (int m = 0; m < 2; ++m) methods_[i][m] = i < rc.dim ? rc.cfg.boundary[i][m] : -1;
    }
    ph_.gamma = rc.gamma;
    ph_.cfl = rc.cfg.cfl;
    integ_ = rc.cfg.integrator;
    fe_ = integ_ == HGPU_INTEGRATOR_FORWARD_EULER;
    stages_ = fe_ ? 1 : tableauOrder(integ_);
    const size_t V = (size_t)rc.grid.V, N = rc.numStates, D = rc.dim, P = D + 2;
    cur_ = DeviceBuffer(sizeof(double) * V * N, true);
    flux_ = DeviceBuffer(sizeof(double) * V * N * D, true);
    sc_ = DeviceBuffer(sizeof(StepConst<double>), true);
    acc_ = DeviceBuffer(sizeof(unsigned long long), true);
    {   // the CFL minimum starts from +Inf (every Roe dtBuffer entry is written, Solver.cpp:217-222)
        const unsigned long long inf = kAccInf;
        cudaCheck(cudaMemcpy(acc_.get(), &inf, sizeof inf, cudaMemcpyHostToDevice), "dt accumulator init");
    }
    health_ = DeviceBuffer(sizeof(unsigned), true);
    lamTmp_ = DeviceBuffer(sizeof(double) * V * N, true);
    if (!fe_) {
        plans_ = buildStagePlans<double>(integ_);
        for (int i = 0; i < plans_.nslots; ++i) slots_.emplace_back(sizeof(double) * V * N, true);
        for (auto& pl : plans_.plans) {
            pl.slot[0] = cur_.as<double>();
            for (int i = 0; i < plans_.nslots; ++i) pl.slot[1 + i] = slots_[i].as<double>();
        }
        alphaBinary_ = tableauAlphaIsBinary(integ_);
    }
    for (int m = 1; m < stages_; ++m) lams_.emplace_back(sizeof(double) * V * N, true);
    // scratch planes (zero: faces outside the flux range are never written and read as 0)
    const size_t sizes[8] = {N * D, N * D, N * D, N * D, N * D, P * D, P * D, P * D};
    for (int i = 0; i < 8; ++i) scratch_.emplace_back(sizeof(double) * V * sizes[i], true);
    S_.gAvg = scratch_[0].as<double>();
    S_.gdqSelf = scratch_[1].as<double>();
    S_.gdqToM = scratch_[2].as<double>();
    S_.gdqToP = scratch_[3].as<double>();
    S_.gDelta = scratch_[4].as<double>();
    S_.gParam = scratch_[5].as<double>();
    S_.gPrimL = scratch_[6].as<double>();
    S_.gPrimR = scratch_[7].as<double>();
    one_.reset(new Tape(makeTape()));
}

RoeAdjoint::Tape RoeAdjoint::makeTape() const {
    const size_t V = (size_t)rc_.grid.V, N = rc_.numStates, D = rc_.dim;
    Tape t;
    t.basis = DeviceBuffer(sizeof(double) * V * D * roeRecordSize((int)D), true);
    for (int k = 0; k < stages_; ++k) {
        t.U.emplace_back(sizeof(double) * V * N, false);
        t.DQ.emplace_back(sizeof(double) * V * N * D, true);
        t.FT.emplace_back(sizeof(double) * V * roeFluxTapePlanes((int)D), false);
    }
    return t;
}

size_t RoeAdjoint::tapeBytes() const {
    const size_t V = (size_t)rc_.grid.V, N = rc_.numStates, D = rc_.dim;
    return sizeof(double) * V * (D * roeRecordSize((int)D) + stages_ * (N + N * D + roeFluxTapePlanes((int)D)));
}

void RoeAdjoint::forward(const double* u_n, double dt, Tape& t, double* u_next, double* dtOut) {
    const Grid& g = rc_.grid;
    const size_t bytes = sizeof(double) * (size_t)g.V * rc_.numStates;
    double* cur = cur_.as<double>();
    StepConst<double>* sc = sc_.as<StepConst<double>>();
    if (u_n != cur) cudaCheck(cudaMemcpyAsync(cur, u_n, bytes, cudaMemcpyDeviceToDevice, stream_), "adjoint input");
    launchBoundary<double>(g, methods_, cur, stream_);
    launchRoeBasis<double>(g, ph_, cur, t.basis.as<double>(), 0, stream_);
    if (dtOut) {                                   // Solver::update's CFL dt
        launchRoeDt<double>(g, ph_, t.basis.as<double>(), acc_.as<unsigned long long>(), health_.as<unsigned>(),
                            stream_);
        launchFinalizeDt<double>(ph_, integ_, 0, 0., acc_.as<unsigned long long>(), kAccInf, sc,
                                 health_.as<unsigned>(), stream_);
        cudaCheck(cudaMemcpyAsync(dtOut, &sc->dt_f64, sizeof(double), cudaMemcpyDeviceToDevice, stream_), "record dt");
    } else {
        launchFinalizeDt<double>(ph_, integ_, 1, dt, acc_.as<unsigned long long>(), 0, sc, health_.as<unsigned>(),
                                 stream_);
    }
    auto stage = [&](int k, const double* in) {
        cudaCheck(cudaMemcpyAsync(t.U[k].get(), in, bytes, cudaMemcpyDeviceToDevice, stream_), "tape stage");
        launchRoeDeltaQ<double>(g, in, t.basis.as<double>(), t.DQ[k].as<double>(), 0, stream_);
        launchRoeFluxRecord(g, rc_.cfg.limiter, in, t.basis.as<double>(), t.DQ[k].as<double>(), sc,
                            flux_.as<double>(), t.FT[k].as<double>(), stream_);
    };
    if (fe_) {
        stage(0, cur);
        CombinePlan<double> plan{};
        plan.fe = 1;
        plan.slot[0] = cur;
        launchDerivCombine<double>(g, ph_, flux_.as<double>(), plan, sc, stream_);
        launchBoundary<double>(g, methods_, cur, stream_);     // the self-gravity pass: ghost refresh, + 0 * dt
        launchZeroAdd<double>(g, cur, sc, stream_);
    } else {
        for (int k = 0; k < stages_; ++k) {
            stage(k, plans_.plans[k].slot[plans_.inputSlot[k]]);
            launchDerivCombine<double>(g, ph_, flux_.as<double>(), plans_.plans[k], sc, stream_);
        }
        if (!alphaBinary_) launchAlphaOnly<double>(g, integ_, cur, sc, stream_);
    }
    if (u_next && u_next != cur)
        cudaCheck(cudaMemcpyAsync(u_next, cur, bytes, cudaMemcpyDeviceToDevice, stream_), "adjoint output");
    cudaCheck(cudaGetLastError(), "adjoint forward launch");
}

void RoeAdjoint::reverse(const Tape& t, double dt, const double* lamNext, double* lamOut) {
    if (lamOut == lamNext) throw ConfigError(HGPU_ERR_ARG, "lambda_n must not alias lambda_next");
    const Grid& g = rc_.grid;
    const size_t bytes = sizeof(double) * (size_t)g.V * rc_.numStates;
    const double* lamS = lamNext;
    if (fe_) {   // u^{n+1} = G(u_1): lambda_1 = G^T lambda^{n+1}  (the + 0 * dt pass is the identity)
        cudaCheck(cudaMemcpyAsync(lamTmp_.get(), lamNext, bytes, cudaMemcpyDeviceToDevice, stream_), "lambda copy");
        launchAdjBoundary(g, methods_, lamTmp_.as<double>(), stream_);
        lamS = lamTmp_.as<double>();
    }
    // the alpha-only pass of tableaus with fractional alphas maps u to sum(alpha) u = u: identity
    double dtdx[3];
    for (int s = 0; s < 3; ++s) dtdx[s] = dt / ph_.dx[s];
    auto lamOf = [&](int m) -> const double* { return m == stages_ ? lamS : lams_[m - 1].as<double>(); };
    for (int k = stages_ - 1; k >= 0; --k) {
        AdjStage st{};
        st.nlam = stages_ - k;
        for (int i = 0; i < st.nlam; ++i) {
            int m = k + 1 + i;   // row m of the tableau forms u_m
            st.lam[i] = lamOf(m);
            st.alpha[i] = fe_ ? 1. : tableauAlpha(integ_, m - 1, k);
            st.coefF[i] = (fe_ ? 1. : tableauBeta(integ_, m - 1, k)) * dt;
        }
        const double* U = t.U[k].as<double>();
        launchAdjFlux(g, ph_, rc_.cfg.limiter, dtdx, U, t.DQ[k].as<double>(), t.basis.as<double>(),
                      t.FT[k].as<double>(), st, S_, k == stages_ - 1, stream_);
        launchAdjDeltaQ(g, ph_, U, t.basis.as<double>(), S_, stream_);
        launchAdjCells(g, st, S_, k == 0 ? lamOut : lams_[k - 1].as<double>(), stream_);
    }
    launchAdjBasis(g, ph_, t.U[0].as<double>(), S_, stream_);
    launchAdjPrims(g, ph_, t.U[0].as<double>(), S_, lamOut, stream_);
    launchAdjBoundary(g, methods_, lamOut, stream_);
    cudaCheck(cudaGetLastError(), "adjoint reverse launch");
}

void RoeAdjoint::step(const double* u_n, const double* lamNext, double* lamOut, double dt) {
    forward(u_n, dt, *one_, nullptr);
    reverse(*one_, dt, lamNext, lamOut);
}

// ---------------- checkpoints ----------------
Checkpoints::Checkpoints(RoeAdjoint* adj, double* state, cudaStream_t stream, int nsteps, int every,
                         std::function<void()> cflStep, const double* cflDt, bool taped)
    : adj_(adj), state_(state), stream_(stream), nsteps_(nsteps), every_(every), taped_(taped),
      cflStep_(std::move(cflStep)), cflDt_(cflDt) {
    if (nsteps < 1 || every < 1) throw ConfigError(HGPU_ERR_ARG, "nsteps and checkpoint interval must be positive");
    every_ = taped ? nsteps : std::min(every, nsteps);
    const auto& rc = adj->config();
    const size_t bytes = sizeof(double) * (size_t)rc.grid.V * rc.numStates;
    if (taped) {   // refuse before allocating what the device cannot hold
        size_t freeB = 0, totalB = 0;
        cudaCheck(cudaMemGetInfo(&freeB, &totalB), "cudaMemGetInfo");
        if ((double)adj->tapeBytes() * nsteps > 0.95 * (double)freeB)
            throw ConfigError(HGPU_ERR_NOMEM, "the tapes of every step do not fit in device memory");
    } else {
        for (int i = 0; i < (nsteps + every_ - 1) / every_; ++i) ckpt_.emplace_back(bytes, false);
    }
    for (int i = 0; i < every_; ++i) tapes_.push_back(adj->makeTape());
    dtDev_ = DeviceBuffer(sizeof(double) * nsteps, true);
    lamA_ = DeviceBuffer(bytes, false);
    lamB_ = DeviceBuffer(bytes, false);
    dts.assign(nsteps, 0.);
    cudaCheck(cudaEventCreate(&e0_), "event");
    cudaCheck(cudaEventCreate(&e1_), "event");
}

Checkpoints::~Checkpoints() {
    if (e0_) cudaEventDestroy(e0_);
    if (e1_) cudaEventDestroy(e1_);
}

void Checkpoints::forward(const double* dtsIn) {
    const auto& rc = adj_->config();
    const size_t bytes = sizeof(double) * (size_t)rc.grid.V * rc.numStates;
    cudaCheck(cudaEventRecord(e0_, stream_), "event");
    if (taped_) {                                   // every step records its own tape
        const double* u = state_;
        for (int i = 0; i < nsteps_; ++i) {
            if (dtsIn) dts[i] = dtsIn[i];
            adj_->forward(u, dtsIn ? dtsIn[i] : 0., tapes_[i], nullptr, dtsIn ? nullptr : dtDev_.as<double>() + i);
            u = adj_->work();
        }
        cudaCheck(cudaMemcpyAsync(state_, u, bytes, cudaMemcpyDeviceToDevice, stream_), "final state");
    }
    for (int i = 0; i < nsteps_ && !taped_; ++i) {
        if (i % every_ == 0)
            cudaCheck(cudaMemcpyAsync(ckpt_[i / every_].get(), state_, bytes, cudaMemcpyDeviceToDevice, stream_),
                      "checkpoint");
        if (dtsIn) {
            dts[i] = dtsIn[i];
            adj_->forward(state_, dtsIn[i], tapes_[0], state_);
        } else {
            cflStep_();
            cudaCheck(cudaMemcpyAsync(dtDev_.as<double>() + i, cflDt_, sizeof(double), cudaMemcpyDeviceToDevice,
                                      stream_),
                      "record dt");
        }
    }
    cudaCheck(cudaEventRecord(e1_, stream_), "event");
    if (!dtsIn)
        cudaCheck(cudaMemcpyAsync(dts.data(), dtDev_.get(), sizeof(double) * nsteps_, cudaMemcpyDeviceToHost, stream_),
                  "dts");
    cudaCheck(cudaStreamSynchronize(stream_), "sync");
    cudaCheck(cudaEventElapsedTime(&forwardMs, e0_, e1_), "elapsed");
    forwardDone_ = true;
}

void Checkpoints::backward(const double* lamT, double* lam0) {
    if (!forwardDone_) throw ConfigError(HGPU_ERR_ARG, "run the checkpointed forward first");
    const auto& rc = adj_->config();
    const size_t bytes = sizeof(double) * (size_t)rc.grid.V * rc.numStates;
    cudaCheck(cudaEventRecord(e0_, stream_), "event");
    double* lam = lamA_.as<double>();
    double* other = lamB_.as<double>();
    cudaCheck(cudaMemcpyAsync(lam, lamT, bytes, cudaMemcpyDeviceToDevice, stream_), "lambda_T");
    const int nseg = (nsteps_ + every_ - 1) / every_;
    for (int seg = nseg - 1; seg >= 0; --seg) {
        const int first = seg * every_, last = std::min(nsteps_, first + every_);
        const double* u = taped_ ? nullptr : ckpt_[seg].as<double>();
        for (int j = first; j < last && !taped_; ++j) {            // recompute, recording tapes, on
            adj_->forward(u, dts[j], tapes_[j - first], nullptr);  // the adjoint's working state
            u = adj_->work();
        }
        for (int j = last - 1; j >= first; --j) {                  // reverse steps
            adj_->reverse(tapes_[j - first], dts[j], lam, other);
            std::swap(lam, other);
        }
    }
    cudaCheck(cudaMemcpyAsync(lam0, lam, bytes, cudaMemcpyDeviceToDevice, stream_), "lambda_0");
    cudaCheck(cudaEventRecord(e1_, stream_), "event");
    cudaCheck(cudaEventSynchronize(e1_), "sync");
    cudaCheck(cudaEventElapsedTime(&backwardMs, e0_, e1_), "elapsed");
}

}  // namespace hgpu
