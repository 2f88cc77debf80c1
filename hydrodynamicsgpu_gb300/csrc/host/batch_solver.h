// batch_solver.h -- host class of a batch of independent Euler problems (batch_solver.cu).
#pragma once
#include <memory>
#include <string>
#include <vector>

#include "../kernels/batch.h"
#include "solver.h"

namespace hgpu {

class BatchBase {
public:
    virtual ~BatchBase() = default;
    virtual void run(int nsteps) = 0;                 // nsteps graph replays of one batched step
    virtual float timedRun(int nsteps) = 0;           // same, device ms (CUDA events on the batch stream)
    virtual void setState(int p, const void* host, size_t count) = 0;
    virtual void getState(int p, void* host, size_t count) = 0;
    virtual void dts(double* out, int n) = 0;
    virtual unsigned readHealth() = 0;
    // read and clear every problem's health word (n = number of problems)
    virtual void readProblemHealth(unsigned* out, int n) = 0;
    virtual void setTuning(const BatchTuning& tu) = 0;
    virtual BatchTuning tuning() const = 0;
    virtual void autotune(const std::string& cachePath, int steps) = 0;
    virtual int problems() const = 0;
    virtual long long totalCells() const = 0;
    virtual int kernelsPerStep() const = 0;
    cudaStream_t stream = nullptr;
};

template <typename real>
class BatchSolver : public BatchBase {
public:
    explicit BatchSolver(const std::vector<hgpu_config>& cfgs);
    ~BatchSolver() override;
    void run(int nsteps) override;
    float timedRun(int nsteps) override;
    void setState(int p, const void* host, size_t count) override;
    void getState(int p, void* host, size_t count) override;
    void dts(double* out, int n) override;
    unsigned readHealth() override;
    void readProblemHealth(unsigned* out, int n) override;
    void setTuning(const BatchTuning& tu) override;
    BatchTuning tuning() const override { return tuning_; }
    void autotune(const std::string& cachePath, int steps) override;
    int problems() const override { return (int)host_.size(); }
    long long totalCells() const override { return totalCells_; }
    int kernelsPerStep() const override { return launches_; }

private:
    static constexpr int kQueues = 32;
    std::vector<ResolvedConfig> rcs_;
    std::vector<BatchProblem<real>> host_;
    int dim_ = 0, N_ = 0, integ_ = 0, nTiles_ = 0, launches_ = 0, kind_ = 0;
    bool hllc_ = false, alphaBinary_ = true;
    long long totalCells_ = 0;
    double tunedMs_ = 0;
    DeviceBuffer state_, faces_, dq_, flux_, probs_, sc_, acc_, health_, healthP_, queues_, tiles_;
    std::vector<DeviceBuffer> work_;
    StagePlans<real> plans_;
    BatchTuning tuning_{};
    cudaGraph_t graph_ = nullptr;
    cudaGraphExec_t exec_ = nullptr;
    cudaEvent_t t0_ = nullptr, t1_ = nullptr;
    void update();
    void ensureGraph();
    void dropGraph();
    void checkProblem(int p, size_t count) const;
    bool splitAvailable() const;             // the two-pass flux exists (FP64 EulerRoe)
    std::string signature() const;
    bool loadTuning(const std::string& path);
};

std::unique_ptr<BatchBase> createBatch(const std::vector<hgpu_config>& cfgs);

}  // namespace hgpu
