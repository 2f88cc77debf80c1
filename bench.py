#!/usr/bin/env python3
"""Benchmark: 2D Euler Roe cell-updates/s on one GB300 (FP64), HydroGPU's KH workload.

Workload (the 2D benchmark configuration): EulerRoe, FP64, 2048x2048 cells (ghosts
included) on [-0.5,0.5]^2, periodic, gamma 1.4, minmod limiter, RK4, CFL 0.5,
Kelvin-Helmholtz shear-layer IC (seeded synthetic noise).  A "step" is one full
Solver::update (all four RK stages).  A cell-update is one interior cell advanced
by one step.

  python bench.py [--gpus N --steps K --warmup W]          # this repository (GB300 kernels)
  python bench.py --impl reference [--steps K --warmup W]   # the reference's kernels on the host CPU

`value` is device time (CUDA events on the solver's stream around K graph
replays, inputs resident in HBM); `e2e` runs the same K steps through the C ABI
(hgpu_update_host) with the state uploaded from and downloaded to page-locked host
memory every step, the copies overlapped with the step in bands.
With N > 1 (torchrun) every rank runs an independent replica on its own GPU
(the workload does not shard across GPUs in the reference; "replicas only").
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "2D Euler Roe cell-updates/s (FP64, 1 GB300) plain vs batched; adjoint/fwd time"
UNIT = "cell-updates/s"
N_STATES = 4
RECORD = 17              # doubles per face in the compact Roe eigenbasis record (2D)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--size", type=int, default=2048)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the 512-problem batched sweep")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint/forward measurement")
    ap.add_argument("--no-gravity", action="store_true", help="skip the self-gravity measurement")
    ap.add_argument("--gravity-size", type=int, default=2048)
    ap.add_argument("--gravity-detail", action="store_true", help="per-kernel breakdown of the self-gravity step")
    ap.add_argument("--batch-problems", type=int, default=512)
    ap.add_argument("--batch-steps", type=int, default=10)
    ap.add_argument("--adjoint-problems", type=int, default=16)
    ap.add_argument("--adjoint-steps", type=int, default=200)
    ap.add_argument("--fd-directions", type=int, default=64)
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)), int(os.environ.get("WORLD_SIZE", 1))


def workload_config(hg_abi, size):
    return hg_abi.make_config(solver="EulerRoe", size=(size, size), xmin=(-.5, -.5), xmax=(.5, .5), gamma=1.4,
                              boundary="PERIODIC", limiter="MinMod", integrator="RungeKutta4", cfl=.5)


def workload_name(size):
    return "KH %dx%d EulerRoe FP64 RK4 minmod periodic CFL 0.5" % (size, size)


# ---------------- clocks during the timed region ----------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.proc = None
        self.lines = []
        self.gpu = gpu_index

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return d.get("hbm_gbs"), "measured"
    except Exception:
        return 6800.0, "fallback"


# ---------------- CPU baselines (the reference's kernels on host cores) ----------------
def cpu_sample(size, warm=1, steps=2):
    """Bounded sample: the same scheme on a size x (size/4) strip of the KH workload."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import pyoracle
    from hydrodynamicsgpu_gb300 import _abi, initconds as ic
    ny = max(64, size // 4)
    cfg = _abi.make_config(solver="EulerRoe", size=(size, ny), boundary="PERIODIC", limiter="MinMod",
                           integrator="RungeKutta4", cfl=.5)
    init = ic.kelvin_helmholtz(size=(size, ny), seed=0).reshape(-1)
    kind = "reference"
    try:
        if not pyoracle.refcl_available(cfg):
            pyoracle.build_refcl(quiet=True)
        solver = pyoracle.Refcl(cfg)
        cores = solver.max_threads()
    except Exception:
        kind = "port"
        solver = pyoracle.Oracle(cfg)
        cores = pyoracle.max_threads()
    solver.set_state(init)
    solver.update(warm)
    t0 = time.perf_counter()
    solver.update(steps)
    dt = time.perf_counter() - t0
    cells = (size - 4) * (ny - 4)
    sample = "%d RK4 steps of the same scheme on a %dx%d strip of the KH workload (after %d warm-up)" % (
        steps, size, ny, warm)
    return {"value": cells * steps / dt, "unit": UNIT, "cores": cores, "kind": kind, "sample": sample}, dt


def run_reference(args):
    rank, local_rank, world = dist_env()
    if world > 1 and rank != 0:
        return 0
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import pyoracle
    from hydrodynamicsgpu_gb300 import _abi, initconds as ic
    size = args.size
    ny = max(64, size // 8)
    cfg = _abi.make_config(solver="EulerRoe", size=(size, ny), boundary="PERIODIC", limiter="MinMod",
                           integrator="RungeKutta4", cfl=.5)
    init = ic.kelvin_helmholtz(size=(size, ny), seed=0).reshape(-1)
    kind = "reference"
    try:
        if not pyoracle.refcl_available(cfg):
            pyoracle.build_refcl(quiet=True)
        solver = pyoracle.Refcl(cfg)
        cores = solver.max_threads()
    except Exception:
        kind = "port"
        solver = pyoracle.Oracle(cfg)
        cores = pyoracle.max_threads()
    solver.set_state(init)
    solver.update(args.warmup)
    t0 = time.perf_counter()
    solver.update(args.steps)
    el = time.perf_counter() - t0
    cells = (size - 4) * (ny - 4)
    value = cells * args.steps / el
    sample = ("each step: one RK4 step of the KH scheme on a %dx%d strip (same per-cell work as %dx%d), "
              "the reference's OpenCL kernels compiled for the host CPU with OpenMP" % (size, ny, size, size))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded KH shear layer)",
            "config": {"workload": workload_name(size), "sample_grid": [size, ny]},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": kind, "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ---------------- GB300 arm ----------------
def algorithmic_bytes_per_cell(kind):
    """Compulsory HBM bytes per interior cell for one launch of each kernel (2D, FP64).
    One 'array' = N_STATES doubles per cell; the eigenbasis record is RECORD doubles per face."""
    s = 8
    face = 2  # faces per cell in 2D
    table = {
        "roe_flux": N_STATES * s + face * RECORD * s + face * N_STATES * s + face * N_STATES * s,
        "roe_delta_q_tilde": N_STATES * s + face * (2 * N_STATES + 3) * s + face * N_STATES * s,
        "roe_eigenbasis": N_STATES * s + face * RECORD * s,
        "flux_divergence_combine": face * N_STATES * s + 4 * N_STATES * s,  # flux + ~4 state-sized arrays (RK4 mean)
        "cfl_min_reduce": face * 2 * s,
        "boundary": 0,
        "finalize_dt": 0,
    }
    return table.get(kind, 0)


def batched_sweep(hg, _abi, ic, args):
    """The batched workload: 512 four-quadrant Riemann problems of uneven sides
    (16*round(exp(U(ln 32, ln 512))/16) cells per axis, ghosts included, seed 2),
    EulerRoe FP64, RK2 midpoint, Superbee, CFL 0.5, periodic or free-flow per problem.
    Timed three ways over the same steps: one batched CUDA graph of persistent
    launches per step; per-problem plain launches issued problem after problem (each
    problem's steps, then the next problem, as a sweep of the single-problem solver
    runs); and per-problem plain launches interleaved step by step, each problem on
    its own stream."""
    cfgs, inits = [], []
    for pr in ic.random_quadrant_problems(n=args.batch_problems, seed=2):
        side = pr["side"]
        cfgs.append(_abi.make_config(solver="EulerRoe", size=(side, side), boundary=pr["boundary"],
                                     limiter="Superbee", integrator="RungeKutta2"))
        inits.append(ic.quadrant((side, side), pr["quadrants"]).reshape(-1))
    interior = sum((c.size[0] - 4) * (c.size[1] - 4) for c in cfgs)
    steps = args.batch_steps
    b = hg.Batch(cfgs)
    for p, x in enumerate(inits):
        b.set_state(p, x)
    t0 = time.perf_counter()
    tuning = b.autotune(os.path.join(REPO, "hydrodynamicsgpu_gb300", ".batch_tuning.txt"), steps=2)
    tune_s = time.perf_counter() - t0
    for p, x in enumerate(inits):
        b.set_state(p, x)
    b.update(3)
    b.problem_health()
    batch_ms = b.timed_update(steps) / steps
    _, total_cells, kps = b.info()
    health = b.health()
    flagged = b.problem_health()
    b.close()
    solvers = [hg.Solver(c) for c in cfgs]
    for s_, x in zip(solvers, inits):
        s_.resetState(x)
        s_.update(2, want_dt=False)
    for s_ in solvers:
        s_.synchronize()
    t0 = time.perf_counter()
    for s_ in solvers:
        s_.update(steps, want_dt=False)
        s_.synchronize()
    seq_ms = (time.perf_counter() - t0) * 1e3 / steps
    t0 = time.perf_counter()
    for _ in range(steps):
        for s_ in solvers:
            s_.update(1, want_dt=False)
    for s_ in solvers:
        s_.synchronize()
    inter_ms = (time.perf_counter() - t0) * 1e3 / steps
    for s_ in solvers:
        s_.close()
    rate = lambda ms: interior / (ms * 1e-3)
    return {
        "workload": "%d four-quadrant Riemann problems, sides 32-512 (seed 2), EulerRoe RK2 Superbee FP64"
                    % len(cfgs),
        "interior_cells": interior, "steps": steps,
        "batched": {"value": rate(batch_ms), "ms_per_step": batch_ms, "kernels_per_step": kps,
                    "tuning": {"tile": list(tuning[:3]), "staged_eigenbasis": tuning[3],
                               "blocks_per_sm": tuning[4], "split_flux": tuning[5], "cells_per_thread": tuning[6]},
                    "autotune_s": tune_s, "health_flags": health,
                    "problems_flagged": {"count": int((flagged != 0).sum()),
                                         "first": [int(i) for i in np.flatnonzero(flagged)[:8]],
                                         "bits": int(np.bitwise_or.reduce(flagged)) if len(flagged) else 0}},
        "plain_sequential": {"value": rate(seq_ms), "ms_per_step": seq_ms},
        "plain_interleaved": {"value": rate(inter_ms), "ms_per_step": inter_ms},
        "speedup_vs_plain_sequential": seq_ms / batch_ms,
        "speedup_vs_plain_interleaved": inter_ms / batch_ms,
        "unit": UNIT, "timing": "batched: CUDA events; plain: host wall clock around the launches + synchronize",
    }


def smooth_fd(hg, _abi, ic, args, n, loss_and_cotangent, loss_difference, pert, ndir=8, eps_list=(1e-6, 1e-5, 1e-4)):
    """The same gradient check on a configuration where the rollout is differentiable:
    a smooth periodic flow with velocities away from zero (no face switches its upwind
    side) and the smooth VanAlbada1 limiter, 512^2, RK2, the same step count; central
    differences at each step size of `eps_list` (at 1e-6 the rounding of the two
    200-step trajectories is a visible part of the difference quotient)."""
    import torch
    f = [ic.smooth_perturbation((n, n), seed=400 + k, amp=1.)[0] for k in range(4)]
    u0 = ic.build_state_euler(2, 1.4, 1. + .2 * f[0], .4 + .05 * f[1], .3 + .05 * f[2], 0.,
                              1. + .1 * f[3]).reshape(-1)
    cfg = _abi.make_config(solver="EulerRoe", size=(n, n), boundary="PERIODIC", limiter="VanAlbada1",
                           integrator="RungeKutta2")
    s_ = hg.Solver(cfg)
    s_.resetState(u0)
    cp = hg.Checkpoints(s_, args.adjoint_steps, 20)
    cp.forward()
    dts = cp.dts()
    uT = s_.getState().copy()
    target = uT.reshape(n, n, N_STATES)[..., 0] + pert
    _, lamT = loss_and_cotangent(uT, target)
    dl = torch.tensor(lamT, device="cuda")
    g = torch.empty_like(dl)
    torch.cuda.synchronize()
    cp.backward(dl.data_ptr(), g.data_ptr())
    s_.synchronize()
    gh = g.cpu().numpy()
    rng = np.random.default_rng(300)
    dirs = []
    for _ in range(ndir):
        d = rng.standard_normal(u0.size)
        dirs.append(d / np.linalg.norm(d))
    out = {"workload": "smooth drifting flow 512^2, VanAlbada1, RK2, %d steps" % args.adjoint_steps}
    for eps in eps_list:
        errs = []
        for d in dirs:
            ends = []
            for sgn in (1, -1):
                s_.resetState(u0 + sgn * eps * d)
                s_.update_frozen_dt(dts)
                ends.append(s_.getState().copy())
            errs.append((loss_difference(ends[0], ends[1], target) / (2 * eps), float(np.dot(gh, d))))
        out["eps_%g" % eps] = fd_stats(errs, eps)
    cp.close()
    s_.close()
    return out


def fd_stats(pairs, eps):
    """(finite difference, adjoint) directional derivatives along unit random directions:
    each error is |fd - ad| over the RMS of ad across the directions (a direction nearly
    orthogonal to the gradient has ad ~ 0 and no meaningful relative error of its own)."""
    fd = np.array([p[0] for p in pairs])
    ad = np.array([p[1] for p in pairs])
    scale = float(np.sqrt(np.mean(ad ** 2)))
    err = np.abs(fd - ad) / scale
    return {"directions": len(pairs), "eps": eps, "rms_directional_derivative": scale,
            "rel_err_median": float(np.median(err)), "rel_err_max": float(err.max()),
            "within_1e-6": int((err <= 1e-6).sum())}


def fp32_measure(hg, _abi, ic, args):
    """FP32 instantiation: the KH workload's throughput, and its error against FP64
    after 100 steps on KH 512^2 (each precision with its own CFL dt), per conserved
    variable as max |u32 - u64| / max |u64|."""
    size = args.size
    cfg = _abi.make_config(solver="EulerRoe", size=(size, size), boundary="PERIODIC", limiter="MinMod",
                           integrator="RungeKutta4", precision=_abi.FP32)
    s_ = hg.Solver(cfg)
    s_.resetState(ic.kelvin_helmholtz(size=(size, size), seed=0).astype(np.float32))
    s_.update(args.warmup, want_dt=False)
    ms = s_.timed_update(args.steps) / args.steps
    s_.close()
    n = 512
    u0 = ic.kelvin_helmholtz(size=(n, n), seed=0).reshape(-1)
    out = {}
    for prec in (_abi.FP64, _abi.FP32):
        c = _abi.make_config(solver="EulerRoe", size=(n, n), boundary="PERIODIC", limiter="MinMod",
                             integrator="RungeKutta4", precision=prec)
        s_ = hg.Solver(c)
        s_.resetState(u0.astype(np.float32) if prec == _abi.FP32 else u0)
        s_.update(100, want_dt=False)
        out[prec] = s_.getState().astype(np.float64).reshape(-1, N_STATES)
        s_.close()
    err = np.max(np.abs(out[_abi.FP32] - out[_abi.FP64]), axis=0) / np.max(np.abs(out[_abi.FP64]), axis=0)
    return {"value": (size - 4) ** 2 / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms,
            "error_vs_fp64_100_steps_512": {"rho": float(err[0]), "mx": float(err[1]), "my": float(err[2]),
                                            "E": float(err[3])}}


def gravity_measure(hg, _abi, ic, args):
    """Self-gravity workload: `gravity_size`^2 (ghosts included) EulerRoe FP64 RK4 MinMod,
    periodic, useGravity with gaussSeidelMaxIter 20 and G = 1 (the reference's defaults,
    res/config.lua:65-74), three seeded Gaussian over-densities at rest (p = 10).  Whole
    steps (Roe pass + self-gravity pass with 4 x 20 relaxation sweeps) timed with CUDA
    events over graph replays; the per-kernel breakdown from event pairs; the
    relaxation sweep's HBM fraction with 32 algorithmic bytes per interior cell and
    sweep (the potential read once per colour, written once, the density read once)."""
    n = args.gravity_size
    cfg = _abi.make_config(solver="EulerRoe", size=(n, n), boundary="PERIODIC", limiter="MinMod",
                           integrator="RungeKutta4", use_gravity=True, gauss_seidel_max_iter=20,
                           gravitational_constant=1.)
    s_ = hg.Solver(cfg)
    t0 = time.perf_counter()
    s_.resetState(ic.gravity_blobs(size=(n, n), seed=7))
    reset_s = time.perf_counter() - t0
    s_.update(args.warmup, want_dt=False)
    ms = s_.timed_update(args.steps) / args.steps
    prof = s_.profile(2)
    kps = s_.kernels_per_step()
    health = s_.health()
    s_.close()
    interior = (n - 4) * (n - 4)
    total = sum(v[1] for v in prof.values())
    breakdown = {k: {"launches": v[0], "ms_per_launch": v[1] / v[0], "share": v[1] / total} for k, v in prof.items()}
    relax = prof.get("poisson_relax")
    peak_gbs, peak_kind = measured_peaks()
    sweep_ms = relax[1] / relax[0] if relax else None
    sweep = None
    if sweep_ms:
        gbs = 32. * interior / (sweep_ms * 1e-3) / 1e9
        sweep = {"ms_per_sweep": sweep_ms, "algorithmic_bytes_per_sweep": 32 * interior, "achieved": gbs,
                 "peak": peak_gbs, "unit": "GB/s", "frac": gbs / peak_gbs, "peak_source": peak_kind}
    return {"workload": "self-gravitating blobs %dx%d, EulerRoe FP64 RK4 MinMod periodic, useGravity, "
                        "gaussSeidelMaxIter 20, G 1" % (n, n),
            "value": interior / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms, "kernels_per_step": kps,
            "reset_s": reset_s, "relax_sweep": sweep, "health_flags": health,
            "kernels": breakdown if args.gravity_detail else None}


def adjoint_measure(hg, _abi, ic, args):
    """Adjoint workload: Kelvin-Helmholtz 512^2 problems (seeds 100..), EulerRoe FP64
    RK2 MinMod periodic, `adjoint_steps` steps with CFL dt recorded and then frozen,
    checkpoints every 20 steps.  forward = checkpointed forward; backward = segment
    recompute + reverse steps.  Loss = mean over interior cells of
    (rho_T - rho_target)^2 with rho_target = rho_T + a smooth 1e-2 perturbation
    (seed 200).  Central differences (eps 1e-6, unit random directions, seed 300) of
    the frozen-dt forward check the gradient of problem 0; the loss difference is formed
    cell by cell (loss_difference)."""
    import torch
    n = 512
    shape = (n, n, N_STATES)
    mask = np.zeros((n, n), dtype=bool)
    mask[2:-2, 2:-2] = True
    pert = ic.smooth_perturbation((n, n), seed=200)[0]

    def loss_and_cotangent(uT, target):
        r = uT.reshape(shape)[..., 0] - target
        cnt = mask.sum()
        lam = np.zeros(shape)
        lam[..., 0][mask] = 2 * r[mask] / cnt
        return float(np.sum(r[mask] ** 2) / cnt), lam.reshape(-1)

    def loss_difference(ua, ub, target):
        """loss(ua) - loss(ub) formed cell by cell, (a - b)(a + b - 2 target): the
        difference of the two sums would lose it to their rounding (the loss is
        ~1e-4, a difference across 2e-6 of a unit direction ~1e-14)."""
        a = ua.reshape(shape)[..., 0][mask]
        b = ub.reshape(shape)[..., 0][mask]
        return float(np.sum((a - b) * (a + b - 2 * target[mask])) / mask.sum())

    fwd_ms = bwd_ms = plain_ms = 0.
    tfwd_ms = tbwd_ms = 0.
    taped_same = True
    taped_error = None
    fd = None
    for k in range(args.adjoint_problems):
        cfg = _abi.make_config(solver="EulerRoe", size=(n, n), boundary="PERIODIC", limiter="MinMod",
                               integrator="RungeKutta2")
        u0 = ic.kelvin_helmholtz(size=(n, n), seed=100 + k).reshape(-1)
        s_ = hg.Solver(cfg)
        s_.resetState(u0)
        if k == 0:
            s_.update(3, want_dt=False)
            s_.resetState(u0)
        plain_ms += s_.timed_update(args.adjoint_steps)
        s_.resetState(u0)
        cp = hg.Checkpoints(s_, args.adjoint_steps, 20)
        cp.forward()
        dts = cp.dts()
        uT = s_.getState().copy()
        target = uT.reshape(shape)[..., 0] + pert
        loss, lamT = loss_and_cotangent(uT, target)
        dl = torch.tensor(lamT, device="cuda")
        g = torch.empty_like(dl)
        torch.cuda.synchronize()
        cp.backward(dl.data_ptr(), g.data_ptr())
        s_.synchronize()
        f, bw = cp.times()
        fwd_ms += f
        bwd_ms += bw
        # the same trajectory with every step's tape recorded during the forward (its
        # tapes must fit on the device: refused with HGPU_ERR_NOMEM otherwise)
        cp.close()
        if taped_error is None:
            s_.resetState(u0)
            try:
                ct = hg.Checkpoints(s_, args.adjoint_steps, taped=True)
            except hg.HgpuError as e:
                taped_error = str(e)
            else:
                ct.forward()
                gt = torch.empty_like(dl)
                torch.cuda.synchronize()
                ct.backward(dl.data_ptr(), gt.data_ptr())
                s_.synchronize()
                f, bw = ct.times()
                tfwd_ms += f
                tbwd_ms += bw
                taped_same = taped_same and np.array_equal(ct.dts(), dts) and bool(torch.equal(gt, g))
                ct.close()
        if k == 0 and args.fd_directions > 0:
            gh = g.cpu().numpy()
            rng = np.random.default_rng(300)
            errs = []
            for _ in range(args.fd_directions):
                d = rng.standard_normal(u0.size)
                d /= np.linalg.norm(d)
                ends = []
                for sgn in (1, -1):
                    s_.resetState(u0 + sgn * 1e-6 * d)
                    s_.update_frozen_dt(dts)
                    ends.append(s_.getState().copy())
                fdv = loss_difference(ends[0], ends[1], target) / 2e-6
                errs.append((fdv, float(np.dot(gh, d))))
            fd = fd_stats(errs, 1e-6)
            fd.update({
                  "note": "MinMod and the upwind choice have kinks; on this noisy state perturbations cross "
                          "some of them, so a difference quotient is not a derivative everywhere"})
        cp.close()
        s_.close()
    fd_smooth = (smooth_fd(hg, _abi, ic, args, n, loss_and_cotangent, loss_difference, pert)
                 if args.fd_directions > 0 else None)
    steps_total = args.adjoint_steps * args.adjoint_problems
    return {
        "workload": "%d x KH 512^2 (seeds 100..), EulerRoe RK2 MinMod FP64, %d steps, checkpoints every 20"
                    % (args.adjoint_problems, args.adjoint_steps),
        "forward_ms_per_step": fwd_ms / steps_total, "plain_forward_ms_per_step": plain_ms / steps_total,
        "backward_ms_per_step": bwd_ms / steps_total,
        "adjoint_over_forward": bwd_ms / fwd_ms, "adjoint_over_plain_forward": bwd_ms / plain_ms,
        "taped": {"unavailable": taped_error} if taped_error else {
            "note": "every step's tape recorded during the forward (hgpu_checkpoint_create_taped): the "
                    "backward runs the reverse steps only",
            "forward_ms_per_step": tfwd_ms / steps_total, "backward_ms_per_step": tbwd_ms / steps_total,
            "forward_over_plain_forward": tfwd_ms / plain_ms,
            "adjoint_over_plain_forward": tbwd_ms / plain_ms,
            "gradient_over_plain_forward": (tfwd_ms + tbwd_ms) / plain_ms,
            "same_dts_and_gradient_as_checkpointed": taped_same},
        "finite_differences": fd,
        "finite_differences_differentiable": fd_smooth,
    }


# DRAM bytes (read + write) per interior cell of one launch, from ncu captures of the
# same kernels on KH 1024x1024 (dram__bytes_read.sum + dram__bytes_write.sum over the
# interior cells); traffic grows with the cells processed, so the bench workload's
# per-launch traffic is this times its interior cells.  roe_flux is its two passes
# together (corrections 148 B + transforms 420 B).
MEASURED_TRAFFIC_PER_CELL = {"roe_flux": 568.0, "roe_delta_q_tilde": 252.0, "roe_eigenbasis": 245.0,
                             "flux_divergence_combine": 123.0}

# Instructions the FP64 unit executes per interior cell of one launch of each kernel of
# the EulerRoe FP64 step (MinMod), from ncu's smsp__inst_executed_pipe_fp64 (warp
# instructions x 32) over the cells of the second of two KH 512x512 RK4 steps of the same
# kernels; roe_flux is its two passes together (corrections 30.57 + transforms 65.55);
# Delta-q-tilde and the combine vary by stage, so theirs are the step's means (Delta-q-
# tilde 29.79 in every stage; the combine 40.87, 32.87, 32.87, 28.34).  763.1 per RK4
# cell-update.
FP64_PIPE_PER_CELL = {"roe_eigenbasis": 112.62, "cfl_min_reduce": 9.92, "roe_delta_q_tilde": 29.79,
                      "roe_flux": 96.12, "flux_divergence_combine": 33.74, "state_check": 1.98}


def fp64_roofline(prof, value, fp64_peak):
    """The step's binding roofline: FP64-unit instructions per cell-update (the table
    above times each kernel's launches per step, from a profile of `steps` steps)
    times cell-updates/s, against the FP64 unit's issue rate measured in this run
    (hgpu_fp64_peak, FMA instructions per second on all SMs)."""
    steps = prof["roe_eigenbasis"][0] if "roe_eigenbasis" in prof else 1
    per_update = sum(FP64_PIPE_PER_CELL.get(k, 0.) * v[0] / steps for k, v in prof.items())
    achieved = per_update * value
    return per_update, achieved, achieved / fp64_peak


def summary_block(value, e2e, roofline, batched, adjoint, fused=None):
    """The headline numbers in a few keys, placed last in the JSON line."""
    out = {"value": value, "e2e": e2e["value"] if e2e else None,
           "fused_stage_ms_per_step": fused["ms_per_step"] if fused else None,
           "fp64_frac": roofline["frac"], "hbm_frac_dominant_kernel": roofline["hbm"]["frac"],
           "hbm_frac_step": roofline["hbm_step"]["frac"]}
    if batched:
        out["batched_ms_per_step"] = batched["batched"]["ms_per_step"]
        out["plain_sequential_ms_per_step"] = batched["plain_sequential"]["ms_per_step"]
        out["plain_interleaved_ms_per_step"] = batched["plain_interleaved"]["ms_per_step"]
        out["batched_speedup_vs_plain_sequential"] = batched["speedup_vs_plain_sequential"]
        out["batched_speedup_vs_plain_interleaved"] = batched["speedup_vs_plain_interleaved"]
    if adjoint:
        out["adjoint_over_forward"] = adjoint["adjoint_over_forward"]
        out["adjoint_over_plain_forward"] = adjoint["adjoint_over_plain_forward"]
        tp = adjoint.get("taped")
        if tp and "unavailable" not in tp:
            out["taped_adjoint_over_plain_forward"] = tp["adjoint_over_plain_forward"]
            out["taped_gradient_over_plain_forward"] = tp["gradient_over_plain_forward"]
        fd = adjoint.get("finite_differences")
        if fd:
            out["fd_within_1e-6"] = "%d/%d" % (fd["within_1e-6"], fd["directions"])
            out["fd_rel_err_median"] = fd["rel_err_median"]
        fds = (adjoint.get("finite_differences_differentiable") or {}).get("eps_1e-06")
        if fds:
            out["fd_differentiable_within_1e-6"] = "%d/%d" % (fds["within_1e-6"], fds["directions"])
    return out


def run_gb300(args):
    from hydrodynamicsgpu_gb300.replicas import Replicas
    reps = Replicas()
    rank, local_rank, world = reps.rank, reps.local_rank, reps.world
    import hydrodynamicsgpu_gb300 as hg
    from hydrodynamicsgpu_gb300 import _abi, initconds as ic
    if not os.path.exists(hg.LIB_PATH):
        import __graft_entry__
        __graft_entry__.build()
    hg.select_device(local_rank)

    size = args.size
    cfg = workload_config(_abi, size)
    init = ic.kelvin_helmholtz(size=(size, size), seed=0).reshape(-1)
    solver = hg.Solver(cfg)
    solver.resetState(init)
    interior = (size - 4) * (size - 4)

    barrier = reps.barrier
    max_over_ranks = reps.max

    # warm-up (also captures the CUDA graph of one step)
    solver.update(args.warmup, want_dt=False)
    solver.synchronize()

    # ---- timed region: K graph replays, CUDA events on the solver's stream ----
    clocks = ClockSampler(local_rank)
    clocks.start()
    time.sleep(0.3)
    barrier()
    solver.synchronize()
    ms = solver.timed_update(args.steps)
    solver.synchronize()
    barrier()
    clk = clocks.stop()
    ms = max_over_ranks(ms)
    kernels_per_step = solver.kernels_per_step()
    ms_per_step = ms / args.steps
    value = interior * args.steps * world / (ms * 1e-3)
    health = solver.health()

    # ---- per-kernel breakdown (plain launches, events around each launch) ----
    prof = solver.profile(2)
    dominant = max(prof.items(), key=lambda kv: kv[1][1])
    dom_name, (dom_launches, dom_total) = dominant
    dom_ms = dom_total / dom_launches
    peak_gbs, peak_kind = measured_peaks()
    bytes_per_launch = algorithmic_bytes_per_cell(dom_name) * interior
    achieved_gbs = bytes_per_launch / (dom_ms * 1e-3) / 1e9
    fp64_peak = hg.fp64_peak()
    traffic = MEASURED_TRAFFIC_PER_CELL.get(dom_name)
    per_update, fp64_achieved, fp64_frac = fp64_roofline(prof, value / world, fp64_peak)
    step_bytes = 17 * N_STATES * 8          # compulsory bytes of an RK4 cell-update (17 state arrays)
    step_gbs = step_bytes * value / world / 1e9
    roofline = {"bound": "fp64", "kernel": "the whole step (each of its kernels is FP64-issue-bound)",
                "achieved": fp64_achieved, "peak": fp64_peak, "unit": "FP64-unit instructions/s",
                "frac": fp64_frac, "peak_source": "hgpu_fp64_peak measured in this run (FMA issue rate, all SMs)",
                "fp64_inst_per_cell_update": per_update,
                "traffic": traffic * interior if traffic else None, "traffic_kernel": dom_name,
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum per interior cell at 1024^2, "
                                  "scaled by interior cells",
                "hbm": {"kernel": dom_name, "achieved": achieved_gbs, "peak": peak_gbs, "unit": "GB/s",
                        "frac": achieved_gbs / peak_gbs, "peak_source": peak_kind,
                        "algorithmic_bytes_per_launch": bytes_per_launch, "avg_launch_ms": dom_ms},
                "hbm_step": {"bytes_per_cell_update": step_bytes, "achieved": step_gbs, "peak": peak_gbs,
                             "unit": "GB/s", "frac": step_gbs / peak_gbs}}
    breakdown = {k: {"launches": v[0], "ms_per_launch": v[1] / v[0], "share": v[1] / sum(x[1] for x in prof.values())}
                 for k, v in prof.items()}

    # ---- the same step with each stage as the two fused per-direction kernels (opt-in
    # path, hgpu_set_fused_stages; same bits) ----
    fused = None
    if rank == 0 and world == 1:
        fs = hg.Solver(cfg)
        fs.set_fused_stages(True)
        fs.resetState(init)
        fs.update(args.warmup, want_dt=False)
        fms = fs.timed_update(args.steps) / args.steps
        fs.close()
        fused = {"ms_per_step": fms, "value": interior / (fms * 1e-3), "unit": UNIT,
                 "vs_default": ms_per_step / fms, "kernels": "x pass + y pass per stage (roe_fused.cu)"}

    # ---- e2e through the C ABI: hgpu_update_host per step = H2D from pinned host, the
    # step, D2H to pinned host and the dt read, the copies overlapped in bands ----
    e2e = None
    if not args.no_e2e:
        n = solver.count
        host_in = hg.PinnedArray(n, np.float64)
        host_out = hg.PinnedArray(n, np.float64)
        host_in.array[:] = init
        e2e_solver = hg.Solver(cfg)
        for _ in range(args.warmup):
            e2e_solver.update_host(host_in.array, 1, out=host_out.array)
        e2e_solver.synchronize()
        barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            e2e_solver.update_host(host_in.array, 1, out=host_out.array)   # H2D, step, D2H, dt (8 B)
        el = time.perf_counter() - t0
        barrier()
        el = max_over_ranks(el)
        e2e = {"value": interior * args.steps * world / el, "unit": UNIT,
               "h2d_bytes_per_step": n * 8, "d2h_bytes_per_step": n * 8 + 8,
               "ms_per_step": el / args.steps * 1e3, "api": "hgpu_update_host (host wall clock)"}
        e2e_solver.close()
        host_in.free()
        host_out.free()

    # ---- CPU baseline (rank 0, N=1 only) ----
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu, _ = cpu_sample(size)

    batched = adjoint = fp32 = gravity = None
    if rank == 0 and world == 1:
        fp32 = fp32_measure(hg, _abi, ic, args)
    if rank == 0 and world == 1 and not args.no_batch:
        batched = batched_sweep(hg, _abi, ic, args)
    if rank == 0 and world == 1 and not args.no_adjoint:
        adjoint = adjoint_measure(hg, _abi, ic, args)
    if rank == 0 and world == 1 and not args.no_gravity:
        gravity = gravity_measure(hg, _abi, ic, args)

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded KH shear layer, random-phase noise)",
        "config": {"workload": workload_name(size), "grid": [size, size], "solver": "EulerRoe",
                   "integrator": "RungeKutta4", "limiter": "MinMod", "boundary": "periodic",
                   "interior_cells": interior, "parallelism": "replicas" if world > 1 else "single GPU",
                   "l2": "inputs larger than L2 (state 134 MB, eigenbasis 1.14 GB, fluxes 268 MB per step)"},
        "roofline": roofline,
        "kernels": breakdown,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "clocks": clk,
        "fp32": fp32,
        "fused_stage": fused,
        "self_gravity": gravity,
        "adjoint": adjoint,
        "batched_sweep": batched,
        "gpu_launches": kernels_per_step * args.steps,
        "health_flags": health,
        "summary": summary_block(value, e2e, roofline, batched, adjoint, fused),
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    solver.close()
    reps.close()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    return run_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
