"""bench.py's arithmetic and line layout, checked without a GPU: the FP64 roofline's
instructions per cell-update, the finite-difference statistics, the clock summary and
the summary block placed last in the JSON line."""
import importlib.util
import os

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(REPO, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def kh_rk4_profile(steps=2):
    """launches of each kernel of `steps` KH RK4 steps (as Solver.profile reports them)"""
    per_step = {"boundary": 2, "roe_eigenbasis": 1, "cfl_min_reduce": 1, "finalize_dt": 1, "roe_delta_q_tilde": 4,
                "roe_flux": 4, "flux_divergence_combine": 4, "state_check": 1}
    return {k: (n * steps, 0.1) for k, n in per_step.items()}


def test_fp64_roofline_counts_the_rk4_step(bench):
    per_update, achieved, frac = bench.fp64_roofline(kh_rk4_profile(), 5.0e8, 5.0e11)
    t = bench.FP64_PIPE_PER_CELL
    expect = (t["roe_eigenbasis"] + t["cfl_min_reduce"] + t["state_check"]
              + 4 * (t["roe_delta_q_tilde"] + t["roe_flux"] + t["flux_divergence_combine"]))
    assert per_update == pytest.approx(expect)
    assert per_update == pytest.approx(763.12, abs=0.01)
    assert achieved == pytest.approx(per_update * 5.0e8)
    assert frac == pytest.approx(achieved / 5.0e11)
    # the profile's step count divides out
    assert bench.fp64_roofline(kh_rk4_profile(steps=5), 5.0e8, 5.0e11)[0] == pytest.approx(per_update)


def test_fd_stats(bench):
    pairs = [(1.0, 1.0), (1.0, 1.0 + 2e-7), (2.0, 2.2), (-1.0, -1.0)]
    st = bench.fd_stats(pairs, 1e-6)
    assert st["directions"] == 4
    assert st["within_1e-6"] == 3


def test_clock_summary_flags_throttling(bench):
    c = bench.ClockSampler(0)
    c.proc = None
    assert c.stop()["reasons"] == ["nvidia-smi unavailable"]

    class Done:
        def terminate(self):
            pass

        def wait(self, timeout=None):
            return 0

    c.proc = Done()
    c.lines = ["0, 2070, 2070, 900.1, 0x0, Not Active, Not Active, Not Active, Not Active",
               "0, 1980, 2070, 1400.0, 0x4, Not Active, Not Active, Not Active, Active",
               "0, 2070, 2070, 1395.2, 0x0, Active, Not Active, Not Active, Not Active"]
    out = c.stop()
    assert out["sm_mhz"] == 2070.0 and out["sm_max_mhz"] == 2070.0 and out["samples"] == 3
    assert out["reasons"] == ["hw_slowdown", "sw_power_cap"]


def test_summary_block_keys(bench):
    roof = {"frac": 0.78, "hbm": {"frac": 0.25}, "hbm_step": {"frac": 0.04}}
    batched = {"batched": {"ms_per_step": 22.0}, "plain_sequential": {"ms_per_step": 73.0},
               "plain_interleaved": {"ms_per_step": 26.4}, "speedup_vs_plain_sequential": 3.3,
               "speedup_vs_plain_interleaved": 1.2}
    adjoint = {"adjoint_over_forward": 2.93, "adjoint_over_plain_forward": 2.96,
               "taped": {"adjoint_over_plain_forward": 1.85, "gradient_over_plain_forward": 3.01},
               "finite_differences": {"within_1e-6": 0, "directions": 64, "rel_err_median": 6e-4},
               "finite_differences_differentiable": {"eps_1e-06": {"within_1e-6": 7, "directions": 8}}}
    out = bench.summary_block(5.4e8, {"value": 5.2e8}, roof, batched, adjoint, {"ms_per_step": 9.3})
    assert out["value"] == 5.4e8 and out["e2e"] == 5.2e8 and out["fp64_frac"] == 0.78
    assert out["batched_speedup_vs_plain_sequential"] == 3.3
    assert out["taped_adjoint_over_plain_forward"] == 1.85
    assert out["fd_within_1e-6"] == "0/64" and out["fd_differentiable_within_1e-6"] == "7/8"


def test_summary_block_without_taped_adjoint(bench):
    roof = {"frac": 0.78, "hbm": {"frac": 0.25}, "hbm_step": {"frac": 0.04}}
    adjoint = {"adjoint_over_forward": 2.93, "adjoint_over_plain_forward": 2.96,
               "taped": {"unavailable": "the tapes of every step do not fit in device memory"}}
    out = bench.summary_block(5.4e8, None, roof, None, adjoint)
    assert out["adjoint_over_plain_forward"] == 2.96
    assert "taped_adjoint_over_plain_forward" not in out
    assert out["e2e"] is None
