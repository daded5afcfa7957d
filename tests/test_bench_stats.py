"""The effective-sample statistics of the benchmark (bench.py: tau_int, chain_stats) on
series whose integrated autocorrelation time is known: per-walker AR(1) processes
x_t = rho x_{t-1} + sqrt(1 - rho^2) e_t have tau_int = (1 + rho) / (1 - rho)."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench   # noqa: E402


def ar1(rho, rows, walkers, seed):
    rng = np.random.default_rng(seed)
    x = np.empty((rows, walkers))
    x[0] = rng.normal(size=walkers)
    s = np.sqrt(1.0 - rho * rho)
    for t in range(1, rows):
        x[t] = rho * x[t - 1] + s * rng.normal(size=walkers)
    return x


@pytest.mark.parametrize("rho", [0.0, 0.5, 0.8, 0.95])
def test_tau_int_of_ar1_processes(rho):
    x = ar1(rho, 4000, 256, seed=int(rho * 100) + 1)
    tau, window, ok = bench.tau_int(x)
    exact = (1 + rho) / (1 - rho)
    assert ok
    assert window >= 5 * tau - 1e-9 or tau == 1.0
    # Sokal's window truncates the tail: a few percent low at most for these lengths
    assert abs(tau - exact) <= 0.06 * exact + 0.05, (tau, exact)


def test_tau_int_reports_an_unconverged_window():
    # tau_int ~ 400 rows against a 300-row series: no window satisfies W >= 5 tau
    x = ar1(0.995, 300, 64, seed=3)
    tau, window, ok = bench.tau_int(x)
    assert not ok
    assert window == 299


def test_chain_stats_standard_error_matches_walker_means():
    rho, rows, walkers = 0.8, 3000, 512
    x = ar1(rho, rows, walkers, seed=11) * 2.0 - 100.0
    st = bench.chain_stats(x, [1.0] * 10, walkers, N=100)
    exact = (1 + rho) / (1 - rho)
    assert st["tau_converged"]
    assert abs(st["tau_int_rows"] - exact) <= 0.06 * exact
    # the SE from tau_int agrees with the spread of the walkers' own means
    se_tau = st["se_per_spin"] * 100
    se_walkers = x.mean(axis=0).std(ddof=1) / np.sqrt(walkers)
    assert abs(se_tau - se_walkers) <= 0.15 * se_walkers
    # ESS/s = walkers / tau / seconds per row (1 ms rows)
    assert st["ess_per_s"] == pytest.approx(walkers / st["tau_int_rows"] / 1e-3)
    assert abs(st["half_drift_in_se"]) < 4.0
    assert st["acf"][1] == pytest.approx(rho, abs=0.02)
