"""bench.py's host-side helpers, on CPU: the algorithmic bytes of a step (the
roofline's numerator), the measured peak it is divided by, the clock summary
that decides whether a run is kept, the energy grid and the L1 error of the
time-to-DOS metric, and the single-rank paths of the rank helpers."""
import json
import os

import numpy as np
import pytest

import bench


def test_step_bytes_of_the_headline_flake():
    # nnz (column + FP32 value) + row pointers + T_{n-1}, T_n, T_{n+1} of 32 FP32 columns
    n, nnz = 9_998_234, 671_688_550
    assert bench.step_bytes(n, nnz, 32) == nnz * 8 + (n + 1) * 8 + 3 * n * 32 * 4 == 9_292_816_136


def test_peak_is_the_measured_copy_bandwidth():
    path = os.path.join(bench.REPO, "MEASURED_PEAKS.json")
    if not os.path.exists(path):
        assert bench.peaks() == (6800.0, "fallback")
        return
    with open(path) as f:
        assert bench.peaks() == (float(json.load(f)["hbm_gbs"]), "measured")


def test_clock_summary_reasons_and_median():
    c = bench.Clocks(0)
    c.lines = ["2070, 2070, 812.3, Not Active, Not Active, Not Active, Active",
               "1965, 2070, 1390.0, Not Active, Not Active, Not Active, Active",
               "2070, 2070, 901.0, Not Active, Not Active, Not Active, Not Active",
               "[N/A], 2070, 0, Not Active, Not Active, Not Active, Not Active",  # unparsable: skipped
               "garbage"]
    s = c.summary()
    assert s == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "samples": 3, "reasons": ["sw_power_cap"]}
    c.lines = ["1200, 2070, 500, Active, Not Active, Active, Not Active"]
    assert c.summary()["reasons"] == ["hw_slowdown", "sw_thermal_slowdown"]


def test_clocks_without_nvidia_smi(monkeypatch):
    monkeypatch.setenv("PATH", "/nonexistent")
    with bench.Clocks(0) as c:
        pass
    assert c.summary() == {"sm_mhz": None, "sm_max_mhz": None, "samples": 0, "reasons": []}


def test_energy_grid_and_l1():
    e = bench.energies(2.0, 0.5)
    assert e.shape == (bench.N_E,)
    np.testing.assert_allclose(e[0], 0.5 + 2.0 * (-1.0 + 1.0 / bench.N_E), rtol=1e-15)
    np.testing.assert_allclose(e + e[::-1], 1.0, rtol=1e-14)  # symmetric about the centre
    ref = np.array([1.0, 2.0, 3.0])
    assert bench.l1(ref + np.array([0.1, -0.2, 0.3]), ref) == pytest.approx(0.6 / 6.0)


def test_single_rank_helpers():
    bench.barrier(None)
    assert bench.max_over_ranks(None, 1.25) == 1.25
