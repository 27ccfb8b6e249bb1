"""bench.py's host logic on the CPU: the clock / throttle-reason summary that decides whether
a bench line stands, the roofline arithmetic, and the CPU-baseline sampling (with the
oracle, on tiny samples)."""
import types

import numpy as np

import bench


def _line(sm, reasons=("Not Active",) * 4):
    return ", ".join(["0", str(sm), "2070", "850.25", "0x0000000000000000", *reasons])


def test_clock_summary_median_and_reasons():
    lines = [_line(2070), _line(2055), _line(1980, ("Not Active", "Not Active", "Not Active", "Active")),
             "garbage", "0, [N/A], 2070, 10, 0x0, Not Active, Not Active, Not Active, Not Active"]
    c = bench.ClockSampler.summarize(lines)
    assert c["samples"] == 3
    assert c["sm_mhz"] == 2055.0 and c["sm_max_mhz"] == 2070.0
    assert c["reasons"] == ["sw_power_cap"]
    hot = bench.ClockSampler.summarize([_line(1500, ("Active", "Not Active", "Active", "Not Active"))])
    assert hot["reasons"] == ["hw_slowdown", "sw_thermal_slowdown"]
    assert bench.ClockSampler.summarize([])["sm_mhz"] is None


def test_roofline_arithmetic():
    _, ka, _, _ = bench.he3_setup()
    per_node = bench.alg_ops_per_node("he3", ka)
    assert 700 < per_node < 900
    r = bench.roofline_for("he3", ka, 2.5e10, {"sm_mhz": 2000.0})
    peak = 4 * 32 * 152 * 2000.0e6 / 1e12
    assert np.isclose(r["peak"], peak) and np.isclose(r["achieved"], 2.5e10 * per_node / 1e12)
    assert np.isclose(r["frac"], r["achieved"] / peak)
    assert r["traffic"] == bench.TRAFFIC_PER_LAUNCH["he3"]
    assert bench.roofline_for("he3", ka, 2.5e10, None, default_workload=False)["traffic"] is None
    # the HO correlator (N/2 lags x N products, every sweep) dominates its count
    _, ka_ho, _, _ = bench.ho_setup()
    assert bench.alg_ops_per_node("ho", ka_ho) > 5 * (8 * (2 + 2 / 7) + 9 + 6)


def test_cpu_baseline_keeps_the_measurement_cadence():
    sysm, ka, extra, _ = bench.ho_setup()
    cb = bench.oracle_cpu_rate(sysm, ka, extra, seconds=0.2, walkers=8)
    assert cb["value"] > 0 and cb["kind"] == "port" and cb["cores"] >= 1
    assert "one measurement every 1 sweep(s)" in cb["sample"]


def test_reference_rate_falls_back_to_the_restatement():
    # the harmonic oscillator, and a configuration other than the prepared sample's, are timed
    # with the oracle's restatement, saying why
    sysm, ka, extra, _ = bench.ho_setup()
    cb = bench.reference_cpu_rate("ho", sysm, dict(ka, nbrOfWalkers=8), extra, seconds=0.2)
    assert cb["kind"] == "port" and cb["value"] > 0 and cb["reference_unavailable"]
    sysm, ka, extra, _ = bench.he3_setup(walkers=8, S=3)
    cb = bench.reference_cpu_rate("he3", sysm, ka, extra, seconds=0.2)
    assert cb["kind"] == "port" and cb["reference_unavailable"]


def test_reference_rate_times_the_prepared_reference_sample():
    import pytest
    from oracle import ref_timing
    if not ref_timing.available("he3"):
        pytest.skip("no prepared reference sample (the reference tree was absent at build time)")
    sysm, ka, extra, _ = bench.he3_setup()
    cb = bench.reference_cpu_rate("he3", sysm, ka, extra, seconds=0.5)
    assert cb["kind"] == "reference" and cb["value"] > 0, cb
    assert "reference_unavailable" not in cb


def test_batch_cpu_baseline_weights_systems_by_their_work():
    from feynsimul_gb300.batch import choose_S, ragged_workload
    from feynsimul_gb300.physical_systems.lm2m2 import Lm2m2Cluster
    wl = ragged_workload(seed=1, n_systems=3, n_range=(3, 4), N_choices=(64,), walker_range=(64, 128))
    b = types.SimpleNamespace(
        systems=[types.SimpleNamespace(bisection_level=choose_S(w["N"], 16, 256, dof=3 * (w["n"] - 1)))
                 for w in wl],
        clusters={n: Lm2m2Cluster(n, 1.0) for n in {w["n"] for w in wl}})
    cb = bench.batch_cpu_rate(wl, b, seconds=0.3, walkers=4)
    assert cb["value"] > 0 and "each of the 3 systems" in cb["sample"]
