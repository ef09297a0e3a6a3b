"""bench.py without a GPU: the reference arm (`--impl reference`) and the
roofline arithmetic of the main arm.  The reference arm's timed host steps
are replaced by fixed durations so that no 2048^2 step runs here; its line
must carry the keys the contract names (impl, metric, value, unit, steps,
warmup, ms_per_step, config, cpu_baseline with its kind, cores and sample,
an e2e block without host-device bytes), and ranks other than 0 print
nothing."""
import argparse
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _args(**kw):
    a = dict(gpus=1, steps=20, warmup=3, cpu_steps=2, cpu_budget=30.0)
    a.update(kw)
    return argparse.Namespace(**a)


def _bench(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench

    calls = []

    def fake_steps(steps, threads, warmup=0, budget_s=None):
        calls.append((steps, threads, warmup, budget_s))
        return [4.0] * steps

    monkeypatch.setattr(bench, "cpu_reference_steps", fake_steps)
    return bench, calls


def test_reference_arm_line(monkeypatch, capsys):
    bench, calls = _bench(monkeypatch)
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    bench.run_reference(_args())
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    (steps, threads, warmup, budget), = calls
    assert steps == 2 and warmup == 3 and budget == 30.0 and threads == (os.cpu_count() or 1)
    assert line["impl"] == "reference"
    assert line["metric"] == bench.METRIC and line["unit"] == "Mcell-steps/s"
    assert line["steps"] == 2 and line["warmup"] == 3 and line["higher_is_better"] is True
    assert abs(line["ms_per_step"] - 4000.0) < 1e-9
    assert abs(line["value"] - bench.W * bench.H / 4.0 / 1e6) < 1e-12
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] == threads and cb["value"] == line["value"]
    assert "sample" in cb and cb["unit"] == line["unit"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["unit"] == line["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
    assert "workload" in line["config"]


def test_reference_arm_warmup_and_steps_are_bounded(monkeypatch, capsys):
    bench, calls = _bench(monkeypatch)
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    bench.run_reference(_args(steps=1, warmup=50, cpu_steps=9))
    (steps, _, warmup, _), = calls
    assert steps == 2 and warmup == 10  # at least 2 timed steps, at most 10 warm-up steps
    capsys.readouterr()


def test_reference_arm_other_ranks_print_nothing(monkeypatch, capsys):
    bench, calls = _bench(monkeypatch)
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("LOCAL_RANK", "1")
    bench.run_reference(_args(gpus=2))
    assert calls == [] and capsys.readouterr().out == ""


def test_step_roofline_arithmetic():
    """The step roofline sums every stage's compulsory bytes per cell (597 B at
    200 sweeps in 8-sweep phases) over the device-timed step, and each stage's
    over its own time; fractions are of the given peak."""
    sys.path.insert(0, ROOT)
    import bench

    n = 2050 * 2050
    stages = {"pressure setup": 0.024, "jacobi sweeps": 0.44, "advect velocity": 0.105,
              "sources+viscosity": 0.01}
    r = bench.step_roofline(stages, n, 0.75, 6759.6)
    assert r["bytes_per_cell"] == 597 == sum(bench.STAGE_BYTES_PER_CELL.values())
    assert abs(r["achieved"] - 597 * n / 0.75e-3 / 1e9) < 1e-6
    assert abs(r["frac"] - r["achieved"] / 6759.6) < 1e-12
    # (a stage of 0 compulsory bytes has no fraction)
    assert set(r["stages"]) == {"pressure setup", "jacobi sweeps", "advect velocity"}
    js = r["stages"]["jacobi sweeps"]
    assert js["bytes_per_cell"] == 16 * 25 and abs(js["gbs"] - 400 * n / 0.44e-3 / 1e9) < 1e-6


def test_jacobi_roofline_is_an_hbm_fraction_and_issue_is_bounded():
    """The dominant kernel's `frac` counts 16 compulsory bytes per cell per
    8-sweep phase over the phase time: at the measured 17.4 us per phase it is
    an HBM fraction below 1, while the per-sweep model (13 B per cell-sweep)
    is reported beside it, above the peak, and not as `frac`; the issue
    fraction from the committed ncu instruction count stays below 1."""
    sys.path.insert(0, ROOT)
    import bench

    n = 2050 * 2050
    tr = bench.committed_traffic()
    r = bench.jacobi_roofline(n, 0.0174, 6759.6, "measured", tr,
                              {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0})
    assert abs(r["achieved"] - 16 * n / 17.4e-6 / 1e9) < 1e-6
    assert 0.3 < r["frac"] < 1.0
    assert r["per_sweep_model"]["ratio_to_peak"] > 1.0
    assert r["bytes_per_launch"] == 16 * n
    if tr and tr.get("warp_inst_per_phase"):
        assert 0.0 < r["issue"]["frac"] < 1.0


def test_clock_summary_reports_active_throttle_reasons():
    """The clocks block of the bench line: the median SM clock of the samples
    taken during the timed region, the maximum clock, and every throttle
    reason seen active in any sample (malformed or unavailable lines are
    skipped)."""
    sys.path.insert(0, ROOT)
    import bench

    s = bench.ClockSampler(0)
    s.lines = [
        "2070, 2070, 910.2, Not Active, Not Active, Not Active, Not Active",
        "2055, 2070, 1380.0, Not Active, Not Active, Not Active, Active",
        "1980, 2070, 1400.0, Not Active, Not Active, Not Active, Active",
        "[N/A], 2070, 0, Not Active, Not Active, Not Active, Not Active",
        "garbage",
    ]
    c = s.summary()
    assert c["samples"] == 3 and c["sm_mhz"] == 2055 and c["sm_max_mhz"] == 2070
    assert c["reasons"] == ["sw_power_cap"]
    s.lines = ["2070, 2070, 900, Not Active, Active, Not Active, Not Active"]
    assert s.summary()["reasons"] == ["hw_thermal_slowdown"]
    s.lines = []
    assert s.summary() == {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
