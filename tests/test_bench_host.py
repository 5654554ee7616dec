"""bench.py's host logic, without a GPU: the figures it reads from the committed ncu summaries,
the clock-sample summary, workload selection, the oracle CPU baseline on a bounded sample, and the
reference arm's JSON line (every key of the line contract)."""
import json
import types

import pytest

import bench


@pytest.fixture
def small_workload():
    bench.select_workload("small")
    yield
    bench.select_workload("frame1080")


def test_profile_figures():
    assert bench._traffic("1080p") > 0
    assert 10 < bench._profile_figure("1080p", "warp instructions per point") < 40
    assert bench._profile_figure("tcgen05", "dram bytes per launch", "gemm_%s.md") > 1e9
    assert bench._profile_figure("no_such_workload", "dram bytes per launch") is None


def test_clock_summary_reasons_and_unsampled():
    c = bench.ClockSampler(0)
    c.lines = ["0, 2070, 2070, 950.1, 0x4, Not Active, Not Active, Not Active, Active",
               "0, 2055, 2070, 990.3, 0x0, Not Active, Not Active, Not Active, Not Active",
               "not a sample line"]
    s = c.summary()
    assert s["samples"] == 2 and s["sm_max_mhz"] == 2070.0 and s["reasons"] == ["sw_power_cap"]
    assert 2055.0 <= s["sm_mhz"] <= 2070.0
    assert bench.ClockSampler(0).summary()["reasons"] == ["unsampled"]


def test_select_workload_sets_the_config():
    try:
        for key, wl in bench.WORKLOADS.items():
            bench.select_workload(key)
            assert bench.CONFIG_NAME == wl["name"] and bench.GENOME == wl["genome"]
            assert (bench.W, bench.H) == (wl["out"][0] * wl["ss"], wl["out"][1] * wl["ss"])
    finally:
        bench.select_workload("frame1080")
    assert (bench.W, bench.H) == (3840, 2160) and bench.POINTS == 1000 * 3840 * 2160


def test_cpu_baseline_bounded_sample(rk, compiler, small_workload):
    xml = rk.Flame.synthesize(compiler, 0, 0, bench.W, bench.H).to_xml()
    v, threads, sample, dt = bench.cpu_baseline(xml, seconds=0.2, threads=2)
    assert v > 0 and threads == 2 and "walkers" in sample and 0 < dt < 30


def test_reference_arm_line(rk, monkeypatch, capsys, small_workload):
    # the timed oracle sample is stubbed: this checks the line, not the oracle's speed
    monkeypatch.setattr(bench, "cpu_baseline", lambda xml, seconds=0, threads=None: (0.05, 4, "stub sample", 1.0))
    assert bench.run_reference(types.SimpleNamespace(steps=2, warmup=1)) == 0
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["impl"] == "reference" and line["value"] == 0.05 and line["unit"] == "Gpoints/s"
    assert line["cpu_baseline"] == {"value": 0.05, "unit": "Gpoints/s", "cores": 4, "kind": "port",
                                    "sample": "stub sample"}
    assert line["e2e"] == {"value": 0.05, "unit": "Gpoints/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert line["config"]["workload"] == bench.WORKLOADS["small"]["name"] and "seed 0" in line["data"]
    assert line["ms_per_step"] == pytest.approx(65536 * 256 / 0.05e9 * 1e3)
