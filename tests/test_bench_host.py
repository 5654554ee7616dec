"""bench.py's host logic, without a GPU: the figures it reads from the committed ncu summaries,
the clock-sample summary, workload selection, the oracle CPU baseline on a bounded sample, and the
reference arm's JSON line (every key of the line contract)."""
import json
import os
import subprocess
import sys
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


def test_cpu_baseline_bounded_sample(small_workload):
    v, threads, sample, dt, vb = bench.cpu_baseline(bench.genome_xml(), seconds=0.2, threads=2)
    assert v > 0 and threads == 2 and "walkers" in sample and 0 < dt < 30 and 0 < vb <= v


def test_reference_arm_line(monkeypatch, capsys, small_workload):
    # the timed oracle sample is stubbed: this checks the line, not the oracle's speed
    monkeypatch.setattr(bench, "cpu_baseline",
                        lambda xml, seconds=0, threads=None, reset=True: (0.05, 4, "stub sample", 1.5, 0.04))
    assert bench.run_reference(types.SimpleNamespace(steps=2, warmup=1, no_badval_reset=False)) == 0
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["impl"] == "reference" and line["value"] == 0.05 and line["unit"] == "Gpoints/s"
    assert line["cpu_baseline"] == {"value": 0.05, "unit": "Gpoints/s", "cores": 4, "kind": "port",
                                    "sample": "stub sample"}
    assert line["e2e"] == {"value": 0.05, "unit": "Gpoints/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    # the same workload definition as the native arm's line, read from the same genome file
    assert line["config"] == bench.workload_config(True)
    assert line["config"]["workload"] == bench.WORKLOADS["small"]["name"] and "small.flam3" in line["data"]
    assert line["ms_per_step"] == pytest.approx(1500.0) and line["binned_gpoints_s"] == 0.04


def test_reference_arm_does_not_load_the_library(tmp_path):
    """The reference arm runs the oracle only: it never imports the product package."""
    code = ("import sys, types, bench\n"
            "bench.select_workload('small')\n"
            "bench.cpu_baseline = lambda xml, seconds=0, threads=None, reset=True: (0.05, 1, 's', 1.0, 0.04)\n"
            "bench.run_reference(types.SimpleNamespace(steps=1, warmup=0, no_badval_reset=False))\n"
            "assert 'refrakt_gb300' not in sys.modules, 'product package imported'\n")
    r = subprocess.run([sys.executable, "-c", code], cwd=bench.ROOT, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr


def test_genome_fixtures_match_the_synthesiser(rk, compiler):
    """tests/golden/genomes/ holds what the library's seeded synthesiser writes (make_genomes.py)."""
    sys.path.insert(0, os.path.join(bench.ROOT, "tests", "golden"))
    import make_genomes
    for name, xml in make_genomes.synthesize_all(rk, compiler).items():
        with open(os.path.join(bench.GENOME_DIR, name + ".flam3")) as f:
            assert f.read() == xml, name


def test_algorithmic_operation_count():
    bench.select_workload("frame1080")
    ops, calls = bench.algorithmic_ops_per_point(bench.genome_xml())
    # affine, colour and screen affine alone are 11 operations; julian / ngon / pdj call pow,
    # atan2, sin, cos
    assert 20 < ops < 200 and 1 < calls < 30
    small_ops, small_calls = bench.algorithmic_ops_per_point(
        '<flame size="8 8" scale="1"><xform weight="1" color="0" coefs="1 0 0 1 0 0" linear="1"/></flame>')
    assert small_calls == 0 and small_ops == 4 + 3 + 2 + 4


def test_fit_splat_tile():
    import numpy as np
    h = np.zeros((100, 200), np.int32)
    h[40:50, 120:135] = 3
    assert bench.fit_splat_tile(h, 1000) == (120, 40, 15, 10)
    h[0, 0] = 1  # a stray hit: the box no longer fits, the square around the densest bin is taken
    x0, y0, w, hh = bench.fit_splat_tile(h, 100)
    assert w == hh == 10 and x0 <= 120 <= x0 + w and y0 <= 40 <= y0 + hh
    assert bench.fit_splat_tile(np.zeros((4, 4)), 100) == (0, 0, 0, 0)
    assert bench.splat_tile_capacity(2048) > 5000 and bench.splat_tile_capacity(4096) > 500
