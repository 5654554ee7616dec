"""Edge cases of the drawing path through the C ABI: zero passes, a one-bin grid, a grid of the
maximum width, drawing before warm-up, walker counts that do not fill the shuffle domain, a
genome edit that forces a new warm-up, and repeated draw calls accumulating exactly."""
import numpy as np
import pytest
import torch

from test_gpu_parity import LINEAR, _bins

pytestmark = pytest.mark.gpu


def test_zero_passes_draw_nothing(rk, compiler):
    f = rk.Flame.from_xml(LINEAR, compiler)
    sim = rk.Sim(4096, seed=1)
    sim.warmup(f, 5)
    bins, hits = _bins(64, 64)
    assert sim.draw_to_bins(f, bins, hits, 64, 64, 0) == 0
    assert int(hits.sum()) == 0 and float(bins.abs().sum()) == 0.0


def test_one_bin_and_widest_grids(rk, compiler):
    f = rk.Flame.from_xml(LINEAR, compiler)
    sim = rk.Sim(4096, seed=2)
    sim.warmup(f, 9)
    bins, hits = _bins(1, 1)
    drawn = sim.draw_to_bins(f, bins, hits, 1, 1, 8)
    assert drawn == int(hits.sum().item())
    bins, hits = _bins(65536, 2)
    drawn = sim.draw_to_bins(f, bins, hits, 65536, 2, 4)
    assert drawn == int(hits.sum().item())


def test_errors_are_reported(rk, compiler):
    f = rk.Flame.from_xml(LINEAR, compiler)
    with pytest.raises(rk.RefraktError):
        rk.Sim(4096 + 256)  # not a multiple of the 4096-slot shuffle domain
    sim = rk.Sim(4096, seed=3)
    bins, hits = _bins(32, 32)
    with pytest.raises(rk.RefraktError):
        sim.draw_to_bins(f, bins, hits, 32, 32, 1)  # before warm-up
    sim.warmup(f, 3)
    f.set_xform_value(0, "weight", 0.7)  # an edit invalidates the warm-up, as in the reference
    assert sim.needs_warmup(f)
    with pytest.raises(rk.RefraktError):
        sim.draw_to_bins(f, bins, hits, 32, 32, 1)
    sim.warmup(f, 3)
    assert sim.draw_to_bins(f, bins, hits, 32, 32, 2) >= 0


def test_draw_calls_accumulate(rk, compiler):
    """Two draw calls of n passes bin as many points as the counters report, into the same bins."""
    f = rk.Flame.synthesize(compiler, rk.SYNTH_SMALL, 0, 128, 128)
    sim = rk.Sim(8192, seed=4)
    sim.warmup(f, 19)
    bins, hits = _bins(128, 128)
    d1 = sim.draw_to_bins(f, bins, hits, 128, 128, 10)
    h1 = hits.clone()
    d2 = sim.draw_to_bins(f, bins, hits, 128, 128, 10)
    assert int(hits.sum()) == d1 + d2 and int(h1.sum()) == d1
    assert torch.all(hits >= h1)
