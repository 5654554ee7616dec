"""The learned density estimator's host-side helpers (refrakt_gb300/learned.py), without a GPU:
the plain-path equivalent by log-log interpolation, the sample-count feature channel, the L1
metric, and the training / held-out genome generator."""
import math

import pytest
import torch

from refrakt_gb300 import learned as LD


def test_plain_equivalent_spp():
    spps = [16, 64, 256, 1024]
    errs = [0.16, 0.08, 0.04, 0.02]  # error halves per 4x samples
    assert abs(LD.plain_equivalent_spp(spps, errs, 0.04) - 256) < 1e-6
    assert abs(LD.plain_equivalent_spp(spps, errs, 0.0565685) - 128) < 0.1
    # unordered input and errors outside the measured range clamp to its ends
    assert abs(LD.plain_equivalent_spp(spps[::-1], errs[::-1], 0.08) - 64) < 1e-6
    assert LD.plain_equivalent_spp(spps, errs, 1.0) == pytest.approx(16)
    assert LD.plain_equivalent_spp(spps, errs, 1e-4) == pytest.approx(1024)


def test_level_channel():
    assert LD.level(1) == 0.0
    assert LD.level(16) == pytest.approx(0.4)
    assert LD.level(1024) == pytest.approx(1.0)
    assert LD.level(125) == pytest.approx(math.log2(125) / 10)


def test_l1_per_image():
    a = torch.zeros(3, 4, 4, 3)
    b = torch.zeros(3, 4, 4, 3)
    b[1] += 0.5
    b[2, 0, 0, 0] = 4.8  # one of 48 values
    assert torch.allclose(LD.l1(a, b), torch.tensor([0.0, 0.5, 0.1]))


@pytest.mark.parametrize("seed", [1000, 1005, 3199])
def test_genome_generator(rk, compiler, seed):
    f = LD.genome(rk, compiler, seed, 512, 512)
    i = f.info()
    assert i["num_xforms"] == 2 + seed % 11 and i["has_final"]
    assert (i["estimator_radius"], i["estimator_min"]) == (LD.DE[0], LD.DE[1])
    assert i["estimator_curve"] == pytest.approx(LD.DE[2])
    # the same seed gives the same genome
    assert LD.genome(rk, compiler, seed, 512, 512).to_xml() == f.to_xml()
