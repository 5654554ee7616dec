"""rf_density_estimate_static: density estimation for callers that cannot allocate device memory
(a plug-in inside a host application that owns the memory pool; a frame loop on a fixed memory
budget).  Its scratch lives in static device arrays of the library; it must give the same result
as rf_density_estimate, call after call, and refuse bin grids beyond its fixed scratch.

Collected last so that, if it fails, a run that stops at the first failure has run the rest."""
import ctypes

import numpy as np
import pytest


def _entry(rk):
    lib = rk.library()
    fn = lib.rf_density_estimate_static
    fn.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int, ctypes.c_int, ctypes.c_float,
                   ctypes.c_void_p, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    return fn


def test_static_scratch_refuses_oversized_grids(rk):
    # the size checks come before any device work, so they need no GPU
    fn = _entry(rk)
    dummy = ctypes.c_void_p(16)
    out = ctypes.c_void_p(32)
    rc = fn(dummy, 4096, 4096, 9, 0, 0.4, out, None)
    assert rc == 5  # RF_ERR_CAPACITY
    assert b"static scratch" in rk.library().rf_last_error()
    # within the bin budget but taller than a launch grid can cover
    rc = fn(dummy, 8, 1000000, 9, 0, 0.4, out, None)
    assert rc == 5 and b"rows" in rk.library().rf_last_error()


@pytest.mark.gpu
def test_static_scratch_matches_allocating_entry_point(rk, compiler):
    import torch
    fn = _entry(rk)
    results = []
    # shared-memory tiles (R <= 12) and the global-memory gather (R = 20; R = 100 reads the last
    # entries of the weight table); a large grid before smaller ones, so a later call that read
    # radii the earlier one left behind would differ
    for W, H, seed, R, mn, curve in [(640, 480, 3, 9, 0, 0.4), (256, 192, 1, 9, 0, 0.4), (320, 200, 2, 5, 1, 0.6),
                                     (64, 48, 4, 20, 0, 0.3), (64, 48, 5, 100, 0, 0.4), (96, 64, 6, 100, 100, 0.4)]:
        f = rk.Flame.synthesize(compiler, rk.SYNTH_SMALL, seed, W, H)
        sim = rk.Sim(16384, seed=seed)
        sim.warmup(f, 19)
        bins = torch.zeros(H, W, 4, device="cuda")
        hits = torch.zeros(H, W, dtype=torch.int32, device="cuda")
        sim.draw_to_bins(f, bins, hits, W, H, 16)
        sim.close()
        want = torch.zeros_like(bins)
        rk.density_estimate(bins, W, H, R, mn, curve, want)
        got = torch.full_like(bins, -1.0)
        rc = fn(ctypes.c_void_p(bins.data_ptr()), W, H, R, mn, curve, ctypes.c_void_p(got.data_ptr()), None)
        assert rc == 0, rk.library().rf_last_error()
        torch.cuda.synchronize()
        g, w = got.cpu().numpy(), want.cpu().numpy()
        assert np.allclose(g, w, rtol=2e-5, atol=1e-6)
        results.append(g)
    assert results[0].shape != results[1].shape
    assert len({r.shape for r in results}) == 5
