"""The denoiser's per-tile fallback policy (host logic, no GPU): the worst tiles by estimated
error are replaced by plain accumulation until the estimated image relMSE fits the budget;
tiles not worse than the target are never replaced."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")


def pipeline(err4, h, w, tile):
    from yapt_gb300.denoise import DenoisePipeline
    p = object.__new__(DenoisePipeline)
    p.h, p.w, p.tile = h, w, tile
    p.tile_err = torch.tensor(np.asarray(err4, np.float32) / 4.0)  # the kernel stores a quarter
    return p


def test_no_fallback_when_the_estimate_fits():
    p = pipeline([2e-4] * 6, 128, 192, 64)
    assert p.fallback_tiles(1e-3, 0.5).sum() == 0


def test_one_bad_tile_is_replaced():
    p = pipeline([1e-4, 1e-4, 5e-2, 1e-4, 1e-4, 1e-4], 128, 192, 64)
    assert p.fallback_tiles(1e-3, 0.5).tolist() == [0, 0, 1, 0, 0, 0]


def test_worst_first_until_the_budget_and_never_below_the_target():
    err = [3e-3, 2e-3, 1.5e-3, 9e-4, 9e-4, 9e-4]
    p = pipeline(err, 128, 192, 64)
    f = p.fallback_tiles(1e-3, 0.5)
    assert f[0] == 1 and f[1] == 1  # worst first
    assert np.all(f[3:] == 0)  # at or below the target: kept
    # ragged edge tiles weigh by their pixel count: the small tile is replaced after the big one
    p = pipeline([5e-3, 5e-3], 64, 80, 64)  # 64x64 and 64x16 pixels
    f = p.fallback_tiles(1e-3, 2.0)  # after the big tile: (1e-3 * 4096 + 5e-3 * 1024) / 5120 = 1.8e-3
    assert f.tolist() == [1, 0]
