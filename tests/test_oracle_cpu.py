"""CPU oracle checks (no GPU): determinism, precision agreement, estimator agreement."""
import numpy as np
import pytest

from yapt_gb300 import configs
from yapt_gb300.runtime import Context


@pytest.fixture(scope="module")
def box(host_luts):
    import pyoracle
    sc = configs.box_scene(0)
    return sc, pyoracle.OracleSceneHandle(sc, host_luts)


def test_oracle_is_deterministic_and_thread_independent(box):
    _, h = box
    p = Context.params("nee", 24, 24, spp=2, max_depth=8, lambda_range=(380, 780))
    a = h.render(p, precision=32, threads=1)["records"]
    b = h.render(p, precision=32, threads=7)["records"]
    assert np.array_equal(a, b)


def test_fp32_and_fp64_oracles_agree_per_sample(box):
    _, h = box
    p = Context.params("nee", 24, 24, spp=2, max_depth=8, lambda_range=(380, 780))
    a = h.render(p, precision=32)["records"][..., 1:5]
    b = h.render(p, precision=64)["records"][..., 1:5]
    rel = np.abs(a - b) / np.maximum(np.abs(b), 1e-6)
    # FP32 vs FP64 of the same paths: almost all agree closely; a few branch flips may differ
    assert np.mean(rel < 1e-3) > 0.995


def test_uni_and_nee_estimate_the_same_image(box):
    _, h = box
    pu = Context.params("uni", 16, 16, spp=256, max_depth=8, lambda_range=(380, 780))
    pn = Context.params("nee", 16, 16, spp=256, max_depth=8, lambda_range=(380, 780))
    fu = h.render(pu, precision=32, records=False, film=True)["film"]
    fn = h.render(pn, precision=32, records=False, film=True)["film"]
    # whole-image Y agrees within the noise of the unidirectional estimator
    assert abs(fu[..., 1].mean() - fn[..., 1].mean()) / fn[..., 1].mean() < 0.08


def test_empty_scene_and_black_env_give_zero(host_luts):
    import pyoracle
    sc = configs.box_scene(0)
    sc.instances = []
    h = pyoracle.OracleSceneHandle(sc, host_luts)
    p = Context.params("uni", 8, 8, spp=1, max_depth=4)
    assert np.all(h.render(p)["records"][..., 1:] == 0)


def test_oracle_bdpt_is_deterministic_and_thread_independent(box):
    _, h = box
    p = Context.params("bdpt", 24, 24, spp=2, max_depth=8, lambda_range=(380, 780), light_vertices=8)
    a = h.render(p, precision=32, threads=1)["records"]
    b = h.render(p, precision=32, threads=5)["records"]
    assert np.array_equal(a, b)
    assert np.all(np.isfinite(a)) and a[..., 6].mean() > 0


def test_oracle_bdpt_and_nee_estimate_the_same_image_in_fp64(box):
    # diffuse box, regularisation off, depth large enough that truncation is negligible:
    # the bidirectional and the NEE estimators converge to the same image
    _, h = box
    kw = dict(max_depth=24, regularize=False, lambda_range=(380, 780))
    W = H = 16
    spp = 192
    nee = h.render(Context.params("nee", W, H, spp=spp, **kw), precision=64)["records"][..., 6].astype(np.float64)
    bd = h.render(Context.params("bdpt", W, H, spp=spp, **kw), precision=64)["records"][..., 6].astype(np.float64)
    for b in (8,):
        mn = nee.reshape(spp, H // b, b, W // b, b).mean(axis=(2, 4))
        mb = bd.reshape(spp, H // b, b, W // b, b).mean(axis=(2, 4))
        se = np.sqrt(mn.var(axis=0, ddof=1) / spp + mb.var(axis=0, ddof=1) / spp)
        z = np.abs(mn.mean(axis=0) - mb.mean(axis=0)) / se
        assert z.max() < 5.0, (z.max(), mn.mean(), mb.mean())
    assert abs(bd.mean() - nee.mean()) / nee.mean() < 0.03


def test_oracle_generates_the_same_tables_as_the_library(built):
    """The oracle library builds its own copy of the precomputed tables, so the timed CPU
    baseline loads no GPU library; the copies equal the library's bit for bit."""
    import pyoracle
    from yapt_gb300 import _native as N
    for name in pyoracle.LUT_NAMES + ["sobol"]:
        assert np.array_equal(pyoracle.host_table(name), N.host_table(name)), name
    assert np.array_equal(pyoracle.host_table("rgb_to_spd", (380, 780)), N.host_table("rgb_to_spd", (380, 780)))


def test_strided_subsample_renders_the_same_pixels_as_the_full_crop(box):
    """oracle_render_strided (the bounded CPU sample of a large request) traces pixel
    (cx + i*s, cy + j*s) exactly as the full render of the crop does."""
    import pyoracle
    _, h = box
    p = pyoracle.render_params("nee", 40, 30, spp_start=3, spp=2, max_depth=8, lambda_range=(380, 780),
                               crop=(5, 4, 23, 17))
    full = h.render(p, precision=32, records=False, film=True)["film"]
    sub = h.render_strided(p, 4, precision=32, film=True)["film"]
    assert sub.shape == (5, 6, 3)
    assert np.array_equal(sub, full[::4, ::4])


def test_subsurface_oracle_is_deterministic_and_estimators_agree():
    """The subsurface layer in the oracle: thread-independent samples, finite values, FP32 and
    FP64 per-sample agreement, and the unidirectional and NEE estimators agree on the image."""
    import pyoracle
    sc = configs.subsurface_box_scene(0)
    h = pyoracle.OracleSceneHandle(sc, pyoracle.own_luts())
    kw = dict(max_depth=8, lambda_range=(380, 780))
    p = pyoracle.render_params("nee", 24, 24, spp=2, **kw)
    h.ensure_rgb_table(p)
    a = h.render(p, precision=32, threads=1)["records"]
    b = h.render(p, precision=32, threads=6)["records"]
    assert np.array_equal(a, b) and np.all(np.isfinite(a))
    d = h.render(p, precision=64)["records"]
    rel = np.abs(a[..., 1:5] - d[..., 1:5]) / np.maximum(np.abs(d[..., 1:5]), 1e-6)
    assert np.mean(rel < 1e-3) > 0.99
    fu = h.render(pyoracle.render_params("uni", 16, 16, spp=256, **kw), precision=32, records=False, film=True)["film"]
    fn = h.render(pyoracle.render_params("nee", 16, 16, spp=256, **kw), precision=32, records=False, film=True)["film"]
    assert abs(fu[..., 1].mean() - fn[..., 1].mean()) / fn[..., 1].mean() < 0.08


def test_bdpt_subsurface_oracle_agrees_with_nee():
    """Subsurface exits as BDPT vertices in the oracle: thread-independent, FP32 and FP64 agree
    per sample, and the bidirectional image agrees with NEE's, which takes the whole subsurface
    event at the entry vertex (a wrong MIS sum over the exit vertices would bias it)."""
    import pyoracle
    sc = configs.subsurface_box_scene(0)
    h = pyoracle.OracleSceneHandle(sc, pyoracle.own_luts())
    kw = dict(max_depth=8, lambda_range=(380, 780))
    p = pyoracle.render_params("bdpt", 24, 24, spp=2, light_vertices=8, **kw)
    h.ensure_rgb_table(p)
    a = h.render(p, precision=32, threads=1)["records"]
    b = h.render(p, precision=32, threads=6)["records"]
    assert np.array_equal(a, b) and np.all(np.isfinite(a))
    d = h.render(p, precision=64)["records"]
    rel = np.abs(a[..., 5:8] - d[..., 5:8]) / np.maximum(np.abs(d[..., 5:8]), 1e-6)
    assert np.mean(rel < 1e-3) > 0.99
    fb = h.render(pyoracle.render_params("bdpt", 32, 32, spp=512, light_vertices=8, **kw), precision=32, records=False,
                  film=True)["film"]
    fn = h.render(pyoracle.render_params("nee", 32, 32, spp=512, **kw), precision=32, records=False, film=True)["film"]
    assert abs(fb[..., 1].mean() - fn[..., 1].mean()) / fn[..., 1].mean() < 0.01
