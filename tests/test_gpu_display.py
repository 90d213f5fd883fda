"""The display path (the reference's tonemap stage: TonemapStage.cpp, gatherLuminanceHistogram.comp,
analyzeLuminanceHistogram.comp, prepareTonemapData.comp, tonemap.frag with ACES) on the GPU,
against a float64 numpy restatement. 8-bit outputs may differ by one step where a value lies on a
rounding boundary (the device uses CUDA's powf/log2f/exp2f); the exposure within 1e-3 relative."""
import numpy as np
import pytest

from yapt_gb300 import configs
from yapt_gb300.runtime import Context

pytestmark = pytest.mark.gpu

M = np.array([[3.2406, -1.5372, -0.4986], [-0.9689, 1.8758, 0.0415], [0.0557, -0.2040, 1.0570]])
ACES_IN = np.array([[0.59719, 0.35458, 0.04823], [0.07600, 0.90834, 0.01566], [0.02840, 0.13383, 0.83777]])
ACES_OUT = np.array([[1.60475, -0.53108, -0.07367], [-0.10208, 1.10813, -0.00605], [-0.00327, -0.07276, 1.07602]])
LUM = np.array([0.2126, 0.7152, 0.0722])


def linear_rgb(xyz):
    c = xyz.astype(np.float64) @ M.T
    lum = c @ LUM
    m = c.min(-1)
    t = np.where(m < 0, np.divide(lum, lum - m, out=np.zeros_like(lum), where=(lum - m) != 0), 1.0)
    return np.where((m < 0)[..., None], lum[..., None] + (c - lum[..., None]) * t[..., None], c)


def aces(c):
    v = c @ ACES_IN.T
    v = (v * (v + 0.0245786) - 0.000090537) / (v * (0.983729 * v + 0.4329510) + 0.238081)
    return np.clip(v @ ACES_OUT.T, 0, 1)


def encode(c):
    c = np.clip(c, 0, 1)
    e = np.where(c <= 0.0031308, 12.92 * c, 1.055 * np.power(c, 1 / 2.4) - 0.055)
    return np.rint(np.clip(e, 0, 1) * 255)


def mean_ev(rgb):
    ev = np.log2(np.maximum(rgb @ LUM, 0) * 8.0 + 1e-300)
    b = np.floor(np.clip(ev + 12.0, 0, 127) + 0.5)
    return float(np.mean(b - 12.0))


@pytest.fixture(scope="module")
def rendered(built):
    c = Context(0)
    c.upload_scene(configs.box_scene(1))
    W, H = 64, 48
    c.film_clear(W, H)
    from yapt_gb300 import _native as N
    c.render(c.params("nee", W, H, spp=16, max_depth=8, lambda_range=(380, 780), flags=N.YG_FLAG_ATROUS_FEATURES))
    xyz, _ = c.film()
    yield c, xyz
    c.close()


@pytest.mark.parametrize("operator", [0, 1])
def test_manual_exposure_with_and_without_aces(rendered, operator):
    c, xyz = rendered
    img, e = c.tonemap(enable=operator, auto_exposure=0, manual_exposure=6.0)
    assert e == pytest.approx(6.0)
    rgb = linear_rgb(xyz) * 6.0
    want = encode(aces(rgb) if operator else rgb)
    assert np.abs(img[..., :3].astype(int) - want).max() <= 1
    assert np.all(img[..., 3] == 255)


def test_auto_exposure_adapts_from_the_first_frame(rendered):
    c, xyz = rendered
    img, e0 = c.tonemap(auto_exposure=1, exposure_compensation=0.5, reset=1)
    assert e0 == pytest.approx(0.5)  # the first frame starts at the parameter value
    target = 0.18 / (2.0 ** (mean_ev(linear_rgb(xyz)) + 0.5) / 8.0)
    e = e0
    for dt in (0.1, 0.25, 1.0):
        _, got = c.tonemap(auto_exposure=1, exposure_compensation=0.5, delta_time=dt, eye_adaptation_speed=2.0)
        e = e + (target - e) * (1 - np.exp(-dt * 2.0))
        assert got == pytest.approx(e, rel=1e-3)  # a pixel on a bucket edge moves the mean EV by 1/npix


def test_denoised_source(rendered):
    c, _ = rendered
    out, _ = c.atrous_denoise()
    img, _ = c.tonemap(enable=1, auto_exposure=0, manual_exposure=4.0, source=1)
    want = encode(aces(linear_rgb(out[..., :3]) * 4.0))
    assert np.abs(img[..., :3].astype(int) - want).max() <= 1


def test_py_yapt_final_color_with_denoise_and_tonemap(built, py_yapt):
    import pyyapt_util as U
    Y = py_yapt
    r = Y.Renderer()
    r.init()
    r.getRendererVariable("Generic.RenderResolution").setFromIntArray([32, 24])
    r.getRendererVariable("World.EnvIntensityScale").setFromFloatArray([0.0])
    sc = Y.Scene()
    sc.init(r)
    objs = U.build_scene(Y, r, sc, U.box(1))
    r.getRendererVariable("Denoise.Mode").setSelectedOption(1)
    r.getRendererVariable("Tonemap.UseAutoExposure").setSelectedOption(0)
    r.getRendererVariable("Tonemap.ManualExposure").setFromFloatArray([5.0])
    sc.update(0.016, 4)
    fc = r.readback(Y.ReadbackTarget.FinalColor).getData()
    img = np.frombuffer(fc.getBytes(), np.uint8).reshape(24, 32, 4)
    assert img[..., :3].max() > 0 and np.all(img[..., 3] == 255)
    r.getRendererVariable("Denoise.Mode").setSelectedOption(2)
    with pytest.raises(Y.YaptError):
        sc.update(0.016, 1)  # the debug views are not built
    del objs
    sc.shutdown()
    r.shutdown()
