"""The a-trous denoiser (the reference's edge-stopping filter, kept as the baseline of the
learned denoiser) on the GPU, through the C ABI, against the FP32 oracle.

Tolerance: the device kernels and the oracle compute every value in the same order with the
same transcendental functions, so the gathered moment sums, the packed features and the
filtered colour are compared bit for bit; a 1e-5 relative bound is allowed on at most
1e-4 of the values for the filtered output (none are expected)."""
import numpy as np
import pytest

from yapt_gb300 import _native as N
from yapt_gb300 import configs
from yapt_gb300.runtime import Context, atrous_params, atrous_run

import test_atrous_cpu as T

pytestmark = pytest.mark.gpu

REL_TOL = 1e-5


def close(a, b, frac=1e-4):
    rel = np.abs(a.astype(np.float64) - b) / np.maximum(np.abs(b.astype(np.float64)), 1e-12)
    bad = float(np.mean(rel > REL_TOL))
    exact = float(np.mean(a == b))
    assert bad <= frac, "%.6f of values beyond %g (exact %.6f)" % (bad, REL_TOL, exact)
    return exact


@pytest.mark.parametrize("w,h,prefilter,passes", [(36, 24, 1, 5), (37, 23, 0, 5), (1, 1, 1, 5), (200, 120, 1, 5),
                                                  (64, 48, 1, 0), (64, 48, 1, 7)])
def test_filter_matches_the_oracle_on_synthetic_inputs(built, w, h, prefilter, passes):
    import pyoracle
    film, odd, mom = T.synthetic(w, h, seed=w * 7 + h, miss_frac=0.15)
    cam = T.camera(w, h)
    p = atrous_params(prefilter=prefilter, passes=passes)
    out, var, feat = atrous_run(film, odd, mom, cam, p)
    o_out, o_var, o_feat = pyoracle.atrous(film, odd, mom, cam, p)
    assert np.array_equal(feat, o_feat), "packed features differ"
    close(out, o_out)
    close(var, o_var)


def gathered(ctx, sc, integrator, w, h, spp, spp_start=0):
    ctx.upload_scene(sc)
    ctx.film_clear(w, h)
    p = ctx.params(integrator, w, h, spp_start=spp_start, spp=spp, max_depth=8, lambda_range=(380, 780),
                   flags=N.YG_FLAG_ATROUS_FEATURES, light_vertices=8 if integrator == "bdpt" else 0)
    rec = ctx.render(p, dump=True)
    return p, rec, ctx.atrous_state()


@pytest.mark.parametrize("integrator,scene", [("nee", "box"), ("uni", "layered"), ("bdpt", "box")])
def test_gathered_moments_and_half_films_match_the_oracle(built, host_luts, integrator, scene):
    import pyoracle
    sc = configs.box_scene(2) if scene == "box" else configs.layered_box_scene(4)
    W, H = 40, 32
    with Context(0) as c:
        p, rec, st = gathered(c, sc, integrator, W, H, spp=6, spp_start=3)
    rgb = N.host_table("rgb_to_spd", (380, 780))
    mom = np.zeros((4, H, W, 4), np.float32)
    pyoracle.OracleSceneHandle(sc, host_luts, rgb).atrous_moments(p, mom)
    assert np.array_equal(st["moments"], mom), "moment sums differ in %d values" % int(np.sum(st["moments"] != mom))
    assert np.all(st["moments"][1, ..., 3] > 0), "closed box: every pixel hits something"
    # odd-indexed samples (global index spp_start + k) summed in order
    odd = np.zeros((H, W, 4), np.float32)
    for k in range(p.spp_count):
        if (p.spp_start + k) & 1:
            odd[..., :3] += rec[k, ..., 5:8]
            odd[..., 3] += np.float32(1)
    assert np.array_equal(st["odd"], odd)
    assert np.all(st["film"][..., 3] == 6)


def test_denoise_of_a_render_matches_the_oracle_and_lowers_the_error(built, host_luts):
    import pyoracle
    sc = configs.box_scene(1)
    W, H = 64, 48
    with Context(0) as c:
        c.upload_scene(sc)
        c.film_clear(W, H)
        ref_p = c.params("nee", W, H, spp_start=0, spp=1024, max_depth=8, lambda_range=(380, 780))
        c.render(ref_p)
        ref, _ = c.film()
        p, rec, st = gathered(c, sc, "nee", W, H, spp=4)
        noisy, _ = c.film()
        out, var = c.atrous_denoise()
        st = c.atrous_state(features=True)
    o_out, o_var, o_feat = pyoracle.atrous(st["film"], st["odd"], st["moments"], sc.camera.struct(), atrous_params())
    assert np.array_equal(st["features"], o_feat)
    close(out, o_out)
    close(var, o_var)

    def relmse(x):
        return float(np.mean((x - ref) ** 2 / (ref ** 2 + 1e-2)))

    # at 4 samples the filter roughly halves the error of this scene (it also bleeds the ceiling
    # light into the dark ceiling pixels beside it, as the reference's filter does: the
    # albedo variance of the mixed pixels at the light's edge relaxes the edge stopping)
    assert relmse(out[..., :3]) < 0.75 * relmse(noisy), (relmse(out[..., :3]), relmse(noisy))


def test_denoise_requires_the_gather_on_every_render(built):
    with Context(0) as c:
        c.upload_scene(configs.box_scene(0))
        W, H = 16, 16
        c.film_clear(W, H)
        with pytest.raises(N.YaptError):
            c.atrous_denoise()  # nothing rendered
        c.render(c.params("nee", W, H, spp=2, flags=N.YG_FLAG_ATROUS_FEATURES))
        c.render(c.params("nee", W, H, spp_start=2, spp=2))  # one render without the gather
        with pytest.raises(N.YaptError):
            c.atrous_denoise()
        c.film_clear(W, H)
        c.render(c.params("nee", W, H, spp=2, flags=N.YG_FLAG_ATROUS_FEATURES))
        c.render(c.params("nee", W, H, spp_start=2, spp=2, flags=N.YG_FLAG_ATROUS_FEATURES))
        out, var = c.atrous_denoise()
        assert np.all(np.isfinite(out)) and np.all(var >= 0)
        with pytest.raises(N.YaptError):
            c.atrous_denoise(atrous_params(color_sigma=float("nan")))
        with pytest.raises(N.YaptError):
            c.render(c.params("nee", W, H, spp=1, flags=N.YG_FLAG_ATROUS_FEATURES | N.YG_FLAG_NO_FILM))
