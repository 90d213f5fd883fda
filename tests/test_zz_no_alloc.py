"""The render entry point that allocates nothing (yg_render_samples_noalloc).

It exists for callers that cannot allocate device memory while rendering (a process
whose device budget is reserved up front, a host application that must not hit
cudaMalloc's implicit synchronisation mid-frame). It must give the same samples as the
allocating entry point yg_render, call after call, although every call reuses one
fixed scratch array. This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

from yapt_gb300 import configs
from yapt_gb300 import _native as N
from yapt_gb300.runtime import Context

pytestmark = pytest.mark.gpu

REL_TOL = 1e-4  # same per-sample tolerance as the other parity tests


def noalloc(lib, ctx, params, out_tensor):
    return lib.yg_render_samples_noalloc(ctx.h, ctypes.byref(params), ctypes.c_void_p(out_tensor.data_ptr()))


def render_noalloc(lib, c, p):
    import torch
    cw, ch = p.crop_w or p.width, p.crop_h or p.height
    out = torch.full((p.spp_count * ch * cw * 4,), float("nan"), device="cuda", dtype=torch.float32)
    N.check(noalloc(lib, c, p, out))
    c.synchronize()
    return out.cpu().numpy().reshape(p.spp_count, ch, cw, 4)


def assert_same_samples(got, ref):
    assert np.all(got[..., 3] == 1.0)
    rel = np.abs(got[..., :3] - ref) / np.maximum(np.abs(ref), 1e-6)
    assert np.all(rel <= REL_TOL), float(rel.max())
    assert np.any(ref > 0)


def test_noalloc_matches_the_allocating_entry_point_on_consecutive_calls(built, host_luts):
    import pyoracle
    lib = N.load()
    sc = configs.random_shapes_scene(3, n_spheres=60)
    W, H = 80, 48
    with Context(0) as c:
        c.upload_scene(sc)
        for (start, spp) in [(0, 3), (3, 2)]:
            p = c.params("nee", W, H, spp_start=start, spp=spp, max_depth=12, lambda_range=(380, 700),
                         flags=N.YG_FLAG_NO_FILM)
            ref = c.render(p, dump=True)[..., 5:8]
            got = render_noalloc(lib, c, p)
            assert_same_samples(got, ref)
            if start == 3:  # the second call also directly against the oracle
                orc = pyoracle.OracleSceneHandle(sc, host_luts).render(p, precision=32)["records"][..., 5:8]
                assert_same_samples(got, orc)


@pytest.mark.parametrize("case", ["several_waves", "crop", "waves_split_planes"])
def test_noalloc_over_several_waves_and_on_a_crop(built, case):
    """128 x 128 x 4 samples run as four waves of the fixed 16,384-path arena; the crop case
    renders a ragged window of a larger image; 96 x 102 x 3 samples split a sample plane and a
    four-row band between two waves and end each plane with a partial band (the slots there keep
    scanline order, the others cover 8 x 4 tiles). All against yg_render's per-sample dump, which
    renders each request as one wave."""
    lib = N.load()
    with Context(0) as c:
        c.upload_scene(configs.box_scene(2))
        if case == "several_waves":
            p = c.params("uni", 128, 128, spp_start=5, spp=4, max_depth=8, lambda_range=(380, 700),
                         flags=N.YG_FLAG_NO_FILM)
        elif case == "crop":
            p = c.params("nee", 200, 120, spp_start=17, spp=3, max_depth=8, lambda_range=(380, 700),
                         flags=N.YG_FLAG_NO_FILM, crop=(37, 21, 61, 43))
        else:
            p = c.params("nee", 96, 102, spp_start=2, spp=3, max_depth=8, lambda_range=(380, 700),
                         flags=N.YG_FLAG_NO_FILM)
        ref = c.render(p, dump=True)[..., 5:8]
        for _ in range(2):  # twice in a row: the array keeps the last call's contents
            assert_same_samples(render_noalloc(lib, c, p), ref)


def test_noalloc_rejects_requests_beyond_its_scratch(built):
    import torch
    lib = N.load()
    with Context(0) as c:
        c.upload_scene(configs.box_scene(0))
        p = c.params("nee", 8, 8, spp=257, max_depth=4, flags=N.YG_FLAG_NO_FILM)
        out = torch.empty(257 * 8 * 8 * 4, device="cuda", dtype=torch.float32)
        rc = noalloc(lib, c, p, out)
        assert rc == -1
        assert b"maximum of 256" in lib.yg_last_error()


def test_noalloc_rejects_materials_whose_textures_were_cleared(built):
    """After yg_clear_textures the device texture table holds freed pointers; a material
    that still refers to a texture must be rejected on the host, before any launch."""
    import torch
    lib = N.load()
    with Context(0) as c:
        c.upload_scene(configs.textured_box_scene(1))
        p = c.params("nee", 16, 16, spp=1, max_depth=4, lambda_range=(380, 700), flags=N.YG_FLAG_NO_FILM)
        c.render(p)  # makes the RGB fit resident for this range
        N.check(c.lib.yg_clear_textures(c.h))
        out = torch.empty(16 * 16 * 4, device="cuda", dtype=torch.float32)
        rc = noalloc(lib, c, p, out)
        assert rc != 0
        assert b"texture" in lib.yg_last_error()
        with pytest.raises(RuntimeError):
            c.render(p)
