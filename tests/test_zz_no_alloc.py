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


def test_noalloc_matches_the_allocating_entry_point_on_consecutive_calls(built):
    import torch
    lib = N.load()
    sc = configs.random_shapes_scene(3, n_spheres=60)
    W, H = 80, 48
    with Context(0) as c:
        c.upload_scene(sc)
        for (start, spp) in [(0, 3), (3, 2)]:
            p = c.params("nee", W, H, spp_start=start, spp=spp, max_depth=12, lambda_range=(380, 700), flags=256)
            ref = c.render(p, dump=True)[..., 5:8]
            out = torch.full((spp * H * W * 4,), float("nan"), device="cuda", dtype=torch.float32)
            N.check(noalloc(lib, c, p, out))
            c.synchronize()
            got = out.cpu().numpy().reshape(spp, H, W, 4)
            assert np.all(got[..., 3] == 1.0)
            rel = np.abs(got[..., :3] - ref) / np.maximum(np.abs(ref), 1e-6)
            assert np.all(rel <= REL_TOL), float(rel.max())
            assert np.any(ref > 0)


def test_noalloc_rejects_requests_beyond_its_scratch(built):
    import torch
    lib = N.load()
    with Context(0) as c:
        c.upload_scene(configs.box_scene(0))
        p = c.params("nee", 8, 8, spp=257, max_depth=4, flags=256)
        out = torch.empty(257 * 8 * 8 * 4, device="cuda", dtype=torch.float32)
        rc = noalloc(lib, c, p, out)
        assert rc == -1
        assert b"maximum of 256" in lib.yg_last_error()
