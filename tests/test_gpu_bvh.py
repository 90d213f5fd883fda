"""The device-built wide BVH: for scenes from 10 to 2 million triangles every child slot's
dequantised box (evaluated in double on the host) contains the triangles under it, every
node and triangle is reachable exactly once, and the depth fits the traversal stack.
Traversal exactness is covered by the per-sample parity tests (uni/NEE/BDPT) against the
oracle, whose BVH is built independently."""
import ctypes as C

import numpy as np
import pytest

from yapt_gb300 import configs
from yapt_gb300 import _native as N
from yapt_gb300.runtime import Context
from yapt_gb300.scene import CameraDesc, Scene

pytestmark = pytest.mark.gpu


def check(ctx):
    n, d, v = C.c_uint64(), C.c_uint64(), C.c_uint64()
    N.check(ctx.lib.yg_bvh_check(ctx.h, C.byref(n), C.byref(d), C.byref(v)))
    return n.value, d.value, v.value


@pytest.mark.parametrize("make", [lambda: configs.box_scene(0), lambda: configs.random_shapes_scene(0),
                                  lambda: configs.caustic_box_scene(0), lambda: configs.serve_scene(7)],
                         ids=["box", "random_shapes", "caustic_box", "serve_2M"])
def test_wide_bvh_contains_its_triangles(built, make):
    sc = make()
    with Context(0) as c:
        c.upload_scene(sc)
        info = c.scene_info()
        nodes, depth, bad = check(c)
    assert bad == 0
    assert info["triangles"] == sc.triangle_count()
    assert 1 <= depth <= 30
    assert nodes <= max(1, info["triangles"])  # fewer wide nodes than triangles


def test_degenerate_and_tiny_scenes(built):
    # one triangle; coplanar duplicates; a zero-area triangle
    sc = Scene()
    p = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 0], [1, 0, 0], [0, 1, 0], [2, 2, 2], [2, 2, 2], [2, 2, 2]],
                 np.float32)
    n = np.tile(np.float32([0, 0, 1]), (9, 1))
    m = sc.add_mesh(p, n, np.arange(9, dtype=np.uint32), submeshes=[(0, 3), (3, 6)])
    mat = sc.add_material(albedo=(0.5, 0.5, 0.5), metalness=0.0)
    sc.add_instance(m, mat, submesh=0)
    sc.camera = CameraDesc(eye=(0.3, 0.3, 2.0), target=(0.3, 0.3, 0.0))
    with Context(0) as c:
        c.upload_scene(sc)
        assert check(c)[2] == 0
        c.film_clear(8, 8)
        c.render(c.params("uni", 8, 8, spp=2, max_depth=3, env_scale=1.0))
        xyz, cnt = c.film()
        assert np.all(np.isfinite(xyz)) and np.all(cnt == 2)
    sc.add_instance(m, mat, submesh=1)
    with Context(0) as c:
        c.upload_scene(sc)
        assert check(c)[2] == 0
        c.film_clear(8, 8)
        c.render(c.params("nee", 8, 8, spp=2, max_depth=3, env_scale=1.0))
        assert np.all(np.isfinite(c.film()[0]))
