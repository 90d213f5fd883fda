"""The debug build's bounds checks (compiled with -DYG_DEBUG_BOUNDS, e.g.
YG_NVCC_EXTRA=-DYG_DEBUG_BOUNDS before the build): node, triangle and queue indices are checked
before they are read and an out-of-range one is counted and skipped. Renders of every
integrator on scenes with instancing, cutouts and subsurface probes must count none. In a
normal build the entry point reports that the checks are not compiled in, and the test is
skipped."""
import ctypes as C

import pytest

from yapt_gb300 import configs
from yapt_gb300 import _native as N
from yapt_gb300.runtime import Context

pytestmark = pytest.mark.gpu


def test_renders_refuse_no_index(built):
    lib = N.load()
    with Context(0) as c:
        c.upload_scene(configs.box_scene(0))
        n = C.c_uint32()
        if lib.yg_debug_bounds_errors(c.h, C.byref(n)) == -4:
            pytest.skip("library built without YG_DEBUG_BOUNDS")
        for scene in (configs.box_scene(1), configs.random_shapes_scene(2, n_spheres=60), configs.subsurface_box_scene(0)):
            c.upload_scene(scene)
            for integ in ("uni", "nee", "bdpt"):
                c.film_clear(32, 32)
                c.render(c.params(integ, 32, 32, spp=2, max_depth=8, lambda_range=(380, 780)))
            N.check(lib.yg_debug_bounds_errors(c.h, C.byref(n)))
            assert n.value == 0
