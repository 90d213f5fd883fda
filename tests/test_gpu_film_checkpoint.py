"""Film checkpoints (yg_film_save / yg_film_restore): a render preempted after some sample
indices resumes on a fresh context from the saved state, and the film it ends with equals,
bit for bit, the film of the render that never stopped (compensated sums, counts, the a-trous
moments and features included). Foreign buffers are rejected with an error."""
import numpy as np
import pytest

from yapt_gb300 import configs
from yapt_gb300 import _native as N
from yapt_gb300.runtime import Context

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("flags", [0, N.YG_FLAG_ATROUS_FEATURES], ids=["film", "atrous"])
def test_resumed_render_equals_the_uninterrupted_one(built, flags):
    scene = configs.box_scene(3)
    W, H = 48, 40
    P = lambda c, s0: c.params("nee", W, H, spp_start=s0, spp=4, max_depth=8, lambda_range=(380, 780), flags=flags)  # noqa: E731
    with Context(0) as a:
        a.upload_scene(scene)
        a.film_clear(W, H)
        a.render(P(a, 0))
        a.render(P(a, 4))
        want_xyz, want_cnt = a.film()
        want_at = a.atrous_denoise()[0] if flags else None
    with Context(0) as b:
        b.upload_scene(scene)
        b.film_clear(W, H)
        b.render(P(b, 0))
        state = b.film_save()
    with Context(0) as c:
        c.upload_scene(scene)
        c.film_restore(state)
        c.render(P(c, 4))
        xyz, cnt = c.film()
        assert np.array_equal(cnt, want_cnt) and np.array_equal(xyz, want_xyz)
        if flags:
            assert np.array_equal(c.atrous_denoise()[0], want_at)


def test_restore_rejects_foreign_buffers(built):
    with Context(0) as c:
        c.upload_scene(configs.box_scene(0))
        with pytest.raises(N.YaptError):
            c.film_restore(bytes(64))
        c.film_clear(8, 8)
        state = c.film_save()
        with pytest.raises(N.YaptError):
            c.film_restore(state[:len(state) // 2])
