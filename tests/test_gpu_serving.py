"""The serving loop on the GPU: continuous batching must not change any result.

Requests of different scenes, sizes, sample counts, depths and integrators are submitted at
once; each result must equal, bit for bit, the film yg_render gives for the same parameters on
a context of its own (the tolerance is zero: every sample depends only on its request, and
films are folded in sample order). Admission must keep the device footprint within the
budget, cancelled and invalid requests must not disturb the others.
"""
import time

import numpy as np
import pytest

from yapt_gb300 import configs
from yapt_gb300 import _native as N
from yapt_gb300.runtime import Context, Server

pytestmark = pytest.mark.gpu

LAMBDA = (380, 780)


def scenes():
    return [configs.box_scene(0), configs.box_scene(5), configs.random_shapes_scene(2, n_spheres=40)]


def request_set():
    P = Context.params
    return [
        (0, P("nee", 64, 48, spp_start=0, spp=6, max_depth=8, lambda_range=LAMBDA)),
        (1, P("uni", 40, 40, spp_start=3, spp=5, max_depth=6, lambda_range=LAMBDA, crop=(8, 4, 24, 30))),
        (2, P("nee", 96, 64, spp_start=1, spp=3, max_depth=12, lambda_range=LAMBDA, seed=7)),
        (0, P("bdpt", 32, 32, spp_start=0, spp=3, max_depth=8, lambda_range=LAMBDA, light_vertices=8)),
        (1, P("nee", 16, 16, spp_start=9, spp=17, max_depth=4, lambda_range=LAMBDA)),
        (2, P("uni", 128, 96, spp_start=0, spp=2, max_depth=10, lambda_range=LAMBDA)),
    ]


def alone(scene, params):
    with Context(0) as c:
        c.upload_scene(scene)
        c.film_clear(params.width, params.height)
        c.render(params)
        return c.film()


@pytest.mark.parametrize("persistent", [False, True], ids=["graph", "persistent"])
def test_results_are_identical_alone_and_in_the_mix(built, persistent):
    scs = scenes()
    reqs = request_set()
    expected = [alone(scs[s], p) for (s, p) in reqs]
    ctxs = [Context(0) for _ in scs]
    for c, sc in zip(ctxs, scs):
        c.upload_scene(sc)
    try:
        with Server(ctxs, lambda_range=LAMBDA, max_depth=12, round_samples=1 << 14, persistent=persistent) as srv:
            ids = [srv.submit(s, p) for (s, p) in reqs]
            for rid in ids:
                info = srv.wait(rid, timeout=120.0)
                assert info["state"] == "done", info
            for rid, (xyz_e, cnt_e) in zip(ids, expected):
                xyz, cnt = srv.result(rid)
                assert np.array_equal(cnt, cnt_e)
                assert np.array_equal(xyz, xyz_e), float(np.abs(xyz - xyz_e).max())
            st = srv.stats()
            total = sum(p.spp_count * (p.crop_w or p.width) * (p.crop_h or p.height) for _, p in reqs)
            assert st["samples"] == total
            assert st["completed"] == len(reqs)
            # continuous batching: several requests shared rounds
            planes = sum(p.spp_count for _, p in reqs if p.integrator != 2)
            assert st["rounds"] < planes
            if persistent:
                assert st["persistent_rounds"] == st["rounds"] and st["graph_replays"] in (0, st["rounds"])
            else:
                assert st["graph_replays"] == st["rounds"] and st["persistent_rounds"] == 0
    finally:
        for c in ctxs:
            c.close()


def test_admission_keeps_the_footprint_within_the_budget(built):
    with Context(0) as c:
        c.upload_scene(configs.box_scene(0))
        film = 64 * 64 * 32
        with Server([c], lambda_range=LAMBDA, memory_budget_bytes=2 * film + 100, round_samples=1 << 12) as srv:
            ids = [srv.submit(0, Context.params("nee", 64, 64, spp_start=i, spp=4, max_depth=6, lambda_range=LAMBDA))
                   for i in range(6)]
            infos = [srv.wait(r, timeout=120.0) for r in ids]
            assert all(i["state"] == "done" for i in infos)
            st = srv.stats()
            assert st["peak_bytes_in_use"] <= 2 * film + 100
            assert st["bytes_in_use"] == 0
            # admission follows arrival order
            admits = [i["t_admit"] for i in infos]
            assert admits == sorted(admits)
            with pytest.raises(N.YaptError):  # could never fit
                srv.submit(0, Context.params("nee", 256, 256, spp=1, lambda_range=LAMBDA))


def test_cancel_and_invalid_requests_leave_the_others_intact(built):
    with Context(0) as c:
        c.upload_scene(configs.box_scene(0))
        p_ok = Context.params("nee", 48, 32, spp=4, max_depth=6, lambda_range=LAMBDA)
        ref = alone(configs.box_scene(0), p_ok)
        with Server([c], lambda_range=LAMBDA, max_depth=8, round_samples=1 << 12) as srv:
            big = srv.submit(0, Context.params("nee", 256, 256, spp=64, max_depth=8, lambda_range=LAMBDA))
            ok = srv.submit(0, p_ok)
            srv.cancel(big)
            with pytest.raises(N.YaptError):  # other spectral range than the server's
                srv.submit(0, Context.params("nee", 8, 8, spp=1, lambda_range=(380, 700)))
            with pytest.raises(N.YaptError):  # depth above the server's
                srv.submit(0, Context.params("nee", 8, 8, spp=1, max_depth=20, lambda_range=LAMBDA))
            with pytest.raises(N.YaptError):  # no such scene
                srv.submit(3, p_ok)
            assert srv.wait(big, timeout=120.0)["state"] == "cancelled"
            assert srv.wait(ok, timeout=120.0)["state"] == "done"
            xyz, cnt = srv.result(ok)
            assert np.array_equal(xyz, ref[0]) and np.array_equal(cnt, ref[1])
            with pytest.raises(N.YaptError):
                srv.result(big)
            srv.release(big)
            st = srv.stats()
            assert st["cancelled"] == 1 and st["bytes_in_use"] == 0


def test_shutdown_with_work_in_flight_returns_promptly(built):
    with Context(0) as c:
        c.upload_scene(configs.box_scene(0))
        srv = Server([c], lambda_range=LAMBDA, max_depth=8)
        for i in range(8):
            srv.submit(0, Context.params("nee", 256, 256, spp_start=64 * i, spp=64, max_depth=8, lambda_range=LAMBDA))
        time.sleep(0.05)
        t = time.time()
        srv.close()
        assert time.time() - t < 30.0


def test_grid_barrier_wait_is_bounded_and_the_context_survives(built):
    """The persistent round's grid barrier: with every block arriving, each block passes it
    three times; with one block that never arrives (the barrier expects one more block than the
    grid), every wait runs out after its poll limit, the kernel reports the time-out and returns,
    and the context renders correctly afterwards."""
    scene = configs.box_scene(0)
    p = Context.params("nee", 32, 32, spp_start=0, spp=2, max_depth=6, lambda_range=LAMBDA)
    xyz_e, cnt_e = alone(scene, p)
    with Context(0) as c:
        blocks, passes, timed = c.grid_barrier_selftest(missing=0, poll_limit=1 << 22)
        assert blocks > 0 and not timed and passes == 3 * blocks
        t = time.time()
        blocks, passes, timed = c.grid_barrier_selftest(missing=1, poll_limit=4096)
        assert timed and passes == 0
        assert time.time() - t < 30.0
        c.upload_scene(scene)
        c.film_clear(32, 32)
        c.render(p)
        xyz, cnt = c.film()
        assert np.array_equal(cnt, cnt_e) and np.array_equal(xyz, xyz_e)


def test_persistent_round_barrier_time_out_fails_only_that_round(built):
    """A persistent round whose barrier waits are allowed a single poll: whether or not the
    barriers time out, every request ends (done with the film yg_render gives, or failed with
    YG_ERR_DEVICE_TIMEOUT); a new server on the same context then completes the request."""
    scene = configs.box_scene(0)
    p = Context.params("nee", 48, 32, spp_start=0, spp=2, max_depth=6, lambda_range=LAMBDA)
    xyz_e, cnt_e = alone(scene, p)
    with Context(0) as c:
        c.upload_scene(scene)
        with Server([c], lambda_range=LAMBDA, max_depth=8, persistent=True, barrier_polls=1) as srv:
            ids = [srv.submit(0, p) for _ in range(3)]
            for rid in ids:
                info = srv.wait(rid, timeout=60.0)
                assert info["state"] in ("done", "failed"), info
                if info["state"] == "failed":
                    assert info["error"] == -6
                else:
                    xyz, cnt = srv.result(rid)
                    assert np.array_equal(cnt, cnt_e) and np.array_equal(xyz, xyz_e)
        with Server([c], lambda_range=LAMBDA, max_depth=8, persistent=True) as srv:
            rid = srv.submit(0, p)
            assert srv.wait(rid, timeout=60.0)["state"] == "done"
            xyz, cnt = srv.result(rid)
            assert np.array_equal(cnt, cnt_e) and np.array_equal(xyz, xyz_e)
