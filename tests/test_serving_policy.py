"""Admission and round planning of the serving loop, on host data only (yg_server_plan).

The policy: queued requests are admitted in arrival order while their film fits the memory
budget and a slot is free (no overtaking, so a large request is never starved); each round
then merges the admitted uni/NEE requests, fewest remaining samples first, in whole sample
planes, up to the round's sample target (a lone first request may exceed it by one plane) and
never beyond the wave capacity; requests passed over for 8 rounds go first; BDPT requests
advance on their own stream and take no planes here.
"""
import pytest

from yapt_gb300.runtime import plan_round

MB = 1 << 20


def item(px, planes, fp=MB, admitted=False, integ="nee", waited=0):
    return dict(pixels=px, planes_left=planes, footprint_bytes=fp, admitted=admitted, integrator=integ,
                rounds_waited=waited)


def test_admission_is_in_arrival_order_within_the_budget(built):
    items = [item(64 * 64, 4, 3 * MB), item(64 * 64, 4, 3 * MB), item(64 * 64, 4, 3 * MB), item(8 * 8, 1, 1)]
    adm, planes, total = plan_round(items, budget_bytes=7 * MB)
    assert adm == [1, 1, 0, 0]  # the small fourth request does not overtake the third
    assert planes[2] == planes[3] == 0
    adm, _, _ = plan_round(items, budget_bytes=100 * MB, max_active=3)
    assert adm == [1, 1, 1, 0]
    adm, _, _ = plan_round(items, budget_bytes=10 * MB, bytes_in_use=8 * MB)
    assert adm == [0, 0, 0, 0]


def test_round_plans_fewest_remaining_samples_first_in_whole_planes(built):
    big = item(1024 * 1024, 64, admitted=True)
    small = item(128 * 128, 4, admitted=True)
    mid = item(256 * 256, 16, admitted=True)
    adm, planes, total = plan_round([big, small, mid], budget_bytes=1 << 40, round_samples=1 << 19)
    assert planes[1] == 4  # the smallest request finishes in this round
    assert planes[2] == ((1 << 19) - 4 * 128 * 128) // (256 * 256)
    assert planes[0] == 0  # a 1M-pixel plane no longer fits the round's target
    assert total == planes[1] * 128 * 128 + planes[2] * 256 * 256 <= 1 << 19


def test_a_lone_large_request_gets_one_plane_beyond_the_round_target(built):
    adm, planes, total = plan_round([item(1024 * 1024, 64, admitted=True)], budget_bytes=1 << 40,
                                    round_samples=1 << 19, wave_capacity=1 << 21)
    assert planes == [1] and total == 1024 * 1024


def test_round_never_exceeds_the_wave_capacity_or_the_remaining_planes(built):
    items = [item(4096, 3, admitted=True), item(4096, 1000, admitted=True)]
    adm, planes, total = plan_round(items, budget_bytes=1 << 40, wave_capacity=1 << 16, round_samples=1 << 20)
    assert planes[0] == 3
    assert total <= 1 << 16 and planes[1] == ((1 << 16) - 3 * 4096) // 4096


def test_requests_passed_over_for_eight_rounds_go_first(built):
    waiting = item(1024 * 1024, 2, admitted=True, waited=8)
    small = item(64 * 64, 1, admitted=True)
    _, planes, _ = plan_round([small, waiting], budget_bytes=1 << 40, round_samples=1 << 19)
    assert planes[1] == 1 and planes[0] == 0


def test_bdpt_requests_take_no_merged_planes_but_are_admitted(built):
    adm, planes, _ = plan_round([item(64 * 64, 8, integ="bdpt"), item(64 * 64, 8)], budget_bytes=1 << 40)
    assert adm == [1, 1] and planes == [0, 8]


def test_invalid_plan_input_is_rejected(built):
    from yapt_gb300 import _native as N
    with pytest.raises(N.YaptError):
        plan_round([item(1 << 22, 1)], budget_bytes=1 << 40, wave_capacity=1 << 21)
