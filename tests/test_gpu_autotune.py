"""Schedule autotuner on the GPU: the distinct schedules of a size, every schedule reproducing
the first one's multislice field, the cached choice taken by plans created afterwards."""
import importlib

import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture()
def at(monkeypatch, tmp_path):
    monkeypatch.setenv("RS_SCHEDULE_CACHE", str(tmp_path / "schedules.json"))
    monkeypatch.delenv("RS_AUTOTUNE", raising=False)
    return importlib.import_module("3d_ravesim_gb300.autotune")


def test_schedule_lists(rs, cuda):
    lib = rs._lib
    # the split-pair family is one schedule where it covers both directions; the compensated
    # family (bit 16) keeps every single-sequence kernel choice
    # per direction: the split-pair passes (one schedule), or (bit 16 rows, bit 32 columns) the
    # single-sequence kernels with their own choices
    # (bits 64 / 128: the dithered rows / columns one per thread group, where split-pair ones exist)
    assert lib.plan_for(4096, 4096, cuda).schedules() == [0, 16, 17, 20, 32, 34, 40, 42, 48, 49, 50, 51, 52, 54,
                                                          56, 57, 58, 59, 60, 62, 64, 96, 98, 104, 106,
                                                          128, 144, 145, 148, 192]
    assert lib.plan_for(2048, 2048, cuda).schedules() == [0, 16, 17, 20, 32, 34, 48, 49, 50, 51, 52, 54,
                                                          64, 96, 98, 128, 144, 145, 148, 192]  # no split
    assert lib.plan_for(8192, 64, cuda).schedules() == [0, 16, 17, 20, 64]  # split-pair rows, 64-point columns
    assert lib.plan_for(16384, 64, cuda).schedules() == [0, 16, 20]  # dithered rows only one per thread group
    # 3*2^k: dithered rows and columns only one per thread group (radix-24 first stage)
    assert lib.plan_for(3072, 3072, cuda).schedules() == [0, 16, 17, 20, 32, 34, 48, 49, 50, 51, 52, 54]
    assert lib.plan_for(72, 40, cuda).schedules() == [0]  # direct-DFT sizes have one schedule
    p = lib.plan_for(1024, 1024, cuda)
    old = p.schedule()
    p.set_schedule(6)
    assert p.schedule() == 6
    p.set_schedule(old)
    with pytest.raises(Exception):
        p.set_schedule(256)


@pytest.mark.parametrize("n", [1024, 1536])
def test_tune_multislice(rs, cuda, at, n):
    c = at.tune_multislice(n, n, cuda, reps=3)
    plan = rs._lib.plan_for(n, n, cuda)
    assert sorted(c.timings_ms) == plan.schedules()
    assert all(t > 0 for t in c.timings_ms.values())
    # the pipelined and per-block kernels compute the same values (the rounding of each step is
    # spelled out), so every schedule reproduces the first one's field
    assert max(c.rel_diff.values()) <= at.MAX_SCHEDULE_DIFF, c.rel_diff
    assert c.mask in plan.schedules()
    assert at.cached_schedule(n, n, cuda) == c.mask
    # a plan created afterwards (another slot) takes the cached schedule
    with rs._lib.plan_slot(7):
        fresh = rs._lib.plan_for(n, n, cuda)
    assert fresh.schedule() == c.mask


def test_autotune_on_first_plan(rs, cuda, at, monkeypatch):
    monkeypatch.setenv("RS_AUTOTUNE", "1")
    with rs._lib.plan_slot(9):
        p = rs._lib.plan_for(768, 768, cuda)
    assert at.cached_schedule(768, 768, cuda) == p.schedule()
    torch.cuda.synchronize()
