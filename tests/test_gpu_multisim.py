"""Batched multisim on the GPU: the fused multi-stream runner against the unfused loop and, for
one item, against the FP64 oracle (point source -> shell sample -> free space -> area_v1)."""
import importlib

import numpy as np
import pytest
import torch

from conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ms():
    return importlib.import_module("3d_ravesim_gb300.multisim")


def small_batch(ms):
    return ms.shell_batch(n_sources_side=2, n_energies=2, sizes=(256, 384, 512), slices=8, fov=128e-6,
                          detector_pixels=256, seed=3)


def test_batched_fused_matches_plain_loop(ms, cuda):
    b = small_batch(ms)
    fused = ms.BatchRunner(b, cuda, streams=3).run()
    plain = ms.BatchRunner(b, cuda, streams=1).run(plain=True)
    assert torch.isfinite(fused).all() and fused.abs().sum() > 0
    assert rel_l2(fused.cpu().numpy(), plain.cpu().numpy()) < 1e-5


def test_batched_item_matches_fp64_oracle(ms, cuda, oracle):
    b = small_batch(ms)
    item = b.items[1]
    runner = ms.BatchRunner(b, cuda, streams=1)
    img = runner.run([item]).cpu().numpy()
    p = ms.item_params(b, item)
    cutoff = b.cutoff_fraction / p.dx
    s = b.sample
    db = ms._scaled_db(b, item.energy)
    u, U = oracle.point_source_2d(item.n, item.n, p.dx, p.dx, b.z_sample, item.x, item.y, p.wl, cutoff)
    u, U = oracle.sample_apply_2d(u, np.asarray(s.grid), db, p.dx, p.dx, p.wl, cutoff, s.pixel_size_x,
                                  s.pixel_size_y, s.pixel_size_z)
    z = s.z_start + s.get_thickness()
    u, U = oracle.propagate_2d(u, p.dx, p.dx, p.wl, p.z_detector - z, cutoff, U=U, skip_fft=True)
    ref = oracle.detector_area_v1(u, p.dx, p.dx, p.detector_pixel_size_x, p.detector_pixel_size_y,
                                  b.detector_pixels, b.detector_pixels, p.z_detector)
    assert rel_l2(img, ref) < 2e-5


def test_batch_graph_replay_matches_eager_run(ms, cuda):
    """The captured batch (accumulators zeroed, items on their streams, the stream sum) replays to
    the eager runner's image bit for bit, and a second replay gives the same image."""
    b = small_batch(ms)
    eager = ms.BatchRunner(b, cuda, streams=2).run().clone()
    runner = ms.BatchRunner(b, cuda, streams=2)
    runner.capture()
    first = runner.replay().clone()
    second = runner.replay().clone()
    assert torch.equal(first, eager)
    assert torch.equal(second, first)


def test_plain_loop_with_cufft_matches_own_ffts(ms, cuda):
    """The cuFFT form of the unfused comparator computes the same batch as the fused runner."""
    b = small_batch(ms)
    fused = ms.BatchRunner(b, cuda, streams=2).run()
    cufft = ms.BatchRunner(b, cuda, streams=1).run(plain="cufft")
    assert rel_l2(cufft.cpu().numpy(), fused.cpu().numpy()) < 1e-5


def test_stacked_apply_equals_separate_calls(ms, cuda):
    """Sample.apply_stacked over three fields gives each field's separate Sample.apply result
    bit for bit with the single-sequence kernels (same row kernel; the batched per-block column
    kernel and the pipelined one compute the same values)."""
    b = small_batch(ms)
    p = ms.item_params(b, b.items[0])
    n = p.nx
    from importlib import import_module
    plan = import_module("3d_ravesim_gb300")._lib.plan_for(n, n, cuda)
    old = plan.schedule()
    plan.set_schedule(old | 48)
    s = b.sample
    s.db_list = ms._scaled_db(b, b.items[0].energy)
    g = torch.Generator(device="cpu").manual_seed(9)
    fields = [torch.polar(torch.ones(n * n), torch.rand(n * n, generator=g) * 3).to(torch.complex64).to(cuda)
              for _ in range(3)]
    cutoff = b.cutoff_fraction / p.dx
    stack = torch.cat(fields).contiguous()
    Ustack = torch.zeros_like(stack)
    s.apply_stacked(stack, Ustack, 3, p, cutoff)
    for k, f in enumerate(fields):
        from importlib import import_module
        rs = import_module("3d_ravesim_gb300")
        u, U = rs.GpuVector(f.clone()), rs.GpuVector.zeros(n * n, cuda)
        s.apply(u, U, p, cutoff, 0, None)
        assert torch.equal(u.vec, stack[k * n * n:(k + 1) * n * n])
        assert torch.equal(U.vec, Ustack[k * n * n:(k + 1) * n * n])
    plan.set_schedule(old)


def test_stacked_batch_matches_per_item_batch(ms, cuda):
    b = ms.shell_batch(n_sources_side=3, n_energies=2, sizes=(256, 384), slices=8, fov=128e-6,
                       detector_pixels=256, seed=5)
    per_item = ms.BatchRunner(b, cuda, streams=2).run().clone()
    stacked = ms.BatchRunner(b, cuda, streams=2).run(stacked=True)
    assert max(len(g) for g in ms.group_items(b.items, 16)) > 1
    # stacked fields run the batched per-block column kernel (compensated twiddles), separate
    # items the split-pair column pipeline (dithered twiddles): equal to FP32 rounding
    assert rel_l2(stacked.cpu().numpy(), per_item.cpu().numpy()) < 1e-6
