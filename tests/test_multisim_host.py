"""Host side of the batched multisim: sampling against big-wave, sharding, and the cross-rank
detector sum on CPU ranks (gloo, world size 2)."""
import importlib
import os

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


@pytest.fixture(scope="module")
def ms():
    return importlib.import_module("3d_ravesim_gb300.multisim")


def test_energy_sampling_matches_reference(ms, golden):
    out = ms.generate_energies_from_spectrum(golden["spectrum_e"], golden["spectrum_i"], np.random.RandomState(11),
                                             (15e3, 40e3), 64)
    np.testing.assert_array_equal(out, golden["spectrum_draw"])


def test_energy_sampling_rejects_narrow_range(ms):
    e = np.arange(10, 51, dtype=np.float64) * 1e3
    with pytest.raises(ValueError, match="Not enough energy points"):
        ms.generate_energies_from_spectrum(e, np.ones_like(e), np.random.RandomState(0), (20e3, 20.5e3), 4)


def test_config2_batch_shape(ms):
    b = ms.shell_batch()
    assert len(b.items) == 1024
    assert set(i.n for i in b.items) == {1024, 1536, 2048, 3072}
    assert all(15e3 <= i.energy < 41e3 for i in b.items)
    xs = sorted(set(round(i.x, 12) for i in b.items))
    assert len(xs) == 64 and max(abs(x) for x in xs) < 20e-6


def test_shard_items_partitions_by_cost(ms):
    b = ms.shell_batch()
    shards = [ms.shard_items(b.items, r, 4) for r in range(4)]
    assert sum(len(s) for s in shards) == len(b.items)
    cost = [sum(i.n ** 2 for i in s) for s in shards]
    assert max(cost) / min(cost) < 1.05
    ids = sorted(id(i) for s in shards for i in s)
    assert ids == sorted(id(i) for i in b.items)


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = importlib.import_module("3d_ravesim_gb300.multisim")
    img = torch.full((8, 8), float(rank + 1), dtype=torch.float64)
    ms.reduce_detector(img)
    q.put((rank, float(img.sum())))
    dist.destroy_process_group()


def test_reduce_detector_two_cpu_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs)
    res = dict(q.get(timeout=5) for _ in range(2))
    assert res == {0: 64 * 3.0, 1: 64 * 3.0}


def _item_image(it, npx=16):
    """Host stand-in for one item's detector image: integer counts (so any summation order gives
    the same float64 sum) placed by the source position and scaled by energy and grid size."""
    img = torch.zeros((npx, npx), dtype=torch.float64)
    ix = int(abs(it.x) * 1e6) % npx
    iy = int(abs(it.y) * 1e6) % npx
    img[iy, ix] += round(it.energy / 1000.0)
    img[(iy + 3) % npx, :] += it.n // 512
    return img


def _sharded_rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = importlib.import_module("3d_ravesim_gb300.multisim")
    b = ms.shell_batch(n_sources_side=4, n_energies=5, slices=4, fov=64e-6)
    seen = []

    def run_items(items):
        seen.extend(items)
        out = torch.zeros((16, 16), dtype=torch.float64)
        for it in items:
            out += _item_image(it)
        return out
    img = ms.run_sharded(b, rank, world, run_items=run_items)
    q.put((rank, img.numpy().tolist(), [(it.x, it.y, it.energy, it.n) for it in seen]))
    dist.destroy_process_group()


def test_sharded_batch_equals_single_rank_sum():
    """Two gloo ranks each run their shard of a 80-item batch; after the one reduce every rank
    holds the single-rank sum of all items bit for bit, and the shards partition the batch."""
    ms = importlib.import_module("3d_ravesim_gb300.multisim")
    b = ms.shell_batch(n_sources_side=4, n_energies=5, slices=4, fov=64e-6)
    whole = torch.zeros((16, 16), dtype=torch.float64)
    for it in b.items:
        whole += _item_image(it)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + (os.getpid() + 7) % 1000
    procs = [ctx.Process(target=_sharded_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = {}
    for _ in range(2):
        rank, img, seen = q.get(timeout=120)
        res[rank] = (np.array(img), seen)
    for p in procs:
        p.join(60)
    assert all(p.exitcode == 0 for p in procs)
    for rank in (0, 1):
        assert np.array_equal(res[rank][0], whole.numpy())
    keys = sorted(res[0][1] + res[1][1])
    assert keys == sorted((it.x, it.y, it.energy, it.n) for it in b.items)
    assert res[0][1] and res[1][1]


def test_group_items_by_size_and_energy():
    import importlib
    ms = importlib.import_module("3d_ravesim_gb300.multisim")
    It = ms.Item
    items = [It(0.0, 0.0, 20e3, 256), It(1.0, 0.0, 20e3, 384), It(2.0, 0.0, 20e3, 256), It(3.0, 0.0, 25e3, 256),
             It(4.0, 0.0, 20e3, 256), It(5.0, 0.0, 20e3, 256)]
    groups = ms.group_items(items, 3)
    assert [[it.x for it in g] for g in groups] == [[0.0, 2.0, 4.0], [5.0], [1.0], [3.0]]
    assert sum(len(g) for g in groups) == len(items)
