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


def test_group_items_by_size_and_energy():
    import importlib
    ms = importlib.import_module("3d_ravesim_gb300.multisim")
    It = ms.Item
    items = [It(0.0, 0.0, 20e3, 256), It(1.0, 0.0, 20e3, 384), It(2.0, 0.0, 20e3, 256), It(3.0, 0.0, 25e3, 256),
             It(4.0, 0.0, 20e3, 256), It(5.0, 0.0, 20e3, 256)]
    groups = ms.group_items(items, 3)
    assert [[it.x for it in g] for g in groups] == [[0.0, 2.0, 4.0], [5.0], [1.0], [3.0]]
    assert sum(len(g) for g in groups) == len(items)
