"""Size-independent properties of the multislice path at the benchmark's full size (the 4096^2
Talbot-Lau workload: 512 voxel slices of 200 seeded blobs), where no FP64 run is affordable:

* linearity: a fixed sample's multislice is a linear map of the entering field, so
  run(a u0 + b u1) = a run(u0) + b run(u1) to FP32 rounding over the 512 slices;
* reproducibility: the same call twice gives the same bits;
* energy: free-space propagation with an inactive cutoff keeps sum |u|^2 (Parseval), and a
  sample without absorption (beta = 0) keeps it too, slice after slice.
"""
import importlib

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def talbot(rs):
    wl = importlib.import_module("3d_ravesim_gb300.workloads")
    return wl.talbot_lau(n=4096, slices=512)


def _field(seed, n, device):
    g = torch.Generator(device="cpu").manual_seed(seed)
    re = torch.randn(n * n, generator=g)
    im = torch.randn(n * n, generator=g)
    return torch.complex(re, im).to(torch.complex64).to(device)


def _run(rs, s, p, cutoff, u0):
    u, U = rs.GpuVector(u0.clone()), rs.GpuVector(torch.empty_like(u0))
    s.apply(u, U, p, cutoff, 0, None)
    torch.cuda.synchronize()
    return u.vec


def test_full_size_multislice_is_linear_and_reproducible(rs, cuda, talbot):
    s, p, cutoff = talbot.elements[1], talbot.params, talbot.cutoff
    n = p.nx
    u0, u1 = _field(1, n, cuda), _field(2, n, cuda)
    a, b = complex(0.6, -0.3), complex(-0.2, 0.9)
    r0 = _run(rs, s, p, cutoff, u0)
    r1 = _run(rs, s, p, cutoff, u1)
    rab = _run(rs, s, p, cutoff, a * u0 + b * u1)
    want = a * r0 + b * r1
    err = float(torch.linalg.vector_norm(rab - want) / torch.linalg.vector_norm(want))
    assert err < 2e-5, err
    assert torch.equal(_run(rs, s, p, cutoff, u0), r0)


def test_full_size_energy_without_absorption(rs, cuda, talbot):
    s, p = talbot.elements[1], talbot.params
    n = p.nx
    u0 = _field(3, n, cuda)
    e0 = float(torch.sum(torch.abs(u0.to(torch.complex128)) ** 2))
    # free space, cutoff beyond every frequency of the grid: Parseval
    u, U = rs.GpuVector(u0.clone()), rs.GpuVector(torch.empty_like(u0))
    rs.propagate_2d(u, U, p.dx, p.dy, p.wl, 0.05, p.chunk_size, 1.0 / p.dx, n, n)
    torch.cuda.synchronize()
    e1 = float(torch.sum(torch.abs(u.vec.to(torch.complex128)) ** 2))
    assert abs(e1 / e0 - 1.0) < 1e-5, e1 / e0
    # the same sample with beta = 0 (phase only) and an inactive cutoff: every step is unitary
    saved = s.db_list
    try:
        s.db_list = np.asarray(saved).real.astype(np.complex128)
        s.invalidate_device_cache()
        r = _run(rs, s, p, 1.0 / p.dx, u0)
    finally:
        s.db_list = saved
        s.invalidate_device_cache()
    e2 = float(torch.sum(torch.abs(r.to(torch.complex128)) ** 2))
    assert abs(e2 / e0 - 1.0) < 1e-4, e2 / e0
