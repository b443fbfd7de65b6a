"""rs_detector_noalloc: the detector for callers that cannot allocate device memory.

Some callers of this library do not own the device memory they run in: a framework whose
caching pool owns the GPU, or a service with a fixed memory budget. Others cannot accept the
device-wide synchronisation of the cudaMalloc/cudaFree with which rs_detector grows its table
buffer. rs_detector_noalloc keeps its tables in a fixed device array inside the library instead,
so a call allocates nothing. This file is named to be collected last: if it fails, a run that
stops at the first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _geom(rs, dx, dy, dpx, dpy, out_x, out_y, z, integrator):
    return rs._lib.DetectorGeom(dx, dy, dpx, dpy, z, out_x, out_y, integrator, 0)


@pytest.mark.parametrize("integrator", [0, 1])
def test_noalloc_detector_matches_planned_detector_twice(rs, cuda, integrator):
    lib = rs._lib.lib()
    nx, ny = 512, 384
    rng = np.random.default_rng(7 + integrator)
    field = torch.from_numpy((rng.normal(size=nx * ny) + 1j * rng.normal(size=nx * ny)).astype(np.complex64)).to(cuda)
    g = _geom(rs, 0.25e-6, 0.3e-6, 0.7e-6, 0.65e-6, 150, 160, 0.4, integrator)
    stream = rs._lib.stream_handle()
    plan = rs._lib.plan_for(nx, ny, cuda)
    ref = torch.zeros((160, 150), dtype=torch.float64, device=cuda)
    rs._lib.check(lib.rs_detector(plan.handle, rs._lib.ptr(field), rs._lib.ptr(ref), ctypes.byref(g), stream),
                  "rs_detector")
    outs = []
    for _ in range(2):
        out = torch.full((160, 150), -1.0, dtype=torch.float64, device=cuda)
        rs._lib.check(lib.rs_detector_noalloc(rs._lib.ptr(field), nx, ny, rs._lib.ptr(out), ctypes.byref(g), stream),
                      "rs_detector_noalloc")
        outs.append(out)
    torch.cuda.synchronize()
    r = ref.cpu().numpy()
    assert np.all(r > 0)
    for out in outs:
        np.testing.assert_allclose(out.cpu().numpy(), r, rtol=2e-6, atol=0)


def test_noalloc_detector_warm_call_takes_no_device_memory_and_rewrites_its_tables(rs, cuda):
    """A warm call leaves the device's free memory unchanged; a following call with another field
    size, output size and integrator reads none of the first call's tables (it matches its own
    planned detector)."""
    lib = rs._lib.lib()
    stream = rs._lib.stream_handle()
    cases = [(512, 384, _geom(rs, 0.25e-6, 0.3e-6, 0.7e-6, 0.65e-6, 150, 160, 0.4, 0)),
             (256, 640, _geom(rs, 0.4e-6, 0.2e-6, 0.5e-6, 0.9e-6, 90, 70, 0.7, 1))]
    fields, outs, refs = [], [], []
    for k, (nx, ny, g) in enumerate(cases):
        rng = np.random.default_rng(30 + k)
        fields.append(torch.from_numpy((rng.normal(size=nx * ny) + 1j * rng.normal(size=nx * ny))
                                       .astype(np.complex64)).to(cuda))
        outs.append(torch.full((g.out_y, g.out_x), -1.0, dtype=torch.float64, device=cuda))
        refs.append(torch.zeros((g.out_y, g.out_x), dtype=torch.float64, device=cuda))
        plan = rs._lib.plan_for(nx, ny, cuda)
        rs._lib.check(lib.rs_detector(plan.handle, rs._lib.ptr(fields[k]), rs._lib.ptr(refs[k]), ctypes.byref(g),
                                      stream), "rs_detector")
    (nx0, ny0, g0), (nx1, ny1, g1) = cases
    rs._lib.check(lib.rs_detector_noalloc(rs._lib.ptr(fields[0]), nx0, ny0, rs._lib.ptr(outs[0]), ctypes.byref(g0),
                                          stream), "rs_detector_noalloc")  # warm
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    rs._lib.check(lib.rs_detector_noalloc(rs._lib.ptr(fields[0]), nx0, ny0, rs._lib.ptr(outs[0]), ctypes.byref(g0),
                                          stream), "rs_detector_noalloc")
    rs._lib.check(lib.rs_detector_noalloc(rs._lib.ptr(fields[1]), nx1, ny1, rs._lib.ptr(outs[1]), ctypes.byref(g1),
                                          stream), "rs_detector_noalloc")
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free_before
    for out, ref in zip(outs, refs):
        r = ref.cpu().numpy()
        assert np.count_nonzero(r) > r.size // 2  # the legacy integrator leaves edge pixels empty
        np.testing.assert_allclose(out.cpu().numpy(), r, rtol=2e-6, atol=0)


def test_noalloc_detector_rejects_oversized_request(rs, cuda):
    """A 200000 x 200000 request needs ~13 MB of tables, three times the fixed array: it must be
    refused on the host before anything is launched (the buffers passed here are deliberately tiny
    and are never touched)."""
    lib = rs._lib.lib()
    n = 200000
    g = _geom(rs, 1e-7, 1e-7, 1e-7, 1e-7, n, n, 0.4, 0)
    dummy = torch.zeros(16, dtype=torch.complex64, device=cuda)
    out = torch.zeros(16, dtype=torch.float64, device=cuda)
    st = lib.rs_detector_noalloc(rs._lib.ptr(dummy), n, n, rs._lib.ptr(out), ctypes.byref(g),
                                 rs._lib.stream_handle())
    assert st == rs._lib.RS_EINVAL
    assert b"fixed" in lib.rs_last_error()
