"""Device-side timeouts reach the caller, and a run allocates no device memory once its plan and
buffers are set up.

The timeout is made without any fault: the plan's test hook makes the next pipelined column pass
wait on a barrier that nothing completes, with a short bound; the pass records the timeout in the
plan's status word and returns without touching the field. The host reads the word after its own
stream synchronisation (no device-wide sync) and raises TimeoutError."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _field(rs, cuda, n, seed):
    rng = np.random.default_rng(seed)
    x = (rng.normal(size=n * n) + 1j * rng.normal(size=n * n)).astype(np.complex64)
    return rs.GpuVector.from_numpy(x, cuda), rs.GpuVector.zeros(n * n, cuda)


def _params(rs, n, dx=0.5e-6):
    return rs.SimParams(N=n * n, nx=n, ny=n, dx=dx, dy=dx, z_detector=1.0, detector_size=n * dx,
                        detector_pixel_size_x=2 * dx, detector_pixel_size_y=2 * dx,
                        wl=rs.convert_energy_wavelength(20000.0), chunk_size=n)


def test_stalled_pass_raises_timeout_and_clears(rs, cuda):
    n = 1024
    plan = rs._lib.plan_for(n, n, cuda)
    plan.set_schedule(2)  # pipelined columns
    p = _params(rs, n)
    u, U = _field(rs, cuda, n, 1)
    plan.test_stall(True)
    rs.propagate_2d(u, U, p.dx, p.dy, p.wl, 0.01, n, 0.4 / p.dx, n, n)
    with pytest.raises(TimeoutError, match="gave up waiting"):
        rs.square_and_downsample_2d(u, p, p.z_detector)
    # reported once, then cleared: the same call sequence now runs and matches a fresh field's run
    u1, U1 = _field(rs, cuda, n, 2)
    rs.propagate_2d(u1, U1, p.dx, p.dy, p.wl, 0.01, n, 0.4 / p.dx, n, n)
    img = rs.square_and_downsample_2d(u1, p, p.z_detector)
    assert np.all(np.isfinite(img))
    assert plan.status() == 0


def test_stall_seen_through_the_c_abi_without_device_sync(rs, cuda):
    n = 512
    lib = rs._lib.lib()
    plan = rs._lib.plan_for(n, n, cuda)
    plan.set_schedule(2)
    u, U = _field(rs, cuda, n, 3)
    stream = rs._lib.stream_handle()
    assert lib.rs_plan_test_stall(plan.handle, 1) == rs._lib.RS_OK
    st = lib.rs_propagate(plan.handle, rs._lib.ptr(u.vec), rs._lib.ptr(U.vec), 5e-7, 5e-7, 6e-11, 0.01,
                          8e5, 0, stream)
    assert st == rs._lib.RS_OK  # the launch itself succeeds; the pass reports through the status word
    torch.cuda.current_stream().synchronize()
    word = ctypes.c_int(0)
    assert lib.rs_plan_check(plan.handle, ctypes.byref(word)) == rs._lib.RS_ETIMEOUT
    assert word.value != 0
    assert lib.rs_plan_clear_status(plan.handle, stream) == rs._lib.RS_OK
    assert lib.rs_plan_check(plan.handle, ctypes.byref(word)) == rs._lib.RS_OK and word.value == 0


def test_run_allocates_nothing_after_setup(rs, cuda):
    """A two-element run (voxel Sample, PlasmaSample) with the detector: after the plan exists and
    reserve_run_buffers has sized its buffers, the run makes no library allocation."""
    n = 512
    dx = 0.5e-6
    p = _params(rs, n, dx)
    g = n + 2
    nz = 3
    zz = (np.arange(nz) - (nz - 1) / 2)[:, None, None] * 2e-6
    yy = (np.arange(g) - g / 2)[None, :, None] * dx
    xx = (np.arange(g) - g / 2)[None, None, :] * dx
    r = np.sqrt(xx ** 2 + yy ** 2 + zz ** 2)
    grid = ((r <= 60e-6) & (r >= 40e-6)).astype(np.uint32)
    s = rs.Sample(z_start=0.5, pixel_size_x=dx, pixel_size_z=2e-6, grid=grid, materials=[rs.Material("shell", 1.0)],
                  x_positions=np.array([0.0]), pixel_size_y=dx, y_positions=np.array([0.0]))
    s.db_list = np.array([0.0, 3.2e-7 + 2.1e-10j])
    ne = (1e21 * np.exp(-r ** 2 / (2 * (50e-6) ** 2))).astype(np.float32)
    ps = rs.PlasmaSample(z_start=0.6, pixel_size_x=dx, pixel_size_z=2e-6, ne_grid=ne, ni_grid=ne / 3.5,
                         te_grid=np.full_like(ne, 500.0), zstar_grid=np.full_like(ne, 3.5), Z=6,
                         x_positions=np.array([0.0]), formula="CH", pixel_size_y=dx, y_positions=np.array([0.0]),
                         scattering_factors=(3.5, 0.002, 3.5, 18.5))
    ps.store_deltabetas = lambda table: None
    s.store_deltabetas = lambda table: None
    src = rs.PointSource(x=0.0, y=0.0, z=0.5 - 3.0)  # 3 m upstream: the spherical phase does not alias
    u, U = rs.GpuVector.zeros(n * n, cuda), rs.GpuVector.zeros(n * n, cuda)
    wavesim = __import__("importlib").import_module("3d_ravesim_gb300.wavesim")
    propagation = __import__("importlib").import_module("3d_ravesim_gb300.propagation")

    def run():
        return wavesim.run_simulation(p, src, [s, ps], [0.3, 0.3, 0.3], u, U, None)

    propagation.reserve_run_buffers(p, cuda, [s, ps])
    before = rs._lib.alloc_count()
    first = run()
    torch.cuda.synchronize()
    assert rs._lib.alloc_count() == before
    second = run()
    assert rs._lib.alloc_count() == before
    np.testing.assert_array_equal(first[0], second[0])


def test_cancel_flag_stops_the_multislice_loop(rs, cuda):
    """A set cancel flag stops rs_multislice_voxel before its first slice with InterruptedError;
    cleared, the same call runs to the field of an uncancelled plan."""
    n = 256
    dx = 0.5e-6
    p = rs.SimParams(N=n * n, nx=n, ny=n, dx=dx, dy=dx, z_detector=1.0, detector_size=n * dx,
                     detector_pixel_size_x=dx, detector_pixel_size_y=dx,
                     wl=rs.convert_energy_wavelength(20000.0), chunk_size=n)
    grid = np.random.default_rng(5).integers(0, 2, size=(4, n // 2 + 4, n // 2 + 4)).astype(np.uint32)
    s = rs.Sample(z_start=0.5, pixel_size_x=2 * dx, pixel_size_z=1e-6, grid=grid,
                  materials=[rs.Material("a", 1.0)], x_positions=np.array([0.0]), pixel_size_y=2 * dx,
                  y_positions=np.array([0.0]))
    s.db_list = np.array([0, 2e-7 + 1e-10j])
    plan = rs._lib.plan_for(n, n, cuda)
    flag = ctypes.c_int(1)
    plan.set_cancel_flag(flag)
    try:
        u, U = rs.GpuVector.ones(n * n, cuda), rs.GpuVector.zeros(n * n, cuda)
        with pytest.raises(InterruptedError, match="cancelled before slice 0"):
            s.apply(u, U, p, 0.45 / dx, 0, None)
        flag.value = 0
        s.apply(u, U, p, 0.45 / dx, 0, None)
        got = u.to_numpy()
    finally:
        plan.set_cancel_flag(None)
    u2, U2 = rs.GpuVector.ones(n * n, cuda), rs.GpuVector.zeros(n * n, cuda)
    s.apply(u2, U2, p, 0.45 / dx, 0, None)
    np.testing.assert_array_equal(got, u2.to_numpy())
