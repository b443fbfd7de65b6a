"""Four-step plans (axes up to 32768): rs_propagate through the length-n/256 and length-256
transforms against the single-pass plan and the FP64 oracle at 4096/8192, the spectrum in
four-step storage order, skip_fft chaining, and at 32768^2 the dz / -dz round trip and
Parseval (no FP64 reference fits the host there)."""

import numpy as np
import pytest
import torch

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def storage_to_natural(n: int) -> np.ndarray:
    """Frequency held by storage entry i of an axis of length n."""
    i = np.arange(n)
    return i // 256 + (n // 256) * (i % 256)


def natural_spectrum(U: np.ndarray) -> np.ndarray:
    ny, nx = U.shape
    out = np.empty_like(U)
    out[np.ix_(storage_to_natural(ny), storage_to_natural(nx))] = U
    return out


def propagate(rs, plan, u, U, dx, dy, wl, dz, f, skip=0):
    rs._lib.check(rs._lib.lib().rs_propagate(plan.handle, rs._lib.ptr(u), rs._lib.ptr(U), dx, dy, wl, dz, f, skip,
                                             rs._lib.stream_handle()), "rs_propagate")


def field(n_y, n_x, seed, device):
    g = torch.Generator(device="cpu").manual_seed(seed)
    re = torch.randn(n_y * n_x, generator=g)
    ph = torch.rand(n_y * n_x, generator=g) * 6.283
    return torch.polar(1 + 0.1 * re, ph).to(torch.complex64).to(device)


@pytest.mark.parametrize("nx,ny", [(4096, 4096), (8192, 4096), (4096, 16384)])
def test_four_step_matches_single_pass(rs, cuda, nx, ny):
    lib = rs._lib
    four = lib.Plan(nx, ny, cuda, flags=lib.RS_PLAN_FOURSTEP)
    std = lib.Plan(nx, ny, cuda)
    assert four.four_step and not std.four_step and std.fast
    dx, dy, wl = 0.1e-6, 0.12e-6, 5e-11
    f = 0.4 / dx  # active cutoff
    u0 = field(ny, nx, 11, cuda)
    u1, U1 = u0.clone(), torch.empty_like(u0)
    u2, U2 = u0.clone(), torch.empty_like(u0)
    with torch.cuda.device(cuda):
        propagate(rs, four, u1, U1, dx, dy, wl, 2e-3, f)
        propagate(rs, std, u2, U2, dx, dy, wl, 2e-3, f)
    torch.cuda.synchronize()
    # both FP32; the four-step W_n twiddles are sincospif values, the single-pass ones compensated
    assert rel_l2(u1.cpu().numpy(), u2.cpu().numpy()) < 4e-6
    Un = natural_spectrum(U1.cpu().numpy().reshape(ny, nx))
    assert rel_l2(Un, U2.cpu().numpy().reshape(ny, nx)) < 4e-6
    # a second step from the stored spectrum (skip_fft) continues both the same way
    with torch.cuda.device(cuda):
        propagate(rs, four, u1, U1, dx, dy, wl, 1e-3, f, skip=1)
        propagate(rs, std, u2, U2, dx, dy, wl, 1e-3, f, skip=1)
    torch.cuda.synchronize()
    assert rel_l2(u1.cpu().numpy(), u2.cpu().numpy()) < 6e-6


def test_four_step_vs_fp64_oracle(rs, cuda, oracle):
    nx = ny = 4096
    lib = rs._lib
    four = lib.Plan(nx, ny, cuda, flags=lib.RS_PLAN_FOURSTEP)
    dx, wl = 0.1e-6, rs.convert_energy_wavelength(25000.0)
    f = 0.45 / dx
    u0 = field(ny, nx, 5, cuda)
    u, U = u0.clone(), torch.empty_like(u0)
    with torch.cuda.device(cuda):
        propagate(rs, four, u, U, dx, dx, wl, 0.01, f)
    ref, _ = oracle.propagate_2d(u0.cpu().numpy().astype(np.complex128).reshape(ny, nx), dx, dx, wl, 0.01, f)
    assert rel_l2(u.cpu().numpy().reshape(ny, nx), ref) < 1e-5


def test_four_step_rejects_other_entry_points(rs, cuda):
    lib = rs._lib
    four = lib.Plan(4096, 4096, cuda, flags=lib.RS_PLAN_FOURSTEP)
    u = torch.zeros(4096 * 4096, dtype=torch.complex64, device=cuda)
    rc = lib.lib().rs_fft2(four.handle, lib.ptr(u), lib.ptr(u), lib.stream_handle())
    assert rc != 0 and b"four-step" in lib.lib().rs_last_error()
    with pytest.raises(Exception):
        lib.Plan(4096, 3072, cuda, flags=lib.RS_PLAN_FOURSTEP)


def test_32768_round_trip_and_parseval(rs, cuda):
    """The 32768^2 sweep: propagate by dz with the cutoff inactive keeps the field's norm
    (Parseval, the transfer function has modulus 1), and -dz brings the field back."""
    n = 32768
    p = rs.SimParams(N=n * n, nx=n, ny=n, dx=50e-9, dy=50e-9, z_detector=1.0, detector_size=n * 50e-9,
                     detector_pixel_size_x=50e-9 * 64, detector_pixel_size_y=50e-9 * 64,
                     wl=rs.convert_energy_wavelength(30000.0), chunk_size=n)
    plan = rs._lib.plan_for(n, n, cuda)
    assert plan.four_step
    u = rs.GpuVector(field(n, n, 3, cuda))
    u0 = u.vec.clone()
    U = rs.GpuVector.zeros(n * n, cuda)
    f = 1.0 / p.dx  # 2 f^2 above every kx^2 + ky^2: no frequency is cut
    rs.propagate_2d(u, U, p.dx, p.dy, p.wl, 1e-4, p.chunk_size, f, n, n)
    n0 = torch.linalg.vector_norm(u0.to(torch.complex128)).item()
    n1 = torch.linalg.vector_norm(u.vec.to(torch.complex128)).item()
    assert abs(n1 / n0 - 1) < 2e-6
    assert (u.vec - u0).abs().max().item() > 1e-3  # the step did something
    rs.propagate_2d(u, U, p.dx, p.dy, p.wl, -1e-4, p.chunk_size, f, n, n)
    err = (torch.linalg.vector_norm((u.vec - u0).to(torch.complex128)) / n0).item()
    assert err < 2e-5
    # detector on the four-step plan's (natural-order) field
    img = rs.square_and_downsample_2d(u, p, 1.0)
    assert img.shape == (512, 512) and np.isfinite(img).all()
    del u, U, u0
    torch.cuda.empty_cache()


def test_32768_spectrum_reads_as_natural_fft2(rs, cuda):
    """At 32768^2 U keeps the four-step plan's storage order on the device, but reads as big-wave's
    U = FFT2(u): bins picked in natural order from U (through the storage index the host reads
    use) equal a direct DFT of the new u at those bins."""
    from importlib import import_module
    vec = import_module("3d_ravesim_gb300.vector")
    n = 32768
    p = rs.SimParams(N=n * n, nx=n, ny=n, dx=50e-9, dy=50e-9, z_detector=1.0, detector_size=n * 50e-9,
                     detector_pixel_size_x=50e-9 * 64, detector_pixel_size_y=50e-9 * 64,
                     wl=rs.convert_energy_wavelength(30000.0), chunk_size=n)
    u = rs.GpuVector(field(n, n, 5, cuda))
    U = rs.GpuVector.zeros(n * n, cuda)
    rs.propagate_2d(u, U, p.dx, p.dy, p.wl, 2e-4, p.chunk_size, 0.45 / p.dx, n, n)
    assert U.spectrum_order == ("four_step", n, n)
    freq = vec.four_step_frequency(n)
    storage_of = np.empty(n, dtype=np.int64)
    storage_of[freq] = np.arange(n)
    rng = np.random.default_rng(11)
    kx = np.concatenate([[0, 1, n - 1, 5000], rng.integers(0, n, 4)])
    ky = np.concatenate([[0, n // 2, 2, 7], rng.integers(0, n, 4)])
    # direct DFT at (ky, kx): X = sum_y e^{-2 pi i ky y/n} sum_x u[y, x] e^{-2 pi i kx x/n}
    xs = torch.arange(n, device=cuda, dtype=torch.float64)
    ex = torch.polar(torch.ones(n, len(kx), device=cuda, dtype=torch.float64),
                     -2 * np.pi * torch.outer(xs, torch.tensor(kx, device=cuda, dtype=torch.float64)) / n)
    rows = u.vec.view(n, n) @ ex.to(torch.complex64)                       # (n, len(kx))
    ey = torch.polar(torch.ones(len(ky), n, device=cuda, dtype=torch.float64),
                     -2 * np.pi * torch.outer(torch.tensor(ky, device=cuda, dtype=torch.float64), xs) / n)
    direct = (ey @ rows.to(torch.complex128)).diagonal().cpu().numpy()     # X[ky[j], kx[j]]
    idx = torch.tensor(storage_of[ky] * n + storage_of[kx], device=cuda)
    got = U.vec[idx].cpu().numpy().astype(np.complex128)
    scale = np.sqrt(float((u.vec.abs() ** 2).sum().item()) * n * n) / n  # typical |X| of the field
    assert np.max(np.abs(got - direct)) / scale < 1e-4
    del u, U, rows, ex, ey
    torch.cuda.empty_cache()


def shell_sample(rs, nz, ny_v, nx_v, pitch, seed=0):
    zz = (np.arange(nz) - (nz - 1) / 2.0)[:, None, None] * pitch
    yy = (np.arange(ny_v) - ny_v / 2.0)[None, :, None] * pitch
    xx = (np.arange(nx_v) - nx_v / 2.0)[None, None, :] * pitch
    r = np.sqrt(xx ** 2 + yy ** 2 + zz ** 2)
    rmax = 0.45 * min(ny_v, nx_v) * pitch
    grid = ((r <= rmax) & (r >= 0.8 * rmax)).astype(np.uint32)
    s = rs.Sample(z_start=0.1, pixel_size_x=pitch, pixel_size_z=2e-6, grid=grid, materials=[rs.Material("A", 1.0)],
                  x_positions=np.array([0.0]), pixel_size_y=pitch, y_positions=np.array([0.0]))
    s.db_list = np.array([0.0, 2.5e-7 + 1.5e-10j])
    return s


@pytest.mark.parametrize("nx,ny,slices", [(1024, 4096, 6)])
def test_split_columns_vs_fp64_oracle(rs, cuda, oracle, nx, ny, slices):
    """Sample.apply with the three-pass columns (RS_SCHED_SPLIT_COLS) against big-wave's FP64
    restatement, and against the single column pass."""
    dx = 0.25e-6
    wl = rs.convert_energy_wavelength(20000.0)
    p = rs.SimParams(N=nx * ny, nx=nx, ny=ny, dx=dx, dy=dx, z_detector=1.0, detector_size=nx * dx,
                     detector_pixel_size_x=dx, detector_pixel_size_y=dx, wl=wl, chunk_size=nx)
    s = shell_sample(rs, slices, ny + 2, nx + 2, dx)
    f = 0.45 / dx
    plan = rs._lib.plan_for(nx, ny, cuda)
    assert 40 in plan.schedules()  # split columns: a choice of the single-sequence column kernels (bit 32)
    g = torch.Generator(device="cpu").manual_seed(2)
    u0 = torch.polar(torch.ones(nx * ny), torch.rand(nx * ny, generator=g) * 0.3).to(torch.complex64)
    out = {}
    old = plan.schedule()
    try:
        for mask in ((old | 32) & ~8, old | 40):
            plan.set_schedule(mask)
            u = rs.GpuVector(u0.clone().to(cuda))
            U = rs.GpuVector.zeros(nx * ny, cuda)
            s.apply(u, U, p, f, 0, None)
            out[mask] = u.to_numpy().reshape(ny, nx)
    finally:
        plan.set_schedule(old)
    single, split = out[(old | 32) & ~8], out[old | 40]
    assert rel_l2(split, single) < 5e-6
    ref, _ = oracle.sample_apply_2d(u0.numpy().astype(np.complex128).reshape(ny, nx), np.asarray(s.grid), s.db_list,
                                    dx, dx, wl, f, s.pixel_size_x, s.pixel_size_y, s.pixel_size_z)
    assert rel_l2(split, ref) < 1e-5
    assert rel_l2(single, ref) < 1e-5


def test_split_columns_16384(rs, cuda):
    """The 16384-point columns of the large-field case: three-pass columns against the single
    per-block column pass over a few voxel slices."""
    nx, ny, slices = 512, 16384, 4
    dx = 50e-9
    wl = rs.convert_energy_wavelength(30000.0)
    p = rs.SimParams(N=nx * ny, nx=nx, ny=ny, dx=dx, dy=dx, z_detector=1.0, detector_size=nx * dx,
                     detector_pixel_size_x=dx, detector_pixel_size_y=dx, wl=wl, chunk_size=nx)
    s = shell_sample(rs, slices, ny + 2, nx + 2, dx)
    plan = rs._lib.plan_for(nx, ny, cuda)
    g = torch.Generator(device="cpu").manual_seed(4)
    u0 = torch.polar(torch.ones(nx * ny), torch.rand(nx * ny, generator=g) * 0.3).to(torch.complex64)
    out = {}
    old = plan.schedule()
    try:
        for mask in (0, 8):
            plan.set_schedule(mask)
            u = rs.GpuVector(u0.clone().to(cuda))
            U = rs.GpuVector.zeros(nx * ny, cuda)
            s.apply(u, U, p, 0.45 / dx, 0, None)
            out[mask] = u.to_numpy()
    finally:
        plan.set_schedule(old)
    assert rel_l2(out[8], out[0]) < 5e-6


def test_point_source_propagate_four_step(rs, cuda):
    """rs_point_source_propagate on a four-step plan (source field, then FFT -> cutoff -> IFFT as a
    four-step propagation of dz = 0) against the single-pass plan."""
    lib = rs._lib
    n = 4096
    four = lib.Plan(n, n, cuda, flags=lib.RS_PLAN_FOURSTEP)
    std = lib.Plan(n, n, cuda)
    dx, wl = 0.1e-6, rs.convert_energy_wavelength(25000.0)
    out = []
    for plan in (four, std):
        u = torch.zeros(n * n, dtype=torch.complex64, device=cuda)
        U = torch.zeros_like(u)
        lib.check(lib.lib().rs_point_source_propagate(plan.handle, lib.ptr(u), lib.ptr(U), dx, dx, 2e-6, -1e-6, 1.0,
                                                     wl, 0.4 / dx, lib.stream_handle()), "point source")
        torch.cuda.synchronize()
        out.append(u.cpu().numpy())
    assert rel_l2(out[0], out[1]) < 4e-6


def test_vacuum_run_32768(rs, cuda):
    """run_simulation with no element at 32768^2 (point source 3 m before the detector): the
    detected energy is the detector's solid angle, area / z^2, as in big-wave's vacuum runs."""
    import importlib
    ws = importlib.import_module("3d_ravesim_gb300.wavesim")
    n, dx, z = 32768, 50e-9, 3.0
    wl = rs.convert_energy_wavelength(30000.0)
    p = rs.SimParams(N=n * n, nx=n, ny=n, dx=dx, dy=dx, z_detector=z, detector_size=4e-4, detector_size_x=4e-4,
                     detector_size_y=4e-4, detector_pixel_size_x=8e-7, detector_pixel_size_y=8e-7, wl=wl,
                     chunk_size=n)
    u, U = rs.GpuVector.zeros(n * n, cuda), rs.GpuVector.zeros(n * n, cuda)
    angle = float(np.arcsin(0.3 / dx * wl))
    img = ws.run_simulation(p, rs.PointSource(x=0.0, y=0.0, z=0.0), [], [angle], u, U, [])[0]
    assert img.shape == (500, 500)
    assert abs(float(img.sum()) / ((4e-4) ** 2 / z ** 2) - 1) < 1e-4
    del u, U
    torch.cuda.empty_cache()
