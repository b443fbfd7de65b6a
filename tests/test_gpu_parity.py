"""CUDA path vs the oracle and vs fixtures produced by big-wave itself.

Tolerances: the GPU path computes in complex64 / FP32 (FP64 only for tables and the
point-source phase). Against FP64 references a single Fresnel step agrees to a relative L2
of ~1e-6; the bounds below leave ~10x margin. Index work (cutoff mask, sample indices) is
checked bit-exactly.
"""
import numpy as np
import pytest
import torch

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def gv(rs, arr, cuda):
    return rs.GpuVector.from_numpy(np.asarray(arr, np.complex64).reshape(-1), cuda)


def host(v, ny, nx):
    torch.cuda.synchronize()
    return v.to_numpy().reshape(ny, nx)


FAST = [(16, 16), (32, 64), (64, 32), (128, 256), (512, 128), (1024, 64), (256, 2048), (4096, 16), (64, 4096),
        (8192, 32), (32, 8192), (16384, 16), (16, 16384),
        (24, 48), (96, 1536), (3072, 64), (1536, 192), (768, 384), (48, 6144), (12288, 16)]
GENERIC = [(40, 28), (72, 72), (24, 16), (48, 64), (3, 3), (4, 4)]


@pytest.mark.parametrize("nx,ny", FAST + GENERIC)
def test_fft2_ifft2_vs_scipy(rs, cuda, nx, ny):
    rng = np.random.default_rng(nx * 7 + ny)
    x = (rng.normal(size=(ny, nx)) + 1j * rng.normal(size=(ny, nx)))
    a, b, c = gv(rs, x, cuda), rs.GpuVector.zeros(nx * ny, cuda), rs.GpuVector.zeros(nx * ny, cuda)
    a.fft2(b, nx, ny)
    b.ifft2(c, nx, ny)
    ref = np.fft.fft2(x)
    assert rel_l2(host(b, ny, nx), ref) < 2e-6
    assert rel_l2(host(c, ny, nx), x) < 2e-6


def test_fft2_fastwave_kats(rs, cuda):
    """fast-wave/test/fwtest.cu:131-230: 3x3 ones and 4x4 arange vs numpy.fft.fft2 literals."""
    a, b = gv(rs, np.ones((3, 3)), cuda), rs.GpuVector.zeros(9, cuda)
    a.fft2(b, 3, 3)
    exp = np.zeros((3, 3))
    exp[0, 0] = 9
    np.testing.assert_allclose(host(b, 3, 3), exp, atol=2e-6)
    m = np.arange(1, 17).reshape(4, 4)
    a, b = gv(rs, m, cuda), rs.GpuVector.zeros(16, cuda)
    a.fft2(b, 4, 4)
    exp4 = np.array([[136, -8 + 8j, -8, -8 - 8j], [-32 + 32j, 0, 0, 0], [-32, 0, 0, 0], [-32 - 32j, 0, 0, 0]])
    np.testing.assert_allclose(host(b, 4, 4), exp4, atol=2e-5)


def test_fft2_in_place(rs, cuda):
    rng = np.random.default_rng(5)
    x = rng.normal(size=(256, 512)) + 1j * rng.normal(size=(256, 512))
    a = gv(rs, x, cuda)
    a.fft2(a, 512, 256)
    assert rel_l2(host(a, 256, 512), np.fft.fft2(x)) < 2e-6


def test_cutoff_matches_golden_bit_exact_mask(rs, cuda, golden):
    nx, ny, dx, dy, f = golden["cutoff_params"]
    nx, ny = int(nx), int(ny)
    v = gv(rs, golden["cutoff_in"], cuda)
    rs.apply_frequency_cutoff_2d(v, f, dx, dy, nx, ny, nx * 4)
    out = host(v, ny, nx)
    ref = golden["cutoff_out"]
    np.testing.assert_array_equal(out == 0, ref == 0)
    np.testing.assert_array_equal(out, ref.astype(np.complex64))


@pytest.mark.parametrize("nx,ny", [(64, 64), (256, 128)])
def test_cutoff_fast_sizes_vs_oracle(rs, cuda, oracle, nx, ny):
    rng = np.random.default_rng(1)
    x = (rng.normal(size=(ny, nx)) + 1j * rng.normal(size=(ny, nx))).astype(np.complex64)
    for f in (0.2e6, 1.7e6, 3.3e6, 1e9):
        v = gv(rs, x, cuda)
        rs.apply_frequency_cutoff_2d(v, f, 1e-7, 1.3e-7, nx, ny, nx)
        np.testing.assert_array_equal(host(v, ny, nx), oracle.apply_frequency_cutoff_2d(x, f, 1e-7, 1.3e-7))


def test_circular_cutoff_axis_and_diagonal(rs, cuda):
    """tests/big_wave_2d/test_p5.py:126-140."""
    nx = ny = 64
    spec = np.zeros((ny, nx), np.complex64)
    spec[0, 14], spec[0, 15], spec[10, 10], spec[10, 11] = 1, 2, 3, 4
    v = gv(rs, spec, cuda)
    rs.apply_frequency_cutoff_2d(v, 10 / nx, 1.0, 1.0, nx, ny, 4 * nx)
    a = host(v, ny, nx)
    assert a[0, 14] == 1 and a[0, 15] == 0 and a[10, 10] == 3 and a[10, 11] == 0


def test_propagate_2d_vs_golden_generic_size(rs, cuda, golden):
    nx, ny, dx, dy, wl, dz1, f1, dz2, f2 = golden["prop_params"]
    nx, ny = int(nx), int(ny)
    for name in ("c128", "c64"):
        u, U = gv(rs, golden[f"prop_{name}_in"], cuda), rs.GpuVector.zeros(nx * ny, cuda)
        rs.propagate_2d(u, U, dx, dy, wl, dz1, nx * 4, f1, nx, ny)
        assert rel_l2(host(u, ny, nx), golden[f"prop_{name}_u"]) < 1e-5
        assert rel_l2(host(U, ny, nx), golden[f"prop_{name}_U"]) < 1e-5
        rs.propagate_2d(u, U, dx, dy, wl, dz2, nx * 4, f2, nx, ny, skip_fft=True)
        assert rel_l2(host(u, ny, nx), golden[f"prop_{name}_skip_u"]) < 1e-5
        assert rel_l2(host(U, ny, nx), golden[f"prop_{name}_skip_U"]) < 1e-5


@pytest.mark.parametrize("nx,ny", [(64, 64), (128, 512), (1024, 1024), (256, 4096), (1536, 1536), (3072, 96),
                                   (24, 3072)])
def test_propagate_2d_fast_sizes_vs_fp64_oracle(rs, cuda, oracle, nx, ny):
    rng = np.random.default_rng(nx + ny)
    x = (rng.normal(size=(ny, nx)) + 1j * rng.normal(size=(ny, nx)))
    dx, dy, wl = 1e-7, 1.3e-7, oracle.convert_energy_wavelength(8000.0)
    u, U = gv(rs, x, cuda), rs.GpuVector.zeros(nx * ny, cuda)
    rs.propagate_2d(u, U, dx, dy, wl, 0.003, nx, 2.0e6, nx, ny)
    ru, rU = oracle.propagate_2d(x.astype(np.complex128), dx, dy, wl, 0.003, 2.0e6)
    assert rel_l2(host(u, ny, nx), ru) < 1e-5
    assert rel_l2(host(U, ny, nx), rU) < 1e-5
    np.testing.assert_array_equal(host(U, ny, nx) == 0, rU == 0)
    rs.propagate_2d(u, U, dx, dy, wl, 0.05, nx, 1.5e6, nx, ny, skip_fft=True)
    ru, rU = oracle.propagate_2d(ru, dx, dy, wl, 0.05, 1.5e6, U=rU, skip_fft=True)
    assert rel_l2(host(u, ny, nx), ru) < 1e-5
    assert rel_l2(host(U, ny, nx), rU) < 1e-5


def test_plane_and_tilted_plane_wave(rs, cuda):
    """tests/big_wave_2d/test_p5.py:84-100 (reference bound 2e-14 in FP64; FP32 here)."""
    nx, ny, dz, wl = 64, 32, 0.7, 0.02
    x = np.arange(nx)[None, :]
    y = np.arange(ny)[:, None]
    for mx, my in ((0, 0), (5, -3)):
        field = np.exp(2j * np.pi * (mx * x / nx + my * y / ny))
        u, U = gv(rs, field, cuda), rs.GpuVector.zeros(nx * ny, cuda)
        rs.propagate_2d(u, U, 1.0, 1.0, wl, dz, nx * 4, 20.0, nx, ny)
        fx, fy = mx / nx, my / ny
        transfer = np.exp(2j * np.pi * dz / wl) * np.exp(-1j * np.pi * wl * dz * (fx * fx + fy * fy))
        assert rel_l2(host(u, ny, nx), field * transfer) < 2e-6


def test_point_source_analytic_vs_golden(rs, cuda, golden):
    nx, ny, dx, dy, z, xs, ys, wl = golden["ps_analytic_params"]
    nx, ny = int(nx), int(ny)
    p = rs.SimParams(N=nx * ny, nx=nx, ny=ny, dx=dx, dy=dy, z_detector=z, detector_size=nx * dx,
                     detector_pixel_size_x=dx, detector_pixel_size_y=dy, wl=wl, chunk_size=nx * 4)
    u = rs.GpuVector.zeros(nx * ny, cuda)
    rs.propagate_analytically_2d(u, z, xs, ys, p)
    a = host(u, ny, nx)
    ref = golden["ps_analytic"]
    assert rel_l2(np.abs(a), np.abs(ref)) < 1e-6
    # the reference rounds the ~1e10 rad carrier in FP64; the GPU reproduces that FP64 phase
    assert np.max(np.abs(np.angle(a * np.conj(ref)))) < 1e-6


def test_point_source_propagate_vs_golden(rs, cuda, golden):
    nx, ny, dx, dy, z, xs, ys, wl, f = golden["ps_prop_params"]
    nx, ny = int(nx), int(ny)
    p = rs.SimParams(N=nx * ny, nx=nx, ny=ny, dx=dx, dy=dy, z_detector=1.0, detector_size=nx * dx,
                     detector_pixel_size_x=dx, detector_pixel_size_y=dy, wl=wl, chunk_size=nx * 8)
    u, U = rs.GpuVector.zeros(nx * ny, cuda), rs.GpuVector.zeros(nx * ny, cuda)
    rs.PointSource(x=xs, y=ys, z=0.0).propagate_to(z, p, f, u, U, None)
    assert rel_l2(host(u, ny, nx), golden["ps_prop_c128_u"]) < 1e-5
    assert rel_l2(host(U, ny, nx), golden["ps_prop_c128_U"]) < 1e-5


@pytest.mark.parametrize("nx,ny", [(256, 256), (512, 1024)])
def test_point_source_fast_vs_oracle(rs, cuda, oracle, nx, ny):
    dx = dy = 0.25e-6
    wl = oracle.convert_energy_wavelength(25000.0)
    p = rs.SimParams(N=nx * ny, nx=nx, ny=ny, dx=dx, dy=dy, z_detector=2.0, detector_size=nx * dx,
                     detector_pixel_size_x=dx, detector_pixel_size_y=dy, wl=wl, chunk_size=nx)
    u, U = rs.GpuVector.zeros(nx * ny, cuda), rs.GpuVector.zeros(nx * ny, cuda)
    rs.propagation.point_source_propagate_2d(u, U, 0.5, 2e-6, -1e-6, p, 0.35 / dx)
    ru, rU = oracle.point_source_2d(nx, ny, dx, dy, 0.5, 2e-6, -1e-6, wl, 0.35 / dx)
    assert rel_l2(host(u, ny, nx), ru) < 1e-5
    assert rel_l2(host(U, ny, nx), rU) < 1e-5


def _sample_from_golden(rs, golden):
    nx, ny, dx, dy, wl, px, py, pz, xp, yp, f, z0 = golden["sample_params"]
    s = rs.Sample(z_start=z0, pixel_size_x=px, pixel_size_z=pz, grid=golden["sample_grid"],
                  materials=[rs.Material("A", 1.0), rs.Material("B", 1.0)], x_positions=np.array([xp]),
                  pixel_size_y=py, y_positions=np.array([yp]))
    s.db_list = golden["sample_db"]
    p = rs.SimParams(N=int(nx * ny), nx=int(nx), ny=int(ny), dx=dx, dy=dy, z_detector=0.1, detector_size=nx * dx,
                     detector_pixel_size_x=dx, detector_pixel_size_y=dy, wl=wl, chunk_size=int(nx) * 8)
    return s, p, f


def test_sample_apply_vs_golden(rs, cuda, golden):
    s, p, f = _sample_from_golden(rs, golden)
    nx, ny = p.nx, p.ny
    for name in ("c128", "c64"):
        u, U = gv(rs, golden[f"sample_{name}_in"], cuda), rs.GpuVector.zeros(nx * ny, cuda)
        s.apply(u, U, p, f, 0, None)
        assert rel_l2(host(u, ny, nx), golden[f"sample_{name}_u"]) < 2e-5
        assert rel_l2(host(U, ny, nx), golden[f"sample_{name}_U"]) < 2e-5


def test_sample_checkpoint_callback_path_matches_fused(rs, cuda, golden):
    s, p, f = _sample_from_golden(rs, golden)
    nx, ny = p.nx, p.ny
    u1, U1 = gv(rs, golden["sample_c128_in"], cuda), rs.GpuVector.zeros(nx * ny, cuda)
    s.apply(u1, U1, p, f, 0, None)
    seen = []
    s._checkpoint_callback = lambda k, z: seen.append(k)
    u2, U2 = gv(rs, golden["sample_c128_in"], cuda), rs.GpuVector.zeros(nx * ny, cuda)
    s.apply(u2, U2, p, f, 0, None)
    del s._checkpoint_callback
    assert seen == list(range(1, s.grid.shape[0] + 1))
    assert rel_l2(host(u2, ny, nx), host(u1, ny, nx)) < 1e-6


@pytest.mark.parametrize("nx,ny,nz", [(256, 256, 12), (512, 256, 5), (384, 192, 4), (16384, 64, 3), (64, 16384, 3)])
def test_sample_fast_sizes_vs_fp64_oracle(rs, cuda, oracle, nx, ny, nz):
    """Shell sample with bilinear (non-aligned) voxels and aligned voxels, both fast-path sizes."""
    rng = np.random.default_rng(nx + nz)
    wl = oracle.convert_energy_wavelength(20000.0)
    dx = dy = 0.5e-6
    for px, py, xp, yp in ((0.5e-6, 0.5e-6, 0.0, 0.0), (0.83e-6, 0.61e-6, 0.37e-6, -0.21e-6)):
        gx, gy = int(nx * dx / px) + 4, int(ny * dy / py) + 4
        z = (np.arange(nz) - (nz - 1) / 2)[:, None, None] * 3.125e-6
        yy = (np.arange(gy) - gy / 2)[None, :, None] * py
        xx = (np.arange(gx) - gx / 2)[None, None, :] * px
        r = np.sqrt(xx ** 2 + yy ** 2 + z ** 2)
        grid = ((r <= 50e-6) & (r >= 35e-6)).astype(np.uint32)
        grid[:, : gy // 3, : gx // 3] = 2
        db = np.array([0, 3.2e-6 + 2.1e-9j, 1.5e-6 + 7e-9j])
        s = rs.Sample(z_start=0.1, pixel_size_x=px, pixel_size_z=3.125e-6, grid=grid,
                      materials=[rs.Material("a", 1), rs.Material("b", 1)], x_positions=np.array([xp]),
                      pixel_size_y=py, y_positions=np.array([yp]))
        s.db_list = db
        p = rs.SimParams(N=nx * ny, nx=nx, ny=ny, dx=dx, dy=dy, z_detector=0.2, detector_size=nx * dx,
                         detector_pixel_size_x=dx, detector_pixel_size_y=dy, wl=wl, chunk_size=nx)
        x = np.exp(1j * rng.uniform(0, 0.2, size=(ny, nx)))
        u, U = gv(rs, x, cuda), rs.GpuVector.zeros(nx * ny, cuda)
        s.apply(u, U, p, 0.45 / dx, 0, None)
        ru, rU = oracle.sample_apply_2d(x.astype(np.complex128), grid, db, dx, dy, wl, 0.45 / dx, px, py,
                                        3.125e-6, xp, yp)
        a = host(u, ny, nx)
        assert rel_l2(a, ru) < 2e-5
        assert rel_l2(host(U, ny, nx), rU) < 2e-5
        assert rel_l2(np.abs(a) ** 2, np.abs(ru) ** 2) < 2e-5


def test_plasma_apply_vs_golden(rs, cuda, golden):
    p = golden["plasma_params"]
    nx, ny, dx, dy, wl, px, py, pz, xp, yp, f = p[:11]
    nx, ny = int(nx), int(ny)
    sf = tuple(p[11:15])
    pl = rs.PlasmaSample(z_start=0.02, pixel_size_x=px, pixel_size_z=pz, ne_grid=golden["plasma_ne"],
                         ni_grid=golden["plasma_ni"], te_grid=golden["plasma_te"], zstar_grid=golden["plasma_zs"],
                         Z=6, x_positions=np.array([xp]), pixel_size_y=py, y_positions=np.array([yp]),
                         scattering_factors=sf)
    sp = rs.SimParams(N=nx * ny, nx=nx, ny=ny, dx=dx, dy=dy, z_detector=0.1, detector_size=nx * dx,
                      detector_pixel_size_x=dx, detector_pixel_size_y=dy, wl=wl, chunk_size=nx * 4)
    u, U = gv(rs, np.ones((ny, nx)), cuda), rs.GpuVector.zeros(nx * ny, cuda)
    pl.apply(u, U, sp, f, 0, None)
    assert rel_l2(host(u, ny, nx), golden["plasma_u"]) < 2e-5
    assert rel_l2(host(U, ny, nx), golden["plasma_U"]) < 2e-5


def _det_params(rs, integ, nx, ny, dx, dy, sx, sy, px, py, z):
    return rs.SimParams(N=nx * ny, nx=nx, ny=ny, dx=dx, dy=dy, z_detector=z, detector_size=sx, detector_size_x=sx,
                        detector_size_y=sy, detector_pixel_size_x=px, detector_pixel_size_y=py, wl=1e-10,
                        chunk_size=nx, detector_integrator=integ)


@pytest.mark.parametrize("integ", ["area_v1", "legacy_fastwave"])
def test_detector_vs_golden(rs, cuda, golden, integ):
    import warnings
    p = _det_params(rs, integ, 11, 7, 0.7, 1.1, 5.2, 5.1, 1.3, 1.7, 8.0)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        out = rs.square_and_downsample_2d(gv(rs, golden[f"det_{integ}_small_in"], cuda), p, 8.0)
    np.testing.assert_allclose(out, golden[f"det_{integ}_small_out"], rtol=2e-6, atol=1e-6)
    p2 = _det_params(rs, integ, 64, 64, 0.25e-6, 0.25e-6, 15e-6, 14e-6, 0.7e-6, 0.6e-6, 0.4)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        out2 = rs.square_and_downsample_2d(gv(rs, golden[f"det_{integ}_64_in"], cuda), p2, 0.4)
    assert out2.shape == golden[f"det_{integ}_64_out"].shape
    assert rel_l2(out2, golden[f"det_{integ}_64_out"]) < 2e-6
    assert p2.detector_last_metadata["integrator"] == integ


def test_detector_uniform_field_preserves_area(rs, cuda):
    """tests/big_wave_2d/test_p3.py:226-247."""
    p = _det_params(rs, "area_v1", 11, 7, 0.7, 1.1, 3.9, 3.4, 1.3, 1.7, 8.0)
    out = rs.square_and_downsample_2d(gv(rs, np.ones((7, 11)), cuda), p, 8.0)
    oy, ox = out.shape
    x = (np.arange(ox) - ox // 2) * 1.3
    y = (np.arange(oy) - oy // 2) * 1.7
    cosine = 8.0 / np.sqrt(x[None, :] ** 2 + y[:, None] ** 2 + 64.0)
    np.testing.assert_allclose(out / cosine, 1.3 * 1.7, rtol=2e-7, atol=2e-7)


def test_run_simulation_vs_golden(rs, cuda, golden):
    """wavesim.run_simulation: point source -> gap -> Sample -> final leg (skip_fft) -> detector."""
    ws = __import__("3d_ravesim_gb300.wavesim", fromlist=["run_simulation"])
    a0, a1, wl = golden["run_params"]
    nx = ny = 64
    p = rs.SimParams(N=nx * ny, nx=nx, ny=ny, dx=0.5e-6, dy=0.5e-6, z_detector=0.65, detector_size=24e-6,
                     detector_size_x=24e-6, detector_size_y=20e-6, detector_pixel_size_x=1.5e-6,
                     detector_pixel_size_y=1.25e-6, wl=wl, chunk_size=nx * 8)
    samp = rs.Sample(z_start=0.5, pixel_size_x=0.5e-6, pixel_size_z=2e-6, grid=golden["run_grid"],
                     materials=[rs.Material("W", 19.3)], x_positions=np.array([0.0]), pixel_size_y=0.5e-6,
                     y_positions=np.array([0.0]))
    table = [(rs.Material("W", 19.3), np.complex128(4.2e-6 + 1.9e-7j))]
    u, U = rs.GpuVector.zeros(nx * ny, cuda), rs.GpuVector.zeros(nx * ny, cuda)
    outs = ws.run_simulation(p, rs.PointSource(x=1e-6, y=0.0, z=0.0), [samp], [a0, a1], u, U, table)
    assert rel_l2(host(u, ny, nx), golden["run_u"]) < 2e-5
    assert rel_l2(outs[0], golden["run_out"]) < 2e-5


def test_fast_plan_covers_both_size_families(rs, cuda):
    for n, fast in ((4096, True), (3072, True), (1536, True), (24, True), (40, False), (72, False)):
        assert rs._lib.plan_for(n, 64, cuda).fast is fast


def test_fresnel_plane_vs_golden(rs, cuda, golden):
    """PointSource.propagate_to with Fresnel scaling (big-wave/source.py:62-95)."""
    nx, ny, dx, dy, dz, xs, ys, wl, f = golden["fp_params"]
    nx, ny = int(nx), int(ny)
    p = rs.SimParams(N=nx * ny, nx=nx, ny=ny, dx=dx, dy=dy, z_detector=1.5, detector_size=nx * dx,
                     detector_pixel_size_x=dx, detector_pixel_size_y=dy, wl=wl, chunk_size=nx * 8,
                     use_fresnel_scaling=True)
    p.configure_fresnel_detector(0.0, 1.0)
    u, U = rs.GpuVector.zeros(nx * ny, cuda), rs.GpuVector.zeros(nx * ny, cuda)
    rs.PointSource(x=xs, y=ys, z=0.0).propagate_to(dz, p, f, u, U, None)
    assert rel_l2(host(u, ny, nx), golden["fp_c128_u"]) < 1e-5
    assert rel_l2(host(U, ny, nx), golden["fp_c128_U"]) < 1e-5


@pytest.mark.parametrize("n", [256, 1024])
def test_fresnel_plane_fast_vs_oracle(rs, cuda, oracle, n):
    dx = 0.25e-6
    wl = rs.convert_energy_wavelength(30000.0)
    p = rs.SimParams(N=n * n, nx=n, ny=n, dx=dx, dy=dx, z_detector=2.0, detector_size=n * dx,
                     detector_pixel_size_x=dx, detector_pixel_size_y=dx, wl=wl, chunk_size=n, use_fresnel_scaling=True)
    p.configure_fresnel_detector(0.0, 1.2)
    u, U = rs.GpuVector.zeros(n * n, cuda), rs.GpuVector.zeros(n * n, cuda)
    rs.PointSource(x=15e-6, y=7e-6, z=0.0).propagate_to(1.2, p, f := 0.4 / dx, u, U, None)
    ru, rU = oracle.fresnel_plane_2d(n, n, dx, dx, 1.2, 15e-6, 7e-6, wl, f)
    assert rel_l2(host(u, n, n), ru) < 1e-5


def test_plasma_plane_path_is_bit_identical(rs, cuda):
    """PlasmaSample.apply on the voxel-only row kernel (the slice plane's delta/beta evaluated
    first) and on the general row kernel (delta/beta evaluated while staging each row) give
    the same field bit for bit."""
    wlmod = __import__("importlib").import_module("3d_ravesim_gb300.workloads")
    w = wlmod.gaussian_plasma(n=512, slices=12, dx=2e-6)
    s, p = w.elements[0], w.params
    plan = rs._lib.plan_for(512, 512, cuda)
    old = plan.schedule()
    out = []
    try:
        for mask in (48, 52):  # single-sequence kernels; 4: the general row kernel
            plan.set_schedule(mask)
            u = rs.GpuVector(torch.ones(512 * 512, dtype=torch.complex64, device=cuda))
            U = rs.GpuVector.zeros(512 * 512, cuda)
            s.apply(u, U, p, w.cutoff, 0, None)
            torch.cuda.synchronize()
            out.append((u.vec.clone(), U.vec.clone()))
    finally:
        plan.set_schedule(old)
    assert torch.equal(out[0][0], out[1][0]) and torch.equal(out[0][1], out[1][1])
