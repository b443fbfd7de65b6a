"""The bulk-copy pipelined passes against the classic passes: same arithmetic in the same order,
so outputs must be bit-identical; and no bounded wait may have given up."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def run_both(rs, cuda, nx, ny, fn):
    plan = rs._lib.plan_for(nx, ny, cuda)
    outs = []
    old = plan.schedule()
    # the single-sequence kernels with compensated twiddles (schedule bits 16 | 32): per-block
    # kernels, pipelined rows, pipelined columns, both
    for mask in (0, 1, 2, 3):
        plan.set_schedule(48 | mask)
        outs.append(fn())
        torch.cuda.synchronize()
    plan.set_schedule(old)
    assert plan.status() == 0
    return outs


@pytest.mark.parametrize("nx,ny", [(4096, 4096), (1024, 2048), (2048, 256), (1536, 1536), (3072, 768), (512, 6144),
                                   (8192, 512)])
def test_fft_and_propagate_pipeline_bit_identical(rs, cuda, nx, ny):
    rng = np.random.default_rng(nx ^ ny)
    x = (rng.normal(size=nx * ny) + 1j * rng.normal(size=nx * ny)).astype(np.complex64)

    def fn():
        a = rs.GpuVector.from_numpy(x, cuda)
        b = rs.GpuVector.zeros(nx * ny, cuda)
        a.fft2(b, nx, ny)
        c = rs.GpuVector.zeros(nx * ny, cuda)
        b.ifft2(c, nx, ny)
        u, U = rs.GpuVector.from_numpy(x, cuda), rs.GpuVector.zeros(nx * ny, cuda)
        rs.propagate_2d(u, U, 1e-7, 1.3e-7, 5e-11, 0.01, nx, 3.0e6, nx, ny)
        rs.propagate_2d(u, U, 1e-7, 1.3e-7, 5e-11, 0.02, nx, 2.5e6, nx, ny, skip_fft=True)
        return [v.to_numpy() for v in (b, c, u, U)]
    runs = run_both(rs, cuda, nx, ny, fn)
    for other in runs[1:]:
        for a, b in zip(runs[0], other):
            np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("n,pitch", [(4096, 1e-6), (2048, 0.5e-6), (1536, 0.37e-6)])
def test_multislice_pipeline_bit_identical(rs, cuda, n, pitch):
    wl = rs.convert_energy_wavelength(25000.0)
    dx = 0.5e-6 if n < 4096 else 0.1e-6
    gl = int(n * dx / pitch) + 4
    rng = np.random.default_rng(n)
    grid = rng.integers(0, 4, size=(6, gl, gl)).astype(np.uint32)
    s = rs.Sample(z_start=0.5, pixel_size_x=pitch, pixel_size_z=1e-6, grid=grid,
                  materials=[rs.Material(str(i), 1.0) for i in range(3)], x_positions=np.array([0.1e-6]),
                  pixel_size_y=pitch, y_positions=np.array([-0.2e-6]))
    s.db_list = np.array([0, 2e-7 + 1e-10j, 4e-7 + 3e-10j, 1e-7 + 2e-9j])
    p = rs.SimParams(N=n * n, nx=n, ny=n, dx=dx, dy=dx, z_detector=1.0, detector_size=n * dx,
                     detector_pixel_size_x=dx, detector_pixel_size_y=dx, wl=wl, chunk_size=n)

    def fn():
        u, U = rs.GpuVector.zeros(n * n, cuda), rs.GpuVector.zeros(n * n, cuda)
        rs.propagation.point_source_propagate_2d(u, U, 0.5, 0.0, 0.0, p, 0.45 / dx)
        s.apply(u, U, p, 0.45 / dx, 0, None)
        return [u.to_numpy(), U.to_numpy()]
    runs = run_both(rs, cuda, n, n, fn)
    for other in runs[1:]:
        for a, b in zip(runs[0], other):
            np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("nx,ny", [(4096, 4096), (1024, 1536), (2048, 2048), (512, 512), (8192, 1024), (16384, 256),
                                   (1536, 1024), (3072, 512), (512, 3072), (768, 384), (384, 6144), (6144, 768)])
def test_split_pair_passes_match_compensated_passes(rs, cuda, nx, ny):
    """The split-pair multislice passes (two rows / two columns per thread group in packed f32x2
    arithmetic, dithered twiddle tables) against the single-sequence passes with compensated
    twiddles on the same 12-slice voxel run: equal to FP32 rounding (both are within the FP64
    accuracy bound; their roundings differ). The dithered rows (bit 64) and columns (bit 128) one
    per thread group give the split-pair passes' values exactly. Rows of 16384 and rows and
    columns of 3*2^k have only the one-per-group dithered form (radix-24 first stage): there the
    default schedule runs it and is held to the same bound against the compensated passes."""
    wl = rs.convert_energy_wavelength(25000.0)
    dx = 0.25e-6
    pitch = 0.7e-6
    gx, gy = int(nx * dx / pitch) + 4, int(ny * dx / pitch) + 4
    rng = np.random.default_rng(nx + 3 * ny)
    grid = rng.integers(0, 4, size=(12, gy, gx)).astype(np.uint32)
    s = rs.Sample(z_start=0.5, pixel_size_x=pitch, pixel_size_z=1e-6, grid=grid,
                  materials=[rs.Material(str(i), 1.0) for i in range(3)], x_positions=np.array([0.1e-6]),
                  pixel_size_y=pitch, y_positions=np.array([-0.2e-6]))
    s.db_list = np.array([0, 2e-7 + 1e-10j, 4e-7 + 3e-10j, 1e-7 + 2e-9j])
    p = rs.SimParams(N=nx * ny, nx=nx, ny=ny, dx=dx, dy=dx, z_detector=1.0, detector_size=nx * dx,
                     detector_pixel_size_x=dx, detector_pixel_size_y=dx, wl=wl, chunk_size=nx)
    plan = rs._lib.plan_for(nx, ny, cuda)
    old = plan.schedule()
    outs = []
    try:
        for mask in (0, 48 | old, 64, 128):
            plan.set_schedule(mask)
            x = rng.normal(size=nx * ny) + 1j * rng.normal(size=nx * ny) if not outs else None
            if x is not None:
                x0 = x.astype(np.complex64)
            u, U = rs.GpuVector.from_numpy(x0, cuda), rs.GpuVector.zeros(nx * ny, cuda)
            s.apply(u, U, p, 0.45 / dx, 0, None)
            outs.append((u.to_numpy(), U.to_numpy()))
    finally:
        plan.set_schedule(old)
    for a, b in zip(outs[0], outs[1]):
        assert np.all(np.isfinite(a))
        assert np.linalg.norm(a - b) / np.linalg.norm(b) < 3e-6
    for single in outs[2:]:
        for a, b in zip(outs[0], single):
            np.testing.assert_array_equal(a, b)
    assert plan.status() == 0


@pytest.mark.parametrize("n", [1024, 2048])
def test_split_pair_rows_store_the_entering_fields(rs, cuda, n):
    """rs_multislice_dbgrid_store and rs_multislice_dbgrid_fields with the split-pair row passes
    (schedule 0) write the same fields, to FP32 rounding, as the single-sequence kernels (48), and
    exactly the fields of the dithered rows one row per thread group (64); the fields-only form
    writes exactly what the storing forward writes."""
    lib = rs._lib
    rng = np.random.default_rng(n)
    nz, nv = 6, n // 4 + 4
    db = torch.from_numpy(np.stack([rng.uniform(0, 3e-7, (nz, nv, nv)), rng.uniform(0, 1e-9, (nz, nv, nv))], -1)
                          .astype(np.float32)).to(cuda)
    dx = 0.5e-6
    geom = lib.VoxelGeom(nz, nv, nv, 4 * dx, 4 * dx, 2e-6, 0.0, 0.0)
    dz = lib.doubles([2e-6] * nz)
    plan = lib.plan_for(n, n, cuda)
    old = plan.schedule()
    u0 = torch.polar(torch.ones(n * n), torch.from_numpy(rng.uniform(0, 6, n * n)).float()).to(torch.complex64).to(cuda)
    out = {}
    try:
        for mask in (0, 48, 64):
            plan.set_schedule(mask)
            for name in ("rs_multislice_dbgrid_store", "rs_multislice_dbgrid_fields"):
                u, U = u0.clone(), torch.empty_like(u0)
                fields = torch.zeros((nz, n * n), dtype=torch.complex64, device=cuda)
                lib.check(getattr(lib.lib(), name)(plan.handle, lib.ptr(u), lib.ptr(U), lib.ptr(db), geom, dx, dx,
                                                   6.2e-11, 0.45 / dx, dz, None, 0, nz, lib.ptr(fields),
                                                   lib.stream_handle()), name)
                torch.cuda.synchronize()
                out[(mask, name)] = fields.cpu().numpy()
    finally:
        plan.set_schedule(old)
    for mask in (0, 48, 64):
        assert np.array_equal(out[(mask, "rs_multislice_dbgrid_store")], out[(mask, "rs_multislice_dbgrid_fields")])
    assert np.array_equal(out[(0, "rs_multislice_dbgrid_store")], out[(64, "rs_multislice_dbgrid_store")])
    a, b = out[(0, "rs_multislice_dbgrid_store")], out[(48, "rs_multislice_dbgrid_store")]
    assert np.array_equal(a[0], b[0])  # the field entering the first slice is the input
    assert np.linalg.norm(a - b) / np.linalg.norm(b) < 3e-6
