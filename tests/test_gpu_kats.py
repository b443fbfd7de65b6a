"""Known-answer tests of the CUDA path, restating the physics checks of the reference's own P5
suite (tests/big_wave_2d/test_p5.py:102-197) with complex64 tolerances: a uniform thin layer
(phase and Beer-Lambert), a square aperture against the Fresnel integrals, an offset thin
slab against its explicit transmission, and the x/y symmetry of a centred hollow capsule."""
import numpy as np
import pytest
import torch
from scipy.special import fresnel

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def params(rs, nx, ny, dx, wl, z):
    return rs.SimParams(N=nx * ny, nx=nx, ny=ny, dx=dx, dy=dx, z_detector=z, detector_size=nx * dx,
                        detector_pixel_size_x=dx, detector_pixel_size_y=dx, wl=wl, chunk_size=nx)


def field(rs, cuda, arr):
    return rs.GpuVector.from_numpy(np.asarray(arr, np.complex64).reshape(-1), cuda)


def host(v, ny, nx):
    torch.cuda.synchronize()
    return v.to_numpy().reshape(ny, nx).astype(np.complex128)


def test_uniform_thin_layer_phase_and_beer_lambert(rs, cuda):
    """test_p5.py:102-124: a uniform layer multiplies a plane wave by material_factor * exp(2 pi i t/wl)."""
    p = params(rs, 32, 16, 1e-6, 1e-10, 0.1)
    t = 2e-7
    db = 1.2e-7 + 2.4e-8j
    grid = np.ones((1, p.ny + 2, p.nx + 2), dtype=np.uint32)
    m = rs.Material("layer", 1.0)
    s = rs.Sample(z_start=0.05, pixel_size_x=p.dx, pixel_size_z=t, grid=grid, materials=[m],
                  x_positions=np.array([0.0]), pixel_size_y=p.dx, y_positions=np.array([0.0]))
    s.db_list = np.array([0.0, db])
    u, U = field(rs, cuda, np.ones(p.N)), rs.GpuVector.zeros(p.N, cuda)
    s.apply(u, U, p, 1.0 / p.dx, 0, None)
    out = host(u, p.ny, p.nx)
    expected = np.exp(-2j * np.pi * t / p.wl * np.conj(db)) * np.exp(2j * np.pi * t / p.wl)
    assert np.max(np.abs(np.angle(out * np.conj(expected)))) < 2e-6
    assert abs(np.mean(np.abs(out) ** 2) - np.exp(-4 * np.pi * t * db.imag / p.wl)) < 2e-6


def test_square_aperture_matches_fresnel_integral(rs, cuda):
    """test_p5.py:140-170: 16 x 16 um aperture, 0.4 m, against the product of Fresnel integrals."""
    p = params(rs, 256, 256, 1e-6, 1e-10, 0.4)
    a = 16
    ap = np.zeros((p.ny, p.nx))
    y0, x0 = p.ny // 2, p.nx // 2
    ap[y0 - a // 2:y0 + a // 2, x0 - a // 2:x0 + a // 2] = 1.0
    u, U = field(rs, cuda, ap), rs.GpuVector.zeros(p.N, cuda)
    rs.propagate_2d(u, U, p.dx, p.dx, p.wl, p.z_detector, p.chunk_size, 1.0 / p.dx, p.nx, p.ny)
    coord = (np.arange(p.nx) - p.nx // 2) * p.dx
    scale = np.sqrt(2.0 / (p.wl * p.z_detector))
    centre = -0.5 * p.dx  # the even, cell-centred aperture spans [-8.5, 7.5] um
    s0, c0 = fresnel(scale * (centre - a * p.dx / 2 - coord))
    s1, c1 = fresnel(scale * (centre + a * p.dx / 2 - coord))
    one = (c1 - c0) + 1j * (s1 - s0)
    expected = np.abs(one[:, None] * one[None, :]) ** 2
    actual = np.abs(host(u, p.ny, p.nx)) ** 2
    central = np.s_[48:-48, 48:-48]
    assert rel_l2(actual[central] / actual.max(), expected[central] / expected.max()) < 0.12


def test_offset_thin_slab_matches_explicit_transmission(rs, cuda, oracle):
    """test_p5.py:172-211: integer-cell offsets select grid[3:3+ny, 8:8+nx]; the sample step equals
    the explicit transmission followed by one Fresnel step of the slab thickness."""
    nx = ny = 64
    wl = rs.convert_energy_wavelength(8000.0)
    p = params(rs, nx, ny, 1e-6, wl, 0.1)
    t = 2e-7
    db = 4.5e-5 + 3.9e-6j  # a dense metal at 8 keV
    grid = np.zeros((1, ny + 12, nx + 12), dtype=np.uint32)
    grid[0, 20:56, 27:45] = 1
    s = rs.Sample(z_start=0.05, pixel_size_x=p.dx, pixel_size_z=t, grid=grid, materials=[rs.Material("W", 19.3)],
                  x_positions=np.array([2 * p.dx]), pixel_size_y=p.dx, y_positions=np.array([-3 * p.dx]))
    s.db_list = np.array([0.0, db])
    cutoff = 0.4 / p.dx
    u, U = field(rs, cuda, np.ones(p.N)), rs.GpuVector.zeros(p.N, cuda)
    s.apply(u, U, p, cutoff, 0, None)
    mask = grid[0, 3:3 + ny, 8:8 + nx]
    ex = np.exp(-2j * np.pi * t / wl * np.conj(db * (mask == 1)))
    ref, _ = oracle.propagate_2d(ex, p.dx, p.dx, wl, t, cutoff)
    assert rel_l2(host(u, ny, nx), ref) < 2e-6


def test_hollow_capsule_is_xy_symmetric_and_not_solid(rs, cuda):
    """test_p5.py:213-254: a centred hollow carbon capsule gives equal centre row and column
    intensities and differs from the solid sphere."""
    nx = ny = 72
    wl = rs.convert_energy_wavelength(8000.0)
    p = params(rs, nx, ny, 0.5e-6, wl, 0.1)
    nz, margin = 7, 8
    shape = (nz, ny + margin, nx + margin)
    z = (np.arange(nz) - (nz - 1) / 2.0)[:, None, None]
    y = (np.arange(shape[1]) - shape[1] / 2.0)[None, :, None]
    x = (np.arange(shape[2]) - shape[2] / 2.0)[None, None, :]
    r = np.sqrt(x * x + y * y + z * z)

    def simulate(grid):
        s = rs.Sample(z_start=0.05, pixel_size_x=p.dx, pixel_size_z=0.25e-6, grid=grid,
                      materials=[rs.Material("C", 2.0)], x_positions=np.array([0.0]), pixel_size_y=p.dx,
                      y_positions=np.array([0.0]))
        s.db_list = np.array([0.0, 4.1e-6 + 4.3e-9j])  # carbon at 8 keV
        u, U = field(rs, cuda, np.ones(p.N)), rs.GpuVector.zeros(p.N, cuda)
        s.apply(u, U, p, 0.4 / p.dx, 0, None)
        return host(u, ny, nx)

    shell = simulate(((r <= 18.0) & (r >= 11.0)).astype(np.uint32))
    solid = simulate((r <= 18.0).astype(np.uint32))
    inten = np.abs(shell) ** 2
    # 72 is not a fast size: the rows and the columns go through the direct O(n^2) FP32 DFT, whose
    # rounding differs between the two axes at the 1e-6 level
    assert rel_l2(inten[ny // 2, :], inten[:, nx // 2]) < 1e-5
    assert rel_l2(shell, solid) > 1e-3
