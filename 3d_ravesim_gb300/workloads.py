"""Seeded synthetic inputs for the benchmark and parity configurations.

* shell_plane_wave (1024^2, 20 keV): plane wave through a voxelised spherical shell (outer radius
  200 um, wall 20 um, delta 3.2e-7, beta 2.1e-10), 128 slices x 3.125 um, then 0.5 m of free space.
* talbot_lau (4096^2, 25 keV): point source 0.5 m upstream, pi-shift Si phase grating (period
  4.2 um, duty 0.5), a 512 x 1 um sample whose delta/beta are a seeded sum of 200 Gaussian blobs
  (sigma 2-20 um, delta peak 1e-7..5e-7, beta = delta/1500) voxelised at 1 um pitch and quantised to
  4095 material levels, then an absorption grating (period 4.2 um, 90 % intensity absorption) at
  the first fractional Talbot distance, then the detector.

Everything is built from numpy.random.default_rng(seed); no dataset is involved.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from .optical_element import Material, Sample
from .propagation import SimParams, convert_energy_wavelength

# delta, beta of Si (2.33 g/cm^3) at 25 keV from the Chantler tables (`chantler.xray_delta_beta`
# over nist_lookup's database), kept as numbers so the workload needs no database.
SI_DELTA_BETA_25KEV = (7.734971368200993e-07, 2.1375609561035094e-09)


@dataclass
class Workload:
    name: str
    params: SimParams
    elements: list
    cutoff: float
    source_xyz: tuple[float, float, float] | None  # None: unit plane wave at the first element
    z_first: float
    info: dict = field(default_factory=dict)

    @property
    def slice_count(self) -> int:
        return sum(int(e.grid.shape[0]) for e in self.elements)


def aligned_voxel_axis(n: int, margin: int = 2) -> np.ndarray:
    """Voxel centres of an axis with voxel pitch == grid pitch and x_len = n + margin (even): the
    reference maps sim index i to voxel index i + margin/2 exactly (optical_element.py:538-546)."""
    length = n + margin
    return np.arange(length) - length / 2.0


def stripe_grating(n: int, dx: float, period_px: int, z_start: float, thickness: float, name: str,
                   duty: float = 0.5) -> Sample:
    """One-slice line grating along x; the y extent is one voxel per field height."""
    length = n + 2
    j = np.arange(length) - 1
    line = ((j % period_px) < int(round(duty * period_px))).astype(np.uint32)
    grid = np.broadcast_to(line, (1, 3, length)).copy()
    return Sample(z_start=z_start, pixel_size_x=dx, pixel_size_z=thickness, grid=grid,
                  materials=[Material(name, 1.0)], x_positions=np.array([0.0]), pixel_size_y=n * dx,
                  y_positions=np.array([0.0]))


def shell_plane_wave(n: int = 1024, slices: int = 128, dx: float = 0.5e-6, energy: float = 20000.0,
                     outer: float = 200e-6, wall: float = 20e-6, thickness: float = 400e-6,
                     z_detector_gap: float = 0.5) -> Workload:
    wl = convert_energy_wavelength(energy)
    pz = thickness / slices
    ax = aligned_voxel_axis(n) * dx
    zc = (np.arange(slices) + 0.5 - slices / 2.0) * pz
    r2_xy = ax[None, :] ** 2 + ax[:, None] ** 2
    grid = np.empty((slices, n + 2, n + 2), dtype=np.uint32)
    for k in range(slices):
        r = np.sqrt(r2_xy + zc[k] ** 2)
        grid[k] = ((r >= outer - wall) & (r <= outer)).astype(np.uint32)
    z0 = 0.1
    sample = Sample(z_start=z0, pixel_size_x=dx, pixel_size_z=pz, grid=grid, materials=[Material("shell", 1.0)],
                    x_positions=np.array([0.0]), pixel_size_y=dx, y_positions=np.array([0.0]))
    sample.db_list = np.array([0.0, 3.2e-7 + 2.1e-10j])
    zd = z0 + thickness + z_detector_gap
    p = SimParams(N=n * n, nx=n, ny=n, dx=dx, dy=dx, z_detector=zd, detector_size=n * dx,
                  detector_pixel_size_x=dx, detector_pixel_size_y=dx, wl=wl, chunk_size=n)
    return Workload("shell_plane_wave", p, [sample], cutoff=0.5 / dx, source_xyz=None, z_first=z0,
                    info={"nx": n, "ny": n, "slices": slices, "energy_ev": energy})


def gaussian_blob_volume(n: int, dx: float, slices: int, pz: float, pitch: float, blobs: int, seed: int,
                         levels: int = 4095):
    """Quantised voxel volume of a sum of 3D Gaussian blobs and its delta+i*beta table."""
    rng = np.random.default_rng(seed)
    fov = n * dx
    depth = slices * pz
    length = int(math.ceil(fov / pitch)) + 4
    length += length % 2
    cx = rng.uniform(-fov / 2, fov / 2, blobs)
    cy = rng.uniform(-fov / 2, fov / 2, blobs)
    cz = rng.uniform(0.0, depth, blobs)
    sig = rng.uniform(2e-6, 20e-6, blobs)
    amp = rng.uniform(1e-7, 5e-7, blobs)
    ax = (np.arange(length) - length / 2.0) * pitch
    gx = np.exp(-np.square(ax[:, None] - cx[None, :]) / (2 * sig ** 2))  # (length, blobs)
    gy = np.exp(-np.square(ax[:, None] - cy[None, :]) / (2 * sig ** 2))
    delta = np.empty((slices, length, length), dtype=np.float64)
    for k in range(slices):
        z = (k + 0.5) * pz
        w = amp * np.exp(-np.square(z - cz) / (2 * sig ** 2))
        delta[k] = (gy * w[None, :]) @ gx.T
    dmax = float(delta.max())
    ids = np.rint(delta * (levels / dmax)).astype(np.uint32)
    table = (np.arange(levels + 1) * (dmax / levels)) * (1.0 + 1j / 1500.0)
    return ids, table.astype(np.complex128), length


def talbot_lau(n: int = 4096, slices: int = 512, seed: int = 0, dx: float = 0.1e-6, energy: float = 25000.0,
               blobs: int = 200, voxel_pitch: float = 1e-6) -> Workload:
    wl = convert_energy_wavelength(energy)
    period = 4.2e-6
    period_px = int(round(period / dx))
    z_g1 = 0.5
    d_si, b_si = SI_DELTA_BETA_25KEV
    t1 = wl / (2.0 * d_si)  # pi phase shift
    g1 = stripe_grating(n, dx, period_px, z_g1, t1, "Si")
    g1.db_list = np.array([0.0, d_si + 1j * b_si])
    pz = 1e-6
    z_s = z_g1 + t1 + 100e-6
    ids, table, length = gaussian_blob_volume(n, dx, slices, pz, voxel_pitch, blobs, seed)
    sample = Sample(z_start=z_s, pixel_size_x=voxel_pitch, pixel_size_z=pz, grid=ids,
                    materials=[Material(f"blob{i}", 1.0) for i in range(len(table) - 1)],
                    x_positions=np.array([0.0]), pixel_size_y=voxel_pitch, y_positions=np.array([0.0]))
    sample.db_list = table
    # first fractional Talbot distance of a pi grating, magnified for the spherical wave
    d_plane = period ** 2 / (8.0 * wl)
    d_t = z_g1 * d_plane / (z_g1 - d_plane)
    t2 = 20e-6
    beta_g2 = math.log(10.0) * wl / (4.0 * math.pi * t2)  # exp(-4 pi beta t / wl) = 0.1
    g2 = stripe_grating(n, dx, period_px, z_g1 + d_t, t2, "absorber")
    g2.db_list = np.array([0.0, 1j * beta_g2])
    z_det = z_g1 + d_t + t2 + 1e-3
    p = SimParams(N=n * n, nx=n, ny=n, dx=dx, dy=dx, z_detector=z_det, detector_size=n * dx,
                  detector_pixel_size_x=1e-6, detector_pixel_size_y=1e-6, wl=wl, chunk_size=n)
    return Workload("talbot_lau", p, [g1, sample, g2], cutoff=0.45 / dx, source_xyz=(0.0, 0.0, 0.0), z_first=z_g1,
                    info={"nx": n, "ny": n, "energy_ev": energy, "sample_slices": slices, "blobs": blobs,
                          "voxel_grid": [slices, length, length], "talbot_distance_m": d_t,
                          "g1_thickness_m": t1, "g2_beta": beta_g2})


def gaussian_plasma(n: int = 2048, slices: int = 256, dx: float = 0.5e-6, energy: float = 8000.0,
                    n0: float = 1e21, length: float = 150e-6, te: float = 500.0, zstar: float = 3.5,
                    pz: float = 2e-6, pitch: float = 2e-6, z_detector_gap: float = 0.2):
    """Differentiable-plasma forward (2048^2, 8 keV, 256 x 2 um slices): a plasma with n_e = n0 exp(-r^2 / 2 L^2) (cm^-3, r from the centre of the
    slab), T_e = 500 eV, Z* = 3.5 and n_i = n_e / Z*, in CH (zbar = 3.5, z2bar = 18.5), so q = 1 and
    only the free-electron refraction and the Kramers absorption contribute."""
    from .plasma_sample import PlasmaSample
    wl = convert_energy_wavelength(energy)
    fov = n * dx
    glen = int(math.ceil(fov / pitch)) + 4
    glen += glen % 2
    ax = (np.arange(glen) - glen / 2.0) * pitch
    zc = (np.arange(slices) + 0.5 - slices / 2.0) * pz
    r2xy = ax[None, :] ** 2 + ax[:, None] ** 2
    ne = np.empty((slices, glen, glen), dtype=np.float32)
    for k in range(slices):
        ne[k] = n0 * np.exp(-(r2xy + zc[k] ** 2) / (2.0 * length ** 2))
    ni = (ne / zstar).astype(np.float32)
    teg = np.full_like(ne, te)
    zs = np.full_like(ne, zstar)
    z0 = 0.1
    sample = PlasmaSample(z_start=z0, pixel_size_x=pitch, pixel_size_z=pz, ne_grid=ne, ni_grid=ni, te_grid=teg,
                          zstar_grid=zs, Z=6, x_positions=np.array([0.0]), formula="CH", pixel_size_y=pitch,
                          y_positions=np.array([0.0]), scattering_factors=(6.0, 0.0, 3.5, 18.5))
    p = SimParams(N=n * n, nx=n, ny=n, dx=dx, dy=dx, z_detector=z0 + slices * pz + z_detector_gap,
                  detector_size=fov, detector_pixel_size_x=dx, detector_pixel_size_y=dx, wl=wl, chunk_size=n)
    return Workload("gaussian_plasma", p, [sample], cutoff=0.45 / dx, source_xyz=None, z_first=z0,
                    info={"nx": n, "ny": n, "slices": slices, "energy_ev": energy, "grid": [slices, glen, glen]})


def capsule_large(n: int = 16384, slices: int = 1024, dx: float = 50e-9, energy: float = 30000.0,
                  seed: int = 0, pitch: float = 2e-6, pz: float = 0.5e-6, lmax: int = 8,
                  amplitude: float = 10e-6, z_source: float = 1.0, z_detector_gap: float = 0.3) -> Workload:
    """Large in-HBM field: 16384^2 complex64 (2 GiB) at 30 keV, point source 1 m upstream, an
    ellipsoidal CH capsule shell (semi-axes 400/400/380 um, 15 um wall, delta 2.5e-7, beta
    1.5e-10) whose outer radius carries a seeded perturbation of real spherical harmonics
    l = 1..lmax scaled to `amplitude` at its largest, voxelised at `pitch` in x/y with one voxel
    plane per slice (slices x pz centred on the capsule; at 1024 x 0.5 um the poles beyond
    +-256 um lie outside the slab), then 0.3 m of free space to the detector."""
    from scipy.special import lpmv
    rng = np.random.default_rng(seed)
    wl = convert_energy_wavelength(energy)
    fov = n * dx
    glen = int(math.ceil(fov / pitch)) + 4
    glen += glen % 2
    ax = (np.arange(glen) - glen / 2.0) * pitch
    zc = (np.arange(slices) + 0.5 - slices / 2.0) * pz
    # perturbation coefficients c_lm, normalised on a coarse (theta, phi) grid
    coeffs = [(l, m, rng.normal(), rng.uniform(0, 2 * np.pi)) for l in range(1, lmax + 1) for m in range(0, l + 1)]

    def dr(ct, ph):
        out = np.zeros(np.broadcast(ct, ph).shape)
        for l, m, c, p0 in coeffs:
            out += c * lpmv(m, l, ct) * np.cos(m * ph + p0)
        return out
    tg, pg = np.meshgrid(np.linspace(-1, 1, 181), np.linspace(0, 2 * np.pi, 361), indexing="ij")
    scale = amplitude / np.max(np.abs(dr(tg, pg)))
    a_xy, c_z, wall = 400e-6, 380e-6, 15e-6
    yy, xx = np.meshgrid(ax, ax, indexing="ij")
    r_xy2 = xx * xx + yy * yy
    ph = np.arctan2(yy, xx)
    grid = np.zeros((slices, glen, glen), dtype=np.uint32)
    for k in range(slices):
        r = np.sqrt(r_xy2 + zc[k] ** 2)
        ct = np.divide(zc[k], r, out=np.zeros_like(r), where=r > 0)
        st2 = 1.0 - ct * ct
        rho = 1.0 / np.sqrt(st2 / a_xy ** 2 + ct * ct / c_z ** 2)
        near = (r <= rho + amplitude) & (r >= rho - wall - amplitude)  # only there can the wall be
        if near.any():
            outer = rho[near] + scale * dr(ct[near], ph[near])
            rn = r[near]
            grid[k][near] = ((rn <= outer) & (rn >= outer - wall)).astype(np.uint32)
    z0 = z_source
    sample = Sample(z_start=z0, pixel_size_x=pitch, pixel_size_z=pz, grid=grid, materials=[Material("CH", 1.0)],
                    x_positions=np.array([0.0]), pixel_size_y=pitch, y_positions=np.array([0.0]))
    sample.db_list = np.array([0.0, 2.5e-7 + 1.5e-10j])
    z_det = z0 + slices * pz + z_detector_gap
    p = SimParams(N=n * n, nx=n, ny=n, dx=dx, dy=dx, z_detector=z_det, detector_size=fov,
                  detector_pixel_size_x=1e-6, detector_pixel_size_y=1e-6, wl=wl, chunk_size=n)
    return Workload("capsule_large", p, [sample], cutoff=0.45 / dx, source_xyz=(0.0, 0.0, 0.0), z_first=z0,
                    info={"nx": n, "ny": n, "energy_ev": energy, "sample_slices": slices,
                          "voxel_grid": [slices, glen, glen]})
