"""GPU drop-in for big-wave's PlasmaSample (big-wave/plasma_sample.py, big-wave/plasma.py).

delta/beta of every voxel corner are evaluated inside the row FFT pass from the
(n_e, n_i, T_e, Z*) grids with the free-electron + bound-electron + Kramers model of
plasma_delta_beta_grid_multi (big-wave/plasma.py:380-434), bilinearly interpolated, zeroed
outside the grid and turned into the transmission (plasma_sample.py:126-233).
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Callable, Optional, Union

import numpy as np
import torch

from . import _lib, chantler
from .optical_element import slice_schedule, upload_grid
from .propagation import SimParams, convert_energy_wavelength, require_row_aligned_chunk_size
from .vector import as_gpu_pair

ScatteringFactors = tuple[float, float, float, float]


def codata_constants() -> tuple[float, float]:
    """(PLANCK_HC [eV*A], R_ELECTRON_CM [cm]) as nist_lookup derives them from scipy.constants
    (nist_lookup/nist_lookup/physical_constants.py)."""
    import scipy.constants as consts
    planck_hc = 1.e10 * consts.Planck * consts.c / consts.e
    r_e_cm = 100.0 * consts.physical_constants["classical electron radius"][0]
    return planck_hc, r_e_cm


def plasma_delta_beta_grid_multi(ne, ni, te, zstar, f1bar, f2eff_bar, zbar, z2bar, energy):
    """Host FP64 restatement of big-wave/plasma.py:380-434 (used for checks and small tables)."""
    planck_hc, r_e = codata_constants()
    ne, ni, te, zstar = (np.asarray(a, dtype=np.float64) for a in (ne, ni, te, zstar))
    if not (ne.shape == ni.shape == te.shape == zstar.shape):
        raise ValueError("plasma grid tiles must have identical shapes")
    if energy <= 0.0:
        raise ValueError(f"energy must be positive, got {energy}")
    lamb_cm = 1.0e-8 * planck_hc / energy
    pref = r_e * lamb_cm * lamb_cm / (2.0 * np.pi)
    delta = ne * pref
    beta = np.zeros(ne.shape)
    q = np.clip(np.where(zbar > 0.0, zstar / zbar if zbar > 0 else 0.0, 0.0), 0.0, 1.0)
    fb = 1.0 - q
    bound = (fb > 0.0) & (ni > 0.0)
    if np.any(bound):
        bs = ni * pref * fb
        delta = delta + np.where(bound, bs * f1bar, 0.0)
        beta += np.where(bound, bs * f2eff_bar, 0.0)
    ff = (ne > 0.0) & (ni > 0.0) & (q > 0.0) & (z2bar > 0.0) & (te > 0.0)
    if np.any(ff):
        nu = energy / 4.135667e-15
        alpha = np.zeros(ne.shape)
        alpha[ff] = 3.7e8 * ne[ff] * ni[ff] * (np.square(q[ff]) * z2bar) / (np.sqrt(te[ff] * 11604.5) * nu ** 3)
        beta += alpha * lamb_cm / (4.0 * np.pi)
    atlen = np.full(ne.shape, np.inf)
    pos = beta > 0.0
    atlen[pos] = lamb_cm / (4.0 * np.pi * beta[pos])
    return delta, beta, atlen


@dataclass
class PlasmaSample:
    """Plasma region on a (nz, ny, nx) mesh (big-wave/plasma_sample.py:40-110).

    The per-energy Chantler scalars (f1bar, f2eff_bar, zbar, z2bar) come from
    `scattering_factors` (a tuple, or a callable energy -> tuple). When it is unset they are
    computed from nist_lookup's Chantler database by this package's own lookup (`chantler`):
    the compound average of `formula`, else the single element Z.
    """

    z_start: float
    pixel_size_x: float
    pixel_size_z: float
    ne_grid: object
    ni_grid: object
    te_grid: object
    zstar_grid: object
    Z: int
    x_positions: np.ndarray
    formula: Optional[str] = None
    pixel_size_y: float = 0.0
    y_positions: Optional[np.ndarray] = None
    scattering_factors: Optional[Union[ScatteringFactors, Callable[[float], ScatteringFactors]]] = None

    def _scattering_factors(self, energy: float) -> ScatteringFactors:
        sf = self.scattering_factors
        if sf is not None:
            return tuple(float(v) for v in (sf(energy) if callable(sf) else sf))  # type: ignore[return-value]
        try:
            chantler.database_path()
        except FileNotFoundError as exc:
            raise RuntimeError(
                "PlasmaSample needs scattering_factors=(f1bar, f2eff_bar, zbar, z2bar) when "
                "nist_lookup's Chantler database is not available") from exc
        if self.formula:
            return chantler.compound_scattering_factors(self.formula, energy)
        return chantler.element_scattering_factors(int(self.Z), energy)

    def _shape(self) -> tuple:
        return tuple(self.ne_grid.shape)

    def check_valid(self) -> None:
        shape = self._shape()
        assert len(shape) == 3, f"the GPU PlasmaSample supports 3D grids (z, y, x), got {shape}"
        assert shape[0] > 0
        for name, g in (("ni", self.ni_grid), ("te", self.te_grid), ("zstar", self.zstar_grid)):
            assert tuple(g.shape) == shape, f"{name}_grid shape mismatch: {tuple(g.shape)} != {shape}"
        assert self.z_start > 0 and self.pixel_size_x > 0 and self.pixel_size_z > 0
        assert self.pixel_size_y > 0, "3D grids require pixel_size_y > 0"
        assert shape[1] >= 2 and shape[2] >= 2

    def get_thickness(self) -> float:
        return self.pixel_size_z * self._shape()[0]

    def store_deltabetas(self, deltabeta_table) -> None:
        """No table to store: the plasma's delta and beta come from its density, temperature and
        charge grids (big-wave's PlasmaSample.store_deltabetas, plasma_sample.py:108-110, stores
        nothing either)."""

    def _device_grids(self, device: torch.device):
        grids = (self.ne_grid, self.ni_grid, self.te_grid, self.zstar_grid)
        cache = getattr(self, "_dev_cache", None)
        if cache is None or cache[0] != device or any(a is not b for a, b in zip(cache[1], grids)):
            dev = []
            for g in grids:
                if isinstance(g, torch.Tensor):
                    t = g.to(device)
                    if t.dtype not in (torch.float32, torch.float64):
                        t = t.to(torch.float64)
                    dev.append(t.contiguous())
                else:
                    a = np.asarray(g)
                    a = a if a.dtype in (np.float32, np.float64) else a.astype(np.float64)
                    dev.append(upload_grid(a, device, "float"))
            f64 = all(t.dtype == torch.float64 for t in dev)
            if not f64:
                dev = [t.to(torch.float32) for t in dev]
            self._dev_cache = (device, grids, dev, f64)
        return self._dev_cache[2], self._dev_cache[3]

    def apply(self, u, U, sim_params: SimParams, cutoff_freq: float, stepping_iteration: int, history) -> None:
        if not (sim_params.is_2d and len(self._shape()) == 3):
            raise NotImplementedError("the GB300 PlasmaSample implements the 2D path (3D grids, ny > 1)")
        self._apply_2d(u, U, sim_params, cutoff_freq, stepping_iteration, history)

    def _apply_2d(self, u, U, sim_params, cutoff_freq, stepping_iteration, history) -> None:
        from .propagation import square_and_downsample_2d
        u, U = as_gpu_pair(u, U)
        energy = convert_energy_wavelength(sim_params.wl)
        nz, gy, gx = self._shape()
        f1bar, f2eff_bar, zbar, z2bar = self._scattering_factors(energy)
        dy_s = self.pixel_size_y if self.pixel_size_y != 0.0 else self.pixel_size_x
        x_pos = float(self.x_positions[stepping_iteration])
        y_pos = float(self.y_positions[stepping_iteration]) if self.y_positions is not None else 0.0
        nx, ny = sim_params.nx, sim_params.ny
        require_row_aligned_chunk_size(sim_params.chunk_size, nx, ny)
        start_slice = int(getattr(self, "_checkpoint_start_slice", 0))
        if start_slice < 0 or start_slice > nz:
            raise ValueError(f"invalid PlasmaSample checkpoint slice {start_slice}/{nz}")
        callback = getattr(self, "_checkpoint_callback", None)
        device = u.vec.device
        grids, f64 = self._device_grids(device)
        planck_hc, r_e = codata_constants()
        pc = _lib.PlasmaConsts(float(f1bar), float(f2eff_bar), float(zbar), float(z2bar), float(energy),
                               planck_hc, r_e)
        dz, cs = slice_schedule(sim_params, self.z_start, self.pixel_size_z, nz)
        dz_c = _lib.doubles(dz)
        cs_c = _lib.doubles(cs) if cs is not None else None
        geom = _lib.VoxelGeom(nz, gy, gx, float(self.pixel_size_x), float(dy_s), float(self.pixel_size_z),
                              x_pos, y_pos)
        plan = _lib.plan_for(nx, ny, device)

        def run(s0: int, s1: int) -> None:
            with torch.cuda.device(device):
                _lib.check(_lib.lib().rs_multislice_plasma(
                    plan.handle, _lib.ptr(u.vec), _lib.ptr(U.vec), *(_lib.ptr(g) for g in grids),
                    1 if f64 else 0, pc, geom, float(sim_params.dx), float(sim_params.get_dy()),
                    float(sim_params.wl), float(cutoff_freq), dz_c, cs_c, s0, s1,
                    _lib.stream_handle()), "PlasmaSample.apply")

        if callback is None and history is None:
            run(start_slice, nz)
            return
        for rowidx in range(start_slice, nz):
            slice_z = self.z_start + rowidx * self.pixel_size_z
            if history is not None:
                history.push(square_and_downsample_2d(u, sim_params, slice_z), slice_z)
            run(rowidx, rowidx + 1)
            if callback is not None:
                callback(rowidx + 1, self.z_start + (rowidx + 1) * self.pixel_size_z)
