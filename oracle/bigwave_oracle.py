"""CPU oracle for big-wave's 2D multislice path — TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py (its CPU-baseline / reference arm) may
import this module, and only as the checker or the timed CPU baseline. The product
(3d_ravesim_gb300) never calls it.

It restates, in numpy on whole (ny, nx) arrays, the arithmetic of big-wave's NumpyVector
path (file:line citations are relative to the RAVE-SIM repository root). Fields keep their
dtype like NumpyVector does: complex64 in -> scipy.fft in single precision, complex128 in ->
the FP64 run every parity test compares against.

Parity pin: tests/golden/make_golden.py runs the reference itself (big-wave imported with
stubs for its optional dependencies) on seeded inputs and stores inputs and outputs in
tests/golden/*.npz; tests/test_oracle_golden.py checks this module against those fixtures.
"""
from __future__ import annotations

import math

import numpy as np
from scipy import fft as spfft

# big-wave/propagation.py:199-201
H_PLANCK = 6.62607004 * 10 ** (-34)
C_0 = 299792458
EV_TO_JOULE = 1.602176634 * 10 ** (-19)


def convert_energy_wavelength(energy_or_wavelength: float) -> float:
    """big-wave/propagation.py:260-262."""
    return H_PLANCK * C_0 / (energy_or_wavelength * EV_TO_JOULE)


def frequency_squared(n: int, spacing: float) -> np.ndarray:
    """big-wave/propagation.py:293-295."""
    return np.square(np.fft.fftfreq(n) / spacing)


def fft2(field: np.ndarray) -> np.ndarray:
    """NumpyVector.fft2 (big-wave/vector.py:341-343)."""
    return spfft.fft2(field)


def ifft2(spec: np.ndarray) -> np.ndarray:
    """NumpyVector.ifft2 (big-wave/vector.py:345-347)."""
    return spfft.ifft2(spec)


def cutoff_mask(nx: int, ny: int, freq: float, dx: float, dy: float) -> np.ndarray:
    """True where big-wave/propagation.py:321-323 zeroes the spectrum (k^2 > 2 f^2)."""
    freq_sq = 2.0 * freq ** 2
    return frequency_squared(ny, dy)[:, None] + frequency_squared(nx, dx)[None, :] > freq_sq


def apply_frequency_cutoff_2d(spec: np.ndarray, freq: float, dx: float, dy: float) -> np.ndarray:
    """big-wave/propagation.py:298-326 (returns a new array)."""
    out = spec.copy()
    out[cutoff_mask(spec.shape[1], spec.shape[0], freq, dx, dy)] = 0.0
    return out


def transfer_function(nx: int, ny: int, dx: float, dy: float, wl: float, dz: float) -> np.ndarray:
    """global_phase * exp(phase_scale * k^2) in complex128 (big-wave/propagation.py:427-436)."""
    kx2 = frequency_squared(nx, dx)
    ky2 = frequency_squared(ny, dy)
    global_phase = np.exp(1j * 2 * np.pi / wl * dz)
    phase_scale = -1j * np.pi * wl * dz
    return global_phase * np.exp(phase_scale * (ky2[:, None] + kx2[None, :]))


def propagate_2d(u: np.ndarray, dx: float, dy: float, wl: float, dz: float, cutoff: float,
                 U: np.ndarray | None = None, skip_fft: bool = False) -> tuple[np.ndarray, np.ndarray]:
    """big-wave/propagation.py:396-442. Returns (u_new, U_new); U_new is the spectrum of u_new."""
    ny, nx = u.shape
    spec = U if skip_fft else fft2(u)
    spec = spec * transfer_function(nx, ny, dx, dy, wl, dz)
    spec = spec.astype(u.dtype, copy=False)  # the in-place tile *= keeps the field dtype
    spec = apply_frequency_cutoff_2d(spec, cutoff, dx, dy)
    return ifft2(spec), spec


def propagate_analytically_2d(nx: int, ny: int, dx: float, dy: float, z: float, xs: float, ys: float,
                              wl: float, dtype=np.complex128) -> np.ndarray:
    """big-wave/propagation.py:458-484: exp(2 pi i r/wl)/r, x = (i - nx/2) dx - xs."""
    x = (np.arange(nx, dtype=np.float64) - nx / 2.0) * dx - xs
    y = (np.arange(ny, dtype=np.float64) - ny / 2.0) * dy - ys
    r = np.sqrt(np.square(y)[:, None] + np.square(x)[None, :] + z ** 2)
    return (np.exp(r * (2j * np.pi / wl)) / r).astype(dtype)


def point_source_2d(nx, ny, dx, dy, z, xs, ys, wl, cutoff, dtype=np.complex128):
    """PointSource.propagate_to in 2D (big-wave/source.py:97-107) without the density check."""
    u = propagate_analytically_2d(nx, ny, dx, dy, z, xs, ys, wl, dtype)
    U = apply_frequency_cutoff_2d(fft2(u), cutoff, dx, dy)
    return ifft2(U), U


def fresnel_plane_2d(nx, ny, dx, dy, dz, xs, ys, wl, cutoff, dtype=np.complex128):
    """Fresnel-scaled source plane, FFT2, cutoff, IFFT2 (big-wave/source.py:62-95)."""
    wave_number = 2.0 * np.pi / wl
    flat = np.arange(nx * ny, dtype=np.int64)
    x = (flat % nx - nx / 2.0) * dx
    y = (flat // nx - ny / 2.0) * dy
    phase = -wave_number * (x * xs + y * ys) / dz
    u = (np.exp(1j * phase) / dz).astype(dtype).reshape(ny, nx)
    U = apply_frequency_cutoff_2d(fft2(u), cutoff, dx, dy)
    return ifft2(U), U


def material_factor(deltabeta, thickness: float, wl: float):
    """big-wave/optical_element.py:39-42."""
    return np.exp(-2j * np.pi * thickness / wl * np.conj(deltabeta))


def sample_axis(n: int, spacing: float, scale: float, pos: float, length: int, pitch: float):
    """Voxel coordinate of every sim column/row (big-wave/optical_element.py:538-546)."""
    sim = (np.arange(n, dtype=np.float64) - n / 2.0) * spacing
    idx = (sim * scale + pos + length * pitch * 0.5) / pitch
    floor_raw = np.floor(idx).astype(np.int64)
    frac = idx - floor_raw
    inside = (idx >= 0.0) & (idx < float(length) - 1.0)
    return np.clip(floor_raw, 0, length - 2), frac, inside


def interpolate_slice(values: np.ndarray, nx, ny, dx, dy, px, py, x_pos, y_pos, scale=1.0):
    """Bilinear interpolation of a (y_len, x_len) complex table, zero outside
    (big-wave/optical_element.py:567-579, plasma_sample.py:212-216)."""
    y_len, x_len = values.shape
    x0, xf, xin = sample_axis(nx, dx, scale, x_pos, x_len, px)
    y0, yf, yin = sample_axis(ny, dy, scale, y_pos, y_len, py)
    X0 = x0[None, :]
    Y0 = y0[:, None]
    v00 = values[Y0, X0]
    v01 = values[Y0, X0 + 1]
    v10 = values[Y0 + 1, X0]
    v11 = values[Y0 + 1, X0 + 1]
    a = v00 * (1.0 - xf[None, :]) + v01 * xf[None, :]
    b = v10 * (1.0 - xf[None, :]) + v11 * xf[None, :]
    out = a * (1.0 - yf[:, None]) + b * yf[:, None]
    out[~(yin[:, None] & xin[None, :])] = 0.0
    return out


def sample_transmission(grid_slice: np.ndarray, db_list: np.ndarray, nx, ny, dx, dy, px, py, pz, wl,
                        x_pos=0.0, y_pos=0.0, scale=1.0) -> np.ndarray:
    """material_factor of the interpolated delta+i*beta of one Sample slice, complex128
    (big-wave/optical_element.py:566-582: the db_list gather, the interpolation, the factor)."""
    db = interpolate_slice(db_list[grid_slice], nx, ny, dx, dy, px, py, x_pos, y_pos, scale)
    return material_factor(db, pz, wl)


def sample_apply_2d(u, grid, db_list, dx, dy, wl, cutoff, px, py, pz, x_pos=0.0, y_pos=0.0,
                    slice_dz=None, start_slice=0):
    """Sample._apply_2d without history/checkpoints (big-wave/optical_element.py:502-596).
    Returns (u, U)."""
    ny, nx = u.shape
    U = None
    for z in range(start_slice, grid.shape[0]):
        t = sample_transmission(grid[z], db_list, nx, ny, dx, dy, px, py, pz, wl, x_pos, y_pos)
        u = (u * t).astype(u.dtype, copy=False)
        dz = pz if slice_dz is None else slice_dz[z]
        u, U = propagate_2d(u, dx, dy, wl, dz, cutoff)
    return u, U


def dbvolume_apply_2d(u, dbvol, dx, dy, wl, cutoff, px, py, pz, x_pos=0.0, y_pos=0.0):
    """Sample._apply_2d with a per-voxel delta+i*beta volume (nz, ny_v, nx_v) complex instead of
    ids + db_list (big-wave/optical_element.py:533-592). Returns (u, U)."""
    ny, nx = u.shape
    U = None
    for z in range(dbvol.shape[0]):
        db = interpolate_slice(dbvol[z], nx, ny, dx, dy, px, py, x_pos, y_pos)
        u = (u * material_factor(db, pz, wl)).astype(u.dtype, copy=False)
        u, U = propagate_2d(u, dx, dy, wl, pz, cutoff)
    return u, U


# ---- plasma (big-wave/plasma.py) ---------------------------------------------------------
def plasma_delta_beta_grid_multi(ne, ni, te, zstar, f1bar, f2eff_bar, zbar, z2bar, energy,
                                 planck_hc, r_electron_cm):
    """big-wave/plasma.py:380-434 (delta, beta)."""
    ne, ni, te, zstar = (np.asarray(a, dtype=np.float64) for a in (ne, ni, te, zstar))
    lamb_cm = 1.0e-8 * planck_hc / energy
    prefactor = r_electron_cm * lamb_cm * lamb_cm / (2.0 * math.pi)
    delta = ne * prefactor
    beta = np.zeros(ne.shape, dtype=np.float64)
    q = np.clip(np.where(zbar > 0.0, zstar / zbar, 0.0), 0.0, 1.0)
    fb = 1.0 - q
    bound = (fb > 0.0) & (ni > 0.0)
    if np.any(bound):
        bs = ni * prefactor * fb
        delta = delta + np.where(bound, bs * f1bar, 0.0)
        beta += np.where(bound, bs * f2eff_bar, 0.0)
    ff = (ne > 0.0) & (ni > 0.0) & (q > 0.0) & (z2bar > 0.0) & (te > 0.0)
    if np.any(ff):
        nu = energy / 4.135667e-15
        alpha = np.zeros(ne.shape, dtype=np.float64)
        alpha[ff] = 3.7e8 * ne[ff] * ni[ff] * (np.square(q[ff]) * z2bar) / (np.sqrt(te[ff] * 11604.5) * nu ** 3)
        beta += alpha * lamb_cm / (4.0 * math.pi)
    return delta, beta


def plasma_apply_2d(u, ne, ni, te, zs, sf, energy, consts, dx, dy, wl, cutoff, px, py, pz,
                    x_pos=0.0, y_pos=0.0):
    """PlasmaSample._apply_2d (big-wave/plasma_sample.py:126-233); sf = (f1bar, f2eff, zbar, z2bar),
    consts = (PLANCK_HC, R_ELECTRON_CM). Returns (u, U)."""
    ny, nx = u.shape
    U = None
    for z in range(ne.shape[0]):
        d, b = plasma_delta_beta_grid_multi(ne[z], ni[z], te[z], zs[z], *sf, energy, *consts)
        db = interpolate_slice(d + 1j * b, nx, ny, dx, dy, px, py, x_pos, y_pos)
        u = (u * material_factor(db, pz, wl)).astype(u.dtype, copy=False)
        u, U = propagate_2d(u, dx, dy, wl, pz, cutoff)
    return u, U


# ---- detector (big-wave/propagation.py:949-1110) -----------------------------------------
def _axis_plan(det, ds, n, sp):
    """Fractional cell range [lo, hi) that each detector pixel covers on one grid axis, clipped to
    the grid (big-wave/propagation.py:949-977, _area_axis_plan)."""
    gl = (-(n // 2) - 0.5) * sp
    gr = gl + n * sp
    lo = det - ds * 0.5
    hi = det + ds * 0.5
    clo = np.clip(lo, gl, gr)
    chi = np.maximum(np.clip(hi, gl, gr), clo)
    slo = (clo - gl) / sp
    shi = (chi - gl) / sp
    ilo = np.floor(slo).astype(np.int64)
    ihi = np.floor(shi).astype(np.int64)
    flo = slo - ilo
    fhi = shi - ihi
    flo[ilo >= n] = 0.0
    fhi[ihi >= n] = 0.0
    ilo[ilo >= n] = n
    ihi[ihi >= n] = n
    return ilo, flo, ihi, fhi, lo, hi


def detector_area_v1(field: np.ndarray, dx, dy, ds_px, ds_py, out_x, out_y, detector_z) -> np.ndarray:
    """_area_v1_stream (big-wave/propagation.py:995-1110): separable exact overlap areas times
    z/sqrt(x^2+y^2+z^2), float64 (out_y, out_x)."""
    ny, nx = field.shape
    x_det = (np.arange(out_x, dtype=np.float64) - out_x // 2) * ds_px
    y_det = (np.arange(out_y, dtype=np.float64) - out_y // 2) * ds_py
    i0, f0, i1, f1, _, _ = _axis_plan(x_det, ds_px, nx, dx)
    _, _, _, _, y_lo, y_hi = _axis_plan(y_det, ds_py, ny, dy)
    # squared in the field's own precision, accumulated in FP64 (propagation.py:1038-1039)
    inten = field.real * field.real + field.imag * field.imag
    prefix = np.zeros((ny, nx + 1))
    np.cumsum(inten, axis=1, dtype=np.float64, out=prefix[:, 1:])

    def at(idx, fr):
        res = prefix[:, idx] * dx
        inner = idx < nx
        res[:, inner] += fr[inner] * dx * inten[:, idx[inner]]
        return res
    xint = at(i1, f1) - at(i0, f0)  # (ny, out_x)
    gyl = (-(ny // 2) - 0.5) * dy
    cell_lo = gyl + np.arange(ny) * dy
    cell_hi = cell_lo + dy
    overlap = np.minimum(cell_hi[None, :], y_hi[:, None]) - np.maximum(cell_lo[None, :], y_lo[:, None])
    overlap = np.where(overlap > 0, overlap, 0.0)  # (out_y, ny)
    cosine = detector_z / np.sqrt(np.square(x_det)[None, :] + np.square(y_det)[:, None] + detector_z ** 2)
    return (overlap @ xint) * cosine


def detector_legacy(field: np.ndarray, dx, dy, ds_px, ds_py, out_x, out_y, detector_z) -> np.ndarray:
    """_legacy_fastwave_stream (big-wave/propagation.py:836-946)."""
    ny, nx = field.shape

    def ranges(out_n, grid_n, ds, sp):
        pos = (np.arange(out_n, dtype=np.float64) - out_n // 2) * ds
        lo = np.trunc((pos - ds * 0.5) / sp).astype(np.int64) + grid_n // 2
        hi = np.trunc((pos + ds * 0.5) / sp).astype(np.int64) + grid_n // 2
        return pos, np.clip(lo, 0, grid_n), np.clip(hi, 0, grid_n)
    x_det, lx, hx = ranges(out_x, nx, ds_px, dx)
    y_det, ly, hy = ranges(out_y, ny, ds_py, dy)
    inten = field.real * field.real + field.imag * field.imag
    prefix = np.zeros((ny, nx + 1))
    np.cumsum(inten, axis=1, dtype=np.float64, out=prefix[:, 1:])
    rows = prefix[:, hx] - prefix[:, lx]  # (ny, out_x)
    gy = np.arange(ny)
    sel = (gy[None, :] >= ly[:, None]) & (gy[None, :] < hy[:, None])
    cosine = detector_z / np.sqrt(np.square(x_det)[None, :] + np.square(y_det)[:, None] + detector_z ** 2)
    return (sel.astype(np.float64) @ rows) * (dx * dy) * cosine


def relative_l2(actual, expected) -> float:
    """tests/big_wave_2d/test_p5.py:44-50."""
    actual = np.asarray(actual)
    expected = np.asarray(expected)
    return float(np.linalg.norm((actual - expected).reshape(-1))
                 / max(np.linalg.norm(expected.reshape(-1)), np.finfo(float).eps))
