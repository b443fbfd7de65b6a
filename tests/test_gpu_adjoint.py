"""Adjoint gradients (no reference counterpart): the hand-written CUDA adjoint against central
finite differences of the FP64 oracle and against torch.fft autograd of the same forward model."""
import importlib

import numpy as np
import pytest
import torch

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def setup_case(rs, cuda, n=64, nz=4, seed=0, every=None, aligned=False):
    adj = importlib.import_module("3d_ravesim_gb300.adjoint")
    rng = np.random.default_rng(seed)
    dx = 0.5e-6
    wl = rs.convert_energy_wavelength(8000.0)
    pitch = 0.85e-6
    nv = int(n * dx / pitch) + 4
    db = np.stack([rng.uniform(0, 2e-6, (nz, nv, nv)), rng.uniform(0, 2e-8, (nz, nv, nv))], -1).astype(np.float32)
    geom = adj.VolumeGeometry(z_start=0.1, pixel_size_x=pitch, pixel_size_y=pitch, pixel_size_z=2e-6,
                              x_pos=0.13e-6, y_pos=-0.07e-6)
    # aligned: one detector pixel per grid cell, so area_v1 is diagonal (w(y, x) * |u|^2)
    ds, size = (dx, n * dx) if aligned else (1.3 * dx, n * dx * 0.9)
    p = rs.SimParams(N=n * n, nx=n, ny=n, dx=dx, dy=dx, z_detector=0.1 + nz * 2e-6 + 0.03, detector_size=size,
                     detector_pixel_size_x=ds, detector_pixel_size_y=ds, wl=wl, chunk_size=n)
    u0 = torch.ones(n * n, dtype=torch.complex64, device=cuda)
    model = adj.MultisliceModel(p, geom, 0.45 / dx, u0, checkpoint_every=every)
    return adj, model, db, p, geom


def oracle_loss(oracle, db, p, geom, cutoff, target):
    n = p.nx
    vol = db[..., 0].astype(np.float64) + 1j * db[..., 1].astype(np.float64)
    u = np.ones((n, n), np.complex128)
    u, U = oracle.dbvolume_apply_2d(u, vol, p.dx, p.dx, p.wl, cutoff, geom.pixel_size_x, geom.pixel_size_y,
                                    geom.pixel_size_z, geom.x_pos, geom.y_pos)
    u, U = oracle.propagate_2d(u, p.dx, p.dx, p.wl, p.z_detector - (geom.z_start + db.shape[0] * geom.pixel_size_z),
                               cutoff, U=U, skip_fft=True)
    I = oracle.detector_area_v1(u, p.dx, p.dx, p.detector_pixel_size_x, p.detector_pixel_size_y, target.shape[1],
                                target.shape[0], p.z_detector)
    return float(np.sum((I - target) ** 2)), I


@pytest.mark.parametrize("every", [None, 1])
def test_adjoint_matches_fp64_finite_differences(rs, cuda, oracle, every):
    adj, model, db, p, geom = setup_case(rs, cuda, every=every)
    dbt = torch.from_numpy(db).to(cuda)
    I = model.forward(dbt)
    rng = np.random.default_rng(5)
    target = (I.cpu().numpy() * rng.uniform(0.9, 1.1, I.shape)).astype(np.float64)
    L0, I_ref = oracle_loss(oracle, db, p, geom, model.cutoff, target)
    assert rel_l2(I.cpu().numpy(), I_ref) < 2e-5
    grad = model.backward(dbt, 2.0 * (I - torch.from_numpy(target).to(cuda))).cpu().numpy()
    nz, nv = db.shape[0], db.shape[1]
    picks = [(int(rng.integers(nz)), int(rng.integers(8, nv - 8)), int(rng.integers(8, nv - 8)), int(c))
             for c in (0, 1) for _ in range(12)]
    fd, ad = [], []
    for k, j, i, c in picks:
        eps = 1e-3 * (2e-6 if c == 0 else 2e-8)
        dp, dm = db.astype(np.float64).copy(), db.astype(np.float64).copy()
        dp[k, j, i, c] += eps
        dm[k, j, i, c] -= eps
        lp, _ = oracle_loss(oracle, dp, p, geom, model.cutoff, target)
        lm, _ = oracle_loss(oracle, dm, p, geom, model.cutoff, target)
        fd.append((lp - lm) / (2 * eps))
        ad.append(grad[k, j, i, c])
    fd, ad = np.array(fd), np.array(ad)
    for c in (0, 1):
        sel = slice(0, 12) if c == 0 else slice(12, 24)
        scale = np.max(np.abs(fd[sel]))
        assert scale > 0
        assert np.max(np.abs(ad[sel] - fd[sel])) / scale < 5e-3, (c, ad[sel], fd[sel])


def torch_field(db, p, geom, cutoff, oracle):
    """The same forward model in complex128 torch ops (torch.fft), with the oracle's sample
    coordinates, so that torch.autograd differentiates it."""
    n, nz, nv = p.nx, db.shape[0], db.shape[1]
    dev = db.device
    x0, xf, xin = oracle.sample_axis(n, p.dx, 1.0, geom.x_pos, nv, geom.pixel_size_x)
    y0, yf, yin = oracle.sample_axis(n, p.dx, 1.0, geom.y_pos, nv, geom.pixel_size_y)
    x0, y0 = torch.from_numpy(x0).to(dev), torch.from_numpy(y0).to(dev)
    xf, yf = torch.from_numpy(xf).to(dev), torch.from_numpy(yf).to(dev)
    inside = torch.from_numpy(yin[:, None] & xin[None, :]).to(dev)

    def H(dz):
        h = oracle.transfer_function(n, n, p.dx, p.dx, p.wl, dz)
        return torch.from_numpy(h * ~oracle.cutoff_mask(n, n, cutoff, p.dx, p.dx)).to(dev)
    h_slice = H(geom.pixel_size_z)
    u = torch.ones((n, n), dtype=torch.complex128, device=dev)
    vol = torch.complex(db[..., 0].double(), db[..., 1].double())
    for z in range(nz):
        v = vol[z]
        a = v[y0][:, x0] * (1 - xf)[None, :] + v[y0][:, x0 + 1] * xf[None, :]
        b = v[y0 + 1][:, x0] * (1 - xf)[None, :] + v[y0 + 1][:, x0 + 1] * xf[None, :]
        d = torch.where(inside, a * (1 - yf)[:, None] + b * yf[:, None], torch.zeros_like(a))
        u = u * torch.exp(-2j * np.pi * geom.pixel_size_z / p.wl * torch.conj(d))
        u = torch.fft.ifft2(torch.fft.fft2(u) * h_slice)
    return torch.fft.ifft2(torch.fft.fft2(u) * H(p.z_detector - (geom.z_start + nz * geom.pixel_size_z)))


def test_adjoint_matches_torch_autograd(rs, cuda, oracle):
    """Every voxel's gradient at once: with one detector pixel per grid cell the area_v1 image is
    w(y, x) |u|^2, whose weights w are read off the oracle detector of a unit field."""
    adj, model, db, p, geom = setup_case(rs, cuda, n=128, nz=6, seed=2, aligned=True)
    n = p.nx
    dbt = torch.from_numpy(db).to(cuda)
    I = model.forward(dbt)
    assert tuple(I.shape) == (n, n)
    det = lambda f: oracle.detector_area_v1(f, p.dx, p.dx, p.dx, p.dx, n, n, p.z_detector)
    w = det(np.ones((n, n), np.complex128))
    f = np.random.default_rng(9).normal(size=(n, n)) + 0j
    assert np.max(np.abs(det(f) - w * np.abs(f) ** 2)) <= 1e-12 * np.max(np.abs(det(f)))
    rng = np.random.default_rng(3)
    target = torch.from_numpy(I.cpu().numpy() * rng.uniform(0.9, 1.1, (n, n))).to(cuda)
    g_ours = model.backward(dbt, 2.0 * (I - target)).double().cpu().numpy()

    dbr = dbt.double().requires_grad_(True)
    u = torch_field(dbr, p, geom, model.cutoff, oracle)
    I_t = torch.from_numpy(w).to(cuda) * (u.real ** 2 + u.imag ** 2)
    assert rel_l2(I_t.detach().cpu().numpy(), I.cpu().numpy()) < 2e-5
    ((I_t - target) ** 2).sum().backward()
    g_ref = dbr.grad.cpu().numpy()
    for c in (0, 1):
        assert rel_l2(g_ours[..., c], g_ref[..., c]) < 2e-3, c
