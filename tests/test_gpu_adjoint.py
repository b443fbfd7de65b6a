"""Adjoint gradients (no reference counterpart): the hand-written CUDA adjoint against central
finite differences of the FP64 oracle and against torch.fft autograd of the same forward model."""
import importlib

import numpy as np
import pytest
import torch

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def setup_case(rs, cuda, n=64, nz=4, seed=0, every=None, aligned=False, pitch=0.85e-6):
    """pitch 0.85 um: voxel rows wider than a third of the row, so the backward takes the per-slice
    path; pitch 2 um: the fused two-pass backward."""
    adj = importlib.import_module("3d_ravesim_gb300.adjoint")
    rng = np.random.default_rng(seed)
    dx = 0.5e-6
    wl = rs.convert_energy_wavelength(8000.0)
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


@pytest.mark.parametrize("every,pitch,path", [(None, 0.85e-6, "per-slice"), (1, 0.85e-6, "per-slice"),
                                              (None, 2e-6, "fused"), (3, 2e-6, "fused"), (0, 2e-6, "fused")])
def test_adjoint_matches_fp64_finite_differences(rs, cuda, oracle, every, pitch, path):
    adj, model, db, p, geom = setup_case(rs, cuda, n=128 if path == "fused" else 64, nz=5, every=every, pitch=pitch)
    dbt = torch.from_numpy(db).to(cuda)
    I = model.forward(dbt)
    rng = np.random.default_rng(5)
    target = (I.cpu().numpy() * rng.uniform(0.9, 1.1, I.shape)).astype(np.float64)
    L0, I_ref = oracle_loss(oracle, db, p, geom, model.cutoff, target)
    assert rel_l2(I.cpu().numpy(), I_ref) < 2e-5
    grad = model.backward(dbt, 2.0 * (I - torch.from_numpy(target).to(cuda))).cpu().numpy()
    assert model.last_backward == path
    nz, nv = db.shape[0], db.shape[1]
    lo, hi = (8, nv - 8) if nv > 24 else (3, nv - 3)
    picks = [(int(rng.integers(nz)), int(rng.integers(lo, hi)), int(rng.integers(lo, hi)), int(c))
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


@pytest.mark.parametrize("pitch,path", [(0.85e-6, "per-slice"), (2e-6, "fused")])
def test_adjoint_matches_torch_autograd(rs, cuda, oracle, pitch, path):
    """Every voxel's gradient at once: with one detector pixel per grid cell the area_v1 image is
    w(y, x) |u|^2, whose weights w are read off the oracle detector of a unit field."""
    adj, model, db, p, geom = setup_case(rs, cuda, n=128, nz=6, seed=2, aligned=True, pitch=pitch)
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
    assert model.last_backward == path

    dbr = dbt.double().requires_grad_(True)
    u = torch_field(dbr, p, geom, model.cutoff, oracle)
    I_t = torch.from_numpy(w).to(cuda) * (u.real ** 2 + u.imag ** 2)
    assert rel_l2(I_t.detach().cpu().numpy(), I.cpu().numpy()) < 2e-5
    ((I_t - target) ** 2).sum().backward()
    g_ref = dbr.grad.cpu().numpy()
    for c in (0, 1):
        assert rel_l2(g_ours[..., c], g_ref[..., c]) < 2e-3, c


def test_plasma_parameter_gradients(rs, cuda, oracle):
    """dL/d(n0, L, T_e) of a Gaussian plasma (n_e = n0 exp(-r^2/2L^2), n_i = n_e/Z*, uniform T_e):
    torch.autograd through gaussian_plasma_db and the hand-written adjoint, against central
    differences of the FP64 oracle forward on the same delta/beta volume."""
    adj = importlib.import_module("3d_ravesim_gb300.adjoint")
    n, nz = 64, 4
    dx = 0.5e-6
    energy = 8000.0
    wl = rs.convert_energy_wavelength(energy)
    pitch = (0.6e-6, 0.6e-6, 2e-6)
    nv = int(n * dx / pitch[0]) + 4
    geom = adj.VolumeGeometry(z_start=0.1, pixel_size_x=pitch[0], pixel_size_y=pitch[1], pixel_size_z=pitch[2])
    p = rs.SimParams(N=n * n, nx=n, ny=n, dx=dx, dy=dx, z_detector=0.1 + nz * pitch[2] + 0.02, detector_size=n * dx,
                     detector_pixel_size_x=dx, detector_pixel_size_y=dx, wl=wl, chunk_size=n)
    u0 = torch.ones(n * n, dtype=torch.complex64, device=cuda)
    model = adj.MultisliceModel(p, geom, 0.45 / dx, u0)
    theta0 = {"n0": 2e22, "length": 8e-6, "te": 50.0}

    def db_of(th, dev, dtype):
        t = {k: torch.tensor(v, dtype=torch.float64, device=dev, requires_grad=dtype == "grad") for k, v in th.items()}
        db = adj.gaussian_plasma_db(t["n0"], t["length"], t["te"], (nz, nv, nv), pitch[::-1], energy)
        return t, db

    th_t, db = db_of(theta0, cuda, "grad")
    I = adj.multislice_intensity(db, model)
    rng = np.random.default_rng(11)
    target = (I.detach() * torch.from_numpy(rng.uniform(0.97, 1.03, tuple(I.shape))).to(cuda)).detach()
    ((I - target) ** 2).sum().backward()
    grads = {k: float(v.grad) for k, v in th_t.items()}
    tgt = target.cpu().numpy()

    def oracle_loss(th):
        _, d = db_of(th, "cpu", "value")
        d = d.double().numpy()
        vol = d[..., 0] + 1j * d[..., 1]
        u, U = oracle.dbvolume_apply_2d(np.ones((n, n), np.complex128), vol, dx, dx, wl, model.cutoff, pitch[0],
                                        pitch[1], pitch[2])
        u, U = oracle.propagate_2d(u, dx, dx, wl, p.z_detector - (geom.z_start + nz * pitch[2]), model.cutoff, U=U,
                                   skip_fft=True)
        Io = oracle.detector_area_v1(u, dx, dx, dx, dx, n, n, p.z_detector)
        return float(np.sum((Io - tgt) ** 2))

    for k, v in theta0.items():
        h = 1e-3 * v
        fd = (oracle_loss({**theta0, k: v + h}) - oracle_loss({**theta0, k: v - h})) / (2 * h)
        assert fd != 0.0
        assert abs(grads[k] - fd) <= 2e-2 * abs(fd), (k, grads[k], fd)


def test_fused_backward_matches_per_slice_at_1024(rs, cuda):
    """The two-pass fused backward against the per-slice adjoint on a larger case (1024^2, 24 slices,
    260^2 voxels, several checkpoint segments and row blocks of 4 rows)."""
    adj = importlib.import_module("3d_ravesim_gb300.adjoint")
    n, nz, dx, pitch = 1024, 24, 0.5e-6, 2e-6
    nv = int(n * dx / pitch) + 4
    rng = np.random.default_rng(21)
    db = np.stack([rng.uniform(0, 2e-6, (nz, nv, nv)), rng.uniform(0, 2e-8, (nz, nv, nv))], -1).astype(np.float32)
    wl = rs.convert_energy_wavelength(8000.0)
    geom = adj.VolumeGeometry(z_start=0.1, pixel_size_x=pitch, pixel_size_y=pitch, pixel_size_z=2e-6)
    p = rs.SimParams(N=n * n, nx=n, ny=n, dx=dx, dy=dx, z_detector=0.1 + nz * 2e-6 + 0.05, detector_size=n * dx,
                     detector_pixel_size_x=2 * dx, detector_pixel_size_y=2 * dx, wl=wl, chunk_size=n)
    model = adj.MultisliceModel(p, geom, 0.45 / dx, torch.ones(n * n, dtype=torch.complex64, device=cuda))
    dbt = torch.from_numpy(db).to(cuda)
    I = model.forward(dbt)
    r = torch.from_numpy(rng.normal(size=tuple(I.shape))).to(cuda)
    g_fused = model.backward(dbt, r).cpu().numpy()
    assert model.last_backward == "fused"
    model.fused = False
    model.forward(dbt)
    g_ref = model.backward(dbt, r).cpu().numpy()
    assert model.last_backward == "per-slice"
    for c in (0, 1):
        assert rel_l2(g_fused[..., c], g_ref[..., c]) < 1e-4, c


def test_auto_checkpointing_keeps_fields_within_budget(rs, cuda):
    """checkpoint_every="auto": every slice's field when they fit the budget, sqrt(nz) segments
    when not; both give the same gradient."""
    grads = {}
    for budget, keeps in ((1 << 40, True), (1, False)):
        adj, model, db, p, geom = setup_case(rs, cuda, n=128, nz=9, every="auto", pitch=2e-6)
        model.memory_budget_bytes = budget
        dbt = torch.from_numpy(db).to(cuda)
        I = model.forward(dbt)
        assert (model.fields is not None) == keeps
        assert model.every == (9 if keeps else 3)
        grads[keeps] = model.backward(dbt, torch.ones_like(I)).cpu().numpy()
        assert model.last_backward == "fused"
    assert rel_l2(grads[True], grads[False]) < 1e-6
