"""Gradients of a multislice detector image with respect to per-voxel delta and beta.

The reference has no gradients; this module differentiates the same forward model (per slice:
bilinear delta+i*beta, transmission exp(-2 pi i t/wl conj(delta + i beta)), Fresnel step with
the circular cutoff; then free space to the detector and the area_v1 integration of |u|^2).

Adjoint (Wirtinger calculus, g = dL/dconj(u)):
  detector      g_f = (D^T r) * u_f                      r = dL/dI  (rs_detector_adjoint)
  Fresnel step  g  = P^H g'   with P^H = step of -dz      (same cutoff mask)
  transmission  dL/dconj(t) = conj(u) * v,  g = conj(t) * v            (rs_adjoint_slice)
                dL/ddelta = 4 pi t/wl Im(conj(conj(u) v) t), dL/dbeta = -4 pi t/wl Re(...)
scattered to the voxels through the bilinear weights. Slice fields are checkpointed every
`checkpoint_every` slices (default ~sqrt(nz)) and recomputed segment by segment on the way back;
checkpoint_every=0 instead keeps the field entering every slice (written by the forward row
pass itself), so the backward needs no recomputation: nz fields of nx*ny*8 bytes, 8.6 GB for
256 slices at 2048^2, which a GB300's HBM holds easily; checkpoint_every="auto" keeps every
field when they fit a memory budget and checkpoints otherwise.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from .propagation import SimParams, propagate_2d, square_and_downsample_2d_device
from .vector import GpuVector


@dataclass
class VolumeGeometry:
    """Placement of a (nz, ny_v, nx_v) voxel volume (big-wave/optical_element.py:383-412)."""

    z_start: float
    pixel_size_x: float
    pixel_size_y: float
    pixel_size_z: float
    x_pos: float = 0.0
    y_pos: float = 0.0


class MultisliceModel:
    """Detector image I(delta, beta) of a field u0 through a delta/beta voxel volume."""

    def __init__(self, params: SimParams, geom: VolumeGeometry, cutoff: float, u0: torch.Tensor,
                 checkpoint_every: int | str | None = None, memory_budget_bytes: int | None = None,
                 keep_tail: int = 2):
        """checkpoint_every: None (about sqrt(nz) slices per segment), a segment length, 0 (keep
        every slice's field), or "auto": keep every field when nz fields fit memory_budget_bytes
        (default: a quarter of the device's free memory at forward time), else sqrt(nz).
        keep_tail: with checkpoints, the number of last segments whose fields the forward keeps
        (the backward starts with them and need not recompute them): 2 * every extra fields."""
        self.p, self.geom, self.cutoff = params, geom, float(cutoff)
        self.u0 = u0
        self.device = u0.device
        if not (checkpoint_every is None or checkpoint_every == "auto" or
                (isinstance(checkpoint_every, int) and checkpoint_every >= 0)):
            raise ValueError(f"checkpoint_every must be None, 'auto' or an int >= 0, got {checkpoint_every!r}")
        self.checkpoint_every = checkpoint_every
        self.memory_budget_bytes = memory_budget_bytes
        if not (isinstance(keep_tail, int) and keep_tail >= 0):
            raise ValueError(f"keep_tail must be an int >= 0, got {keep_tail!r}")
        self.keep_tail = keep_tail
        n = params.nx * params.ny
        self.u = GpuVector(torch.empty(n, dtype=torch.complex64, device=self.device))
        self.U = GpuVector(torch.empty(n, dtype=torch.complex64, device=self.device))
        self.checkpoints: dict[int, torch.Tensor] = {}
        self.tail: dict[int, torch.Tensor] = {}  # first slice -> fields entering a kept segment's slices
        self.u_final = None
        self.last_backward = None  # "fused" (two passes per slice) or "per-slice"
        self.fused = True          # False forces the per-slice backward
        self.fields: torch.Tensor | None = None  # checkpoint_every == 0: every slice's entering field

    # -- helpers ------------------------------------------------------------------------------
    def _vgeom(self, db: torch.Tensor) -> _lib.VoxelGeom:
        nz, nyv, nxv, _ = db.shape
        g = self.geom
        return _lib.VoxelGeom(nz, nyv, nxv, g.pixel_size_x, g.pixel_size_y, g.pixel_size_z, g.x_pos, g.y_pos)

    def _dz(self, nz: int):
        return np.full(nz, self.geom.pixel_size_z, dtype=np.float64)

    def _final_dz(self, nz: int) -> float:
        return self.p.z_detector - (self.geom.z_start + nz * self.geom.pixel_size_z)

    def _step_slices(self, db: torch.Tensor, s0: int, s1: int) -> None:
        p = self.p
        plan = _lib.plan_for(p.nx, p.ny, self.device)
        with torch.cuda.device(self.device):
            _lib.check(_lib.lib().rs_multislice_dbgrid(
                plan.handle, _lib.ptr(self.u.vec), _lib.ptr(self.U.vec), _lib.ptr(db), self._vgeom(db),
                float(p.dx), float(p.get_dy()), float(p.wl), self.cutoff, _lib.doubles(self._dz(db.shape[0])), None,
                s0, s1, _lib.stream_handle()), "rs_multislice_dbgrid")

    # -- forward / backward ---------------------------------------------------------------------
    def forward(self, db: torch.Tensor) -> torch.Tensor:
        """float64 detector image; db is (nz, ny_v, nx_v, 2) float32 (delta, beta) on the device."""
        if db.dtype != torch.float32 or db.dim() != 4 or db.shape[3] != 2 or not db.is_contiguous():
            raise ValueError("db must be a contiguous (nz, ny_v, nx_v, 2) float32 tensor")
        nz = db.shape[0]
        self.u.vec.copy_(self.u0.reshape(-1))
        self.checkpoints = {}
        self.fields = None
        start = self.u.vec.clone()
        mode = self.checkpoint_every
        if mode == "auto":
            need = nz * self.p.nx * self.p.ny * 8
            budget = self.memory_budget_bytes
            if budget is None:
                budget = torch.cuda.mem_get_info(self.device)[0] // 4
            mode = 0 if need <= budget else None
        if mode == 0 and self.fused and self._forward_store_all(db):
            self.every = nz
            self.checkpoints[0] = start  # lets the per-slice backward recompute if it is forced
        else:
            every = mode or max(1, int(round(math.sqrt(nz))))
            self.every = every
            self.tail = {}
            starts = list(range(0, nz, every))
            for s0 in starts:
                self.checkpoints[s0] = self.u.vec.clone()
                s1 = min(nz, s0 + every)
                # the last keep_tail segments keep their fields as they run: the backward starts
                # with them and then needs no recomputation of them
                if s0 in starts[max(0, len(starts) - self.keep_tail):] and self.fused and self._store_segment(db, s0, s1):
                    continue
                self._step_slices(db, s0, s1)
        p = self.p
        propagate_2d(self.u, self.U, p.dx, p.get_dy(), p.wl, self._final_dz(nz), p.chunk_size, self.cutoff,
                     p.nx, p.ny, skip_fft=True)
        self.u_final = self.u.vec.clone()
        return square_and_downsample_2d_device(self.u, p, p.z_detector)

    def backward(self, db: torch.Tensor, dI: torch.Tensor) -> torch.Tensor:
        """dL/d(delta, beta) for the upstream gradient dI = dL/dI of the last forward call."""
        p = self.p
        nz = db.shape[0]
        lib = _lib.lib()
        plan = _lib.plan_for(p.nx, p.ny, self.device)
        st = _lib.stream_handle()
        grad = torch.zeros_like(db)
        r = dI.to(torch.float64).contiguous()
        dx, dy = float(p.dx), float(p.get_dy())
        ds_px, ds_py, det_z, _ = p.effective_detector_geometry(p.z_detector)
        out_y, out_x = r.shape
        dgeom = _lib.DetectorGeom(dx, dy, ds_px, ds_py, det_z, out_x, out_y,
                                  0 if p.detector_integrator == "area_v1" else 1, 0)
        g = GpuVector(torch.empty_like(self.u.vec))
        scratch = GpuVector(torch.empty_like(self.u.vec))
        with torch.cuda.device(self.device):
            _lib.check(lib.rs_detector_adjoint(plan.handle, _lib.ptr(self.u_final), _lib.ptr(g.vec), _lib.ptr(r),
                                               dgeom, st), "rs_detector_adjoint")
        # P_final^H
        propagate_2d(g, scratch, p.dx, p.get_dy(), p.wl, -self._final_dz(nz), p.chunk_size, self.cutoff, p.nx, p.ny)
        vg = self._vgeom(db)
        if self.fused and self._backward_fused(db, g, grad, vg, plan, st):
            self.last_backward = "fused"
            return grad
        self.last_backward = "per-slice"
        for s0 in sorted(self.checkpoints, reverse=True):
            s1 = min(nz, s0 + self.every)
            # recompute the fields entering slices s0 .. s1-1 from the checkpoint
            self.u.vec.copy_(self.checkpoints[s0])
            fields = []
            for k in range(s0, s1):
                fields.append(self.u.vec.clone())
                if k + 1 < s1:
                    self._step_slices(db, k, k + 1)
            for k in range(s1 - 1, s0 - 1, -1):
                propagate_2d(g, scratch, p.dx, p.get_dy(), p.wl, -self.geom.pixel_size_z, p.chunk_size, self.cutoff,
                             p.nx, p.ny)
                with torch.cuda.device(self.device):
                    _lib.check(lib.rs_adjoint_slice(plan.handle, _lib.ptr(g.vec), _lib.ptr(fields[k - s0]),
                                                    _lib.ptr(db), vg, dx, dy, float(p.wl), k, 1.0, _lib.ptr(grad), st),
                               "rs_adjoint_slice")
        return grad


    def _store_segment(self, db: torch.Tensor, s0: int, s1: int) -> bool:
        """Slices s0..s1-1 keeping the field entering each (self.tail); False if unsupported."""
        p = self.p
        plan = _lib.plan_for(p.nx, p.ny, self.device)
        if not plan.fast or p.nx & (p.nx - 1) or 2 * db.shape[2] > p.nx + p.nx // 16:
            return False
        fields = torch.empty((s1 - s0, p.nx * p.ny), dtype=torch.complex64, device=self.device)
        with torch.cuda.device(self.device):
            rc = _lib.lib().rs_multislice_dbgrid_store(
                plan.handle, _lib.ptr(self.u.vec), _lib.ptr(self.U.vec), _lib.ptr(db), self._vgeom(db),
                float(p.dx), float(p.get_dy()), float(p.wl), self.cutoff, _lib.doubles(self._dz(db.shape[0])), None,
                s0, s1, _lib.ptr(fields), _lib.stream_handle())
        if rc == _lib.RS_EUNSUPPORTED:
            return False
        _lib.check(rc, "rs_multislice_dbgrid_store")
        self.tail[s0] = fields
        return True

    def _forward_store_all(self, db: torch.Tensor) -> bool:
        """The whole forward in one fused call that also keeps every slice's entering field;
        False (nothing run) when the size is not supported by the fused adjoint."""
        p = self.p
        nz = db.shape[0]
        plan = _lib.plan_for(p.nx, p.ny, self.device)
        if not plan.fast or p.nx & (p.nx - 1) or 2 * db.shape[2] > p.nx + p.nx // 16:
            return False
        self.fields = torch.empty((nz, p.nx * p.ny), dtype=torch.complex64, device=self.device)
        with torch.cuda.device(self.device):
            _lib.check(_lib.lib().rs_multislice_dbgrid_store(
                plan.handle, _lib.ptr(self.u.vec), _lib.ptr(self.U.vec), _lib.ptr(db), self._vgeom(db),
                float(p.dx), float(p.get_dy()), float(p.wl), self.cutoff, _lib.doubles(self._dz(nz)), None, 0, nz,
                _lib.ptr(self.fields), _lib.stream_handle()), "rs_multislice_dbgrid_store")
        return True

    def _backward_fused(self, db, g, grad, vg, plan, st) -> bool:
        """Backward sweep in two fused passes per slice (rs_adjoint_multislice_dbgrid), each segment's
        fields recomputed from its checkpoint by rs_multislice_dbgrid_store. False when the size is
        not supported by the fused kernels (the caller then takes the per-slice path)."""
        p = self.p
        lib = _lib.lib()
        nz = db.shape[0]
        n = p.nx * p.ny
        dz = _lib.doubles(self._dz(nz))
        if self.fields is not None:  # every field kept by the forward: one sweep, nothing recomputed
            with torch.cuda.device(self.device):
                _lib.check(lib.rs_adjoint_multislice_dbgrid(plan.handle, _lib.ptr(g.vec), _lib.ptr(db), vg,
                                                            float(p.dx), float(p.get_dy()), float(p.wl), self.cutoff,
                                                            dz, None, 0, nz, _lib.ptr(self.fields), _lib.ptr(grad),
                                                            st), "rs_adjoint_multislice_dbgrid")
            return True
        tail = self.tail or {}
        scratch = None
        order = sorted(self.checkpoints, reverse=True)
        for i, s0 in enumerate(order):
            s1 = min(nz, s0 + self.every)
            # g stays transformed along x from one segment to the next
            gflags = (1 if i > 0 else 0) | (2 if i + 1 < len(order) else 0)
            with torch.cuda.device(self.device):
                fields = tail.get(s0)  # a kept segment's fields are still there
                if fields is None:
                    if scratch is None:
                        scratch = torch.empty((self.every, n), dtype=torch.complex64, device=self.device)
                    fields = scratch
                    self.u.vec.copy_(self.checkpoints[s0])
                    rc = lib.rs_multislice_dbgrid_fields(plan.handle, _lib.ptr(self.u.vec), _lib.ptr(self.U.vec),
                                                         _lib.ptr(db), vg, float(p.dx), float(p.get_dy()),
                                                         float(p.wl), self.cutoff, dz, None, s0, s1,
                                                         _lib.ptr(fields), st)
                    if rc == _lib.RS_EUNSUPPORTED:
                        return False
                    _lib.check(rc, "rs_multislice_dbgrid_fields")
                rc = lib.rs_adjoint_multislice_dbgrid_ex(plan.handle, _lib.ptr(g.vec), _lib.ptr(db), vg,
                                                         float(p.dx), float(p.get_dy()), float(p.wl), self.cutoff,
                                                         dz, None, s0, s1, _lib.ptr(fields), _lib.ptr(grad), gflags,
                                                         st)
                if rc == _lib.RS_EUNSUPPORTED:
                    return False
                _lib.check(rc, "rs_adjoint_multislice_dbgrid")
        return True


class _MultisliceIntensity(torch.autograd.Function):
    @staticmethod
    def forward(ctx, db: torch.Tensor, model: MultisliceModel) -> torch.Tensor:
        ctx.model = model
        ctx.save_for_backward(db)
        return model.forward(db.detach().contiguous())

    @staticmethod
    def backward(ctx, dI: torch.Tensor):
        (db,) = ctx.saved_tensors
        return ctx.model.backward(db.detach().contiguous(), dI), None


def multislice_intensity(db: torch.Tensor, model: MultisliceModel) -> torch.Tensor:
    """Differentiable detector image: torch.autograd sees dI/d(db) through the hand-written adjoint."""
    return _MultisliceIntensity.apply(db, model)


def gaussian_plasma_db(n0: torch.Tensor, length: torch.Tensor, te: torch.Tensor, shape: tuple[int, int, int],
                       pitch: tuple[float, float, float], energy: float, zstar: float = 3.5, z2bar: float = 18.5,
                       zbar: float = 3.5) -> torch.Tensor:
    """(nz, ny_v, nx_v, 2) float32 delta/beta of n_e = n0 exp(-r^2/2L^2), n_i = n_e/Z*, uniform T_e, in
    torch (so n0, L, T_e receive gradients): delta = r_e lambda^2/(2 pi) n_e and the Kramers beta of
    big-wave/plasma.py:380-434 with q = Z*/zbar = 1 (no bound electrons)."""
    import scipy.constants as consts
    planck_hc = 1.e10 * consts.Planck * consts.c / consts.e
    r_e = 100.0 * consts.physical_constants["classical electron radius"][0]
    dev = n0.device
    nz, ny, nx = shape
    pz, py, px = pitch
    z = (torch.arange(nz, device=dev, dtype=torch.float64) + 0.5 - nz / 2.0) * pz
    y = (torch.arange(ny, device=dev, dtype=torch.float64) - ny / 2.0) * py
    x = (torch.arange(nx, device=dev, dtype=torch.float64) - nx / 2.0) * px
    r2 = z[:, None, None] ** 2 + y[None, :, None] ** 2 + x[None, None, :] ** 2
    ne = n0 * torch.exp(-r2 / (2.0 * length ** 2))
    ni = ne / zstar
    lamb_cm = 1.0e-8 * planck_hc / energy
    pref = r_e * lamb_cm * lamb_cm / (2.0 * math.pi)
    q = min(max(zstar / zbar, 0.0), 1.0)
    nu = energy / 4.135667e-15
    delta = ne * pref
    alpha = 3.7e8 * ne * ni * (q * q * z2bar) / (torch.sqrt(te * 11604.5) * nu ** 3)
    beta = alpha * lamb_cm / (4.0 * math.pi)
    return torch.stack([delta, beta], dim=-1).to(torch.float32).contiguous()
