"""GpuVector: big-wave's Vector protocol (big-wave/vector.py:13-90) on a CUDA complex64 tensor.

The field is a flat (nx*ny,) torch.complex64 tensor in HBM, laid out row-major exactly like
NumpyVector.vec.reshape(ny, nx) (big-wave/vector.py:341-347). fft2/ifft2 run the native
Stockham kernels; the chunked read/write/modify callbacks are host round trips kept for
API compatibility (tests, small diagnostics), not for the hot path.
"""
from __future__ import annotations

from typing import Callable

import numpy as np
import torch

from . import _lib


FOUR_STEP_N2 = 256  # the second factor of a four-step axis (n = n1 * 256)


def four_step_frequency(n: int) -> np.ndarray:
    """Frequency index held by each storage entry of a four-step axis of length n: entry i holds
    frequency i // 256 + (n // 256) * (i % 256)."""
    i = np.arange(n)
    return i // FOUR_STEP_N2 + (n // FOUR_STEP_N2) * (i % FOUR_STEP_N2)


def natural_from_four_step(flat: np.ndarray, nx: int, ny: int) -> np.ndarray:
    """A spectrum in four-step storage order (both axes) as the natural-order flat array."""
    out = np.empty((ny, nx), dtype=flat.dtype)
    out[np.ix_(four_step_frequency(ny), four_step_frequency(nx))] = np.asarray(flat).reshape(ny, nx)
    return out.reshape(-1)


def four_step_from_natural(flat: np.ndarray, nx: int, ny: int) -> np.ndarray:
    nat = np.asarray(flat).reshape(ny, nx)
    return np.ascontiguousarray(nat[np.ix_(four_step_frequency(ny), four_step_frequency(nx))]).reshape(-1)


class GpuVector:
    """A complex64 wave field resident on one CUDA device.

    spectrum_order is None when the tensor holds its values in natural order, or
    ("four_step", nx, ny) when it holds a spectrum that a four-step plan (axes of 32768) left in
    four-step storage order. Every host read (to_numpy, the chunked callbacks, checkpoints) sees
    the natural order either way, so U = FFT2(u) holds for callers as in big-wave."""

    spectrum_order = None

    def __init__(self, vec: torch.Tensor):
        if not isinstance(vec, torch.Tensor):
            raise TypeError("GpuVector wraps a torch.Tensor; use GpuVector.from_numpy for arrays")
        if vec.dtype != torch.complex64:
            raise TypeError(f"GpuVector holds complex64 fields only, got {vec.dtype}")
        if not vec.is_cuda:
            raise TypeError("GpuVector must live on a CUDA device (there is no CPU fallback)")
        if vec.dim() != 1 or not vec.is_contiguous():
            raise ValueError("GpuVector expects a flat contiguous tensor")
        self.vec = vec

    # -- construction -------------------------------------------------------------------
    @classmethod
    def zeros(cls, n: int, device: str | torch.device = "cuda") -> "GpuVector":
        return cls(torch.zeros(int(n), dtype=torch.complex64, device=device))

    @classmethod
    def ones(cls, n: int, device: str | torch.device = "cuda") -> "GpuVector":
        return cls(torch.ones(int(n), dtype=torch.complex64, device=device))

    @classmethod
    def from_numpy(cls, arr: np.ndarray, device: str | torch.device = "cuda") -> "GpuVector":
        a = np.ascontiguousarray(np.asarray(arr).reshape(-1))
        if a.dtype != np.complex64:
            if not np.iscomplexobj(a) and a.dtype.kind not in "fiu":
                raise TypeError(f"cannot build a complex64 field from {a.dtype}")
            a = a.astype(np.complex64)
        return cls(torch.from_numpy(a).to(device))

    def to_numpy(self) -> np.ndarray:
        host = self.vec.detach().cpu().numpy()
        if self.spectrum_order is not None:
            _, nx, ny = self.spectrum_order
            host = natural_from_four_step(host, nx, ny)
        return host

    def load_natural(self, host: np.ndarray) -> None:
        """Copy a natural-order host array into the field, in this vector's storage order."""
        a = np.ascontiguousarray(np.asarray(host, dtype=np.complex64).reshape(-1))
        if self.spectrum_order is not None:
            _, nx, ny = self.spectrum_order
            a = four_step_from_natural(a, nx, ny)
        self.vec.copy_(torch.from_numpy(a).to(self.device))

    @property
    def device(self) -> torch.device:
        return self.vec.device

    # -- Vector protocol ------------------------------------------------------------------
    def __len__(self) -> int:
        return int(self.vec.numel())

    @property
    def dtype(self) -> np.dtype:
        return np.dtype(np.complex64)

    def fft(self, destination: "GpuVector"):
        raise NotImplementedError("1D propagation is outside the GB300 2D path")

    def ifft(self, destination: "GpuVector"):
        raise NotImplementedError("1D propagation is outside the GB300 2D path")

    def fft2(self, destination: "GpuVector", nx: int, ny: int) -> None:
        """destination = scipy.fft.fft2(self.reshape(ny, nx)).reshape(-1) (unnormalised)."""
        self._check_2d(destination, nx, ny)
        plan = _lib.plan_for(nx, ny, self.device)
        with torch.cuda.device(self.device):
            _lib.check(_lib.lib().rs_fft2(plan.handle, _lib.ptr(self.vec), _lib.ptr(destination.vec),
                                          _lib.stream_handle()), "fft2")

    def ifft2(self, destination: "GpuVector", nx: int, ny: int) -> None:
        """destination = scipy.fft.ifft2(self.reshape(ny, nx)).reshape(-1) (1/N normalised)."""
        self._check_2d(destination, nx, ny)
        plan = _lib.plan_for(nx, ny, self.device)
        with torch.cuda.device(self.device):
            _lib.check(_lib.lib().rs_ifft2(plan.handle, _lib.ptr(self.vec), _lib.ptr(destination.vec),
                                           _lib.stream_handle()), "ifft2")

    def write_chunked(self, chunk_size: int, fn: Callable[[int, np.ndarray], None]) -> None:
        self.modify_chunked(chunk_size, fn)

    def modify_chunked(self, chunk_size: int, fn: Callable[[int, np.ndarray], None]) -> None:
        host = self.to_numpy()
        for i in range(0, len(host), chunk_size):
            chunk = host[i:i + chunk_size]
            fn(i, chunk)
            host[i:i + chunk_size] = chunk
        self.load_natural(host)

    def read_chunked(self, chunk_size: int, fn: Callable[[int, np.ndarray], None]) -> None:
        host = self.to_numpy()
        for i in range(0, len(host), chunk_size):
            fn(i, host[i:i + chunk_size])

    def copy(self) -> "GpuVector":
        c = GpuVector(self.vec.clone())
        c.spectrum_order = self.spectrum_order
        return c

    def copy_to(self, destination: "GpuVector") -> None:
        if len(destination) != len(self) or destination.device != self.device:
            destination.vec = self.vec.clone()
        else:
            destination.vec.copy_(self.vec)
        destination.spectrum_order = self.spectrum_order

    def drop(self) -> None:
        self.vec = torch.empty(0, dtype=torch.complex64, device=self.device)
        self.spectrum_order = None

    # -- helpers --------------------------------------------------------------------------
    def _check_2d(self, destination: "GpuVector", nx: int, ny: int) -> None:
        require_gpu(destination, "destination")
        if len(self) != nx * ny:
            raise ValueError(f"vector length {len(self)} does not match nx*ny={nx * ny}")
        if len(destination) != nx * ny:
            destination.vec = torch.empty(nx * ny, dtype=torch.complex64, device=self.device)
        if destination.device != self.device:
            raise ValueError("source and destination live on different devices")


def require_gpu(v, name: str) -> GpuVector:
    if not isinstance(v, GpuVector):
        raise TypeError(f"{name} must be a GpuVector (complex64 on CUDA), got {type(v).__name__}")
    return v


def as_gpu_pair(u, U) -> tuple[GpuVector, GpuVector]:
    u = require_gpu(u, "u")
    U = require_gpu(U, "U")
    if len(U) != len(u):
        # big-wave's U "doesn't have to be a valid vector": allocate it like NumpyVector.fft2 would
        U.vec = torch.empty(len(u), dtype=torch.complex64, device=u.device)
    if u.device != U.device:
        raise ValueError("u and U live on different devices")
    if u.vec.data_ptr() == U.vec.data_ptr():
        raise ValueError("u and U must be distinct buffers")
    return u, U
