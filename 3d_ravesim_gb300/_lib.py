"""ctypes binding of librs_fresnel.so (C ABI in include/rs_fresnel.h).

This is the only module that talks to the native library. There is no CPU fallback: if the
library is missing or fails to load, every call raises RuntimeError.
"""
from __future__ import annotations

import contextlib
import ctypes
import threading
import weakref
from pathlib import Path

import torch

from . import _build

RS_OK, RS_EINVAL, RS_ENOMEM, RS_ECUDA, RS_EUNSUPPORTED, RS_ETIMEOUT, RS_ECANCELLED = range(7)

c_int, c_uint, c_double, c_void_p = ctypes.c_int, ctypes.c_uint, ctypes.c_double, ctypes.c_void_p


class VoxelGeom(ctypes.Structure):
    _fields_ = [("nz", c_int), ("ny_v", c_int), ("nx_v", c_int),
                ("pixel_size_x", c_double), ("pixel_size_y", c_double), ("pixel_size_z", c_double),
                ("x_pos", c_double), ("y_pos", c_double)]


class PlasmaConsts(ctypes.Structure):
    _fields_ = [("f1bar", c_double), ("f2eff_bar", c_double), ("zbar", c_double), ("z2bar", c_double),
                ("energy_ev", c_double), ("planck_hc", c_double), ("r_electron_cm", c_double)]


class DetectorGeom(ctypes.Structure):
    _fields_ = [("dx", c_double), ("dy", c_double), ("ds_px", c_double), ("ds_py", c_double),
                ("detector_z", c_double), ("out_x", c_int), ("out_y", c_int),
                ("integrator", c_int), ("accumulate", c_int)]


_P = c_void_p
_DP = ctypes.POINTER(c_double)
_SIGS = {
    "rs_version": ([], ctypes.c_char_p),
    "rs_last_error": ([], ctypes.c_char_p),
    "rs_plan_create": ([c_int, c_int, c_uint, ctypes.POINTER(c_void_p)], c_int),
    "rs_plan_destroy": ([_P], c_int),
    "rs_plan_is_fast": ([_P], c_int),
    "rs_fft2": ([_P, _P, _P, _P], c_int),
    "rs_ifft2": ([_P, _P, _P, _P], c_int),
    "rs_apply_cutoff": ([_P, _P, c_double, c_double, c_double, _P], c_int),
    "rs_apply_transfer": ([_P, _P, c_double, c_double, c_double, c_double, c_double, _P], c_int),
    "rs_propagate": ([_P, _P, _P, c_double, c_double, c_double, c_double, c_double, c_int, _P], c_int),
    "rs_point_source": ([_P, _P, c_double, c_double, c_double, c_double, c_double, c_double, _P], c_int),
    "rs_point_source_propagate": ([_P, _P, _P, c_double, c_double, c_double, c_double, c_double,
                                   c_double, c_double, _P], c_int),
    "rs_fresnel_plane": ([_P, _P, c_double, c_double, c_double, c_double, c_double, c_double, _P], c_int),
    "rs_fresnel_plane_propagate": ([_P, _P, _P, c_double, c_double, c_double, c_double, c_double, c_double,
                                    c_double, _P], c_int),
    "rs_multislice_voxel": ([_P, _P, _P, _P, c_int, _P, c_int, ctypes.POINTER(VoxelGeom), c_double,
                             c_double, c_double, c_double, _DP, _DP, c_int, c_int, _P], c_int),
    "rs_multislice_voxel_stacked": ([_P, c_int, _P, _P, _P, c_int, _P, c_int, ctypes.POINTER(VoxelGeom),
                                     c_double, c_double, c_double, c_double, _DP, _DP, c_int, c_int, _P], c_int),
    "rs_multislice_plasma": ([_P, _P, _P, _P, _P, _P, _P, c_int, ctypes.POINTER(PlasmaConsts),
                              ctypes.POINTER(VoxelGeom), c_double, c_double, c_double, c_double,
                              _DP, _DP, c_int, c_int, _P], c_int),
    "rs_detector": ([_P, _P, _P, ctypes.POINTER(DetectorGeom), _P], c_int),
    "rs_multislice_dbgrid": ([_P, _P, _P, _P, ctypes.POINTER(VoxelGeom), c_double, c_double, c_double, c_double,
                              _DP, _DP, c_int, c_int, _P], c_int),
    "rs_multislice_dbgrid_store": ([_P, _P, _P, _P, ctypes.POINTER(VoxelGeom), c_double, c_double, c_double,
                                    c_double, _DP, _DP, c_int, c_int, _P, _P], c_int),
    "rs_adjoint_multislice_dbgrid_ex": ([_P, _P, _P, ctypes.POINTER(VoxelGeom), c_double, c_double, c_double,
                                         c_double, _DP, _DP, c_int, c_int, _P, _P, c_uint, _P], c_int),
    "rs_multislice_dbgrid_fields": ([_P, _P, _P, _P, ctypes.POINTER(VoxelGeom), c_double, c_double, c_double,
                                     c_double, _DP, _DP, c_int, c_int, _P, _P], c_int),
    "rs_adjoint_multislice_dbgrid": ([_P, _P, _P, ctypes.POINTER(VoxelGeom), c_double, c_double, c_double, c_double,
                                      _DP, _DP, c_int, c_int, _P, _P, _P], c_int),
    "rs_adjoint_slice": ([_P, _P, _P, _P, ctypes.POINTER(VoxelGeom), c_double, c_double, c_double, c_int, c_double,
                          _P, _P], c_int),
    "rs_detector_adjoint": ([_P, _P, _P, _P, ctypes.POINTER(DetectorGeom), _P], c_int),
    "rs_plan_set_pipeline": ([_P, c_int], c_int),
    "rs_plan_set_cancel_flag": ([_P, ctypes.POINTER(c_int)], c_int),
    "rs_plan_set_schedule": ([_P, c_int], c_int),
    "rs_plan_is_four_step": ([_P], c_int),
    "rs_plan_get_schedule": ([_P, ctypes.POINTER(c_int)], c_int),
    "rs_plan_schedules": ([_P, ctypes.POINTER(c_int), c_int, ctypes.POINTER(c_int)], c_int),
    "rs_plan_status": ([_P, ctypes.POINTER(c_int)], c_int),
    "rs_plan_check": ([_P, ctypes.POINTER(c_int)], c_int),
    "rs_plan_clear_status": ([_P, _P], c_int),
    "rs_plan_test_stall": ([_P, c_int], c_int),
    "rs_detector_table_bytes": ([c_int, c_int, ctypes.POINTER(DetectorGeom), ctypes.POINTER(ctypes.c_size_t)], c_int),
    "rs_plan_reserve": ([_P, ctypes.c_size_t, ctypes.c_size_t], c_int),
    "rs_alloc_count": ([ctypes.POINTER(ctypes.c_ulonglong)], c_int),
    "rs_detector_noalloc": ([_P, c_int, c_int, _P, ctypes.POINTER(DetectorGeom), _P], c_int),
    "rs_launch_count": ([ctypes.POINTER(ctypes.c_ulonglong)], c_int),
    "rs_plan_profile": ([_P, c_int], c_int),
    "rs_plan_profile_read": ([_P, _DP, _DP, ctypes.POINTER(c_int), ctypes.POINTER(c_int)], c_int),
    "rs_apply_transmission_voxel": ([_P, _P, _P, c_int, _P, c_int, ctypes.POINTER(VoxelGeom),
                                     c_double, c_double, c_double, c_int, c_double, _P], c_int),
}

RS_PLAN_FOURSTEP = 1  # rs_plan_create flag (include/rs_fresnel.h)

_lib = None
_lock = threading.Lock()


def library_path() -> Path:
    return _build.LIB


def lib() -> ctypes.CDLL:
    """Load (building first if the sources are newer) the native library."""
    global _lib
    if _lib is None:
        with _lock:
            if _lib is None:
                path = _build.build()
                handle = ctypes.CDLL(str(path))
                for name, (argtypes, restype) in _SIGS.items():
                    fn = getattr(handle, name)
                    fn.argtypes = argtypes
                    fn.restype = restype
                _lib = handle
    return _lib


def exported_symbols() -> list[str]:
    return list(_SIGS)


def check(status: int, what: str) -> None:
    if status == RS_OK:
        return
    msg = lib().rs_last_error().decode(errors="replace")
    text = f"{what}: {msg}"
    if status == RS_EINVAL:
        raise ValueError(text)
    if status == RS_ECANCELLED:
        raise InterruptedError(text)
    if status == RS_ETIMEOUT:
        raise TimeoutError(text)
    if status == RS_ENOMEM:
        raise MemoryError(text)
    if status == RS_EUNSUPPORTED:
        raise NotImplementedError(text)
    raise RuntimeError(text)


def stream_handle(device: torch.device | None = None) -> c_void_p:
    return c_void_p(torch.cuda.current_stream(device).cuda_stream)


def ptr(t: torch.Tensor) -> c_void_p:
    return c_void_p(t.data_ptr())


class Plan:
    """Owns one rs_plan (twiddles, transfer and geometry tables) for an (nx, ny) field."""

    def __init__(self, nx: int, ny: int, device: torch.device, flags: int = 0):
        """flags: 0, or RS_PLAN_FOURSTEP for a four-step plan at axes of 4096..16384 (axes of
        32768 always get one)."""
        self.nx, self.ny, self.device = int(nx), int(ny), device
        handle = c_void_p()
        with torch.cuda.device(device):
            check(lib().rs_plan_create(self.nx, self.ny, int(flags), ctypes.byref(handle)), "rs_plan_create")
        self.handle = handle
        self.fast = bool(lib().rs_plan_is_fast(handle))
        self.four_step = bool(lib().rs_plan_is_four_step(handle))
        self._finalizer = weakref.finalize(self, Plan._destroy, handle, device)

    def set_pipeline(self, enable: bool | int) -> None:
        """Pass variants: True = bulk-copy pipelined rows and columns, False = per-block kernels, or a
        mask (bit 0 rows, bit 1 columns)."""
        mask = (3 if enable else 0) if isinstance(enable, bool) else int(enable)
        with torch.cuda.device(self.device):
            check(lib().rs_plan_set_pipeline(self.handle, mask), "rs_plan_set_pipeline")

    def set_cancel_flag(self, flag: "ctypes.c_int | None") -> None:
        """Host flag the multislice loops read before each slice: non-zero stops the call with
        InterruptedError (the field is then not a result). None turns the check off. The caller
        keeps `flag` alive while it is set."""
        self._cancel_flag = flag  # referenced here so the library never reads freed memory
        check(lib().rs_plan_set_cancel_flag(self.handle, ctypes.byref(flag) if flag is not None else None),
              "rs_plan_set_cancel_flag")

    def set_schedule(self, mask: int) -> None:
        """Pass schedule bits: 1 pipelined rows, 2 pipelined columns, 4 general row kernel,
        8 split (three-pass) columns, 16 / 32 compensated rows / columns, 64 / 128 dithered
        rows / columns one per thread group."""
        with torch.cuda.device(self.device):
            check(lib().rs_plan_set_schedule(self.handle, int(mask)), "rs_plan_set_schedule")

    def schedule(self) -> int:
        m = c_int(0)
        check(lib().rs_plan_get_schedule(self.handle, ctypes.byref(m)), "rs_plan_get_schedule")
        return m.value

    def schedules(self) -> list[int]:
        """The schedule masks that are distinct for this plan's sizes."""
        buf = (c_int * 256)()
        n = c_int(0)
        check(lib().rs_plan_schedules(self.handle, buf, 256, ctypes.byref(n)), "rs_plan_schedules")
        return [buf[i] for i in range(min(n.value, 256))]

    def status(self) -> int:
        """Synchronise and return the device status word (0 = no bounded wait gave up)."""
        st = c_int(0)
        with torch.cuda.device(self.device):
            check(lib().rs_plan_status(self.handle, ctypes.byref(st)), "rs_plan_status")
        return st.value

    def check(self) -> None:
        """Raise TimeoutError if a pipelined pass of this plan gave up waiting for a bulk copy.
        No device synchronisation: the answer is as of the last call whose stream the caller has
        synchronised. The status is cleared after it is reported once."""
        st = c_int(0)
        code = lib().rs_plan_check(self.handle, ctypes.byref(st))
        if code != RS_OK:
            msg = lib().rs_last_error().decode(errors="replace")
            self.clear_status()
            check(code, f"plan {self.nx}x{self.ny}: {msg}")

    def clear_status(self) -> None:
        with torch.cuda.device(self.device):
            check(lib().rs_plan_clear_status(self.handle, stream_handle(self.device)), "rs_plan_clear_status")

    def test_stall(self, enable: bool = True) -> None:
        """Test hook: the next pipelined column pass times out on purpose (bounded, no fault)."""
        check(lib().rs_plan_test_stall(self.handle, int(bool(enable))), "rs_plan_test_stall")

    def reserve(self, detector_table_bytes: int = 0, plasma_plane_voxels: int = 0) -> None:
        """Grow the plan's detector-table and plasma-plane buffers now, so a run allocates nothing."""
        with torch.cuda.device(self.device):
            check(lib().rs_plan_reserve(self.handle, int(detector_table_bytes), int(plasma_plane_voxels)),
                  "rs_plan_reserve")

    @staticmethod
    def _destroy(handle: c_void_p, device: torch.device) -> None:
        # a finaliser: it may run at interpreter exit, after torch's CUDA state or this module's
        # globals are gone, where there is nothing left to free and nobody to report to
        try:
            with torch.cuda.device(device):
                lib().rs_plan_destroy(handle)
        except Exception:  # noqa: BLE001
            pass


_plans: dict[tuple[int, int, int, int], Plan] = {}
_slot = threading.local()


@contextlib.contextmanager
def plan_slot(k: int):
    """Inside this context, plan_for returns the plans of slot k: work issued on different CUDA
    streams must use different slots, because a plan's tables are rewritten by each call."""
    prev = getattr(_slot, "k", 0)
    _slot.k = int(k)
    try:
        yield
    finally:
        _slot.k = prev


def plan_for(nx: int, ny: int, device: torch.device, slot: int | None = None) -> Plan:
    """Cached plan per (nx, ny, device, slot). Plans are not shared between threads or streams."""
    idx = device.index if device.index is not None else torch.cuda.current_device()
    k = getattr(_slot, "k", 0) if slot is None else int(slot)
    key = (int(nx), int(ny), idx, k)
    p = _plans.get(key)
    if p is None:
        p = Plan(nx, ny, torch.device("cuda", idx))
        _plans[key] = p
        from . import autotune
        autotune.apply_to_plan(p)  # the cached pass schedule of this device and size, if any
    return p


def check_plans(device: torch.device | None = None) -> None:
    """After a host synchronisation: raise TimeoutError if any pass of this device's plans gave up
    waiting for a bulk copy (see Plan.check)."""
    idx = None if device is None else (device.index if device.index is not None else torch.cuda.current_device())
    for (nx, ny, d, k), p in list(_plans.items()):
        if idx is None or d == idx:
            p.check()


def detector_table_bytes(nx: int, ny: int, geom: DetectorGeom) -> int:
    n = ctypes.c_size_t(0)
    check(lib().rs_detector_table_bytes(int(nx), int(ny), ctypes.byref(geom), ctypes.byref(n)),
          "rs_detector_table_bytes")
    return int(n.value)


def alloc_count() -> int:
    """Device and pinned-host allocations made by the native library so far in this process."""
    n = ctypes.c_ulonglong(0)
    check(lib().rs_alloc_count(ctypes.byref(n)), "rs_alloc_count")
    return int(n.value)


def launch_count() -> int:
    n = ctypes.c_ulonglong(0)
    check(lib().rs_launch_count(ctypes.byref(n)), "rs_launch_count")
    return int(n.value)


def doubles(values) -> ctypes.Array:
    arr = (c_double * len(values))(*[float(v) for v in values])
    return arr
