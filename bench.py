"""Benchmark: fused multislice slice-steps/s at 4096^2 complex64 on GB300.

Workload (one "step"): the Talbot-Lau single-source configuration at 4096 x 4096 complex64 —
point source 0.5 m upstream (exp(2 pi i r/wl)/r, FP64 phase), pi-shift Si phase grating,
512 x 1 um Gaussian-blob voxel sample, absorption grating at the first fractional Talbot
distance, free space to the detector, area_v1 detector — run through the package's public API
(Sample.apply / propagate_2d / square_and_downsample_2d) on inputs already resident in HBM.
value = transmission slices per second (514 per step: 1 + 512 + 1); the source, free-space legs
and detector are inside the timed region but not counted.

Also reported: the same workload end to end with host inputs (e2e), the unfused "plain" form on
the same GPU (our own FFT passes as separate kernels, and a cuFFT-based variant via torch.fft),
the dominant kernels' achieved HBM bandwidth vs the measured peak, the CPU oracle on the host
cores, and the FP64 relative L2 error of a truncated run.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
from __future__ import annotations

import argparse
import importlib
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "fused slice-steps/s at 4096^2 c64 (Talbot-Lau, 512-slice blob sample)"
UNIT = "slice-steps/s"
# fast-wave (CUDA + cuFFT) published 43.25 ms per layer at 4096^2 c64 (RTX 5070 Ti Laptop)
PUBLISHED_MS_PER_LAYER = 43.25


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per launch of each fused-pass kernel
# at 4096^2, from ncu captures of this workload's multislice loop (every launch is a whole-field
# pass, so a capture of a few slices gives the per-launch figure of the full run). --dram-csv
# replaces them with the figures of a capture given on the command line.
# row_pass_kernel: the dithered rows one per thread group (the default row pass; 208.5 MB with
# compensated twiddles too), col_pipe_kernel: the dithered columns one per thread group (215.1 MB
# compensated), col_x2_pipe_kernel: the split-pair columns (the default column pass).
NCU_DRAM_BYTES_4096 = {"row_pass_kernel": 208.5e6, "col_pipe_kernel": 215.2e6,
                       "row_x2_kernel": 208.7e6, "col_x2_pipe_kernel": 212.1e6}


def pass_kernels(mask: int, n: int) -> dict:
    """Kernel that runs the multislice row / column passes of an n x n plan under a schedule mask."""
    x2_rows = n in (256, 512, 1024, 2048, 4096, 8192)
    x2_cols = n in (256, 512, 1024, 2048, 4096)
    single = (384, 768, 1536, 3072, 6144)  # dithered rows / columns only one per thread group
    if (x2_rows or n in single + (16384,)) and not mask & 16:
        # 64: dithered, one row per group (the only dithered form at 16384 and 3*2^k)
        rows = "row_pass_kernel" if mask & 64 or not x2_rows else "row_x2_kernel"
    else:
        rows = "row_pipe_kernel" if mask & 1 else "row_pass_kernel"
    if (x2_cols or n in single) and not mask & 32:
        # 128: dithered, one column per group (the only dithered form at 3*2^k)
        cols = "col_pipe_kernel" if mask & 128 or not x2_cols else "col_x2_pipe_kernel"
    else:
        cols = "col_pipe_kernel" if mask & 2 and not mask & 8 else "col_pass_kernel"
    return {"row_pass": rows, "col_pass": cols}


def dram_bytes_from_csv(path: str) -> dict:
    """Mean dram__bytes_read.sum + dram__bytes_write.sum per launch, by kernel (template arguments
    dropped), from an ncu --csv log of those two metrics."""
    import csv
    from collections import defaultdict
    per = defaultdict(lambda: defaultdict(float))
    with open(path, newline="") as f:
        rows = [r for r in csv.reader(f) if len(r) > 10]
    hdr = rows[0]
    ki, mi, vi, ii = (hdr.index(k) for k in ("Kernel Name", "Metric Name", "Metric Value", "ID"))
    for r in rows[1:]:
        if r[mi] in ("dram__bytes_read.sum", "dram__bytes_write.sum"):
            name = r[ki].split("<")[0].split("(")[0].replace("void ", "").split("::")[-1]
            per[name][r[ii]] += float(r[vi].replace(",", ""))
    return {k: sum(v.values()) / len(v) for k, v in per.items()}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=4096, help="field size (default 4096)")
    ap.add_argument("--slices", type=int, default=512)
    ap.add_argument("--sweep-only", action="store_true",
                    help="run only the FFT + propagate sweep of a four-step plan and print its JSON")
    ap.add_argument("--sweep-n", type=int, default=32768, help="field size of the sweep (four-step plan)")
    ap.add_argument("--schedule", default="auto",
                    help="pass schedule of the field's plan: 'auto' (tuned at start-up) or a mask (1 pipelined "
                         "rows, 2 pipelined columns, 4 general row kernel, 8 split columns)")
    ap.add_argument("--no-extras", action="store_true", help="skip plain/e2e/cpu/accuracy legs")
    ap.add_argument("--dram-csv", default=None,
                    help="ncu --csv log of dram__bytes_read.sum and dram__bytes_write.sum for the pass kernels: "
                         "roofline.traffic from that capture instead of the built-in figures")
    ap.add_argument("--workload", default="talbot", choices=["talbot", "capsule"],
                    help="talbot: the 4096^2 Talbot-Lau benchmark (default); capsule: the 16384^2 "
                         "capsule field (--n 16384 --slices 1024), timed without the extra legs")
    return ap.parse_args()


# ------------------------------------------------------------------------------- helpers
class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for name, flag in zip(names, parts[3:7]):
                if flag.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak_hbm() -> tuple[float, str]:
    path = ROOT / "MEASURED_PEAKS.json"
    if path.exists():
        return float(json.loads(path.read_text())["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ------------------------------------------------------------------------------ our arm
class Pipeline:
    """The Talbot-Lau run through the public API on one device."""

    def __init__(self, rs, wl, device):
        import torch
        self.rs, self.w, self.dev = rs, wl, device
        self.p = wl.params
        n = self.p.nx
        self.u = rs.GpuVector.zeros(n * n, device)
        self.U = rs.GpuVector.zeros(n * n, device)
        self.det = None
        for el in wl.elements:  # upload grids once: inputs resident in HBM
            el.grid = torch.from_numpy(np.ascontiguousarray(el.grid).view(np.int32)).to(device)
            el.grid_is_signed = False

    def run(self, det_out=None):
        rs, p, w = self.rs, self.p, self.w
        u, U = self.u, self.U
        z = w.z_first
        if w.source_xyz is None:  # unit plane wave at the first element
            u.vec.fill_(1.0)
            valid = False
        else:
            rs.propagation.point_source_propagate_2d(u, U, z - w.source_xyz[2], w.source_xyz[0], w.source_xyz[1],
                                                     p, w.cutoff)
            valid = False
        for el in w.elements:
            if z < el.z_start:
                rs.propagate_2d(u, U, p.dx, p.get_dy(), p.wl, el.z_start - z, p.chunk_size, w.cutoff, p.nx, p.ny,
                                skip_fft=valid)
            el.apply(u, U, p, w.cutoff, 0, None)
            valid = True
            z = el.z_start + el.get_thickness()
        rs.propagate_2d(u, U, p.dx, p.get_dy(), p.wl, p.z_detector - z, p.chunk_size, w.cutoff, p.nx, p.ny,
                        skip_fft=True)
        return rs.propagation.square_and_downsample_2d_device(u, p, p.z_detector, out=det_out)


def l2_flush_buffer(torch, device):
    return torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=device)


def schedule_name(mask: int, n: int = 4096) -> str:
    """Readable form of a pass-schedule mask of an n x n plan (bits: 1 pipelined rows, 2 pipelined
    columns, 4 general row kernel, 8 split columns, 16 / 32 single-sequence compensated rows /
    columns instead of the dithered passes, for the sizes that have them, 64 / 128 the dithered
    rows / columns one per thread group, the only dithered form at 16384 (rows) and 3*2^k)."""
    single = n in (384, 768, 1536, 3072, 6144)
    x2_rows = n in (256, 512, 1024, 2048, 4096, 8192)
    x2_cols = n in (256, 512, 1024, 2048, 4096)
    if (x2_rows or single or n == 16384) and not mask & 16:
        rows = "rows:dithered-single" if mask & 64 or not x2_rows else "rows:split-pair"
    else:
        rows = "rows:pipelined" if mask & 1 else ("rows:per-block" if mask & 4 else "rows:per-block-voxel")
    if (x2_cols or single) and not mask & 32:
        cols = "cols:dithered-single" if mask & 128 or not x2_cols else "cols:split-pair"
    else:
        cols = "cols:pipelined" if mask & 2 else "cols:per-block"
        if mask & 8:
            cols = "cols:split-3-pass (last slice " + cols.split(":")[1] + ")"
    return f"{rows},{cols}"


def time_steps(torch, fn, steps, flush, stream):
    """Sum of per-step CUDA-event times; the L2 flush between steps is outside the events."""
    total = 0.0
    for _ in range(steps):
        flush.fill_(1.0)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        b.record(stream)
        b.synchronize()
        total += a.elapsed_time(b)
    return total


def plain_slice_rate(rs, torch, wl, device, slices: int, use_cufft: bool) -> float:
    """Unfused form on the same GPU: per slice T multiply, FFT2, H*mask, IFFT2 as separate
    launches (fast-wave's per-slice sequence, fast-wave/src/simulation.cpp:597-733)."""
    lib = rs._lib
    p = wl.params
    n = p.nx
    sample = wl.elements[1]
    plan = lib.plan_for(n, n, device)
    u = torch.ones(n * n, dtype=torch.complex64, device=device)
    U = torch.empty_like(u)
    geom = lib.VoxelGeom(int(sample.grid.shape[0]), int(sample.grid.shape[1]), int(sample.grid.shape[2]),
                         sample.pixel_size_x, sample.pixel_size_y or sample.pixel_size_x, sample.pixel_size_z, 0.0, 0.0)
    _, db = sample._device_inputs(device)
    st = lib.stream_handle()
    L = lib.lib()

    def one(k):
        lib.check(L.rs_apply_transmission_voxel(plan.handle, lib.ptr(u), lib.ptr(sample.grid), 0, lib.ptr(db),
                                                len(sample.db_list), geom, p.dx, p.dx, p.wl, k, 1.0, st), "T")
        if use_cufft:
            torch.fft.fft2(u.view(n, n), out=U.view(n, n))
            lib.check(L.rs_apply_transfer(plan.handle, lib.ptr(U), p.dx, p.dx, p.wl, sample.pixel_size_z,
                                          wl.cutoff, st), "H")
            torch.fft.ifft2(U.view(n, n), out=u.view(n, n))
        else:
            lib.check(L.rs_fft2(plan.handle, lib.ptr(u), lib.ptr(U), st), "fft2")
            lib.check(L.rs_apply_transfer(plan.handle, lib.ptr(U), p.dx, p.dx, p.wl, sample.pixel_size_z,
                                          wl.cutoff, st), "H")
            lib.check(L.rs_ifft2(plan.handle, lib.ptr(U), lib.ptr(u), st), "ifft2")

    for k in range(3):
        one(k)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for k in range(slices):
        one(k % int(sample.grid.shape[0]))
    b.record()
    b.synchronize()
    return slices / (a.elapsed_time(b) / 1e3)


def cpu_baseline(n: int, samples: int = 2) -> dict:
    """The oracle's complex64 slice-step (big-wave's NumpyVector path restated) on the host, at the
    benchmark's field size, scipy.fft with its default single worker as big-wave calls it."""
    from oracle import bigwave_oracle as orc
    rs_wl = importlib.import_module("3d_ravesim_gb300.workloads")
    w = rs_wl.talbot_lau(n=n, slices=8, blobs=20)
    s = w.elements[1]
    p = w.params
    grid = np.asarray(s.grid)
    u = np.ones((n, n), np.complex64)
    t0 = time.perf_counter()
    for k in range(samples):
        t = orc.sample_transmission(grid[k], s.db_list, n, n, p.dx, p.dx, s.pixel_size_x, s.pixel_size_y,
                                    s.pixel_size_z, p.wl)
        u = (u * t).astype(np.complex64)
        u, _ = orc.propagate_2d(u, p.dx, p.dx, p.wl, s.pixel_size_z, w.cutoff)
    dt = time.perf_counter() - t0
    return {"value": samples / dt, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"{samples} Sample slice-steps at {n}^2 complex64 (oracle restatement of big-wave's "
                      f"NumpyVector path, scipy.fft default 1 worker), {dt:.1f} s"}


def accuracy_check(rs, torch, device, n: int, slices: int = 4, workload: str = "talbot") -> dict:
    """Relative L2 of field and detector intensity vs the FP64 oracle on the benchmark geometry at
    n^2 with `slices` sample slices (a full 512-slice FP64 run at 4096^2 takes hours on the CPU,
    at 1024^2 about half a minute); workload "shell" is the plane-wave shell case (1024^2, 128 slices)."""
    from scipy import fft as spfft

    from oracle import bigwave_oracle as orc
    wlmod = importlib.import_module("3d_ravesim_gb300.workloads")
    if workload == "shell":
        w = wlmod.shell_plane_wave(n=n, slices=slices)
    else:
        w = wlmod.talbot_lau(n=n, slices=slices)
    pipe = Pipeline(rs, w, device)
    det = pipe.run()
    torch.cuda.synchronize()
    gpu_u = pipe.u.to_numpy().reshape(n, n)
    gpu_det = det.cpu().numpy()
    p = w.params
    with spfft.set_workers(os.cpu_count() or 1):
        z = w.z_first
        if w.source_xyz is None:
            u, U = np.ones((n, n), np.complex128), None
        else:
            u, U = orc.point_source_2d(n, n, p.dx, p.dx, z, 0.0, 0.0, p.wl, w.cutoff)
        valid = False
        for el in w.elements:
            if z < el.z_start:
                u, U = orc.propagate_2d(u, p.dx, p.dx, p.wl, el.z_start - z, w.cutoff, U=U if valid else None,
                                        skip_fft=valid)
            grid = np.asarray(el.grid.cpu().numpy() if hasattr(el.grid, "cpu") else el.grid).view(np.uint32)
            u, U = orc.sample_apply_2d(u, grid, el.db_list, p.dx, p.dx, p.wl, w.cutoff, el.pixel_size_x,
                                       el.pixel_size_y or el.pixel_size_x, el.pixel_size_z)
            valid = True
            z = el.z_start + el.get_thickness()
        u, U = orc.propagate_2d(u, p.dx, p.dx, p.wl, p.z_detector - z, w.cutoff, U=U, skip_fft=True)
    ref_det = orc.detector_area_v1(u, p.dx, p.dx, p.detector_pixel_size_x, p.detector_pixel_size_y,
                                   gpu_det.shape[1], gpu_det.shape[0], p.z_detector)
    name = "shell plane wave" if workload == "shell" else "Talbot-Lau"
    return {"case": f"{name} {n}^2 with {slices} sample slices vs FP64 oracle",
            "field_rel_l2": orc.relative_l2(gpu_u, u),
            "intensity_rel_l2": orc.relative_l2(np.abs(gpu_u) ** 2, np.abs(u) ** 2),
            "detector_rel_l2": orc.relative_l2(gpu_det, ref_det)}


def accuracy_plasma(rs, torch, device, n: int = 512, slices: int = 256) -> dict:
    """The differentiable-plasma forward (Gaussian CH plasma, 8 keV, 256 x 2 um slices, the same 1.02 mm field)
    at 512^2 (2 um pixels) through PlasmaSample.apply and the final leg, against the FP64
    oracle's PlasmaSample restatement (big-wave/plasma_sample.py:126-233)."""
    from scipy import fft as spfft

    from oracle import bigwave_oracle as orc
    wlmod = importlib.import_module("3d_ravesim_gb300.workloads")
    psmod = importlib.import_module("3d_ravesim_gb300.plasma_sample")
    w = wlmod.gaussian_plasma(n=n, slices=slices, dx=2e-6)
    s, p = w.elements[0], w.params
    u, U = rs.GpuVector(torch.ones(n * n, dtype=torch.complex64, device=device)), rs.GpuVector.zeros(n * n, device)
    s.apply(u, U, p, w.cutoff, 0, None)
    z = s.z_start + s.get_thickness()
    rs.propagate_2d(u, U, p.dx, p.dy, p.wl, p.z_detector - z, p.chunk_size, w.cutoff, n, n, skip_fft=True)
    gpu_det = rs.square_and_downsample_2d(u, p, p.z_detector)
    gpu_u = u.to_numpy().reshape(n, n)
    energy = rs.convert_energy_wavelength(p.wl)
    with spfft.set_workers(os.cpu_count() or 1):
        ru, rU = orc.plasma_apply_2d(np.ones((n, n), np.complex128), s.ne_grid, s.ni_grid, s.te_grid, s.zstar_grid,
                                     s.scattering_factors, energy, psmod.codata_constants(), p.dx, p.dx, p.wl,
                                     w.cutoff, s.pixel_size_x, s.pixel_size_y, s.pixel_size_z)
        ru, _ = orc.propagate_2d(ru, p.dx, p.dx, p.wl, p.z_detector - z, w.cutoff, U=rU, skip_fft=True)
    ref_det = orc.detector_area_v1(ru, p.dx, p.dx, p.detector_pixel_size_x, p.detector_pixel_size_y,
                                   gpu_det.shape[1], gpu_det.shape[0], p.z_detector)
    return {"case": f"Gaussian plasma (2048^2-case geometry) {n}^2 with {slices} slices vs FP64 oracle",
            "field_rel_l2": orc.relative_l2(gpu_u, ru),
            "intensity_rel_l2": orc.relative_l2(np.abs(gpu_u) ** 2, np.abs(ru) ** 2),
            "detector_rel_l2": orc.relative_l2(gpu_det, ref_det)}


def accuracy_multisim_item(rs, torch, device) -> dict:
    """One item of the multisim batch (the first 1024^2 one: point source, 64-slice shell, 10 m to
    the 2048^2 detector) through the batch runner, against the FP64 oracle chain."""
    from scipy import fft as spfft

    from oracle import bigwave_oracle as orc
    ms = importlib.import_module("3d_ravesim_gb300.multisim")
    b = ms.shell_batch()
    item = next(it for it in b.items if it.n == 1024)
    runner = ms.BatchRunner(b, device, streams=1)
    img = runner.run([item]).cpu().numpy()
    gpu_u = runner._buffers(0, item.n)[0].to_numpy().reshape(item.n, item.n)
    p = ms.item_params(b, item)
    cutoff = b.cutoff_fraction / p.dx
    smp = b.sample
    db = ms._scaled_db(b, item.energy)
    with spfft.set_workers(os.cpu_count() or 1):
        u, U = orc.point_source_2d(item.n, item.n, p.dx, p.dx, b.z_sample, item.x, item.y, p.wl, cutoff)
        u, U = orc.sample_apply_2d(u, np.asarray(smp.grid), db, p.dx, p.dx, p.wl, cutoff, smp.pixel_size_x,
                                   smp.pixel_size_y, smp.pixel_size_z)
        z = smp.z_start + smp.get_thickness()
        u, U = orc.propagate_2d(u, p.dx, p.dx, p.wl, p.z_detector - z, cutoff, U=U, skip_fft=True)
    ref = orc.detector_area_v1(u, p.dx, p.dx, p.detector_pixel_size_x, p.detector_pixel_size_y,
                               b.detector_pixels, b.detector_pixels, p.z_detector)
    return {"case": f"multisim item 1024^2, {smp.grid.shape[0]} slices, {item.energy:.0f} eV "
                    "vs FP64 oracle",
            "field_rel_l2": orc.relative_l2(gpu_u, u),
            "intensity_rel_l2": orc.relative_l2(np.abs(gpu_u) ** 2, np.abs(u) ** 2),
            "detector_rel_l2": orc.relative_l2(img, ref)}


def adjoint_cost(rs, torch, device, n: int = 2048, slices: int = 256, checkpoint_every=None) -> dict:
    """Gradient cost of the differentiable plasma workload (2048^2, 8 keV, 256 x 2 um slices of a
    Gaussian plasma, n0 = 1e21 cm^-3, L = 150 um, T_e = 500 eV): one forward pass against one
    forward + adjoint (loss L2, gradients to every voxel's delta/beta and to n0, L, T_e)."""
    adj = importlib.import_module("3d_ravesim_gb300.adjoint")
    energy, dx, pz, pitch = 8000.0, 0.5e-6, 2e-6, 2e-6
    wl = rs.convert_energy_wavelength(energy)
    glen = int(math.ceil(n * dx / pitch)) + 4
    glen += glen % 2
    geom = adj.VolumeGeometry(z_start=0.1, pixel_size_x=pitch, pixel_size_y=pitch, pixel_size_z=pz)
    p = rs.SimParams(N=n * n, nx=n, ny=n, dx=dx, dy=dx, z_detector=0.1 + slices * pz + 0.2, detector_size=n * dx,
                     detector_pixel_size_x=dx, detector_pixel_size_y=dx, wl=wl, chunk_size=n)
    u0 = torch.ones(n * n, dtype=torch.complex64, device=device)
    model = adj.MultisliceModel(p, geom, 0.45 / dx, u0, checkpoint_every=checkpoint_every)
    th = [torch.tensor(v, dtype=torch.float64, device=device, requires_grad=True) for v in (1e21, 150e-6, 500.0)]

    def fwd(params=th):
        db = adj.gaussian_plasma_db(params[0], params[1], params[2], (slices, glen, glen), (pz, pitch, pitch), energy)
        return adj.multislice_intensity(db, model)
    # target: the intensity of slightly different parameters with Poisson noise at 1e4 photons/pixel
    with torch.no_grad():
        truth = fwd([torch.tensor(v, dtype=torch.float64, device=device) for v in (1.05e21, 145e-6, 550.0)])
        scale = 1e4 / truth.mean()
        gen = torch.Generator(device=device).manual_seed(0)
        target = torch.poisson(truth * scale, generator=gen) / scale

    def grad():
        for t in th:
            t.grad = None
        ((fwd() - target) ** 2).sum().backward()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    with torch.no_grad():
        fwd()
    grad()
    torch.cuda.synchronize()
    ev[0].record()
    with torch.no_grad():
        fwd()
    ev[1].record()
    grad()
    ev[2].record()
    ev[2].synchronize()
    f_ms, g_ms = ev[0].elapsed_time(ev[1]), ev[1].elapsed_time(ev[2])
    return {"case": f"Gaussian plasma {n}^2, {slices} slices, grid {[slices, glen, glen]}; L2 loss against a "
            "Poisson-noisy (1e4 photons/pixel) image of n0 = 1.05e21, L = 145 um, T_e = 550 eV",
            "backward": model.last_backward, "forward_ms": round(f_ms, 2),
            "forward_plus_gradient_ms": round(g_ms, 2), "ratio": round(g_ms / f_ms, 2),
            "checkpoint_every": model.every if checkpoint_every != 0 else "every field kept",
            "grad_n0_L_Te": [float(t.grad) for t in th]}


def plasma_forward_rate(rs, torch, device, n: int = 2048, slices: int = 256, steps: int = 3) -> dict:
    """The differentiable-plasma forward through PlasmaSample.apply: 2048^2, 8 keV, 256 x 2 um slices of a Gaussian
    plasma (n_e, n_i, T_e, Z* grids of 516^2 float32 per slice, delta/beta evaluated in the row pass)."""
    wlmod = importlib.import_module("3d_ravesim_gb300.workloads")
    w = wlmod.gaussian_plasma(n=n, slices=slices)
    s = w.elements[0]
    p = w.params
    u, U = rs.GpuVector.zeros(n * n, device), rs.GpuVector.zeros(n * n, device)

    def run():
        u.vec.fill_(1.0)
        s.apply(u, U, p, w.cutoff, 0, None)
    run()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(steps):
        run()
    b.record()
    b.synchronize()
    ms = a.elapsed_time(b) / steps
    return {"case": f"Gaussian plasma {n}^2, {slices} slices, grids {w.info['grid']} float32 x4",
            "ms_per_run": round(ms, 2), "slice_steps_per_s": round(slices / (ms / 1e3), 1)}


def multisim_cost(rs, torch, device, items: int = 128) -> dict:
    """Batched multisim (64 jittered sources x 16 Kramers energies, grid sizes from {1024, 1536,
    2048, 3072}^2, 64-slice shell, 2048^2 area_v1 detector summed incoherently): the first `items`
    items through the fused multi-stream runner (eager and as one CUDA graph) and through the
    loops of the plain unfused form (own FFTs, cuFFT); then the full 1024-item batch through the
    fused runner and the plain loop."""
    ms = importlib.import_module("3d_ravesim_gb300.multisim")
    b = ms.shell_batch(max_items=items)
    fused = ms.BatchRunner(b, device, streams=2)  # 2 streams measured faster than 4 or 8 (0.96 vs 1.03 vs 1.05 s)
    plain = ms.BatchRunner(b, device, streams=1)
    plain_cufft = ms.BatchRunner(b, device, streams=1)
    fused.run(b.items[:4])
    plain.run(b.items[:1], plain=True)
    plain_cufft.run(b.items[:4], plain="cufft")  # cuFFT plans of every size
    fused.zero()
    plain.zero()
    plain_cufft.zero()
    out = {}
    for name, runner, kw in (("fused", fused, {}), ("plain_loop", plain, {"plain": True}),
                             ("plain_loop_cufft", plain_cufft, {"plain": "cufft"})):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        runner.run(**kw)
        torch.cuda.synchronize()
        out[name + "_s"] = round(time.perf_counter() - t0, 3)
    # the same batch captured as one CUDA graph (items on 2 streams, the detector sum inside),
    # launched once per batch
    graphed = ms.BatchRunner(b, device, streams=2)
    t0 = time.perf_counter()
    graphed.capture()
    capture_s = time.perf_counter() - t0
    graphed.replay()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    graphed.replay()
    out["fused_graph_s"] = round(time.perf_counter() - t0, 3)
    del graphed
    # the full batch (1024 items) through the fused runner (per item, and with the items of one
    # size and energy stacked into one field stack per launch) and the plain loop
    full = ms.shell_batch()
    per_item = ms.BatchRunner(full, device, streams=2)
    per_item.run(full.items[:4])
    stacked = ms.BatchRunner(full, device, streams=2)
    stacked.run(full.items[:40], stacked=True)
    plain_full = ms.BatchRunner(full, device, streams=1)
    plain_full.run(full.items[:1], plain=True)
    full_out = {}
    for name, runner, kw in (("fused", per_item, {}), ("fused_stacked", stacked, {"stacked": True}),
                             ("plain_loop", plain_full, {"plain": True})):
        runner.zero()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        runner.run(**kw)
        torch.cuda.synchronize()
        full_out[name + "_s"] = round(time.perf_counter() - t0, 3)
    n_full = len(full.items)
    del per_item, stacked, plain_full
    torch.cuda.empty_cache()
    # per grid size: 64 items of one size (4 x 4 jittered sources x 4 energies of the same spectrum,
    # so the stacks hold 16 items as in the full batch), stacked against the plain loop, to show
    # where the ratio comes from
    by_size = {}
    for n in b.info["sizes"]:
        one = ms.shell_batch(n_sources_side=4, n_energies=4, sizes=(n,))
        t = {}
        for name, streams, kw in (("stacked", 2, {"stacked": True}), ("plain", 1, {"plain": True})):
            r = ms.BatchRunner(one, device, streams=streams)
            r.run(one.items[:2], **({"plain": True} if name == "plain" else {}))
            if name == "stacked":
                r.run(one.items[:16], stacked=True)
            r.zero()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            r.run(**kw)
            torch.cuda.synchronize()
            t[name] = time.perf_counter() - t0
            del r
        torch.cuda.empty_cache()
        by_size[str(n)] = {"stacked_items_per_s": round(64 / t["stacked"], 2),
                           "plain_loop_items_per_s": round(64 / t["plain"], 2),
                           "speedup": round(t["plain"] / t["stacked"], 2)}
    slices = b.sample.grid.shape[0]
    res = {"case": f"{items} of 1024 items, sizes {b.info['sizes']}, {slices} slices each",
           "fused_items_per_s": round(items / out["fused_s"], 2),
           "fused_graph_items_per_s": round(items / out["fused_graph_s"], 2),
           "plain_loop_items_per_s": round(items / out["plain_loop_s"], 2),
           "plain_loop_cufft_items_per_s": round(items / out["plain_loop_cufft_s"], 2),
           "speedup": round(out["plain_loop_s"] / min(out["fused_s"], out["fused_graph_s"]), 2),
           "speedup_vs_cufft_loop": round(out["plain_loop_cufft_s"] / min(out["fused_s"], out["fused_graph_s"]), 2),
           "graph_capture_s": round(capture_s, 2), **out,
           "full_batch": {"items": n_full,
                          "fused_items_per_s": round(n_full / full_out["fused_s"], 2),
                          "fused_stacked_items_per_s": round(n_full / full_out["fused_stacked_s"], 2),
                          "plain_loop_items_per_s": round(n_full / full_out["plain_loop_s"], 2),
                          "speedup": round(full_out["plain_loop_s"] /
                                           min(full_out["fused_s"], full_out["fused_stacked_s"]), 2),
                          **full_out},
           "by_size_64_items": by_size}
    return res


def sweep_32768(rs, torch, device, reps: int = 5, n: int = 32768) -> dict:
    """One FFT + propagate sweep at 32768^2 complex64 (8 GiB per field, the large-field case's
    roofline check): rs_propagate on a four-step plan, 30 keV, 50 nm pixels, 0.5 um step, the
    circular cutoff active. The field (8 GiB) is far larger than L2, so no flush is needed.
    A smaller n (4096..16384) runs the same passes on a four-step plan of that size."""
    lib = rs._lib
    plan = lib.plan_for(n, n, device) if n > 16384 else lib.Plan(n, n, device, flags=lib.RS_PLAN_FOURSTEP)
    g = torch.Generator(device="cpu").manual_seed(0)
    u = torch.polar(torch.ones(n * n // 64), torch.rand(n * n // 64, generator=g) * 6.283).to(torch.complex64)
    u = u.to(device).repeat(64)
    U = torch.empty_like(u)
    dx, wl = 50e-9, rs.convert_energy_wavelength(30000.0)
    f = 0.45 / dx
    st = lib.stream_handle()
    L = lib.lib()

    def step(skip):
        lib.check(L.rs_propagate(plan.handle, lib.ptr(u), lib.ptr(U), dx, dx, wl, 0.5e-6, f, skip, st), "propagate")

    step(0)
    step(1)
    torch.cuda.synchronize()
    out = {}
    for skip, name in ((0, "fft_propagate"), (1, "propagate_skip_fft")):
        ts = []
        for _ in range(reps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            step(skip)
            b.record()
            b.synchronize()
            ts.append(a.elapsed_time(b))
        ms = float(np.median(ts))
        passes = 7 if skip == 0 else 4
        out[name] = {"ms": round(ms, 3), "passes": passes,
                     "pass_traffic_GB_s": round(passes * 16 * n * n / (ms * 1e-3) / 1e9, 1),
                     "slice_step_GB_s": round(32 * n * n / (ms * 1e-3) / 1e9, 1)}
    peak, kind = measured_peak_hbm()
    for v in out.values():
        v["pass_traffic_frac"] = round(v["pass_traffic_GB_s"] / peak, 3)
        v["slice_step_frac"] = round(v["slice_step_GB_s"] / peak, 3)
    del u, U
    torch.cuda.empty_cache()
    return {"case": f"{n}^2 c64 four-step plan (length-{n // 256} and length-256 transforms per axis), "
                    "30 keV, 50 nm pixels, dz 0.5 um, cutoff 0.45/dx",
            "peak_GB_s": peak, "peak_kind": kind,
            "slice_step_bytes": "32 B per pixel (2 field round trips, the single-pass minimum)",
            "pass_bytes": "16 B per pixel per pass", **out}


def run_ours(args):
    import torch
    import torch.distributed as dist

    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local = int(os.environ.get("LOCAL_RANK", 0))
    if world > 1:
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    rs = importlib.import_module("3d_ravesim_gb300")
    rs.build()
    if args.sweep_only:
        if rank == 0:
            print(json.dumps({"sweep": sweep_32768(rs, torch, device, n=args.sweep_n)}))
        return
    wlmod = importlib.import_module("3d_ravesim_gb300.workloads")
    if args.workload == "capsule":
        w = wlmod.capsule_large(n=args.n, slices=args.slices)
        args.no_extras = True
    else:
        w = wlmod.talbot_lau(n=args.n, slices=args.slices)
    pipe = Pipeline(rs, w, device)
    # pass schedule of the field's plan: every distinct schedule timed on a few seeded voxel
    # slices of this size, the fastest kept (nothing is read from or written to the cache file)
    autotune = importlib.import_module("3d_ravesim_gb300.autotune")
    if args.schedule == "auto":
        tuned = autotune.tune_multislice(w.params.nx, w.params.ny, device, store=False)
    else:
        tuned = autotune.Choice(int(args.schedule), {}, 0, {})
    rs._lib.plan_for(w.params.nx, w.params.ny, device).set_schedule(tuned.mask)
    stream = torch.cuda.current_stream(device)
    flush = l2_flush_buffer(torch, device)
    det = torch.zeros((int(w.params.get_detector_size_y() // w.params.detector_pixel_size_y),
                       int(w.params.get_detector_size_x() // w.params.detector_pixel_size_x)),
                      dtype=torch.float64, device=device)
    for _ in range(args.warmup):
        pipe.run(det)
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    launches0 = rs._lib.launch_count()
    barrier()
    with ClockSampler(local) as clocks:
        total_ms = time_steps(torch, lambda: pipe.run(det), args.steps, flush, stream)
    barrier()
    launches = rs._lib.launch_count() - launches0
    t = torch.tensor([total_ms], dtype=torch.float64, device=device)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    total_ms = float(t.item())
    slices_per_step = w.slice_count
    value = world * slices_per_step * args.steps / (total_ms / 1e3)

    # dominant kernels: per-pass CUDA-event timing of one run (same stream)
    plan = rs._lib.plan_for(w.params.nx, w.params.ny, device)
    L = rs._lib.lib()
    rs._lib.check(L.rs_plan_profile(plan.handle, 1), "profile")
    flush.fill_(1.0)
    pipe.run(det)
    import ctypes
    row_ms, col_ms = ctypes.c_double(), ctypes.c_double()
    nr, nc = ctypes.c_int(), ctypes.c_int()
    rs._lib.check(L.rs_plan_profile_read(plan.handle, ctypes.byref(row_ms), ctypes.byref(col_ms), ctypes.byref(nr),
                                         ctypes.byref(nc)), "profile_read")
    rs._lib.check(L.rs_plan_profile(plan.handle, 0), "profile")
    n = w.params.nx
    field_bytes = 8 * n * n
    peak, peak_kind = measured_peak_hbm()
    row_avg = row_ms.value / max(nr.value, 1)
    col_avg = col_ms.value / max(nc.value, 1)
    # algorithmic bytes per launch: read + write of the field (16 B/pixel); the row pass also reads
    # the voxel slice it gathers (4 B per voxel of the (y_len, x_len) plane)
    vox = w.info["voxel_grid"]
    row_bytes = 2 * field_bytes + 4 * vox[1] * vox[2]
    col_bytes = 2 * field_bytes
    row_gbs = row_bytes / (row_avg * 1e-3) / 1e9
    col_gbs = col_bytes / (col_avg * 1e-3) / 1e9
    dom = "col_pass" if col_ms.value >= row_ms.value else "row_pass"
    kernels = pass_kernels(tuned.mask, n)
    if args.dram_csv:
        traffic = dram_bytes_from_csv(args.dram_csv)
        traffic_source = "ncu dram__bytes_read.sum + dram__bytes_write.sum per launch, capture given by --dram-csv"
    else:
        traffic = NCU_DRAM_BYTES_4096 if n == 4096 else {}
        traffic_source = ("ncu dram__bytes_read.sum + dram__bytes_write.sum per launch of this kernel, one "
                          "capture of this workload's multislice loop at 4096^2" if n == 4096 else None)
    achieved = col_gbs if dom == "col_pass" else row_gbs
    roofline = {"bound": "hbm", "kernel": f"{dom} (fused {'column FFT*H*IFFT' if dom == 'col_pass' else 'row IFFT*T*FFT'})",
                "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                "peak_kind": peak_kind,
                "traffic": traffic.get(kernels[dom]),
                "traffic_source": traffic_source,
                "kernels": kernels,
                "row_pass": {"avg_us": round(row_avg * 1e3, 2), "GB_s": round(row_gbs, 1), "launches": nr.value,
                             "algorithmic_bytes": row_bytes},
                "col_pass": {"avg_us": round(col_avg * 1e3, 2), "GB_s": round(col_gbs, 1), "launches": nc.value,
                             "algorithmic_bytes": col_bytes},
                "slice_step_frac": round((2 * field_bytes * 2) / ((row_avg + col_avg) * 1e-3) / 1e9 / peak, 4)}

    talbot = args.workload == "talbot"
    line = {"metric": METRIC if talbot else f"fused slice-steps/s at {n}^2 c64 (capsule, {args.slices} slices)",
            "value": round(value, 2), "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": round(value / (1e3 / PUBLISHED_MS_PER_LAYER), 2) if talbot else None,
            "dtype": "c64 (fp32 complex)",
            "data": "synthetic (seeded Talbot-Lau: point source, gratings, 200-blob voxel sample)" if talbot else
                    "synthetic (point source 1 m upstream, seeded spherical-harmonic-perturbed CH capsule shell)",
            "config": {**workload_config(w, n, slices_per_step, args.slices, vox, talbot),
                       "l2": "256 MiB buffer written between timed steps (flush outside the events)",
                       "parallelism": f"replicas x{world} (one field per GPU)"},
            "roofline": roofline, "gpu_launches": launches, "clocks": clocks.summary(),
            "schedule": {"mask": tuned.mask, "passes": schedule_name(tuned.mask, n),
                         "tuned_ms_per_schedule": {schedule_name(m, n): round(t, 3)
                                                   for m, t in sorted(tuned.timings_ms.items())},
                         "tuned_on": f"{tuned.slices} seeded voxel slices at {n}^2" if tuned.slices else "given",
                         "max_rel_diff_between_schedules": max(tuned.rel_diff.values(), default=None)}}

    if rank == 0 and not args.no_extras:
        # e2e: every step copies its voxel grids in from pinned host memory and the detector image
        # out. The grids are double-buffered: each step starts the copy of the next step's grids
        # on a copy stream and then computes on the buffer copied during the previous step, so
        # each timed step holds one full upload, one run and one download.
        host_grids = [torch.from_numpy(np.ascontiguousarray(el.grid.cpu().numpy())).pin_memory() for el in w.elements]
        host_det = torch.empty(det.shape, dtype=torch.float64).pin_memory()
        h2d = sum(g.numel() * 4 for g in host_grids)
        d2h = host_det.numel() * 8
        copy_stream = torch.cuda.Stream(device)
        bufs = [[el.grid for el in w.elements], [torch.empty_like(el.grid) for el in w.elements]]
        ready = [torch.cuda.Event(), torch.cuda.Event()]
        used = [torch.cuda.Event(), torch.cuda.Event()]
        state = {"k": 0}

        def upload(k):
            b = k % 2
            with torch.cuda.stream(copy_stream):
                copy_stream.wait_event(used[b])  # the step that last read buffer b has finished
                for dst, hg in zip(bufs[b], host_grids):
                    dst.copy_(hg, non_blocking=True)
                ready[b].record(copy_stream)

        def e2e_step():
            k = state["k"]
            b = k % 2
            stream.wait_event(ready[b])
            for el, g in zip(w.elements, bufs[b]):
                el.grid = g
            upload(k + 1)
            pipe.run(det)
            used[b].record(stream)
            host_det.copy_(det, non_blocking=True)
            state["k"] = k + 1
        for b in (0, 1):
            used[b].record(stream)
        upload(0)
        e2e_step()
        e2e_step()  # both buffers' grids validated once (Sample caches the id check per grid object)
        torch.cuda.synchronize()
        e2e_ms = time_steps(torch, e2e_step, args.steps, flush, stream)
        line["e2e"] = {"value": round(slices_per_step * args.steps / (e2e_ms / 1e3), 2), "unit": UNIT,
                       "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                       "path": "Sample.apply/propagate_2d/square_and_downsample_2d (C ABI); pinned host grids "
                               "copied in on a second stream, double-buffered, overlapping the previous step"}
        # plain (unfused) comparators on the same GPU
        plain = plain_slice_rate(rs, torch, w, device, 64, use_cufft=False)
        cufft = plain_slice_rate(rs, torch, w, device, 64, use_cufft=True)
        fused_rate = slices_per_step / (row_ms.value + col_ms.value) * 1e3 if (nr.value and nc.value) else None
        line["plain"] = {"own_fft_unfused": round(plain, 1), "cufft_unfused": round(cufft, 1),
                         "fused_sample_slices": round(fused_rate, 1) if fused_rate else None, "unit": UNIT,
                         "note": "unfused = T kernel, FFT2, H*mask, IFFT2 as separate launches per slice"}
        line["plasma_forward"] = plasma_forward_rate(rs, torch, device)
        line["adjoint"] = [adjoint_cost(rs, torch, device), adjoint_cost(rs, torch, device, checkpoint_every=0)]
        line["multisim"] = multisim_cost(rs, torch, device)
        line["sweep_32768"] = sweep_32768(rs, torch, device)
        line["cpu_baseline"] = cpu_baseline(n)
        # the full slice count at 1024^2 (errors that repeat every slice add up over 514 of them),
        # and the benchmark size itself truncated to 4 sample slices
        line["accuracy"] = [accuracy_check(rs, torch, device, 1024, slices=args.slices),
                            accuracy_check(rs, torch, device, min(n, 4096)),
                            accuracy_check(rs, torch, device, 1024, slices=128, workload="shell"),
                            accuracy_multisim_item(rs, torch, device),
                            accuracy_plasma(rs, torch, device)]
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def workload_config(w, n: int, slices_per_step: int, sample_slices: int, vox, talbot: bool = True) -> dict:
    """The workload-defining part of a line's config, the same for both arms."""
    return {"workload": f"{'talbot_lau' if talbot else 'capsule'}_{n}x{n}_c64", "nx": n, "ny": n,
            "slices_per_step": slices_per_step, "sample_slices": sample_slices, "voxel_grid": vox,
            "energy_ev": w.info["energy_ev"]}


# ----------------------------------------------------------------------- reference arm
def run_reference(args):
    """The reference's CPU algorithm (the oracle restatement of big-wave's NumpyVector path) on the
    host cores, scipy.fft with all host threads, on the same Talbot-Lau workload as the GPU arm;
    one step = one Sample slice-step of it (a bounded sample of the run's 514)."""
    rank = int(os.environ.get("RANK", 0))
    if rank != 0:
        return
    from scipy import fft as spfft

    from oracle import bigwave_oracle as orc
    wlmod = importlib.import_module("3d_ravesim_gb300.workloads")
    n = args.n
    w = wlmod.talbot_lau(n=n, slices=args.slices)
    s = w.elements[1]
    p = w.params
    grid = np.asarray(s.grid)
    cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)
    u = np.ones((n, n), np.complex64)

    def step(k):
        nonlocal u
        t = orc.sample_transmission(grid[k % grid.shape[0]], s.db_list, n, n, p.dx, p.dx, s.pixel_size_x,
                                    s.pixel_size_y, s.pixel_size_z, p.wl)
        u = (u * t).astype(np.complex64)
        u, _ = orc.propagate_2d(u, p.dx, p.dx, p.wl, s.pixel_size_z, w.cutoff)

    with spfft.set_workers(cores):
        for k in range(args.warmup):
            step(k)
        t0 = time.perf_counter()
        for k in range(args.steps):
            step(k)
        dt = time.perf_counter() - t0
    value = args.steps / dt
    line = {"impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dt / args.steps * 1e3, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c64",
            "data": "synthetic (seeded Talbot-Lau: point source, gratings, 200-blob voxel sample)",
            "config": {**workload_config(w, n, args.slices + 2, args.slices, w.info["voxel_grid"]),
                       "parallelism": f"host cores x{cores}"},
            "cpu_baseline": {"value": round(value, 4), "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{args.steps} Sample slice-steps (sample slices 0..{args.steps - 1}, after "
                                       f"{args.warmup} warm-up steps) of the {n}^2 c64 run, scipy.fft "
                                       f"workers={cores}"},
            "e2e": {"value": round(value, 4), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    else:
        run_ours(a)
