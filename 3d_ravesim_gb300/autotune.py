"""Pass-schedule autotuner.

Every fast size has several schedules of the two fused passes (`Plan.schedules()`, bits of
`Plan.set_schedule`): the column passes as one block per strip of columns or as the persistent
TMA-box pipeline; the row passes as one block per row group (with or without the voxel-only
specialisation) or as the persistent bulk-copy pipeline; for 4096..16384-point columns, the
column pass may also run as three shorter four-step passes. All compute the same transform; which
is fastest depends on the size (threads per transform, shared memory per strip,
resident blocks). `tune_multislice` times each schedule on a seeded multislice run of the
size (CUDA events on the launching stream, median of `reps`), measures each schedule's field
against the first schedule's (a schedule further than FP32 rounding from it is never picked),
and records the fastest in a JSON cache keyed by the device and the size. `Plan`s created afterwards (`_lib.plan_for`) take the cached schedule;
with RS_AUTOTUNE=1 in the environment a size that has no entry is tuned when its first plan is
created. The cache file is RS_SCHEDULE_CACHE, else ~/.cache/rs_fresnel/schedules.json.

`tune_batch_streams` picks the number of CUDA streams of the batched multisim the same way.
"""
from __future__ import annotations

import json
import os
import statistics
import tempfile
import threading
from dataclasses import dataclass
from pathlib import Path
from typing import Callable

import torch

CACHE_VERSION = 1
MAX_SCHEDULE_DIFF = 1e-6
SCHED_COMPENSATED = 48  # RS_SCHED_COMP_ROWS | RS_SCHED_COMP_COLS of include/rs_fresnel.h
_lock = threading.Lock()
_tuning = threading.local()


def cache_path() -> Path:
    env = os.environ.get("RS_SCHEDULE_CACHE")
    if env:
        return Path(env)
    return Path.home() / ".cache" / "rs_fresnel" / "schedules.json"


def device_key(device: torch.device) -> str:
    props = torch.cuda.get_device_properties(device)
    return f"{props.name}|sm{props.major}{props.minor}|{props.multi_processor_count}sm"


def entry_key(dev_key: str, nx: int, ny: int, workload: str) -> str:
    return f"{dev_key}|{int(nx)}x{int(ny)}|{workload}"


def load_cache(path: Path | None = None) -> dict:
    path = cache_path() if path is None else Path(path)
    try:
        data = json.loads(path.read_text(encoding="utf-8"))
    except (OSError, ValueError):
        return {}
    if not isinstance(data, dict) or data.get("version") != CACHE_VERSION:
        return {}
    entries = data.get("entries", {})
    return entries if isinstance(entries, dict) else {}


def store_entry(key: str, value: dict, path: Path | None = None) -> None:
    """Add one entry; the file is replaced atomically so concurrent readers see old or new."""
    path = cache_path() if path is None else Path(path)
    with _lock:
        entries = load_cache(path)
        entries[key] = value
        path.parent.mkdir(parents=True, exist_ok=True)
        fd, tmp = tempfile.mkstemp(prefix=path.name, dir=path.parent)
        with os.fdopen(fd, "w", encoding="utf-8") as f:
            json.dump({"version": CACHE_VERSION, "entries": entries}, f, indent=1, sort_keys=True)
        os.replace(tmp, path)


def pick_fastest(timings: dict[int, float]) -> int:
    """Fastest schedule; ties (within 1 %) go to the lower mask, the simpler kernels."""
    best = min(timings.values())
    return min(m for m, t in timings.items() if t <= best * 1.01)


def time_schedules(set_schedule: Callable[[int], None], run: Callable[[], None], masks: list[int],
                   reps: int = 5, warmup: int = 2, stream: torch.cuda.Stream | None = None) -> dict[int, float]:
    """Median CUDA-event milliseconds of `run` under each schedule mask."""
    stream = torch.cuda.current_stream() if stream is None else stream
    out = {}
    for m in masks:
        set_schedule(m)
        for _ in range(warmup):
            run()
        times = []
        for _ in range(reps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            run()
            b.record(stream)
            b.synchronize()
            times.append(a.elapsed_time(b))
        out[m] = statistics.median(times)
    return out


@dataclass
class Choice:
    mask: int
    timings_ms: dict[int, float]
    slices: int
    rel_diff: dict[int, float]  # relative L2 distance of each schedule's field from its family's first

    def as_json(self) -> dict:
        return {"mask": self.mask, "slices": self.slices,
                "timings_ms": {str(k): round(v, 4) for k, v in sorted(self.timings_ms.items())},
                "rel_diff": {str(k): v for k, v in sorted(self.rel_diff.items())}}


def _workload(nx: int, ny: int, device: torch.device, slices: int):
    """Seeded voxel multislice of the plan's size: random-phase field, a (slices, ny+2, nx+2)
    grid of ids 0..2 (voxel pitch = grid pitch) and a two-material table."""
    g = torch.Generator(device="cpu").manual_seed(nx * 7919 + ny)
    phase = torch.rand(nx * ny, generator=g, dtype=torch.float32) * 6.2831855
    u0 = torch.polar(torch.ones_like(phase), phase).to(torch.complex64).to(device)
    grid = torch.randint(0, 3, (slices, ny + 2, nx + 2), generator=g, dtype=torch.int32).to(device)
    db = torch.tensor([[0.0, 0.0], [3.2e-7, 2.1e-10], [1.1e-6, 4.0e-9]], dtype=torch.float32, device=device)
    return u0, grid, db


def tune_multislice(nx: int, ny: int, device: torch.device | str = "cuda", slices: int | None = None,
                    reps: int = 5, store: bool = True, plan=None) -> Choice:
    """Time every distinct schedule of an (nx, ny) plan on `slices` voxel slices and cache the
    fastest of those that reproduce the first schedule's field."""
    from . import _lib
    device = torch.device(device)
    if slices is None:  # 16 slices' worth of a 4096^2 grid, at least 2, at most 16: per-slice
        # differences of a few microseconds then outweigh the run's fixed start and end
        slices = int(max(2, min(16, (16 * 4096 * 4096) // (nx * ny))))
    if plan is None:
        _tuning.active = True
        try:
            plan = _lib.plan_for(nx, ny, device)
        finally:
            _tuning.active = False
    masks = plan.schedules()
    previous = plan.schedule()
    u0, grid, db = _workload(nx, ny, device, slices)
    u = torch.empty_like(u0)
    U = torch.empty_like(u0)
    dx = 0.5e-6
    wl = 6.2e-11
    geom = _lib.VoxelGeom(slices, ny + 2, nx + 2, dx, dx, 1e-6, 0.0, 0.0)
    dz = _lib.doubles([1e-6] * slices)
    L = _lib.lib()

    def run():
        u.copy_(u0)
        with torch.cuda.device(device):
            _lib.check(L.rs_multislice_voxel(plan.handle, _lib.ptr(u), _lib.ptr(U), _lib.ptr(grid), 0, _lib.ptr(db),
                                             3, geom, dx, dx, wl, 0.45 / dx, dz, None, 0, slices,
                                             _lib.stream_handle(device)), "autotune multislice")

    diffs: dict[int, float] = {}
    try:
        with torch.cuda.device(device):
            timings = time_schedules(plan.set_schedule, run, masks, reps=reps)
            # Each schedule's field against the first schedule of its family: per direction, the
            # split-pair passes with dithered twiddles or (COMP bits) the single-sequence passes.
            # Within a family the kernels compute the same values; the two families differ at
            # the FP32 rounding level and are both within the accuracy bound, so the fastest
            # schedule of either is eligible.
            references: dict[int, torch.Tensor] = {}
            for m in masks:
                plan.set_schedule(m)
                run()
                torch.cuda.synchronize(device)
                fam = m & SCHED_COMPENSATED
                if fam not in references:
                    references[fam] = u.clone()
                    diffs[m] = 0.0
                else:
                    ref = references[fam]
                    diffs[m] = float(torch.linalg.vector_norm(u - ref) / torch.linalg.vector_norm(ref))
    finally:
        plan.set_schedule(previous)
    # a schedule that does not reproduce its family's first field to FP32 rounding is never picked
    eligible = {m: t for m, t in timings.items() if diffs[m] <= MAX_SCHEDULE_DIFF}
    choice = Choice(pick_fastest(eligible), timings, slices, diffs)
    if store:
        store_entry(entry_key(device_key(device), nx, ny, "multislice"), choice.as_json())
    return choice


def cached_schedule(nx: int, ny: int, device: torch.device, workload: str = "multislice") -> int | None:
    entry = load_cache().get(entry_key(device_key(device), nx, ny, workload))
    if isinstance(entry, dict) and isinstance(entry.get("mask"), int):
        return entry["mask"]
    return None


def apply_to_plan(plan) -> None:
    """Called for every new plan: set the cached schedule, or tune first when RS_AUTOTUNE=1."""
    if getattr(_tuning, "active", False):
        return
    try:
        mask = cached_schedule(plan.nx, plan.ny, plan.device)
    except (RuntimeError, AssertionError):
        return
    if mask is None and os.environ.get("RS_AUTOTUNE", "") in ("1", "on", "true"):
        mask = tune_multislice(plan.nx, plan.ny, plan.device, plan=plan).mask
    if mask is not None and mask in plan.schedules():
        plan.set_schedule(mask)


def tune_batch_streams(batch, device: torch.device | str = "cuda", candidates=(1, 2, 3, 4), items: int = 16,
                       store: bool = True) -> tuple[int, dict[int, float]]:
    """Wall time of `items` batch items (cycled over the batch's sizes) with each stream count;
    returns the fastest count and the seconds per configuration."""
    import time

    from .multisim import BatchRunner
    device = torch.device(device)
    sample = batch.items[:items]
    out = {}
    for k in candidates:
        runner = BatchRunner(batch, device, streams=k)
        runner.run(sample[: 2 * k])  # plans, tables and buffers of every stream
        torch.cuda.synchronize(device)
        t0 = time.perf_counter()
        runner.run(sample)
        torch.cuda.synchronize(device)
        out[k] = time.perf_counter() - t0
        del runner
    best = min(out.values())
    pick = min(k for k, t in out.items() if t <= best * 1.01)
    if store:
        sizes = "-".join(str(s) for s in sorted({it.n for it in sample}))
        store_entry(entry_key(device_key(device), 0, 0, f"multisim_streams_{sizes}"),
                    {"streams": pick, "seconds": {str(k): round(v, 5) for k, v in out.items()}, "items": len(sample)})
    return pick, out

