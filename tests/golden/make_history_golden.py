"""Generate tests/golden/history_golden.npz by running big-wave's own history code
(big-wave/history.py:52-435 and the history branches of wavesim.py:188-300) on seeded inputs:

* ``_history_z_steps`` for a set of (dz, history dz) pairs;
* a memory-storage History fed seeded frames through an ROI and a downsample, with its
  stacked frames, z list and metadata;
* run_simulation with a (History, dz) pair on a 64x64 point source -> 4-slice Sample -> gap ->
  2-slice Sample -> final-leg case, complex128: the analytic source frames, the gap and
  final-leg frames every history dz, and one frame per sample slice.

    python tests/golden/make_history_golden.py [/path/to/RAVE-SIM]
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parent))
from make_golden import import_reference  # noqa: E402

OUT = Path(__file__).resolve().parent / "history_golden.npz"
Z_STEP_CASES = [(1.0, 0.3), (1.0, 0.25), (0.9, 0.2), (0.05, 0.2), (0.31, 0.1), (2.0, 0.7), (1e-3, 1e-3)]


def main(root: Path) -> None:
    prop, oe, _ps, src, vec, ws, _ms = import_reference(root)
    import history as hist_mod
    NV = vec.NumpyVector
    rng = np.random.default_rng(4242)
    g: dict[str, np.ndarray] = {}

    steps = [hist_mod._history_z_steps(dz, hdz) for dz, hdz in Z_STEP_CASES]
    g["zsteps_cases"] = np.array(Z_STEP_CASES)
    g["zsteps_lengths"] = np.array([len(s) for s in steps])
    g["zsteps_values"] = np.concatenate(steps)

    frames = rng.normal(size=(5, 10, 12))
    h = hist_mod.History(roi=(1, 9, 2, 11), downsample=(2, 3))
    for i, f in enumerate(frames):
        h.push(f.copy(), 0.1 * (i + 1))
    g["mem_frames_in"] = frames
    g["mem_history"] = h.get_history()
    g["mem_z"] = np.array(h.get_z())
    g["mem_metadata"] = np.array(json.dumps(h.metadata(), sort_keys=True))

    nx = ny = 64
    wl20 = prop.convert_energy_wavelength(20000.0)
    pr = prop.SimParams(N=nx * ny, nx=nx, ny=ny, dx=0.5e-6, dy=0.5e-6, z_detector=0.65, detector_size=24e-6,
                        detector_size_x=24e-6, detector_size_y=20e-6, detector_pixel_size_x=1.5e-6,
                        detector_pixel_size_y=1.25e-6, wl=wl20, chunk_size=nx * 8)
    grid = np.zeros((4, 66, 66), np.uint32)
    yy, xx = np.mgrid[0:66, 0:66]
    grid[:, (yy - 33) ** 2 + (xx - 30) ** 2 < 100] = 1
    samp = oe.Sample(z_start=0.5, pixel_size_x=0.5e-6, pixel_size_z=2e-6, grid=grid,
                     materials=[oe.Material("W", 19.3)], x_positions=np.array([0.0]),
                     pixel_size_y=0.5e-6, y_positions=np.array([0.0]))
    table = [(oe.Material("W", 19.3), np.complex128(4.2e-6 + 1.9e-7j))]
    grid2 = np.zeros((2, 66, 66), np.uint32)
    grid2[:, (yy - 28) ** 2 + (xx - 36) ** 2 < 64] = 1
    samp2 = oe.Sample(z_start=0.56, pixel_size_x=0.5e-6, pixel_size_z=2e-6, grid=grid2,
                      materials=[oe.Material("W", 19.3)], x_positions=np.array([0.0]),
                      pixel_size_y=0.5e-6, y_positions=np.array([0.0]))
    u, U = NV(np.zeros(pr.N, np.complex128)), NV(np.zeros(pr.N, np.complex128))
    angles = [f * np.arcsin(pr.wl / (2 * pr.dx)) for f in (0.6, 0.7, 0.65)]
    hist_dz = 0.07
    hr = hist_mod.History()
    # frames: the source's analytic intensity every 0.07 m up to the first sample (0.5 m), one
    # per slice of each sample, the 0.052 m gap between the samples and the final leg
    source_obj = src.PointSource(x=1e-6, y=0.0, z=0.0)
    elements = [samp, samp2]
    outs = ws.run_simulation(pr, source_obj, elements, angles, u, U, table, Path("."), Path("."), False,
                             history=(hr, hist_dz))
    g["run_history"] = hr.get_history()
    g["run_history_z"] = np.array(hr.get_z())
    g["run_out"] = outs[0]
    g["run_grid"], g["run_grid2"] = grid, grid2
    g["run_params"] = np.array([*angles, wl20, hist_dz])
    np.savez_compressed(OUT, **{k: np.array(v, copy=True) for k, v in g.items()})
    print(f"wrote {OUT} ({OUT.stat().st_size / 1024:.0f} KiB, {len(g)} arrays)")


if __name__ == "__main__":
    sys.path.insert(0, str(Path(__file__).resolve().parent))
    from _refroot import reference_root
    main(reference_root())
