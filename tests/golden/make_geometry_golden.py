"""Generate tests/golden/geometry.json: big-wave's SimParams geometry (big-wave/propagation.py:
100-196: get_dy, detector sizes, configure_fresnel_detector, fresnel_transverse_scale,
effective_slice_dz, effective_final_dz, effective_detector_geometry) for a plain, a
Fresnel-scaled and a cone-beam configuration over a set of planes and steps, with the error
messages where big-wave raises; and its Nyquist helpers grid_density_check_2d and max_dx
(204-248) on a set of grids.

    python tests/golden/make_geometry_golden.py [/path/to/RAVE-SIM]
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

sys.path.insert(0, str(Path(__file__).resolve().parent))
from make_golden import import_reference  # noqa: E402

OUT = Path(__file__).resolve().parent / "geometry.json"

BASE = dict(N=64 * 32, nx=64, ny=32, dx=1e-6, z_detector=1.1, detector_size=64e-6,
            detector_pixel_size_x=2e-6, detector_pixel_size_y=2e-6, wl=5e-11, chunk_size=64)
CONFIGS = [
    {"name": "plain", "params": {}, "fresnel": [0.0, 0.4]},
    {"name": "plain, explicit dy and detector sizes",
     "params": {"dy": 1.5e-6, "detector_size_x": 50e-6, "detector_size_y": 30e-6}, "fresnel": None},
    {"name": "Fresnel scaling", "params": {"use_fresnel_scaling": True}, "fresnel": [-0.3, 0.2]},
    {"name": "cone-beam BPM", "params": {"use_cone_beam_bpm": True}, "fresnel": [0.0, 0.5]},
    {"name": "cone-beam BPM, source downstream of the plane", "params": {"use_cone_beam_bpm": True},
     "fresnel": [0.6, 0.8]},
]
PLANES = [-0.1, 0.25, 0.5, 0.75, 1.0, 1.1, 1.2]
STEPS = [1e-6, 2.5e-4, 0.05]
BAD_FRESNEL = [[0.5, 0.2], [0.0, 1.5]]
NYQUIST = [  # dz, x_source, Nx, dx, y_source, Ny, dy, wl
    [1.0, 0.0, 1024, 1e-7, 0.0, 1024, 1e-7, 5e-11],
    [1.0, 2e-5, 4096, 1e-7, -3e-5, 2048, 1e-7, 5e-11],
    [0.05, 0.0, 4096, 1e-7, 0.0, 4096, 1e-7, 5e-11],
    [0.5, 1e-4, 8192, 5e-8, 0.0, 8192, 5e-8, 4e-11],
    [2.0, 0.0, 16384, 2e-7, 0.0, 16384, 2e-7, 6e-11],
]
MAX_DX = [[1.0, 0.0, 4096, 5e-11], [0.1, 1e-5, 8192, 4e-11], [0.5, 0.0, 32768, 6e-11], [3.0, 2e-4, 1024, 1e-10]]


def attempt(fn, *args):
    try:
        v = fn(*args)
        return list(v) if isinstance(v, tuple) else v
    except ValueError as e:
        return {"error": str(e)}


def main(root: Path) -> None:
    prop, *_ = import_reference(root)
    out = {"base": BASE, "planes": PLANES, "steps": STEPS, "configs": [], "bad_fresnel": [],
           "nyquist": [], "max_dx": []}
    for cfg in CONFIGS:
        p = prop.SimParams(**BASE, **cfg["params"])
        if cfg["fresnel"] is not None:
            p.configure_fresnel_detector(*cfg["fresnel"])
        rec = {**cfg, "dy": p.get_dy(), "nx": p.nx, "is_2d": p.is_2d,
               "use_fresnel_scaling": p.use_fresnel_scaling,
               "detector_size": [p.get_detector_size_x(), p.get_detector_size_y()],
               "magnification": p.fresnel_magnification, "effective_z": p.fresnel_effective_z,
               "scale": [attempt(p.fresnel_transverse_scale, z) for z in PLANES],
               "slice_dz": [[attempt(p.effective_slice_dz, z, dz) for dz in STEPS] for z in PLANES],
               "final_dz": [attempt(p.effective_final_dz, z) for z in PLANES],
               "detector_geometry": [attempt(p.effective_detector_geometry, z) for z in PLANES]}
        out["configs"].append(rec)
    for zs in BAD_FRESNEL:
        p = prop.SimParams(**BASE, use_fresnel_scaling=True)
        out["bad_fresnel"].append({"args": zs, "result": attempt(p.configure_fresnel_detector, *zs)})
    for args in NYQUIST:
        out["nyquist"].append({"args": args, "result": attempt(prop.grid_density_check_2d, *args)})
    for args in MAX_DX:
        out["max_dx"].append({"args": args, "result": prop.max_dx(*args)})
    OUT.write_text(json.dumps(out, indent=1))
    print("wrote", OUT)


if __name__ == "__main__":
    sys.path.insert(0, str(Path(__file__).resolve().parent))
    from _refroot import reference_root
    main(reference_root())
