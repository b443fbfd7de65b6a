"""Generate tests/golden/detector_meta.json: the metadata big-wave's own 2D detector records in
``SimParams.detector_last_metadata`` (big-wave/propagation.py:919-946 for legacy_fastwave,
1087-1110 for area_v1) and the RuntimeWarnings it raises, for seeded small fields over a set of
geometries: both integrators, integer and non-integer pixel/grid ratios, detectors larger than
the grid (zero-count / zero-coverage pixels), unequal dx and dy, and a Fresnel-scaled detector.

    python tests/golden/make_detector_meta_golden.py [/path/to/RAVE-SIM]
"""
from __future__ import annotations

import json
import sys
import warnings
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parent))
from make_golden import import_reference  # noqa: E402

OUT = Path(__file__).resolve().parent / "detector_meta.json"

# SimParams keyword arguments (big-wave's field names), an optional Fresnel configuration
# (z_source, z_sample) and the plane the detector integrates at
CASES = [
    {"name": "area_v1 integer ratio, dy != dx",
     "params": dict(nx=48, ny=32, dx=1e-6, dy=1.5e-6, detector_size_x=48e-6, detector_size_y=48e-6,
                    detector_pixel_size_x=2e-6, detector_pixel_size_y=3e-6, z_detector=1.0),
     "integrator": "area_v1", "current_z": 1.0},
    {"name": "area_v1 non-integer ratio, detector wider than the grid",
     "params": dict(nx=40, ny=24, dx=1e-6, dy=1e-6, detector_size_x=60e-6, detector_size_y=40e-6,
                    detector_pixel_size_x=1.5e-6, detector_pixel_size_y=2.5e-6, z_detector=0.7),
     "integrator": "area_v1", "current_z": 0.7},
    {"name": "area_v1 inside the grid, off-detector plane",
     "params": dict(nx=64, ny=64, dx=0.5e-6, dy=0.5e-6, detector_size_x=20e-6, detector_size_y=10e-6,
                    detector_pixel_size_x=1e-6, detector_pixel_size_y=0.75e-6, z_detector=2.0),
     "integrator": "area_v1", "current_z": 1.25},
    {"name": "legacy_fastwave integer ratio",
     "params": dict(nx=48, ny=32, dx=1e-6, dy=1e-6, detector_size_x=32e-6, detector_size_y=24e-6,
                    detector_pixel_size_x=2e-6, detector_pixel_size_y=2e-6, z_detector=1.0),
     "integrator": "legacy_fastwave", "current_z": 1.0},
    {"name": "legacy_fastwave non-integer ratio, zero-count pixels",
     "params": dict(nx=40, ny=24, dx=1e-6, dy=1e-6, detector_size_x=60e-6, detector_size_y=36e-6,
                    detector_pixel_size_x=1.5e-6, detector_pixel_size_y=1.7e-6, z_detector=1.0),
     "integrator": "legacy_fastwave", "current_z": 1.0},
    {"name": "area_v1 Fresnel-scaled detector",
     "params": dict(nx=64, ny=48, dx=1e-6, dy=1e-6, detector_size_x=120e-6, detector_size_y=96e-6,
                    detector_pixel_size_x=4e-6, detector_pixel_size_y=4e-6, z_detector=2.0,
                    use_fresnel_scaling=True),
     "fresnel": [0.0, 0.5], "integrator": "area_v1", "current_z": 2.0},
    {"name": "legacy_fastwave Fresnel-scaled detector",
     "params": dict(nx=64, ny=48, dx=1e-6, dy=1e-6, detector_size_x=96e-6, detector_size_y=72e-6,
                    detector_pixel_size_x=3e-6, detector_pixel_size_y=3e-6, z_detector=1.5,
                    use_fresnel_scaling=True),
     "fresnel": [-0.5, 0.25], "integrator": "legacy_fastwave", "current_z": 1.5},
]


def main(root: Path) -> None:
    prop, _oe, _ps, _src, vec, *_ = import_reference(root)
    rng = np.random.default_rng(7)
    out = []
    for case in CASES:
        kw = dict(case["params"])
        nx, ny = kw["nx"], kw["ny"]
        p = prop.SimParams(N=nx * ny, wl=1e-10, chunk_size=nx, detector_size=kw["detector_size_x"],
                           detector_integrator=case["integrator"], **kw)
        if "fresnel" in case:
            p.configure_fresnel_detector(*case["fresnel"])
        field = (rng.normal(size=nx * ny) + 1j * rng.normal(size=nx * ny)).astype(np.complex64)
        u = vec.NumpyVector(field)
        with warnings.catch_warnings(record=True) as caught:
            warnings.simplefilter("always")
            prop.square_and_downsample_2d(u, p, case["current_z"])
        meta = dict(p.detector_last_metadata)
        meta.pop("output_storage")  # where the image lives (host memory here)
        out.append({**case, "metadata": meta,
                    "warnings": [str(w.message) for w in caught if issubclass(w.category, RuntimeWarning)]})
    OUT.write_text(json.dumps(out, indent=1))
    print("wrote", OUT)


if __name__ == "__main__":
    sys.path.insert(0, str(Path(__file__).resolve().parent))
    from _refroot import reference_root
    main(reference_root())
