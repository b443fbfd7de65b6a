"""Input configurations of the prepared-directory fixtures (tests/golden/setup_ref*/), shared by
tests/golden/make_setup_golden.py, which runs big-wave's setup_simulation on them, and the tests,
which run this package's setup_simulation on them. The element grids are seeded (write_inputs);
each fixture directory holds the copies the setup made."""
from __future__ import annotations

from pathlib import Path

import numpy as np


def _sample(z_start, grid_path, materials=(["W", 19.3], ["Au", 19.32]), dz=1e-6):
    return {"type": "sample", "z_start": z_start, "pixel_size_x": 4e-7, "pixel_size_y": 4e-7,
            "pixel_size_z": dz, "grid_path": grid_path, "materials": [list(m) for m in materials],
            "x_positions": [0.0], "y_positions": [0.0]}


def _plasma(z_start, prefix, dz, **chem):
    return {"type": "plasma_sample", "z_start": z_start, "pixel_size_x": 4e-7, "pixel_size_y": 4e-7,
            "pixel_size_z": dz, **{f"{k}_grid_path": f"{prefix}_{k}.npy" for k in ("ne", "ni", "te", "zstar")},
            "x_positions": [0.0], "y_positions": [0.0], **chem}


def config_dict() -> dict:
    return {
        "sim_params": {"N": 256 * 256, "nx": 256, "ny": 256, "dx": 2e-7, "dy": 2e-7, "z_detector": 1.0,
                       "detector_size": 12.8e-6, "detector_size_x": 12.8e-6, "detector_size_y": 12.8e-6,
                       "detector_pixel_size_x": 0.8e-6, "detector_pixel_size_y": 0.8e-6, "chunk_size": 256},
        "elements": [_sample(0.5, "grid.npy")],
        "dtype": "c8",
        "use_disk_vector": False,
        "save_final_u_vectors": False,
        "multisource": {"type": "points", "nr_source_points": 5, "energy_range": [15000.0, 30000.0],
                        "x_range": [-2e-6, 2e-6], "y_range": [-1e-6, 1e-6], "z": 0.0, "seed": 42},
    }


def config_plasma() -> dict:
    # three 2 cm elements (4 slices of 5 mm) from z = 0.5 m; the detector right behind the last
    return {
        "sim_params": {"N": 512 * 512, "ny": 512, "dx": 1e-7, "dy": 1e-7, "z_detector": 0.56,
                       "detector_size": 2.56e-6, "detector_size_x": 2.56e-6, "detector_size_y": 5.12e-6,
                       "detector_pixel_size_x": 0.32e-6, "detector_pixel_size_y": 0.64e-6, "chunk_size": "auto"},
        "runtime": {"big_wave": {"memory_budget_gb": 2.0, "detector_integrator": "legacy_fastwave"}},
        "elements": [_sample(0.5, "grid.npy", (["SiO2", 2.2], ["W", 19.3]), dz=5e-3),
                     _plasma(0.52, "pa", 5e-3, formula="CH"),
                     _plasma(0.54, "pb", 5e-3, Z=13)],
        "dtype": "c16",
        "use_disk_vector": False,
        "save_final_u_vectors": False,
        "multisource": {"type": "points", "nr_source_points": 3, "energy_range": [8000.0, 12000.0],
                        "x_range": [-1e-6, 3e-6], "z": 0.2, "seed": 7},
    }


def config_fresnel() -> dict:
    return {
        "sim_params": {"N": 256 * 256, "nx": 256, "ny": 256, "dx": 2e-7, "dy": 2e-7, "z_detector": 2.0,
                       "detector_size": 1e-4, "detector_size_x": 1e-4, "detector_size_y": 8e-5,
                       "detector_pixel_size_x": 2e-6, "detector_pixel_size_y": 2e-6, "chunk_size": 4096,
                       "use_fresnel_scaling": True},
        "elements": [_sample(0.5, "grid.npy")],
        "dtype": "c8",
        "use_disk_vector": False,
        "save_final_u_vectors": False,
        "multisource": {"type": "points", "nr_source_points": 4, "energy_range": [20000.0, 25000.0],
                        "x_range": [-1e-6, 1e-6], "y_range": [-2e-6, 0.0], "z": 0.0, "seed": 11},
    }


def config_exit() -> dict:
    return {
        "sim_params": {"N": 256 * 256, "nx": 256, "ny": 256, "dx": 2e-7, "dy": 2e-7, "z_detector": 1.0,
                       "detector_size": 12.8e-6, "detector_size_x": 12.8e-6, "detector_size_y": 12.8e-6,
                       "detector_pixel_size_x": 0.8e-6, "detector_pixel_size_y": 0.8e-6, "chunk_size": 512},
        "elements": [_sample(0.5, "grid.npy"), {"type": "save_and_exit", "z_start": 0.6},
                     _sample(0.6, "grid2.npy", (["Au", 19.32],))],
        "dtype": "c8",
        "use_disk_vector": False,
        "save_final_u_vectors": True,
        "multisource": {"type": "points", "nr_source_points": 2, "energy_range": [15000.0, 16000.0],
                        "x_range": [-1e-6, 1e-6], "z": 0.0, "seed": 3},
    }


CASES = {"setup_ref": config_dict, "setup_ref_plasma": config_plasma, "setup_ref_fresnel": config_fresnel,
         "setup_ref_exit": config_exit}


def write_inputs(tmp: Path) -> None:
    """Seeded element grids shared by the cases."""
    rng = np.random.default_rng(3)
    np.save(tmp / "grid.npy", rng.integers(0, 3, size=(4, 12, 12), dtype=np.uint32))
    np.save(tmp / "grid2.npy", rng.integers(0, 2, size=(2, 10, 10), dtype=np.uint32))
    for prefix in ("pa", "pb"):
        shape = (4, 8, 8)
        np.save(tmp / f"{prefix}_ne.npy", rng.uniform(1e19, 1e21, size=shape))
        np.save(tmp / f"{prefix}_ni.npy", rng.uniform(1e18, 1e20, size=shape))
        np.save(tmp / f"{prefix}_te.npy", rng.uniform(1.0, 50.0, size=shape))
        np.save(tmp / f"{prefix}_zstar.npy", rng.uniform(0.5, 3.0, size=shape))


# cases whose source 0 big-wave also runs (tests/golden/setup_runs.npz)
RUN_CASES = ("setup_ref_plasma", "setup_ref_fresnel", "setup_ref_exit")


def _with(base: dict, **changes) -> dict:
    """A copy of `base` with top-level keys, or sim_params / multisource entries ("sp_x", "ms_x"),
    replaced."""
    import copy
    out = copy.deepcopy(base)
    for key, value in changes.items():
        if key.startswith("sp_"):
            out["sim_params"][key[3:]] = value
        elif key.startswith("ms_"):
            out["multisource"][key[3:]] = value
        else:
            out[key] = value
    return out


def error_cases() -> dict:
    """Inputs big-wave's setup_simulation rejects, each with the exception it raises (recorded in
    tests/golden/setup_errors.json)."""
    base = config_dict()
    return {
        "nx_not_power_of_two": _with(base, sp_N=384 * 256, sp_nx=384),
        "detector_bigger_than_grid": _with(base, sp_detector_size=1e-4, sp_detector_size_x=1e-4),
        "source_nyquist_exceeded": _with(base, sp_dx=4e-7, sp_dy=4e-7, sp_z_detector=0.5 + 6e-6,
                                         elements=[_sample(0.5, "grid.npy")]),
        "reflections_at_boundary": _with(base, ms_x_range=[-4e-6, 4e-6], sp_detector_size=2.56e-5,
                                         sp_detector_size_x=2.56e-5, sp_detector_size_y=2.56e-5),
        "thin_fresnel_two_elements": _with(config_fresnel(), elements=[_sample(0.5, "grid.npy"),
                                                                       _sample(0.6, "grid2.npy", (["Au", 19.32],))]),
        "cutoff_beyond_nyquist": _with(base, sp_z_detector=0.5 + 1.4e-5),
        "unknown_multisource": _with(base, ms_type="cloud"),
        "y_range_not_a_pair": _with(base, ms_y_range=[0.0]),
        "overlapping_elements": _with(base, elements=[_sample(0.5, "grid.npy"), _sample(0.5 + 1e-6, "grid2.npy")]),
        "bad_chunk_size": _with(base, sp_chunk_size=1.5),
    }
