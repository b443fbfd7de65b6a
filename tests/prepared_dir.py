"""Writes a simulation directory in the layout big-wave's setup_simulation prepares
(big-wave/multisim.py:1233-1397): config.yaml, computed.yaml, the grids next to them and one
00000000/subconfig.yaml. The case is the recorded two-sample run of
tests/golden/history_golden.npz."""
from pathlib import Path

import numpy as np


def write_prepared_dir(yio, root: Path, golden, dtype: str = "c8") -> Path:
    sim = root / "sim"
    (sim / "00000000").mkdir(parents=True)
    np.save(sim / "grid_a.npy", golden["run_grid"])
    np.save(sim / "grid_b.npy", golden["run_grid2"])
    a0, a1, a2, _wl, _hdz = golden["run_params"]
    common = {"pixel_size_x": 5e-07, "pixel_size_z": 2e-06, "pixel_size_y": 5e-07,
              "materials": [["W", 19.3]], "x_positions": [0.0], "y_positions": [0.0]}
    config = {
        "sim_params": {"N": 4096, "nx": 64, "ny": 64, "dx": 5e-07, "dy": 5e-07, "z_detector": 0.65,
                       "detector_size": 2.4e-05, "detector_size_x": 2.4e-05, "detector_size_y": 2e-05,
                       "detector_pixel_size_x": 1.5e-06, "detector_pixel_size_y": 1.25e-06, "chunk_size": 512,
                       "detector_integrator": "area_v1", "use_fresnel_scaling": False},
        "elements": [{"type": "sample", "z_start": 0.5, "grid_path": "grid_a.npy", **common},
                     {"type": "sample", "z_start": 0.56, "grid_path": "grid_b.npy", **common}],
        "dtype": dtype, "use_disk_vector": False, "save_final_u_vectors": False,
        "multisource": {"y_range": [0.0, 0.0]},
        "runtime": {"big_wave": {"history": {"storage": "memory"}}},
    }
    yio.save(sim / "config.yaml", config)
    yio.save(sim / "computed.yaml", {"cutoff_angles": [float(a0), float(a1), float(a2)],
                                     "provenance": {"algorithm_version": "big-wave-2d-p4-v1"}})
    yio.save(sim / "00000000" / "subconfig.yaml", {
        "source": {"type": "point", "x": 1e-06, "y": 0.0, "z": 0.0}, "energy": 20000.0,
        "deltabeta_table": [[["W", 19.3], [4.2e-06, 1.9e-07]]]})
    return sim
