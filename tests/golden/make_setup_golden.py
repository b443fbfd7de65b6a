"""Generate tests/golden/setup_ref/: a simulation directory prepared by big-wave's own
setup_simulation (big-wave/multisim.py:727-1397) for a 256 x 256 run with one voxel sample and
five point sources (uniform energies in 15-30 keV, Gaussian source positions, seed 42), so the
tests can check this package's source sampling and its parsing of a real prepared directory.

big-wave needs two things this container does not have, which the script supplies:
* ruamel.yaml: config.load / config.save go through a stand-in backed by this package's
  yaml_io (so the YAML text is yaml_io's; the values are big-wave's);
* nist_lookup's xray_delta_beta (sqlalchemy): the delta-beta tables come from the Chantler
  restatement in chantler_constants.py over nist_lookup's own xrayref.db.

    python tests/golden/make_setup_golden.py [/path/to/RAVE-SIM]
"""
from __future__ import annotations

import importlib
import shutil
import sqlite3
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
sys.path.insert(0, str(HERE.parents[1]))
from chantler_constants import delta_beta  # noqa: E402
from make_golden import import_reference  # noqa: E402

OUT = HERE / "setup_ref"


def config_dict() -> dict:
    return {
        "sim_params": {"N": 256 * 256, "nx": 256, "ny": 256, "dx": 2e-7, "dy": 2e-7, "z_detector": 1.0,
                       "detector_size": 12.8e-6, "detector_size_x": 12.8e-6, "detector_size_y": 12.8e-6,
                       "detector_pixel_size_x": 0.8e-6, "detector_pixel_size_y": 0.8e-6, "chunk_size": 256},
        "elements": [{"type": "sample", "z_start": 0.5, "pixel_size_x": 4e-7, "pixel_size_y": 4e-7,
                      "pixel_size_z": 1e-6, "grid_path": "grid.npy",
                      "materials": [["W", 19.3], ["Au", 19.32]], "x_positions": [0.0],
                      "y_positions": [0.0]}],
        "dtype": "c8",
        "multisource": {"type": "points", "nr_source_points": 5, "energy_range": [15000.0, 30000.0],
                        "x_range": [-2e-6, 2e-6], "y_range": [-1e-6, 1e-6], "z": 0.0, "seed": 42},
    }


def main(root: Path) -> None:
    _prop, oe, _ps, _src, _vec, _ws, ms = import_reference(root)
    import config as bw_config
    yio = importlib.import_module("3d_ravesim_gb300.yaml_io")

    class YamlStandIn:
        def __init__(self, typ=None):
            pass

        def indent(self, **kw):
            pass

        def load(self, path):
            return yio.load(path)

        def dump(self, dct, f):
            f.write(yio.dumps(dct))

    bw_config.YAML = YamlStandIn
    db = sqlite3.connect(f"file:{root / 'nist_lookup' / 'nist_lookup' / 'xrayref.db'}?mode=ro", uri=True)

    def xray_delta_beta(material, density, energy, *a, **k):
        d, b = delta_beta(db, {material: 1}, density, energy)
        return d, b, None

    oe.xray_delta_beta = xray_delta_beta
    rng = np.random.default_rng(3)
    with tempfile.TemporaryDirectory() as tmp:
        tmp = Path(tmp)
        grid = rng.integers(0, 3, size=(4, 12, 12), dtype=np.uint32)
        np.save(tmp / "grid.npy", grid)
        sim = ms.setup_simulation(config_dict(), tmp, tmp / "out")
        if OUT.exists():
            shutil.rmtree(OUT)
        shutil.copytree(sim, OUT)
    print("wrote", OUT)


if __name__ == "__main__":
    sys.path.insert(0, str(Path(__file__).resolve().parent))
    from _refroot import reference_root
    main(reference_root())
