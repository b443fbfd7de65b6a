"""Generate tests/golden/rundir_ref/: files of a per-source run directory written by big-wave's
own helpers (big-wave/multisim.py:43-70 and 125-215), so the tests can check that
`multisim.save_detector_outputs` and `multisim.point_source_geometry_2d` write the same bytes and
values:

* ``detected.npy``: big-wave's _save_detector_outputs of two seeded float64 phase images;
* ``detected_inputs.npy``: those two images;
* ``source_geometry.json``: point_source_geometry_2d for explicit and missing source.y.

    python tests/golden/make_rundir_golden.py [/path/to/RAVE-SIM]
"""
from __future__ import annotations

import json
import shutil
import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parent))
from make_golden import import_reference  # noqa: E402

OUT = Path(__file__).resolve().parent / "rundir_ref"
SOURCES = [({"type": "point", "x": 1.5e-06, "y": -2.25e-06, "z": -0.5}, {"y_range": [-1e-05, 1e-05]}),
           ({"type": "point", "x": 3e-06, "z": 0.0}, {"y_range": [0.0, 0.0]}),
           ({"type": "point", "x": 0.0, "y": 0.0, "z": 0.0}, {})]


def main(root: Path) -> None:
    *_, ms = import_reference(root)
    rng = np.random.default_rng(99)
    if OUT.exists():
        shutil.rmtree(OUT)
    OUT.mkdir()
    images = [rng.random((5, 7)), rng.random((5, 7))]
    ms._save_detector_outputs(OUT / "detected.npy", [im.copy() for im in images])
    np.save(OUT / "detected_inputs.npy", np.stack(images))
    geoms = [ms.point_source_geometry_2d(s, m) for s, m in SOURCES]
    (OUT / "source_geometry.json").write_text(json.dumps({"inputs": SOURCES, "outputs": geoms}, indent=1))
    print("wrote", OUT)


if __name__ == "__main__":
    sys.path.insert(0, str(Path(__file__).resolve().parent))
    from _refroot import reference_root
    main(reference_root())
