"""Write tests/golden/p5_fingerprints.json from big-wave's recorded P5 convergence runs
(tests/big_wave_2d/p5_results/{vacuum,sample,plasma}_convergence_{4096,8192,16384}.json,
produced by tests/big_wave_2d/p5_benchmark.py with big-wave's own complex64 path): per run the
mode, grid, pixel, cutoff, detected energy, peak and the 256-pixel centre-row fingerprint.
For the plasma runs it adds the carbon scattering factors (f1bar, f2eff_bar, zbar, z2bar) at
the run's energy from the Chantler tables (restated in chantler_constants.py), which
PlasmaSample takes from nist_lookup in big-wave (big-wave/plasma.py:50-56, 185-195).

    python tests/golden/make_p5_fingerprints.py [/path/to/RAVE-SIM]
"""
from __future__ import annotations

import json
import sqlite3
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
from chantler_constants import chantler  # noqa: E402

OUT = HERE / "p5_fingerprints.json"
KEYS = ("mode", "nx", "ny", "dx", "cutoff_frequency", "detected_energy", "detected_peak", "detected_shape",
        "centerline_256", "centerline_start_pixel", "integrator", "dtype")


def energy_of_wavelength(wl: float) -> float:
    """big-wave/propagation.py:199-201 (CODATA 2014 h, exact c and e)."""
    return 6.62607004e-34 * 299792458 / (wl * 1.602176634e-19)


def main(root: Path) -> None:
    runs = []
    for mode in ("vacuum", "sample", "plasma"):
        for n in (4096, 8192, 16384):
            rec = json.loads((root / "tests/big_wave_2d/p5_results" / f"{mode}_convergence_{n}.json").read_text())
            assert rec["status"] == "passed"
            runs.append({k: rec[k] for k in KEYS})
    energy = energy_of_wavelength(1e-9)
    db = sqlite3.connect(f"file:{root / 'nist_lookup' / 'nist_lookup' / 'xrayref.db'}?mode=ro", uri=True)
    f1 = chantler(db, "C", energy, "f1") + 6
    f2 = chantler(db, "C", energy, "f2")
    mu_photo = chantler(db, "C", energy, "mu_photo")
    mu_total = chantler(db, "C", energy, "mu_total")
    out = {"source": "tests/big_wave_2d/p5_results (big-wave, complex64, bfpy FFT, area_v1 detector)",
           "setup": {"wavelength": 1e-9, "z_detector": 10.0, "detector_size": 4e-4, "detector_pixel": 8e-7,
                     "source": [1e-6, -1.4e-6, 0.0], "element_z_start": 5.0, "tile_rows": 32},
           "plasma_scattering_factors": {"energy_ev": energy, "C": [f1, f2 * (mu_total / mu_photo), 6.0, 36.0]},
           "runs": runs}
    OUT.write_text(json.dumps(out, indent=1) + "\n")
    print("wrote", OUT, len(runs), "runs")


if __name__ == "__main__":
    sys.path.insert(0, str(Path(__file__).resolve().parent))
    from _refroot import reference_root
    main(reference_root())
