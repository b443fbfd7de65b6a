"""delta/beta of the grating and filter materials used by the synthetic workloads, from the
Chantler tables of nist_lookup (restated with sqlite3: nist_lookup/nist_lookup/xraydb.py:382-414,
xraydb_plugin.py:116-185). Writes chantler_constants.json beside this file.

    python tests/golden/chantler_constants.py [/path/to/RAVE-SIM]
"""
import json
import math
import sqlite3
import sys
from pathlib import Path

import numpy as np
import scipy.constants as consts
from scipy.interpolate import UnivariateSpline

PLANCK_HC = 1.e10 * consts.Planck * consts.c / consts.e
R_ELECTRON_CM = 100.0 * consts.physical_constants["classical electron radius"][0]
AVOGADRO = consts.Avogadro


def chantler(db, element, energy, column):
    row = db.execute(f"select energy, {column} from Chantler where element = ?", (element,)).fetchone()
    te = np.array(json.loads(row[0]))
    ty = np.array(json.loads(row[1]))
    idx = np.where(te <= energy)[0]
    lo = max(0, -5 + idx.max())
    hi = min(len(te), 6 + idx.max())
    te, ty = te[lo:hi], ty[lo:hi]
    if column == "f1":
        return float(UnivariateSpline(te, ty, s=1)(energy))
    return float(np.exp(np.interp(np.log(energy), np.log(te), np.log(ty))))


def delta_beta(db, formula: dict, density, energy):
    lamb_cm = 1.e-8 * PLANCK_HC / energy
    d = b = mass = 0.0
    for sym, n in formula.items():
        z, m = db.execute("select atomic_number, molar_mass from elements where element = ?", (sym,)).fetchone()
        f1 = chantler(db, sym, energy, "f1") + z
        f2 = chantler(db, sym, energy, "f2")
        ratio = chantler(db, sym, energy, "mu_total") / chantler(db, sym, energy, "mu_photo")
        w = density * n * AVOGADRO
        d += w * f1
        b += w * f2 * ratio
        mass += n * m
    scale = lamb_cm * lamb_cm * R_ELECTRON_CM / (2 * math.pi * mass)
    return d * scale, b * scale


def main(root: Path):
    db = sqlite3.connect(f"file:{root / 'nist_lookup' / 'nist_lookup' / 'xrayref.db'}?mode=ro", uri=True)
    out = {}
    for e in (15000.0, 20000.0, 25000.0, 30000.0, 40000.0):
        out[f"Si_2.33_{int(e)}"] = delta_beta(db, {"Si": 1}, 2.33, e)
        out[f"Au_19.32_{int(e)}"] = delta_beta(db, {"Au": 1}, 19.32, e)
        out[f"Al_2.70_{int(e)}"] = delta_beta(db, {"Al": 1}, 2.70, e)
        mu_al = chantler(db, "Al", e, "mu_total")  # cm^2/g
        out[f"Al_mu_total_{int(e)}"] = mu_al
    out["Al_mu_total_10_50keV_1keV_steps"] = [chantler(db, "Al", 1000.0 * e, "mu_total") for e in range(10, 51)]
    path = Path(__file__).resolve().parent / "chantler_constants.json"
    path.write_text(json.dumps(out, indent=1))
    print(json.dumps({k: v for k, v in out.items() if not isinstance(v, list)}, indent=1))


if __name__ == "__main__":
    sys.path.insert(0, str(Path(__file__).resolve().parent))
    from _refroot import reference_root
    main(reference_root())
