"""A small synthetic Chantler database with the schema of nist_lookup's xrayref.db.

Deterministic (no random numbers): six elements whose tables are smooth functions of energy
with an absorption edge, tabulated on log-spaced grids of different lengths. The fixture script
make_chantler_golden.py runs nist_lookup's and big-wave's own code on it, and the CPU tests run
this package's lookup on the same file, so the lookup's arithmetic (table window, f1 spline,
log-log interpolation, compound averages, formula counts) is pinned without the real database.
"""
from __future__ import annotations

import json
import math
import sqlite3
from pathlib import Path

# symbol: (Z, molar mass, density, edge energy [eV], number of table points)
ELEMENTS = {
    "H": (1, 1.0079, 0.071, 14.0, 70),
    "C": (6, 12.011, 2.26, 284.0, 90),
    "O": (8, 15.999, 1.43, 543.0, 95),
    "Si": (14, 28.086, 2.33, 1839.0, 110),
    "Cu": (29, 63.546, 8.96, 8979.0, 187),
    "Au": (79, 196.97, 19.32, 11919.0, 160),
}
ISXRAYDB_TABLES = ("Waasmaier", "Coster_Kronig", "KeskiRahkonen_Krause", "photoabsorption", "scattering")


def _table(z: int, edge: float, n: int):
    lo, hi = math.log(10.0 + z), math.log(4.3e5)
    energy = [math.exp(lo + (hi - lo) * i / (n - 1)) for i in range(n)]
    f1, f2, photo, incoh, total = [], [], [], [], []
    for e in energy:
        r = e / edge
        jump = 1.0 if e < edge else 6.5
        # a dip of f1 at the edge, decaying photoabsorption with a jump, a slowly varying
        # incoherent term; the values only need to be positive where the tables are logged
        f1.append(-z * 0.35 * math.exp(-abs(math.log(r)) * 3.0) + 0.02 * z * math.sin(3.0 * math.log(e)))
        p = jump * z ** 3.2 * 2.0e4 / e ** 2.7
        f2.append(p * e / (z * 1.0e3) + 1e-6)
        photo.append(p)
        incoh.append(0.02 * z * (1.0 + math.log1p(e / 1e4)))
        total.append(p + incoh[-1] + 0.01 * z)
    return energy, f1, f2, photo, incoh, total


def build(path: Path) -> Path:
    path = Path(path)
    if path.exists():
        path.unlink()
    db = sqlite3.connect(str(path))
    db.execute("create table elements (atomic_number integer primary key, element text, molar_mass real, "
               "density real)")
    db.execute("create table Chantler (id integer primary key, element text, sigma_mu real, mue_f2 real, "
               "density real, corr_henke float, corr_cl35 float, corr_nucl float, energy text, f1 text, "
               "f2 text, mu_photo text, mu_incoh text, mu_total text)")
    for name in ISXRAYDB_TABLES:
        db.execute(f"create table {name} (id integer primary key, element text)")
    for i, (sym, (z, mass, rho, edge, n)) in enumerate(ELEMENTS.items()):
        db.execute("insert into elements values (?, ?, ?, ?)", (z, sym, mass, rho))
        cols = [json.dumps(c) for c in _table(z, edge, n)]
        db.execute("insert into Chantler values (?, ?, 0, 0, ?, 0, 0, 0, ?, ?, ?, ?, ?, ?)", (i + 1, sym, rho, *cols))
    db.commit()
    db.close()
    return path
