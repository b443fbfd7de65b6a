"""Write tests/golden/chantler_golden.json: big-wave's own per-energy plasma scattering factors
(big-wave/plasma.py:241-266 for a formula, big-wave/plasma_sample.py:68-83 for a bare Z) and
nist_lookup's own xray_delta_beta (nist_lookup/nist_lookup/xraydb_plugin.py:136-185), computed by
the unmodified reference modules.

nist_lookup reads its sqlite database through SQLAlchemy, which is not installed here; this
script gives it a minimal stand-in (`_FakeSqlAlchemy` below: table reflection, an
equality filter and `.all()` over sqlite3 rows) so that nist_lookup's own Chantler code
(xraydb.py:382-414: the table window, the s=1 spline for f1 and the log-log interpolation of the
other columns) runs as written.

    python tests/golden/make_chantler_golden.py /path/to/RAVE-SIM   (or set $RAVESIM_REFERENCE)
"""
from __future__ import annotations

import json
import sqlite3
import sys
import types
from pathlib import Path

OUT = Path(__file__).resolve().parent / "chantler_golden.json"

FORMULAS = ("C", "CH", "C8H8", "H2O", "SiO2", "Fe2O3", "CaMg(CO3)2")
ZS = (6, 13, 29, 79)          # C, Al, Cu, Au through the bare-Z path
ENERGIES = (8000.0, 9000.0, 15000.0, 25000.0, 30000.0, 40000.0)
MATERIALS = (("Si", 2.33), ("Au", 19.32), ("Al", 2.70), ("CH", 1.05), ("Be", 1.85), ("SiO2", 2.2))
# the synthetic database of synthetic_xrayref.py (energies on and near its edges)
SYN_FORMULAS = ("C", "CH", "H2O", "SiO2", "C8H8O", "Au", "CuO", "(CH2)3Si2O", "Au0.25Cu0.75")
SYN_ZS = (1, 6, 14, 29, 79)
SYN_ENERGIES = (300.0, 2000.0, 8000.0, 8979.0, 9000.0, 11919.0, 25000.0, 30000.0)
SYN_MATERIALS = (("Si", 2.33), ("Au", 19.32), ("CH", 1.05), ("SiO2", 2.2), ("CuO", 6.3))


def _fake_sqlalchemy():
    class Col:
        def __init__(self, table, name):
            self.table, self.name = table, name

        def __eq__(self, other):
            return (self.name, other)

        __hash__ = object.__hash__

    class Engine:
        def __init__(self, url):
            self.path = url.split("sqlite:///", 1)[1]
            self.db = sqlite3.connect(f"file:{self.path}?mode=ro", uri=True)

        def connect(self):
            return self

    class MetaData:
        def __init__(self):
            self.tables = {}

        def reflect(self, bind):
            self.tables = {n: (bind, n) for (n,) in bind.db.execute("select name from sqlite_master where type='table'")}

    class Query:
        def __init__(self, engine, cls):
            self.engine, self.cls, self.where = engine, cls, []

        def filter(self, pred):
            self.where.append(pred)
            return self

        def all(self):
            table = self.cls.__table_name__
            sql = f"select * from {table}"
            if self.where:
                sql += " where " + " and ".join(f"{c} = ?" for c, _ in self.where)
            cur = self.engine.db.execute(sql, [v for _, v in self.where])
            names = [d[0] for d in cur.description]
            rows = []
            for r in cur.fetchall():
                o = object.__new__(self.cls)
                o.__dict__.update(zip(names, r))
                rows.append(o)
            return rows

    class Session:
        def __init__(self, engine):
            self.engine = engine

        def query(self, cls):
            return Query(self.engine, cls)

    class Registry:
        def map_imperatively(self, cls, table):
            engine, name = table
            cls.__table_name__ = name
            for (col,) in [(row[1],) for row in engine.db.execute(f"pragma table_info({name})")]:
                setattr(cls, col, Col(name, col))

    sa = types.ModuleType("sqlalchemy")
    sa.MetaData = MetaData
    sa.create_engine = lambda url, **kw: Engine(url)
    orm = types.ModuleType("sqlalchemy.orm")
    orm.sessionmaker = lambda bind, **kw: (lambda: Session(bind))
    orm.registry = Registry
    pool = types.ModuleType("sqlalchemy.pool")
    pool.SingletonThreadPool = object
    dialects = types.ModuleType("sqlalchemy.dialects")
    sqlite_d = types.ModuleType("sqlalchemy.dialects.sqlite")
    sa.orm, sa.pool, sa.dialects, dialects.sqlite = orm, pool, dialects, sqlite_d
    return {"sqlalchemy": sa, "sqlalchemy.orm": orm, "sqlalchemy.pool": pool,
            "sqlalchemy.dialects": dialects, "sqlalchemy.dialects.sqlite": sqlite_d}


def _cases(plasma, plasma_sample, xray_delta_beta, xdb, formulas, zs, energies, materials) -> dict:
    out = {"formula": {}, "Z": {}, "delta_beta": {}}
    for f in formulas:
        out["formula"][f] = {repr(e): [float(v) for v in plasma.compound_scattering_factors(f, e)]
                             for e in energies}
    for z in zs:
        ps = object.__new__(plasma_sample.PlasmaSample)
        ps.formula, ps.Z = None, z
        out["Z"][str(z)] = {repr(e): [float(v) for v in ps._scattering_factors(e)] for e in energies}
    for mat, rho in materials:
        out["delta_beta"][f"{mat}@{rho}"] = {repr(e): [float(v) for v in xray_delta_beta(mat, rho, e, xdb=xdb)]
                                             for e in energies}
    return out


def main(root: Path) -> None:
    import tempfile
    sys.modules.update(_fake_sqlalchemy())
    sys.path[:0] = [str(root / "big-wave"), str(root / "nist_lookup"), str(Path(__file__).resolve().parent)]
    import plasma
    import plasma_sample
    from nist_lookup.xraydb import xrayDB
    from nist_lookup.xraydb_plugin import Scatterer, xray_delta_beta
    import synthetic_xrayref

    real = xrayDB()
    out = {"real": _cases(plasma, plasma_sample, xray_delta_beta, real, FORMULAS, ZS, ENERGIES, MATERIALS)}
    with tempfile.TemporaryDirectory() as tmp:
        syn = xrayDB(str(synthetic_xrayref.build(Path(tmp) / "synthetic.db")))
        plasma._lazy_import_xraydb()
        plasma._Scatterer = lambda symbol, energy: Scatterer(symbol, energy, syn)
        plasma._xrayDB = lambda: syn
        plasma._scatterer_cache.clear()
        out["synthetic"] = _cases(plasma, plasma_sample, xray_delta_beta, syn, SYN_FORMULAS, SYN_ZS,
                                  SYN_ENERGIES, SYN_MATERIALS)
    OUT.write_text(json.dumps(out, indent=1) + "\n")
    print(f"wrote {OUT}")


if __name__ == "__main__":
    sys.path.insert(0, str(Path(__file__).resolve().parent))
    from _refroot import reference_root
    main(reference_root())
