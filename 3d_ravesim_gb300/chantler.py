"""Chantler anomalous scattering factors, read from nist_lookup's xrayref.db with sqlite3.

big-wave takes the per-energy scalars of a plasma (f1bar, f2eff_bar, zbar, z2bar) and the
delta/beta of neutral materials from nist_lookup, whose database layer needs SQLAlchemy. This
module restates the arithmetic on the same database file with the standard library:

* one tabulated column at one energy (nist_lookup/nist_lookup/xraydb.py:382-414): the window of
  table points [last <= E - 5, last <= E + 6); f1 by a smoothing spline (s = 1) through it, the
  other columns by linear interpolation in log-log;
* an element's scatterer (nist_lookup/nist_lookup/xraydb_plugin.py:116-133): f1 + Z, f2,
  mu_photo, mu_total, the atomic number and molar mass from the `elements` table;
* compound factors (big-wave/plasma.py:241-266) and the single-element fallback of
  big-wave/plasma_sample.py:68-83;
* the refractive-index decrements of a material (nist_lookup/nist_lookup/xraydb_plugin.py:136-185);
* chemical formulas parsed to element counts, in order of first appearance (the contract of
  nist_lookup/nist_lookup/chemparser.py: element symbols, integer or decimal counts, nested
  parentheses).

The database is found at $RAVESIM_XRAYREF_DB, else beside an installed `nist_lookup` package
(found without importing it), else wherever `set_database` points.
"""
from __future__ import annotations

import functools
import importlib.util
import json
import math
import os
import re
import sqlite3
import threading
from pathlib import Path
from typing import NamedTuple

import numpy as np

ENV = "RAVESIM_XRAYREF_DB"
_override: Path | None = None
_local = threading.local()


def set_database(path) -> None:
    """Use the Chantler database at `path` (None: back to the environment / package search)."""
    global _override
    _override = None if path is None else Path(path)
    _local.__dict__.clear()
    _element_table.cache_clear()
    _elements.cache_clear()
    scatterer.cache_clear()


def database_path() -> Path:
    if _override is not None:
        return _override
    env = os.environ.get(ENV)
    if env:
        return Path(env)
    try:
        spec = importlib.util.find_spec("nist_lookup")
    except (ImportError, ValueError):
        spec = None
    for loc in (spec.submodule_search_locations or []) if spec else []:
        for cand in (Path(loc) / "xrayref.db", Path(loc) / "nist_lookup" / "xrayref.db"):
            if cand.is_file():
                return cand
    raise FileNotFoundError(
        f"nist_lookup's Chantler database (xrayref.db) was not found: set ${ENV}, install nist_lookup, "
        "or call chantler.set_database(path)")


def _conn() -> sqlite3.Connection:
    path = database_path()
    c = getattr(_local, "conn", None)
    if c is None or getattr(_local, "path", None) != path:
        if not path.is_file():
            raise FileNotFoundError(f"Chantler database '{path}' not found")
        c = sqlite3.connect(f"file:{path}?mode=ro", uri=True, check_same_thread=False)
        _local.conn, _local.path = c, path
    return c


# ------------------------------------------------------------------------- elements table
@functools.lru_cache(maxsize=None)
def _elements() -> tuple[dict, dict]:
    """({symbol: (Z, molar mass)}, {Z: symbol}) from the `elements` table."""
    by_sym, by_z = {}, {}
    for z, sym, mass in _conn().execute("select atomic_number, element, molar_mass from elements"):
        by_sym[sym] = (int(z), float(mass))
        by_z[int(z)] = sym
    return by_sym, by_z


def _element_row(symbol: str) -> tuple[int, float]:
    row = _elements()[0].get(symbol.title())
    if row is None:
        raise ValueError(f"element {symbol!r} is not in the Chantler database")
    return row


def atomic_number(symbol: str) -> int:
    return _element_row(symbol)[0]


def molar_mass(symbol: str) -> float:
    return _element_row(symbol)[1]


def atomic_symbol(z: int) -> str:
    sym = _elements()[1].get(int(z))
    if sym is None:
        raise ValueError(f"no element with atomic number {z} in the Chantler database")
    return sym


_symbol_cache: dict[int, str] = {13: "Al"}  # big-wave seeds its cache the same way (plasma.py:36)


def element_symbol(z: int) -> str:
    """Atomic symbol of Z (big-wave/plasma.py:58-64)."""
    z = int(z)
    if z not in _symbol_cache:
        _symbol_cache[z] = atomic_symbol(z)
    return _symbol_cache[z]


# ------------------------------------------------------------------------- Chantler columns
_COLUMNS = ("f1", "f2", "mu_photo", "mu_incoh", "mu_total")


@functools.lru_cache(maxsize=None)
def _element_table(symbol: str) -> dict:
    cols = ", ".join(("energy",) + _COLUMNS)
    row = _conn().execute(f"select {cols} from Chantler where element = ?", (symbol.title(),)).fetchone()
    if row is None:
        raise ValueError(f"element {symbol!r} has no Chantler table")
    return {name: np.array(json.loads(text)) for name, text in zip(("energy",) + _COLUMNS, row)}


def chantler_value(symbol: str, energy: float, column: str) -> float:
    """One Chantler column of `symbol` at `energy` [eV] (xraydb.py:382-414 for a scalar energy)."""
    from scipy.interpolate import UnivariateSpline
    if column == "mu":
        column = "mu_total"
    if column not in _COLUMNS:
        raise ValueError(f"unknown Chantler column {column!r}")
    tab = _element_table(symbol)
    e = np.array([float(energy)])
    te_all = tab["energy"]
    below = np.nonzero(te_all <= e[0])[0]
    if below.size == 0:
        raise ValueError(f"{energy} eV is below the Chantler table of {symbol}")
    last = int(below[-1])
    window = slice(max(0, last - 5), min(te_all.size, last + 6))
    te, ty = te_all[window], tab[column][window]
    if column == "f1":
        out = UnivariateSpline(te, ty, s=1)(e)
    else:
        out = np.exp(np.interp(np.log(e), np.log(te), np.log(ty)))
    return out[0]


class Scatterer(NamedTuple):
    """An element at one energy (xraydb_plugin.py:116-133); f1 includes Z."""
    symbol: str
    number: int
    mass: float
    f1: float
    f2: float
    mu_photo: float
    mu_total: float


@functools.lru_cache(maxsize=None)
def scatterer(symbol: str, energy: float) -> Scatterer:
    z, mass = _element_row(symbol)
    return Scatterer(symbol, z, mass, chantler_value(symbol, energy, "f1") + z,
                     chantler_value(symbol, energy, "f2"), chantler_value(symbol, energy, "mu_photo"),
                     chantler_value(symbol, energy, "mu_total"))


# ------------------------------------------------------------------------- formulas
_KNOWN = frozenset((
    "H He Li Be B C N O F Ne Na Mg Al Si P S Cl Ar K Ca Sc Ti V Cr Mn Fe Co Ni Cu Zn Ga Ge As Se Br "
    "Kr Rb Sr Y Zr Nb Mo Tc Ru Rh Pd Ag Cd In Sn Sb Te I Xe Cs Ba La Ce Pr Nd Pm Sm Eu Gd Tb Dy Ho Er "
    "Tm Yb Lu Hf Ta W Re Os Ir Pt Au Hg Tl Pb Bi Po At Rn Fr Ra Ac Th Pa U Np Pu Am Cm Bk Cf Es Fm Md "
    "No Lr Unq Unp Unh Uns D T").split())
_TOKEN = re.compile(r"(?P<name>[A-Z][a-z]*)|(?P<num>[0-9]+\.?[0-9]*(?:[eE][-+]?[0-9]+)?)|(?P<open>\()|(?P<close>\))")


def chemparse(formula: str) -> dict:
    """{symbol: count} of a chemical formula, symbols in order of first appearance.

    A count multiplies the element or parenthesised group before it (default 1); counts of
    nested groups multiply from the outside in. Unknown symbols, unbalanced parentheses and
    stray characters raise ValueError.
    """
    toks: list[tuple[str, object]] = []
    pos = 0
    while pos < len(formula):
        m = _TOKEN.match(formula, pos)
        if m is None:
            raise ValueError(f"unrecognized element or number in {formula!r} at {pos}")
        kind = m.lastgroup
        toks.append((kind, float(m.group()) if kind == "num" else m.group()))
        pos = m.end()
    toks.append(("end", None))
    i = 0

    def sequence():
        # items (an element or a parenthesised sequence), each with an optional count
        nonlocal i
        items = []
        while toks[i][0] in ("name", "open"):
            kind, val = toks[i]
            i += 1
            if kind == "open":
                val = sequence()
                if toks[i][0] != "close":
                    raise ValueError(f"expected ')' in {formula!r}")
                i += 1
            elif val not in _KNOWN:
                raise ValueError(f"'{val}' is not an element symbol ({formula!r})")
            count = 1
            if toks[i][0] == "num":
                count = toks[i][1]
                i += 1
            items.append((val, count))
        return items

    top = sequence()
    if toks[i][0] != "end":
        raise ValueError(f"expected end of input in {formula!r}")
    out: dict = {}

    def emit(items, weight):
        for val, count in items:
            w = weight * count
            if isinstance(val, str):
                out[val] = out.get(val, 0) + w
            else:
                emit(val, w)

    emit(top, 1)
    return out


# ------------------------------------------------------------------------- factors
def compound_scattering_factors(formula: str, energy: float) -> tuple[float, float, float, float]:
    """(f1bar, f2eff_bar, zbar, z2bar): atom-fraction averages over the formula's elements of
    f1 (+Z), f2 * mu_total / mu_photo, Z and Z^2 (big-wave/plasma.py:241-266)."""
    comp = chemparse(formula)
    total = float(sum(comp.values()))
    if total <= 0:
        raise ValueError(f"empty composition for formula {formula!r}")
    f1bar = f2eff_bar = zbar = z2bar = 0.0
    for symbol, count in comp.items():
        s = scatterer(symbol, energy)
        x = float(count) / total
        f1bar += x * s.f1
        f2eff_bar += x * s.f2 * (s.mu_total / s.mu_photo)
        zbar += x * s.number
        z2bar += x * (s.number ** 2)
    return f1bar, f2eff_bar, zbar, z2bar


def element_scattering_factors(z: int, energy: float) -> tuple[float, float, float, float]:
    """The single-element fallback of big-wave/plasma_sample.py:74-83 (no formula given)."""
    s = scatterer(element_symbol(z), energy)
    return s.f1, s.f2 * (s.mu_total / s.mu_photo), float(z), float(z) * float(z)


def xray_delta_beta(material: str, density: float, energy: float, photo_only: bool = False):
    """(delta, beta, attenuation length [cm]) of a material of `density` [g/cm^3] at `energy`
    [eV] (nist_lookup/nist_lookup/xraydb_plugin.py:136-185)."""
    from .plasma_sample import codata_constants
    import scipy.constants as consts
    planck_hc, r_e_cm = codata_constants()
    lamb_cm = 1.e-8 * planck_hc / energy
    parts = [(n, scatterer(sym, energy)) for sym, n in chemparse(material).items()]
    total_mass = delta = beta_photo = beta_total = 0
    for n, s in parts:
        weight = density * n * consts.Avogadro
        delta += weight * s.f1
        beta_photo += weight * s.f2
        beta_total += weight * s.f2 * (s.mu_total / s.mu_photo)
        total_mass += n * s.mass
    scale = lamb_cm * lamb_cm * r_e_cm / (2 * math.pi * total_mass)
    delta = delta * scale
    beta = (beta_photo if photo_only else beta_total) * scale
    return delta, beta, lamb_cm / (4 * math.pi * beta)
