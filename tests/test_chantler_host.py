"""The package's own Chantler lookup against big-wave's and nist_lookup's outputs
(tests/golden/chantler_golden.json, written by tests/golden/make_chantler_golden.py running the
reference modules): plasma scattering factors for formulas (big-wave/plasma.py:241-266) and bare
Z (big-wave/plasma_sample.py:68-83), and xray_delta_beta (nist_lookup xraydb_plugin.py:136-185).
The synthetic database is rebuilt here from tests/golden/synthetic_xrayref.py, so those cases
always run; the real-database cases run where nist_lookup's xrayref.db can be found."""
import importlib
import json
import sys
from pathlib import Path

import pytest

GOLDEN_DIR = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLDEN_DIR))
import synthetic_xrayref  # noqa: E402

GOLDEN = json.loads((GOLDEN_DIR / "chantler_golden.json").read_text())


@pytest.fixture(scope="module")
def ch():
    return importlib.import_module("3d_ravesim_gb300.chantler")


@pytest.fixture(scope="module")
def syn_db(ch, tmp_path_factory):
    path = synthetic_xrayref.build(tmp_path_factory.mktemp("xrayref") / "synthetic.db")
    ch.set_database(path)
    yield path
    ch.set_database(None)


def _check_all(ch, ps_cls, gold):
    for f, by_e in gold["formula"].items():
        for e, want in by_e.items():
            assert list(ch.compound_scattering_factors(f, float(e))) == want, (f, e)
            ps = object.__new__(ps_cls)
            ps.formula, ps.Z, ps.scattering_factors = f, 0, None
            assert list(ps._scattering_factors(float(e))) == want, (f, e)
    for z, by_e in gold["Z"].items():
        for e, want in by_e.items():
            ps = object.__new__(ps_cls)
            ps.formula, ps.Z, ps.scattering_factors = None, int(z), None
            assert list(ps._scattering_factors(float(e))) == want, (z, e)
    for key, by_e in gold["delta_beta"].items():
        mat, rho = key.split("@")
        for e, want in by_e.items():
            assert list(ch.xray_delta_beta(mat, float(rho), float(e))) == want, (key, e)


def test_synthetic_database_matches_reference_bit_for_bit(ch, syn_db):
    ps_cls = importlib.import_module("3d_ravesim_gb300.plasma_sample").PlasmaSample
    _check_all(ch, ps_cls, GOLDEN["synthetic"])
    assert "plasma" not in sys.modules and "nist_lookup.xraydb" not in sys.modules


def test_real_database_matches_reference_bit_for_bit(ch):
    ch.set_database(None)
    try:
        ch.database_path()
    except FileNotFoundError:
        pytest.skip("nist_lookup's xrayref.db is not installed here (set RAVESIM_XRAYREF_DB)")
    ps_cls = importlib.import_module("3d_ravesim_gb300.plasma_sample").PlasmaSample
    _check_all(ch, ps_cls, GOLDEN["real"])


@pytest.mark.parametrize("formula,want", [
    ("H2O", {"H": 2.0, "O": 1}),
    ("Mn(SO4)2(H2O)7", {"Mn": 1, "S": 2.0, "O": 15.0, "H": 14.0}),
    ("La1.9Sr0.1CuO4", {"La": 1.9, "Sr": 0.1, "Cu": 1, "O": 4.0}),
    ("CaMg(CO3)2", {"Ca": 1, "Mg": 1, "C": 2.0, "O": 6.0}),
    ("((CH2)2O)3", {"C": 6.0, "H": 12.0, "O": 3.0}),
    ("", {}),
])
def test_formula_counts_in_order_of_appearance(ch, formula, want):
    got = ch.chemparse(formula)
    assert list(got.items()) == list(want.items())


@pytest.mark.parametrize("bad", ["2H", "Xx", "H(", "H)", "h2o", "(H2O", "H2O)", "H-2"])
def test_malformed_formulas_raise(ch, bad):
    with pytest.raises(ValueError):
        ch.chemparse(bad)


def test_empty_composition_and_missing_database(ch, syn_db, tmp_path):
    with pytest.raises(ValueError, match="empty composition"):
        ch.compound_scattering_factors("", 8000.0)
    ps_mod = importlib.import_module("3d_ravesim_gb300.plasma_sample")
    ch.set_database(tmp_path / "absent.db")
    try:
        ps = object.__new__(ps_mod.PlasmaSample)
        ps.formula, ps.Z, ps.scattering_factors = "CH", 0, None
        with pytest.raises((RuntimeError, FileNotFoundError)):
            ps._scattering_factors(8000.0)
    finally:
        ch.set_database(syn_db)
