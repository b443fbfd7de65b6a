"""This package's setup_simulation against directories that big-wave's own setup_simulation
prepared from the same inputs (tests/golden/setup_ref*/, written by
tests/golden/make_setup_golden.py from the configurations in tests/golden/setup_cases.py):
config.yaml, computed.yaml (all but the provenance revision) and every subconfig.yaml must hold
the same values, and the element grids must be copied alike.

The delta/beta tables and plasma scattering factors come from the Chantler database. Where
nist_lookup's xrayref.db is not found, the lookups are answered from the fixture's own values
(the Chantler arithmetic is pinned bit for bit by test_chantler_host.py), so everything else of
the setup is still checked."""
import builtins
import importlib
import json
import sys
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLDEN))
from setup_cases import CASES  # noqa: E402


@pytest.fixture(scope="module")
def mods():
    names = ("prepare", "config", "chantler", "propagation", "multisim")
    return {n: importlib.import_module(f"3d_ravesim_gb300.{n}") for n in names}


def _fixture_lookups(ref: Path, cfg):
    """Chantler answers recorded in a prepared directory's subconfigs."""
    db, factors = {}, {}
    for sub in sorted(ref.glob("[0-9]" * 8)):
        s = cfg.load(sub / "subconfig.yaml")
        e = float(s["energy"])
        for (mat, rho), (d, b) in s["deltabeta_table"]:
            db[(mat, float(rho), e)] = (d, b)
        for entry in s.get("plasma_optics_table") or []:
            factors[(entry["formula"], e)] = tuple(entry[k] for k in ("f1bar", "f2eff_bar", "zbar", "z2bar"))
    return db, factors


@pytest.fixture
def chantler_answers(mods, monkeypatch):
    ch = mods["chantler"]
    try:
        ch.database_path()
        return lambda ref: None
    except FileNotFoundError:
        pass

    def install(ref: Path):
        db, factors = _fixture_lookups(ref, mods["config"])
        monkeypatch.setattr(ch, "xray_delta_beta", lambda m, rho, e, photo_only=False: (*db[(m, rho, e)], None))
        monkeypatch.setattr(ch, "compound_scattering_factors", lambda f, e: factors[(f, e)])
        monkeypatch.setattr(ch, "element_scattering_factors", lambda z, e: factors[(None, e)])
    return install


def _tree(path: Path) -> list[str]:
    return sorted(str(p.relative_to(path)) for p in path.rglob("*"))


@pytest.mark.parametrize("name", sorted(CASES))
def test_setup_simulation_writes_the_reference_directory(mods, chantler_answers, tmp_path, name):
    cfg, prep = mods["config"], mods["prepare"]
    ref = GOLDEN / name
    chantler_answers(ref)
    sim = prep.setup_simulation(CASES[name](), ref, tmp_path / "out")
    assert sim.parent.parent.parent == tmp_path / "out" and len(sim.name) == 21  # <year>/<month>/<stamp>
    assert _tree(sim) == _tree(ref)
    for grid in ref.glob("*.npy"):
        assert np.array_equal(np.load(sim / grid.name), np.load(grid))
    assert cfg.load(sim / "config.yaml") == cfg.load(ref / "config.yaml")
    got, want = cfg.load(sim / "computed.yaml"), cfg.load(ref / "computed.yaml")
    assert got.pop("provenance")["algorithm_version"] == want.pop("provenance")["algorithm_version"]
    assert got == want
    for sub in ref.glob("[0-9]" * 8):
        assert cfg.load(sim / sub.name / "subconfig.yaml") == cfg.load(sub / "subconfig.yaml"), sub.name


def test_prepared_plasma_directory_runs_without_the_database(mods, tmp_path):
    """run_single_simulation takes the plasma factors recorded at setup (subconfig's
    plasma_optics_table) when the elements carry none."""
    cfg, ms = mods["config"], mods["multisim"]
    ref = GOLDEN / "setup_ref_plasma"
    dct = cfg.load(ref / "config.yaml")
    sub = cfg.load(ref / "00000001" / "subconfig.yaml")
    elements = [cfg.parse_optical_element(el, ref) for el in dct["elements"]]
    ms.use_plasma_optics_table(elements, sub["plasma_optics_table"])
    plasma = [el for el in elements if type(el).__name__ == "PlasmaSample"]
    assert [el.formula for el in plasma] == ["CH", None]
    for el, entry in zip(plasma, sub["plasma_optics_table"]):
        assert el.scattering_factors == tuple(entry[k] for k in ("f1bar", "f2eff_bar", "zbar", "z2bar"))
        assert el._scattering_factors(float(sub["energy"])) == el.scattering_factors
    with pytest.raises(ValueError, match="2 plasma_sample elements"):
        ms.use_plasma_optics_table([cfg.parse_optical_element(el, ref) for el in dct["elements"]],
                                   sub["plasma_optics_table"][:1])


def test_save_and_exit_cuts_the_run(mods):
    cfg = mods["config"]
    ref = GOLDEN / "setup_ref_exit"
    dct, computed = cfg.load(ref / "config.yaml"), cfg.load(ref / "computed.yaml")
    assert [el["type"] for el in dct["elements"]] == ["sample"]
    assert dct["sim_params"]["z_detector"] == 0.6 and dct["save_final_u_vectors"] is True
    assert len(computed["cutoff_angles"]) == 4  # the angles still cover the full element list and the marker


def test_compute_cutoff_angles_rules(mods):
    prop = mods["propagation"]
    kw = dict(detector_size=1e-5, dx=1e-7, energy_range=(10e3, 20e3), z_source=0.0, z_distances=[0.5, 0.6],
              element_heights=[1e-3, 1e-3], z_detector=1.0, max_x=2e-6)
    angles, widths = prop.compute_cutoff_angles(**kw)
    assert angles == sorted(angles) and len(angles) == len(widths) == 3
    slope0 = (5e-6 + 2e-6) / 1.0
    assert angles[0] == float(np.arctan(slope0)) and widths[0] == 2e-6 + slope0 * 0.5
    # the detector directly behind the last element: its leg keeps the previous slope
    a2, w2 = prop.compute_cutoff_angles(**{**kw, "z_detector": 0.601})
    assert a2[-1] == a2[-2] and w2[-1] == w2[-2] + np.tan(a2[-2]) * 1e-3
    with pytest.raises(ValueError, match="same z coordinate as the detector"):
        prop.compute_cutoff_angles(**{**kw, "z_distances": [0.5, 1.0], "z_detector": 1.0})
    with pytest.raises(ValueError, match="sampled to coarsly"):
        prop.compute_cutoff_angles(**{**kw, "dx": 1.0})


def test_resolve_sim_params_rules(mods):
    cfg = mods["config"]
    base = {"sim_params": {"N": 1024 * 512, "ny": 512, "dx": 1e-7, "z_detector": 1.0, "detector_pixel_size_x": 1e-6,
                           "detector_pixel_size_y": 1e-6}, "dtype": "c8"}
    sim = cfg.resolve_sim_params(base)
    # auto: a quarter of 6 GB at 256 + 4*8 bytes per point, capped at 256 rows
    assert sim["nx"] == 1024 and sim["chunk_size"] == 256 * 1024 and sim["memory_budget_gb"] == 6.0
    assert sim["fft2_backend"] == "scipy_in_memory" and sim["detector_integrator"] == "area_v1"
    small = cfg.resolve_sim_params({**base, "runtime": {"big_wave": {"memory_budget_gb": 0.27}}})
    assert small["chunk_size"] == int(0.27 * 1024 ** 3 * 0.25 // (1024 * 288)) * 1024
    explicit = cfg.resolve_sim_params({**base, "sim_params": {**base["sim_params"], "chunk_size": 3000}})
    assert explicit["chunk_size"] == 2 * 1024  # rounded down to whole rows
    for bad, msg in (({"dtype": "c4"}, "dtype must be"),
                     ({"runtime": {"big_wave": {"memory_budget_gb": "x"}}}, "positive number"),
                     ({"runtime": {"big_wave": {"memory_budget_gb": -1}}}, "positive and finite"),
                     ({"runtime": {"big_wave": {"fft2_backend": "cufft"}}}, "unsupported fft2_backend"),
                     ({"runtime": {"big_wave": {"fft2_backend": "bfpy_ooc"}}}, "requires use_disk_vector"),
                     ({"runtime": {"big_wave": {"detector_integrator": "x"}}}, "unsupported detector_integrator"),
                     ({"runtime": {"big_wave": {"save_debug_wavefields": "yes"}}}, "must be a boolean"),
                     ({"runtime": {"big_wave": {"chunk_size": 1.5}}}, "positive integer or 'auto'"),
                     ({"dtype": "c16", "runtime": {"big_wave": {"chunk_size": 1 << 40, "memory_budget_gb": 0.28}}},
                      "P0 memory gate")):
        with pytest.raises(ValueError, match=msg):
            cfg.resolve_sim_params({**base, **bad})


ERRORS = json.loads((GOLDEN / "setup_errors.json").read_text())


@pytest.mark.parametrize("name", sorted(ERRORS))
def test_setup_simulation_rejects_like_bigwave(mods, chantler_answers, tmp_path, name):
    """The inputs big-wave's setup_simulation rejects raise the same exception type and message
    here, and leave no simulation directory behind."""
    from setup_cases import error_cases
    kind, message = ERRORS[name]
    chantler_answers(GOLDEN / "setup_ref")
    with pytest.raises(getattr(builtins, kind)) as exc:  # setup_ref_exit/ holds both grids
        mods["prepare"].setup_simulation(error_cases()[name], GOLDEN / "setup_ref_exit", tmp_path / "out")
    assert str(exc.value) == message
    assert not (tmp_path / "out").exists()


RULES = json.loads((GOLDEN / "setup_rules.json").read_text())


def test_compute_cutoff_angles_matches_bigwave_bit_for_bit(mods):
    """60 seeded geometries (0-3 elements, the detector right behind the last element in some)
    through big-wave's compute_cutoff_angles and this package's: the same angles and beam
    half-widths to the last bit, or the same exception."""
    prop = mods["propagation"]
    for case in RULES["compute_cutoff_angles"]:
        args = {**case["args"], "energy_range": tuple(case["args"]["energy_range"])}
        if "error" in case:
            with pytest.raises(getattr(builtins, case["error"][0])) as exc:
                prop.compute_cutoff_angles(**args)
            assert str(exc.value) == case["error"][1]
            continue
        angles, widths = prop.compute_cutoff_angles(**args)
        assert angles == case["angles"] and widths == case["widths"], case["args"]


def test_resolve_sim_params_matches_bigwave(mods):
    """40 seeded sim_params / runtime requests (explicit and auto chunk sizes, budgets, dtypes)
    resolved as big-wave resolves them, or rejected with its message."""
    cfg = mods["config"]
    for case in RULES["resolve_sim_params"]:
        if "error" in case:
            with pytest.raises(getattr(builtins, case["error"][0])) as exc:
                cfg.resolve_sim_params(case["dct"])
            assert str(exc.value) == case["error"][1]
            continue
        assert cfg.resolve_sim_params(case["dct"]) == case["out"], case["dct"]
