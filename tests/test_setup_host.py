"""A simulation directory prepared by big-wave's own setup_simulation (tests/golden/setup_ref/,
written by tests/golden/make_setup_golden.py): this package draws the same source points and
energies from the multisource settings, and its parsers read every file of the directory."""
import importlib
from pathlib import Path

import numpy as np
import pytest

REF = Path(__file__).parent / "golden" / "setup_ref"


@pytest.fixture(scope="module")
def mods():
    return (importlib.import_module("3d_ravesim_gb300.multisim"), importlib.import_module("3d_ravesim_gb300.config"))


def test_source_points_match_bigwave_setup(mods):
    ms, cfg = mods
    config, computed = cfg.load(REF / "config.yaml"), cfg.load(REF / "computed.yaml")
    points = ms.sample_source_points(config["multisource"])
    assert points == computed["source_points"]
    for i, pt in enumerate(points):
        sub = cfg.load(REF / f"{i:08}" / "subconfig.yaml")
        assert sub["source"] == {"type": "point", "x": pt["x"], "y": pt["y"], "z": pt["z"]}
        assert sub["energy"] == pt["energy"]
    s = computed["source_sampling"]
    assert (s["x_mean"], s["x_sigma"], s["y_mean"], s["y_sigma"], s["seed"]) == (0.0, 2e-6, 0.0, 1e-6, 42)


def test_prepared_directory_parses(mods):
    ms, cfg = mods
    config, computed = cfg.load(REF / "config.yaml"), cfg.load(REF / "computed.yaml")
    p = cfg.parse_sim_params(config["sim_params"])
    assert (p.nx, p.ny, p.dx, p.get_dy(), p.z_detector, p.chunk_size) == (256, 256, 2e-7, 2e-7, 1.0, 256)
    assert p.detector_integrator == "area_v1" and not p.use_fresnel_scaling
    assert cfg.field_dtype(config) == np.complex64
    elements = [cfg.parse_optical_element(el, REF) for el in config["elements"]]
    assert len(elements) == 1 and elements[0].grid.shape == (4, 12, 12) and elements[0].grid.dtype == np.uint32
    assert [m.mat for m in elements[0].materials] == ["W", "Au"]
    assert len(computed["cutoff_angles"]) == len(elements) + 1 and all(a > 0 for a in computed["cutoff_angles"])
    for i in range(config["multisource"]["nr_source_points"]):
        sub = cfg.load(REF / f"{i:08}" / "subconfig.yaml")
        src = cfg.parse_source(sub["source"])
        assert (src.x, src.y, src.z) == (sub["source"]["x"], sub["source"]["y"], sub["source"]["z"])
        table = cfg.parse_deltabeta_table(sub["deltabeta_table"])
        assert [m.mat for m, _ in table] == ["W", "Au"]
        assert all(db.real > 0 and db.imag > 0 for _, db in table)


def test_source_sampling_checks_like_bigwave(mods):
    ms, _ = mods
    base = {"nr_source_points": 3, "energy_range": [15e3, 20e3], "x_range": [-1e-6, 1e-6], "z": 0.0, "seed": 1}
    with pytest.raises(ValueError, match="exactly two values"):
        ms.sample_source_points({**base, "y_range": [0.0]})
    with pytest.raises(ValueError, match="finite and increasing"):
        ms.sample_source_points({**base, "y_range": [1e-6, -1e-6]})
    with pytest.raises(ValueError, match="only supported for 2D"):
        ms.sample_source_points({**base, "y_range": [-1e-6, 1e-6]}, is_2d=False)
    pts = ms.sample_source_points(base)  # no y_range: every source on y = 0
    assert [p["y"] for p in pts] == [0.0] * 3 and all(15e3 <= p["energy"] < 20e3 for p in pts)
    e, inten = ms.kramers_spectrum()
    spec = ms.sample_source_points(base, spectrum=(e, inten))
    draw = ms.generate_energies_from_spectrum(e, inten, np.random.RandomState(1), (15e3, 20e3), 3)
    assert [p["energy"] for p in spec] == list(draw) and [p["x"] for p in spec] == [p["x"] for p in pts]
