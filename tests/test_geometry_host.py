"""SimParams geometry and the Nyquist helpers against big-wave's own values
(tests/golden/geometry.json, written by tests/golden/make_geometry_golden.py): plain,
Fresnel-scaled and cone-beam configurations over planes inside, at and beyond the detector,
with big-wave's error messages where it raises. Host arithmetic only; values compare exactly."""
import importlib
import json
from pathlib import Path

import pytest

G = json.loads((Path(__file__).parent / "golden" / "geometry.json").read_text())


def attempt(fn, *args):
    try:
        v = fn(*args)
        return list(v) if isinstance(v, tuple) else v
    except ValueError as e:
        return {"error": str(e)}


@pytest.mark.parametrize("cfg", G["configs"], ids=[c["name"] for c in G["configs"]])
def test_simparams_geometry_matches_bigwave(rs, cfg):
    p = rs.SimParams(**G["base"], **cfg["params"])
    if cfg["fresnel"] is not None:
        p.configure_fresnel_detector(*cfg["fresnel"])
    assert (p.get_dy(), p.nx, p.is_2d, p.use_fresnel_scaling) == (cfg["dy"], cfg["nx"], cfg["is_2d"],
                                                                   cfg["use_fresnel_scaling"])
    assert [p.get_detector_size_x(), p.get_detector_size_y()] == cfg["detector_size"]
    assert (p.fresnel_magnification, p.fresnel_effective_z) == (cfg["magnification"], cfg["effective_z"])
    planes, steps = G["planes"], G["steps"]
    assert [attempt(p.fresnel_transverse_scale, z) for z in planes] == cfg["scale"]
    assert [[attempt(p.effective_slice_dz, z, dz) for dz in steps] for z in planes] == cfg["slice_dz"]
    assert [attempt(p.effective_final_dz, z) for z in planes] == cfg["final_dz"]
    assert [attempt(p.effective_detector_geometry, z) for z in planes] == cfg["detector_geometry"]


def test_fresnel_configuration_errors_match_bigwave(rs):
    for case in G["bad_fresnel"]:
        p = rs.SimParams(**G["base"], use_fresnel_scaling=True)
        assert attempt(p.configure_fresnel_detector, *case["args"]) == case["result"]


def test_nyquist_helpers_match_bigwave():
    prop = importlib.import_module("3d_ravesim_gb300.propagation")
    results = [attempt(prop.grid_density_check_2d, *c["args"]) for c in G["nyquist"]]
    assert results == [c["result"] for c in G["nyquist"]]
    assert any(r is None for r in results) and any(r is not None for r in results)
    for c in G["max_dx"]:
        dx = prop.max_dx(*c["args"])
        assert dx == c["result"]
        dz, xs, n, wl = c["args"]
        prop.grid_density_check(dz, xs, n, dx, wl)  # the returned dx passes the check
