"""Detector metadata against big-wave's own (tests/golden/detector_meta.json, written by
tests/golden/make_detector_meta_golden.py from big-wave's square_and_downsample_2d): output
shape, effective geometry (Fresnel magnification included), legacy count map and pixel ratios,
area_v1 coverage, and the RuntimeWarnings. The metadata is host arithmetic, so no GPU is needed;
the image itself is compared on the GPU (test_gpu_parity.py)."""
import importlib
import json
import warnings
from pathlib import Path

import pytest

GOLDEN = json.loads((Path(__file__).parent / "golden" / "detector_meta.json").read_text())


@pytest.mark.parametrize("case", GOLDEN, ids=[c["name"] for c in GOLDEN])
def test_detector_metadata_matches_bigwave(rs, case):
    prop = importlib.import_module("3d_ravesim_gb300.propagation")
    kw = dict(case["params"])
    nx, ny = kw["nx"], kw["ny"]
    p = rs.SimParams(N=nx * ny, wl=1e-10, chunk_size=nx, detector_size=kw["detector_size_x"],
                     detector_integrator=case["integrator"], **kw)
    if "fresnel" in case:
        p.configure_fresnel_detector(*case["fresnel"])
    with warnings.catch_warnings(record=True) as caught:
        warnings.simplefilter("always")
        geo = prop._detector_geometry(p, case["current_z"])
        meta = prop._detector_metadata(p, geo)
    assert meta.pop("output_storage") == "device"
    # a JSON round trip, as the golden took: tuples become lists, floats keep every bit
    assert json.loads(json.dumps(meta)) == case["metadata"]
    assert [str(w.message) for w in caught if issubclass(w.category, RuntimeWarning)] == case["warnings"]


def test_golden_covers_both_integrators_and_fresnel_scaling():
    kinds = {(c["integrator"], c["metadata"]["effective_geometry"]["fresnel_scaled"]) for c in GOLDEN}
    assert kinds == {("area_v1", False), ("area_v1", True), ("legacy_fastwave", False), ("legacy_fastwave", True)}
    assert any(c["warnings"] for c in GOLDEN if c["integrator"] == "area_v1")
    assert any(c["metadata"]["count_map"]["non_uniform"] for c in GOLDEN if c["integrator"] == "legacy_fastwave")
