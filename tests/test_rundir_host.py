"""Per-source run-directory files on the host: detected.npy byte-identical to big-wave's
_save_detector_outputs, point-source geometry equal to big-wave's (tests/golden/rundir_ref was
written by big-wave, tests/golden/make_rundir_golden.py), the YAML layout of the metadata files,
and the history-option checks (big-wave/multisim.py:43-70, 125-257)."""
import importlib
import json
import math
from pathlib import Path

import numpy as np
import pytest
import torch

REF = Path(__file__).resolve().parent / "golden" / "rundir_ref"


@pytest.fixture(scope="module")
def ms():
    return importlib.import_module("3d_ravesim_gb300.multisim")


@pytest.fixture(scope="module")
def yio():
    return importlib.import_module("3d_ravesim_gb300.yaml_io")


def test_detected_npy_bytes_match_bigwave(ms, tmp_path):
    images = np.load(REF / "detected_inputs.npy")
    ms.save_detector_outputs(tmp_path / "detected.npy", [im for im in images])
    assert (tmp_path / "detected.npy").read_bytes() == (REF / "detected.npy").read_bytes()
    # CUDA-tensor outputs take the same route through the host (CPU tensors stand in here)
    ms.save_detector_outputs(tmp_path / "d2.npy", [torch.from_numpy(im) for im in images])
    assert (tmp_path / "d2.npy").read_bytes() == (REF / "detected.npy").read_bytes()
    assert not list(tmp_path.glob("*.part"))


def test_detected_npy_errors(ms, tmp_path):
    with pytest.raises(ValueError):
        ms.save_detector_outputs(tmp_path / "d.npy", [])
    with pytest.raises(ValueError):
        ms.save_detector_outputs(tmp_path / "d.npy", [np.zeros((2, 3)), np.zeros((3, 2))])
    assert not (tmp_path / "d.npy").exists() and not list(tmp_path.glob("*.part"))


def test_point_source_geometry_matches_bigwave(ms):
    ref = json.loads((REF / "source_geometry.json").read_text())
    for (src, multi), out in zip(ref["inputs"], ref["outputs"]):
        assert ms.point_source_geometry_2d(src, multi) == out
    with pytest.raises(ValueError):
        ms.point_source_geometry_2d({"x": 0.0, "z": 0.0}, {"y_range": [-1e-6, 1e-6]})
    with pytest.raises(ValueError):
        ms.point_source_geometry_2d({"x": math.inf, "y": 0.0, "z": 0.0}, {})
    assert ms.get_sub_dir("/tmp/sim", 12) == Path("/tmp/sim/00000012")


def test_yaml_layout_and_round_trip(yio):
    meta = {"integrator": "area_v1", "version": 1, "streaming": True, "output_shape": [16, 16],
            "effective_geometry": {"dx": 5e-07, "current_z": 0.65, "fresnel_scaled": False},
            "coverage_area": {"min": 0.0, "max": 1.875e-12, "zero_pixels": 0}, "roi_yxyx": None,
            "phase_steps": 1, "name": "it's: quoted", "numeric_text": "1.5", "empty": [], "nested_list": [[1, 2], [3]],
            "maps": [{"a": 1, "b": "x"}, {"c": -.5}], "specials": [math.inf, -math.inf], "neg": -3}
    text = yio.dumps(meta)
    assert text.splitlines()[:8] == [
        "integrator: area_v1", "version: 1", "streaming: true", "output_shape:", "  - 16", "  - 16",
        "effective_geometry:", "  dx: 5e-07"]
    assert "roi_yxyx:\n" in text and "name: 'it''s: quoted'" in text and "numeric_text: '1.5'" in text
    assert "maps:\n  - a: 1\n    b: x\n  - c: -0.5\n" in text
    back = yio.loads(text)
    assert back == meta
    nan = yio.loads(yio.dumps({"v": math.nan}))["v"]
    assert math.isnan(nan)


def test_yaml_reads_other_block_styles(yio):
    text = "# comment\na: 1   # trailing\nb:\n- x\n- 'y z'\nc: [1, 2.5, true]\nd: {}\ne: ~\nf: \"q\\tq\"\n"
    assert yio.loads(text) == {"a": 1, "b": ["x", "y z"], "c": [1, 2.5, True], "d": {}, "e": None, "f": "q\tq"}


def test_history_options(ms, rs):
    p = rs.SimParams(N=64, nx=8, ny=8, dx=1e-6, dy=1e-6, z_detector=1.0, detector_size=8e-6,
                     detector_pixel_size_x=1e-6, detector_pixel_size_y=1e-6, wl=1e-10, chunk_size=8,
                     memory_budget_gb=1.0)
    o = ms.resolve_history_options({"downsample": 2, "roi": [0, 4, 0, 4]}, p, False)
    assert o == {"storage": "auto", "memory_budget_bytes": int(102.4 * 1024 ** 2), "max_frames": None,
                 "downsample": (2, 2), "roi": (0, 4, 0, 4)}
    assert ms.resolve_history_options(None, p, True)["storage"] == "hdf5"
    for bad in ({"bogus": 1}, {"storage": "disk"}, {"memory_budget_mb": -1}, {"max_frames": 0},
                {"downsample": [1, 0]}, {"roi": [0, 1, 2]}):
        with pytest.raises(ValueError):
            ms.resolve_history_options(bad, p, False)
    with pytest.raises(ValueError):
        ms.resolve_history_options({"storage": "memory"}, p, True)
