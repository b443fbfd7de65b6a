"""Prepared-simulation parsing on the host (big-wave/config.py:45-520): a directory in
setup_simulation's layout read back into SimParams, Samples, the point source and the
delta-beta table, and the reference's validation errors."""
import importlib
import warnings
from pathlib import Path

import numpy as np
import pytest

from prepared_dir import write_prepared_dir

GOLDEN = Path(__file__).resolve().parent / "golden" / "history_golden.npz"


@pytest.fixture(scope="module")
def cfg():
    return importlib.import_module("3d_ravesim_gb300.config")


@pytest.fixture(scope="module")
def yio():
    return importlib.import_module("3d_ravesim_gb300.yaml_io")


def test_prepared_directory_parses(cfg, yio, tmp_path):
    g = np.load(GOLDEN)
    sim = write_prepared_dir(yio, tmp_path, g)
    dct = cfg.load(sim / "config.yaml")
    p = cfg.parse_sim_params(dct["sim_params"])
    assert (p.nx, p.ny, p.N, p.chunk_size) == (64, 64, 4096, 512) and p.is_2d
    assert p.dx == 5e-07 and p.detector_size_y == 2e-05 and p.wl == 0.0
    els = [cfg.parse_optical_element(e, sim) for e in dct["elements"]]
    assert [e.z_start for e in els] == [0.5, 0.56]
    assert isinstance(els[0].grid, np.memmap) and els[0].grid.shape == (4, 66, 66)
    np.testing.assert_array_equal(np.asarray(els[1].grid), g["run_grid2"])
    assert els[0].materials[0].mat == "W" and els[0].materials[0].density == 19.3
    sub = cfg.load(sim / "00000000" / "subconfig.yaml")
    src = cfg.parse_source(sub["source"])
    assert (src.x, src.y, src.z) == (1e-06, 0.0, 0.0)
    table = cfg.parse_deltabeta_table(sub["deltabeta_table"])
    assert table[0][0].mat == "W" and table[0][1] == np.complex128(4.2e-6 + 1.9e-7j)
    assert cfg.get_runtime_big_wave(dct) == {"history": {"storage": "memory"}}
    assert cfg.parse_dtype(dct) == np.complex64
    assert [float(a) for a in cfg.load(sim / "computed.yaml")["cutoff_angles"]] == list(g["run_params"][:3])


def test_parser_errors(cfg, tmp_path):
    with pytest.raises(KeyError, match="does not exist"):
        cfg.get_float({"a": 1}, ["b"])
    with pytest.raises(AssertionError):
        cfg.get_int({"N": 4096.0}, ["N"])
    with pytest.raises(AssertionError):
        cfg.get_float({"dx": "1e-6"}, ["dx"])
    assert cfg.get_bool_value(" Yes ", "f") is True and cfg.get_bool_value("0", "f") is False
    with pytest.raises(ValueError):
        cfg.get_bool_value(2, "f")
    with pytest.raises(ValueError):
        cfg.parse_dtype({"dtype": "c32"})
    assert cfg.parse_dtype({}) == np.complex128
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        assert cfg.field_dtype({"dtype": "c16"}) == np.complex64
    assert any("complex64" in str(x.message) for x in w)
    with pytest.raises(NotImplementedError):
        cfg.parse_optical_element({"type": "grating"}, tmp_path)
    with pytest.raises(ValueError):
        cfg.parse_optical_element({"type": "lens"}, tmp_path)
    with pytest.raises(NotImplementedError):
        cfg.parse_source({"type": "vector", "input_path": "u.npy", "z": 0.0})
    np.save(tmp_path / "f.npy", np.zeros((2, 4, 4), np.float32))
    with pytest.raises(AssertionError):
        cfg.parse_optical_element({"type": "sample", "grid_path": "f.npy", "materials": [], "z_start": 0.1,
                                   "pixel_size_x": 1e-6, "pixel_size_z": 1e-6, "x_positions": [0.0]}, tmp_path)


def test_yaml_reads_tagged_tuples(yio):
    text = ("deltabeta_table:\n  - !!python/tuple\n    - !!python/tuple\n      - W\n      - 19.3\n"
            "    - !!python/tuple\n      - 4.2e-06\n      - 1.9e-07\nenergy: 20000.0\n")
    assert yio.loads(text) == {"deltabeta_table": [[["W", 19.3], [4.2e-06, 1.9e-07]]], "energy": 20000.0}
