"""The host restatement of big-wave's plasma delta/beta model (plasma_sample.
plasma_delta_beta_grid_multi) against big-wave's own outputs (tests/golden/plasma_db_golden.npz,
written by tests/golden/make_plasma_db_golden.py), edge cases included; and the oracle's
copy of the same model. The in-kernel evaluation is compared on the GPU (test_gpu_parity.py)."""
import importlib
from pathlib import Path

import numpy as np
import pytest

G = np.load(Path(__file__).parent / "golden" / "plasma_db_golden.npz")


def test_plasma_model_matches_bigwave():
    ps = importlib.import_module("3d_ravesim_gb300.plasma_sample")
    grids = (G["ne"], G["ni"], G["te"], G["zstar"])
    for i, sc in enumerate(G["scalars"]):
        for j, e in enumerate(G["energies"]):
            d, b, a = ps.plasma_delta_beta_grid_multi(*grids, *sc, float(e))
            np.testing.assert_allclose(d, G[f"delta_{i}_{j}"], rtol=1e-15, atol=0)
            np.testing.assert_allclose(b, G[f"beta_{i}_{j}"], rtol=1e-15, atol=0)
            np.testing.assert_allclose(a, G[f"atlen_{i}_{j}"], rtol=1e-15, atol=0)
    # the edge rows are in the golden: a vacuum corner has delta = beta = 0 and no attenuation
    assert G["delta_0_0"][0, 0] == 0.0 and np.isinf(G["atlen_0_0"][0, 0])


def test_oracle_plasma_model_matches_bigwave(oracle):
    ps = importlib.import_module("3d_ravesim_gb300.plasma_sample")
    consts = ps.codata_constants()
    grids = (G["ne"], G["ni"], G["te"], G["zstar"])
    for i, sc in enumerate(G["scalars"]):
        for j, e in enumerate(G["energies"]):
            with np.errstate(divide="ignore", invalid="ignore"):  # zstar / zbar where zbar = 0, discarded
                d, b = oracle.plasma_delta_beta_grid_multi(*grids, *sc, float(e), *consts)
            np.testing.assert_allclose(d, G[f"delta_{i}_{j}"], rtol=1e-15, atol=0)
            np.testing.assert_allclose(b, G[f"beta_{i}_{j}"], rtol=1e-15, atol=0)


def test_plasma_model_rejects_bad_input():
    ps = importlib.import_module("3d_ravesim_gb300.plasma_sample")
    z = np.zeros((2, 2))
    with pytest.raises(ValueError, match="identical shapes"):
        ps.plasma_delta_beta_grid_multi(z, z, z, np.zeros((2, 3)), 1.0, 0.1, 1.0, 1.0, 1e4)
    with pytest.raises(ValueError, match="energy must be positive"):
        ps.plasma_delta_beta_grid_multi(z, z, z, z, 1.0, 0.1, 1.0, 1.0, 0.0)
