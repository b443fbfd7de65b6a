"""Prepared directories run end to end on the GPU against big-wave's own runs of them: big-wave's
setup_simulation prepared tests/golden/setup_ref_{plasma,fresnel,exit}/ (the same files this
package's setup_simulation writes, test_prepare_host.py) and big-wave's run_single_simulation ran
source 0 of each (tests/golden/setup_runs.npz, written by tests/golden/make_setup_golden.py).
Here multisim.run_single_simulation runs the same source on complex64 GPU fields:

* plasma: a voxel sample and two plasma samples, the legacy_fastwave detector; the plasma
  scattering factors come from the subconfig's plasma_optics_table (no Chantler database is
  needed where this runs);
* fresnel: the thin-sample Fresnel similarity frame, the detector larger than the grid;
* exit: the run ends at the save_and_exit marker and keeps the field (u_0000.npy).
"""
import importlib
import shutil
import sys
from pathlib import Path

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLDEN))
from setup_cases import CASES, RUN_CASES  # noqa: E402


@pytest.mark.parametrize("name", RUN_CASES)
def test_prepared_directory_runs_like_bigwave(rs, cuda, tmp_path, name):
    ms = importlib.import_module("3d_ravesim_gb300.multisim")
    runs = np.load(GOLDEN / "setup_runs.npz")
    sim = tmp_path / name
    shutil.copytree(GOLDEN / name, sim)
    outs = ms.run_single_simulation(sim, 0, tmp_path / "scratch", device=cuda)
    det = np.load(sim / "00000000" / "detected.npy")
    want = runs[f"{name}_detected"]
    assert det.shape == want.shape and det.dtype == np.float64
    np.testing.assert_array_equal(det[0], outs[0])
    # complex64 fields against big-wave's NumPy run (complex128 for the plasma case)
    assert rel_l2(det, want) < 2e-5, rel_l2(det, want)
    if f"{name}_u_sub" in runs:
        n = CASES[name]()["sim_params"]
        u = np.load(sim / "00000000" / "u_0000.npy")
        assert u.dtype == np.complex64 and u.shape == (n["N"],)
        assert rel_l2(u.reshape(n["ny"], n["nx"])[::4, ::4], runs[f"{name}_u_sub"]) < 2e-5
