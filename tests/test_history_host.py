"""z-history on the host, against big-wave's own History (tests/golden/history_golden.npz was
written by big-wave/history.py through tests/golden/make_history_golden.py): the z-step rule,
ROI/downsample/metadata of a memory History, the analytic point-source frames, and the
validation errors."""
import importlib
import json
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden" / "history_golden.npz"


@pytest.fixture(scope="module")
def hm():
    return importlib.import_module("3d_ravesim_gb300.history")


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


def test_z_steps_match_bigwave(hm, golden):
    vals = golden["zsteps_values"]
    off = 0
    for (dz, hdz), n in zip(golden["zsteps_cases"], golden["zsteps_lengths"]):
        mine = hm._history_z_steps(float(dz), float(hdz))
        np.testing.assert_array_equal(mine, vals[off:off + n])
        off += n


def test_z_steps_match_bigwave_broadly(hm):
    """186 (dz, hist_dz) pairs from big-wave's own rule (tests/golden/make_history_zsteps_golden.py):
    exact and inexact multiples, tails just above and below half a step, dz below one step."""
    import json
    from pathlib import Path
    cases = json.loads((Path(__file__).parent / "golden" / "history_zsteps.json").read_text())
    assert len(cases) > 150
    for c in cases:
        z = hm._history_z_steps(c["dz"], c["hist_dz"])
        assert z.dtype == np.float64 and z.tolist() == c["z"], (c["dz"], c["hist_dz"])


def test_memory_history_matches_bigwave(hm, golden):
    h = hm.History(roi=(1, 9, 2, 11), downsample=(2, 3))
    for i, f in enumerate(golden["mem_frames_in"]):
        h.push(f.copy(), 0.1 * (i + 1))
    np.testing.assert_array_equal(h.get_history(), golden["mem_history"])
    np.testing.assert_array_equal(np.array(h.get_z()), golden["mem_z"])
    assert json.dumps(h.metadata(), sort_keys=True) == str(golden["mem_metadata"])
    assert not h.is_streaming and len(h) == 5


def test_analytic_source_frames_match_bigwave(rs, hm, golden):
    """The first frames of the recorded run are PointSource's analytic history (host FP64,
    big-wave/history.py:348-367)."""
    a0, a1, a2, wl, hdz = golden["run_params"]
    p = rs.SimParams(N=64 * 64, nx=64, ny=64, dx=0.5e-6, dy=0.5e-6, z_detector=0.65, detector_size=24e-6,
                     detector_size_x=24e-6, detector_size_y=20e-6, detector_pixel_size_x=1.5e-6,
                     detector_pixel_size_y=1.25e-6, wl=wl, chunk_size=64 * 8)
    h = hm.History()
    zs = np.arange(0, 0.5, hdz)[1:]
    hm.generate_analytic_history_2d(h, zs, 1e-6, 0.0, p, np.sin(a0) / wl)
    n = len(zs)
    # same arithmetic as the reference; numpy's pow may round the last bit differently on
    # another CPU architecture than the one that wrote the fixture
    np.testing.assert_allclose(h.get_history(), golden["run_history"][:n], rtol=1e-14, atol=0)
    np.testing.assert_array_equal(np.array(h.get_z()), golden["run_history_z"][:n])


def test_history_validation(hm):
    with pytest.raises(ValueError):
        hm.History(memory_budget_bytes=-1)
    with pytest.raises(ValueError):
        hm.History(max_frames=0)
    with pytest.raises(ValueError):
        hm.History(roi=(3, 1, 0, 2))
    with pytest.raises(ValueError):
        hm.History(downsample=(0, 1))
    h = hm.History(max_frames=1)
    h.push(np.zeros((4, 4)), 0.1)
    with pytest.raises(RuntimeError):
        h.push(np.zeros((4, 4)), 0.2)
    h = hm.History()
    h.push(np.zeros((4, 4)), 0.1)
    with pytest.raises(ValueError):
        h.push(np.zeros((4, 5)), 0.2)
    with pytest.raises(ValueError):
        h.push(np.zeros((2, 2, 2)), 0.2)
    with pytest.raises(InterruptedError):
        hm.History(cancel_token=True).push(np.zeros((4, 4)), 0.1)
    with pytest.raises(ValueError):
        hm.History(roi=(0, 8, 0, 8)).push(np.zeros((4, 4)), 0.1)


def test_progress_and_1d_frames(hm):
    seen = []
    h = hm.History(max_frames=3, progress_cb=lambda *a: seen.append(a))
    for i in range(3):
        h.push(np.arange(5.0) + i, 0.5 * i)
    assert seen == [("history_frame", 1, 3), ("history_frame", 2, 3), ("history_frame", 3, 3)]
    assert h.get_history().shape == (5, 3)  # 1D frames stack as (x, z)
    assert h.metadata()["format_version"] == 1 and h.metadata()["axis_order"] == ["x", "z"]


def test_streaming_is_refused(hm, tmp_path):
    """A History big-wave would stream to HDF5 (storage path and budget 0, or a budget the frames
    outgrow, or resuming a stream) says so before writing anything."""
    h = hm.History(storage_path=tmp_path / "history.h5", memory_budget_bytes=0)
    with pytest.raises(RuntimeError, match="h5py"):
        h.push(np.zeros((4, 4)), 0.1)
    h = hm.History(storage_path=tmp_path / "history.h5", memory_budget_bytes=200)
    h.push(np.zeros((4, 4)), 0.1)
    with pytest.raises(RuntimeError, match="in memory"):
        h.push(np.zeros((4, 4)), 0.2)
    (tmp_path / "old.h5").write_bytes(b"")
    with pytest.raises(RuntimeError):
        hm.History(storage_path=tmp_path / "old.h5", resume=True)
    # under budget it stays in memory
    h = hm.History(storage_path=tmp_path / "history.h5", memory_budget_bytes=1 << 20)
    h.push(np.zeros((4, 4)), 0.1)
    assert not h.is_streaming and not (tmp_path / "history.h5").exists()
