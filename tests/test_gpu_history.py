"""run_simulation with a (History, dz) pair on the GPU against big-wave's own recorded run
(tests/golden/history_golden.npz): the source's analytic frames, one frame per sample slice, the
gap between two samples and the final leg every history dz (big-wave/wavesim.py:188-300,
big-wave/history.py:348-435)."""
import importlib
from pathlib import Path

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden" / "history_golden.npz"


def test_run_history_vs_bigwave(rs, cuda):
    g = np.load(GOLDEN)
    hm = importlib.import_module("3d_ravesim_gb300.history")
    ws = importlib.import_module("3d_ravesim_gb300.wavesim")
    a0, a1, a2, wl, hdz = g["run_params"]
    nx = ny = 64
    p = rs.SimParams(N=nx * ny, nx=nx, ny=ny, dx=0.5e-6, dy=0.5e-6, z_detector=0.65, detector_size=24e-6,
                     detector_size_x=24e-6, detector_size_y=20e-6, detector_pixel_size_x=1.5e-6,
                     detector_pixel_size_y=1.25e-6, wl=wl, chunk_size=nx * 8)
    common = dict(pixel_size_x=0.5e-6, pixel_size_z=2e-6, materials=[rs.Material("W", 19.3)],
                  x_positions=np.array([0.0]), pixel_size_y=0.5e-6, y_positions=np.array([0.0]))
    s1 = rs.Sample(z_start=0.5, grid=g["run_grid"], **common)
    s2 = rs.Sample(z_start=0.56, grid=g["run_grid2"], **common)
    table = [(rs.Material("W", 19.3), np.complex128(4.2e-6 + 1.9e-7j))]
    u, U = rs.GpuVector.zeros(nx * ny, cuda), rs.GpuVector.zeros(nx * ny, cuda)
    h = hm.History()
    outs = ws.run_simulation(p, rs.PointSource(x=1e-6, y=0.0, z=0.0), [s1, s2], [a0, a1, a2], u, U, table,
                             history=(h, float(hdz)))
    ref, ref_z = g["run_history"], g["run_history_z"]
    np.testing.assert_array_equal(np.array(h.get_z()), ref_z)
    frames = h.get_history()
    assert frames.shape == ref.shape
    n_analytic = len(np.arange(0, 0.5, hdz)[1:])
    # host FP64 with the reference's arithmetic; numpy's pow may differ in the last bit between
    # CPU architectures
    np.testing.assert_allclose(frames[:n_analytic], ref[:n_analytic], rtol=1e-14, atol=0)
    for k in range(n_analytic, len(ref)):
        assert rel_l2(frames[k], ref[k]) < 2e-5, (k, ref_z[k])
    assert rel_l2(outs[0], g["run_out"]) < 2e-5


def test_history_frames_equal_direct_propagation(rs, cuda):
    """Each recorded plane of propagate_with_history_2d is the start spectrum propagated by the
    plane's full offset, so it matches one propagate_2d call of that length (to FP32 rounding:
    the direct call fuses the forward column transform with the transfer function)."""
    hm = importlib.import_module("3d_ravesim_gb300.history")
    n = 256
    wl = rs.convert_energy_wavelength(15000.0)
    p = rs.SimParams(N=n * n, nx=n, ny=n, dx=0.4e-6, dy=0.4e-6, z_detector=1.0, detector_size=n * 0.4e-6,
                     detector_pixel_size_x=0.8e-6, detector_pixel_size_y=0.8e-6, wl=wl, chunk_size=n * 8)
    rng = np.random.default_rng(5)
    u0 = (np.exp(1j * rng.uniform(0, 1, size=n * n)) * (1 + 0.1 * rng.normal(size=n * n))).astype(np.complex64)
    f = 0.45 / p.dx
    u, U = rs.GpuVector.from_numpy(u0, cuda), rs.GpuVector.zeros(n * n, cuda)
    h = hm.History()
    hm.propagate_with_history_2d(u, U, p, 0.031, f, 0.2, False, (h, 0.01))
    zs = hm._history_z_steps(0.031, 0.01)
    assert np.allclose(h.get_z(), zs[1:] + 0.2)
    for k, dz in enumerate(zs[1:]):
        v, V = rs.GpuVector.from_numpy(u0, cuda), rs.GpuVector.zeros(n * n, cuda)
        rs.propagate_2d(v, V, p.dx, p.dy, p.wl, float(dz), p.chunk_size, f, n, n)
        direct = rs.square_and_downsample_2d(v, p, float(zs[k + 1] + 0.2))
        assert rel_l2(h.get_history()[k], direct) < 1e-5
    # the field left behind is the last plane's
    v, V = rs.GpuVector.from_numpy(u0, cuda), rs.GpuVector.zeros(n * n, cuda)
    rs.propagate_2d(v, V, p.dx, p.dy, p.wl, 0.031, p.chunk_size, f, n, n)
    assert rel_l2(u.to_numpy(), v.to_numpy()) < 1e-5


def test_run_single_source_writes_run_directory(rs, cuda, tmp_path):
    """multisim.run_single_source on the recorded two-sample case: the run directory holds
    big-wave's files with the same images (big-wave/multisim.py:258-519)."""
    g = np.load(GOLDEN)
    ms = importlib.import_module("3d_ravesim_gb300.multisim")
    yio = importlib.import_module("3d_ravesim_gb300.yaml_io")
    a0, a1, a2, wl, hdz = g["run_params"]
    nx = ny = 64
    p = rs.SimParams(N=nx * ny, nx=nx, ny=ny, dx=0.5e-6, dy=0.5e-6, z_detector=0.65, detector_size=24e-6,
                     detector_size_x=24e-6, detector_size_y=20e-6, detector_pixel_size_x=1.5e-6,
                     detector_pixel_size_y=1.25e-6, wl=1.0, chunk_size=nx * 8)
    common = dict(pixel_size_x=0.5e-6, pixel_size_z=2e-6, materials=[rs.Material("W", 19.3)],
                  x_positions=np.array([0.0]), pixel_size_y=0.5e-6, y_positions=np.array([0.0]))
    elements = [rs.Sample(z_start=0.5, grid=g["run_grid"], **common),
                rs.Sample(z_start=0.56, grid=g["run_grid2"], **common)]
    table = [(rs.Material("W", 19.3), np.complex128(4.2e-6 + 1.9e-7j))]
    sub = ms.get_sub_dir(tmp_path / "sim", 3)
    outs = ms.run_single_source(sub, p, rs.PointSource(x=1e-6, y=0.0, z=0.0), elements, [a0, a1, a2], table,
                                energy=20000.0, source_idx=3, source_dct={"type": "point", "x": 1e-6, "y": 0.0,
                                                                          "z": 0.0},
                                device=cuda, history_dz=float(hdz), history_options={"storage": "memory"},
                                checkpoint_dir=tmp_path / "ck")
    assert p.wl == wl
    det = np.load(sub / "detected.npy")
    assert det.shape == (1, 16, 16) and det.dtype == np.float64
    np.testing.assert_array_equal(det[0], outs[0])
    assert rel_l2(det[0], g["run_out"]) < 2e-5
    hist = np.load(sub / "history.npy")
    np.testing.assert_array_equal(np.load(sub / "history_z.npy"), g["run_history_z"])
    assert hist.shape == g["run_history"].shape
    assert rel_l2(hist, g["run_history"]) < 2e-5
    assert np.load(sub / "history_x.npy").shape == (16,) and np.load(sub / "history_y.npy").shape == (16,)
    meta = yio.load(sub / "detector_metadata.yaml")
    assert meta["phase_steps"] == 1 and meta["integrator"] == "area_v1" and meta["output_shape"] == [16, 16]
    assert meta["source_geometry"] == yio.load(sub / "source_geometry.yaml")
    assert meta["source_geometry"] == {"type": "point", "units": "m", "x": 1e-6, "y": 0.0, "z": 0.0,
                                       "y_origin": "explicit"}
    hmeta = yio.load(sub / "history_metadata.yaml")
    assert hmeta["frames"] == len(g["run_history_z"]) and hmeta["storage"] == "npy"
    manifest = (tmp_path / "ck" / "00000003" / "manifest.json").read_text()
    assert '"status": "complete"' in manifest


def test_run_single_simulation_from_prepared_directory(rs, cuda, tmp_path):
    """multisim.run_single_simulation on a directory in setup_simulation's layout gives
    big-wave's recorded image and history."""
    from prepared_dir import write_prepared_dir
    g = np.load(GOLDEN)
    ms = importlib.import_module("3d_ravesim_gb300.multisim")
    yio = importlib.import_module("3d_ravesim_gb300.yaml_io")
    sim = write_prepared_dir(yio, tmp_path, g)
    outs = ms.run_single_simulation(sim, 0, tmp_path / "scratch", history_dz=float(g["run_params"][4]), device=cuda)
    sub = sim / "00000000"
    det = np.load(sub / "detected.npy")
    np.testing.assert_array_equal(det[0], outs[0])
    assert rel_l2(det[0], g["run_out"]) < 2e-5
    assert rel_l2(np.load(sub / "history.npy"), g["run_history"]) < 2e-5
    meta = yio.load(sub / "detector_metadata.yaml")
    assert meta["source_geometry"]["y_origin"] == "explicit" and meta["phase_steps"] == 1
