"""run_simulation with run checkpoints on GPU fields: an interrupted run resumed from its last
checkpoint (big-wave/wavesim.py:155-310) ends in the same detector image as an uninterrupted one."""
import importlib

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def case(rs, cuda):
    nx = ny = 128
    wl = rs.convert_energy_wavelength(20000.0)
    p = rs.SimParams(N=nx * ny, nx=nx, ny=ny, dx=0.5e-6, dy=0.5e-6, z_detector=1.15, detector_size=nx * 0.5e-6,
                     detector_pixel_size_x=1e-6, detector_pixel_size_y=1e-6, wl=wl, chunk_size=nx)
    z = (np.arange(12) - 5.5)[:, None, None]
    yy = (np.arange(ny + 4) - (ny + 4) / 2)[None, :, None]
    xx = (np.arange(nx + 4) - (nx + 4) / 2)[None, None, :]
    r = np.sqrt(xx ** 2 + yy ** 2 + (4 * z) ** 2)
    grid = ((r <= 40) & (r >= 28)).astype(np.uint32)
    samp = rs.Sample(z_start=1.0, pixel_size_x=0.5e-6, pixel_size_z=2e-6, grid=grid, materials=[rs.Material("C", 2.0)],
                     x_positions=np.array([0.0]), pixel_size_y=0.5e-6, y_positions=np.array([0.0]))
    table = [(rs.Material("C", 2.0), np.complex128(4.1e-6 + 4.3e-9j))]
    fp = {"N": nx * ny, "nx": nx, "ny": ny, "dtype": np.dtype(np.complex64).str, "wavelength": wl,
          "z_detector": p.z_detector, "source_index": 0}
    return p, samp, table, fp, [0.2, 0.2]


def run(rs, cuda, p, samp, table, angles, **kw):
    ws = importlib.import_module("3d_ravesim_gb300.wavesim")
    u, U = rs.GpuVector.zeros(p.N, cuda), rs.GpuVector.zeros(p.N, cuda)
    outs = ws.run_simulation(p, rs.PointSource(x=1e-6, y=0.0, z=0.0), [samp], angles, u, U, table, **kw)
    torch.cuda.synchronize()
    return outs[0]


def test_interrupted_run_resumes_to_the_same_image(rs, cuda, tmp_path):
    ck = importlib.import_module("3d_ravesim_gb300.checkpoint")
    p, samp, table, fp, angles = case(rs, cuda)
    straight = run(rs, cuda, p, samp, table, angles, checkpoint=ck.RunCheckpoint(tmp_path / "a", fp))

    class StopAfter:  # cancels the save that follows the second committed slice checkpoint
        def __init__(self):
            self.commits, self.is_set = 0, False

        def __call__(self, stage, done, total):
            if stage == "checkpoint_commit":
                self.commits += 1
                self.is_set = self.commits >= 3  # source stage, slice 5, slice 10
    stop = StopAfter()
    with pytest.raises(InterruptedError):
        run(rs, cuda, p, samp, table, angles,
            checkpoint=ck.RunCheckpoint(tmp_path / "b", fp, progress_cb=stop, cancel_token=stop))
    state = ck.RunCheckpoint(tmp_path / "b", fp).load(rs.GpuVector.zeros(p.N, cuda), rs.GpuVector.zeros(p.N, cuda))
    assert (state.element_index, state.slice_index, state.stage) == (0, 10, "element_slice")
    resumed = run(rs, cuda, p, samp, table, angles, checkpoint=ck.RunCheckpoint(tmp_path / "b", fp),
                  resume_checkpoint=True)
    np.testing.assert_array_equal(resumed, straight)
