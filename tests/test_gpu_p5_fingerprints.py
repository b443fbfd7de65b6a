"""Full-size runs against big-wave's own recorded P5 convergence runs
(tests/golden/p5_fingerprints.json, written by make_p5_fingerprints.py from
tests/big_wave_2d/p5_results): a point source 5 m before a uniform voxel sample or plasma
layer (or vacuum), the detector 10 m from the source, 4096^2 / 8192^2 / 16384^2 complex64.
The detected energy, the peak and the 256-pixel centre-row fingerprint are compared with
big-wave's values (its complex64 FFTs and ours round differently, so the tolerances are
FP32-level, not bit-exact)."""
import json
import math
from pathlib import Path

import numpy as np
import pytest
import torch

from conftest import rel_l2

pytestmark = pytest.mark.gpu
FIX = json.loads((Path(__file__).resolve().parent / "golden" / "p5_fingerprints.json").read_text())


def elements_for(rs, mode: str):
    """big-wave's p5_benchmark.make_element (tests/big_wave_2d/p5_benchmark.py:69-111)."""
    if mode == "vacuum":
        return [], []
    n = 258
    pitch = 4e-4 / (n - 2)
    if mode == "sample":
        mat = rs.Material("P5-benchmark", 1.0)
        s = rs.Sample(z_start=5.0, pixel_size_x=pitch, pixel_size_y=pitch, pixel_size_z=1e-6,
                      grid=np.ones((1, n, n), dtype=np.uint32), materials=[mat], x_positions=np.array([0.0]),
                      y_positions=np.array([0.0]))
        return [s], [(mat, np.complex128(1.2e-7 + 2.4e-9j))]
    shape = (4, n, n)
    sf = tuple(FIX["plasma_scattering_factors"]["C"])
    p = rs.PlasmaSample(z_start=5.0, pixel_size_x=pitch, pixel_size_y=pitch, pixel_size_z=1e-6,
                        ne_grid=np.full(shape, 2e19, np.float32), ni_grid=np.full(shape, 1e19, np.float32),
                        te_grid=np.full(shape, 200.0, np.float32), zstar_grid=np.full(shape, 2.0, np.float32),
                        Z=6, x_positions=np.array([0.0]), y_positions=np.array([0.0]), scattering_factors=sf)
    return [p], []


@pytest.mark.parametrize("run", FIX["runs"], ids=lambda r: f"{r['mode']}-{r['nx']}")
def test_matches_bigwave_recorded_run(rs, cuda, run):
    import importlib
    ws = importlib.import_module("3d_ravesim_gb300.wavesim")
    setup = FIX["setup"]
    nx, ny, dx = run["nx"], run["ny"], run["dx"]
    wl = setup["wavelength"]
    p = rs.SimParams(N=nx * ny, nx=nx, ny=ny, dx=dx, dy=dx, z_detector=setup["z_detector"],
                     detector_size=setup["detector_size"], detector_size_x=setup["detector_size"],
                     detector_size_y=setup["detector_size"], detector_pixel_size_x=setup["detector_pixel"],
                     detector_pixel_size_y=setup["detector_pixel"], wl=wl, chunk_size=nx * setup["tile_rows"],
                     detector_integrator=run["integrator"])
    elements, table = elements_for(rs, run["mode"])
    angle = math.asin(run["cutoff_frequency"] * wl)
    u, U = rs.GpuVector.zeros(nx * ny, cuda), rs.GpuVector.zeros(nx * ny, cuda)
    x, y, z = setup["source"]
    out = ws.run_simulation(p, rs.PointSource(x=x, y=y, z=z), elements, [angle] * (len(elements) + 1), u, U,
                            table)[0]
    assert list(out.shape) == run["detected_shape"][1:]
    energy, peak = float(np.sum(out)), float(np.max(out))
    w = 256
    s0 = run["centerline_start_pixel"]
    line = out[out.shape[0] // 2, s0:s0 + w]
    assert abs(energy / run["detected_energy"] - 1) < 2e-6, (energy, run["detected_energy"])
    assert abs(peak / run["detected_peak"] - 1) < 2e-5, (peak, run["detected_peak"])
    assert rel_l2(line, np.array(run["centerline_256"])) < 2e-5
    del u, U
    torch.cuda.empty_cache()
