"""Host-side behaviour of the drop-in API that needs no GPU: validation, errors, geometry."""
import math

import numpy as np
import pytest
import torch


def test_simparams_checks_like_reference(rs):
    with pytest.raises(ValueError, match="N must be positive"):
        rs.SimParams(N=0, dx=1e-6, z_detector=1, detector_size=1e-5, detector_pixel_size_x=1e-6,
                     detector_pixel_size_y=1e-6, wl=1e-10, chunk_size=4)
    with pytest.raises(ValueError, match="must equal nx"):
        rs.SimParams(N=100, nx=7, ny=10, dx=1e-6, z_detector=1, detector_size=1e-5, detector_pixel_size_x=1e-6,
                     detector_pixel_size_y=1e-6, wl=1e-10, chunk_size=10)
    p = rs.SimParams(N=64 * 32, ny=32, dx=1e-6, z_detector=1, detector_size=1e-5, detector_pixel_size_x=1e-6,
                     detector_pixel_size_y=1e-6, wl=1e-10, chunk_size=64)
    assert p.nx == 64 and p.is_2d and p.get_dy() == 1e-6
    with pytest.raises(ValueError, match="unsupported detector_integrator"):
        rs.SimParams(N=4, dx=1, z_detector=1, detector_size=1, detector_pixel_size_x=1, detector_pixel_size_y=1,
                     wl=1, chunk_size=1, detector_integrator="nope")


def test_energy_wavelength_roundtrip(rs, oracle):
    for e in (8000.0, 20000.0, 25000.0, 30000.0):
        assert rs.convert_energy_wavelength(e) == oracle.convert_energy_wavelength(e)
    assert math.isclose(rs.convert_energy_wavelength(20000.0), 0.61992e-10, rel_tol=1e-4)


def test_row_alignment_is_enforced(rs):
    prop = rs.propagation
    with pytest.raises(ValueError, match="complete rows"):
        prop.require_row_aligned_chunk_size(17, 16, 8)
    with pytest.raises(ValueError, match="must not exceed"):
        prop.require_row_aligned_chunk_size(16 * 9, 16, 8)


def test_gpu_vector_fails_loudly_without_cuda(rs):
    with pytest.raises(TypeError, match="CUDA"):
        rs.GpuVector(torch.zeros(16, dtype=torch.complex64))
    with pytest.raises(TypeError, match="complex64"):
        rs.GpuVector(torch.zeros(16, dtype=torch.complex128))


def test_propagate_rejects_numpy_vectors(rs):
    class FakeNumpyVector:
        vec = np.zeros(64, np.complex64)
    with pytest.raises(TypeError, match="GpuVector"):
        rs.propagate_2d(FakeNumpyVector(), FakeNumpyVector(), 1e-6, 1e-6, 1e-10, 0.1, 8, 1e5, 8, 8)


def test_slice_schedule_matches_cone_beam_geometry(rs):
    from importlib import import_module
    oe = import_module("3d_ravesim_gb300.optical_element")
    p = rs.SimParams(N=64, ny=8, dx=1e-6, z_detector=2.0, detector_size=8e-6, detector_pixel_size_x=1e-6,
                     detector_pixel_size_y=1e-6, wl=1e-10, chunk_size=8)
    dz, cs = oe.slice_schedule(p, 0.5, 1e-6, 4)
    assert np.all(dz == 1e-6) and cs is None
    p2 = rs.SimParams(N=64, ny=8, dx=1e-6, z_detector=2.0, detector_size=8e-6, detector_pixel_size_x=1e-6,
                      detector_pixel_size_y=1e-6, wl=1e-10, chunk_size=8, use_cone_beam_bpm=True)
    p2.configure_fresnel_detector(0.0, 0.5)
    dz2, cs2 = oe.slice_schedule(p2, 0.5, 1e-6, 4)
    assert cs2 is not None and cs2[0] > 1.0
    assert dz2[0] == pytest.approx(1e-6 / (p2.fresnel_transverse_scale(0.5) * p2.fresnel_transverse_scale(0.5 + 1e-6)))


def test_multislice_model_rejects_bad_checkpoint_setting():
    import importlib
    import torch
    adj = importlib.import_module("3d_ravesim_gb300.adjoint")
    rs = importlib.import_module("3d_ravesim_gb300")
    p = rs.SimParams(N=64 * 64, nx=64, ny=64, dx=1e-6, dy=1e-6, z_detector=1.0, detector_size=64e-6,
                     detector_pixel_size_x=1e-6, detector_pixel_size_y=1e-6, wl=1e-10, chunk_size=64)
    geom = adj.VolumeGeometry(z_start=0.1, pixel_size_x=1e-6, pixel_size_y=1e-6, pixel_size_z=1e-6)
    for bad in (-1, "sqrt", 2.5):
        with pytest.raises(ValueError):
            adj.MultisliceModel(p, geom, 1e5, torch.ones(64 * 64, dtype=torch.complex64), checkpoint_every=bad)


def test_four_step_storage_order_round_trip():
    """The natural <-> four-step storage reordering of spectra: entry i of an axis holds frequency
    i // 256 + (n // 256) * (i % 256), and the two conversions invert each other."""
    import importlib
    import numpy as np
    vec = importlib.import_module("3d_ravesim_gb300.vector")
    nx, ny = 1024, 512
    f = vec.four_step_frequency(nx)
    assert sorted(f) == list(range(nx)) and f[1] == nx // 256 and f[256] == 1
    rng = np.random.default_rng(0)
    nat = (rng.normal(size=nx * ny) + 1j * rng.normal(size=nx * ny)).astype(np.complex64)
    st = vec.four_step_from_natural(nat, nx, ny)
    fy, fx = vec.four_step_frequency(ny), vec.four_step_frequency(nx)
    assert st.reshape(ny, nx)[3, 7] == nat.reshape(ny, nx)[fy[3], fx[7]]
    assert np.array_equal(vec.natural_from_four_step(st, nx, ny), nat)
