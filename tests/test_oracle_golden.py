"""The CPU oracle against fixtures produced by running big-wave itself (tests/golden/make_golden.py)."""
import warnings

import numpy as np
import pytest

from conftest import rel_l2


def test_fft2_matches_numpyvector(golden, oracle):
    for name in ("c128_32x64", "c64_64x128"):
        x = golden[f"fft2_{name}_in"]
        out = oracle.fft2(x)
        assert out.dtype == x.dtype
        np.testing.assert_array_equal(out, golden[f"fft2_{name}_out"])
        np.testing.assert_array_equal(oracle.ifft2(out), golden[f"fft2_{name}_inv"])


def test_cutoff_bit_exact(golden, oracle):
    nx, ny, dx, dy, f = golden["cutoff_params"]
    out = oracle.apply_frequency_cutoff_2d(golden["cutoff_in"], f, dx, dy)
    np.testing.assert_array_equal(out, golden["cutoff_out"])
    assert np.count_nonzero(out == 0) > 0  # the mask is active


@pytest.mark.parametrize("name", ["c128", "c64"])
def test_propagate_2d(golden, oracle, name):
    nx, ny, dx, dy, wl, dz1, f1, dz2, f2 = golden["prop_params"]
    u, U = oracle.propagate_2d(golden[f"prop_{name}_in"], dx, dy, wl, dz1, f1)
    tol = 1e-13 if name == "c128" else 1e-6
    assert u.dtype == golden[f"prop_{name}_u"].dtype
    assert rel_l2(u, golden[f"prop_{name}_u"]) < tol
    assert rel_l2(U, golden[f"prop_{name}_U"]) < tol
    u2, U2 = oracle.propagate_2d(u, dx, dy, wl, dz2, f2, U=U, skip_fft=True)
    assert rel_l2(u2, golden[f"prop_{name}_skip_u"]) < tol
    assert rel_l2(U2, golden[f"prop_{name}_skip_U"]) < tol


def test_point_source(golden, oracle):
    nx, ny, dx, dy, z, xs, ys, wl = golden["ps_analytic_params"]
    u = oracle.propagate_analytically_2d(int(nx), int(ny), dx, dy, z, xs, ys, wl)
    np.testing.assert_array_equal(u, golden["ps_analytic"])
    nx, ny, dx, dy, z, xs, ys, wl, f = golden["ps_prop_params"]
    for name, dt in (("c128", np.complex128), ("c64", np.complex64)):
        u, U = oracle.point_source_2d(int(nx), int(ny), dx, dy, z, xs, ys, wl, f, dt)
        assert rel_l2(u, golden[f"ps_prop_{name}_u"]) < (1e-14 if dt == np.complex128 else 1e-7)
        assert rel_l2(U, golden[f"ps_prop_{name}_U"]) < (1e-14 if dt == np.complex128 else 1e-7)


@pytest.mark.parametrize("name", ["c128", "c64"])
def test_sample_apply(golden, oracle, name):
    nx, ny, dx, dy, wl, px, py, pz, xp, yp, f, z0 = golden["sample_params"]
    u, U = oracle.sample_apply_2d(golden[f"sample_{name}_in"], golden["sample_grid"], golden["sample_db"],
                                  dx, dy, wl, f, px, py, pz, xp, yp)
    tol = 1e-13 if name == "c128" else 2e-6
    assert rel_l2(u, golden[f"sample_{name}_u"]) < tol
    assert rel_l2(U, golden[f"sample_{name}_U"]) < tol


def test_plasma_apply(golden, oracle):
    p = golden["plasma_params"]
    nx, ny, dx, dy, wl, px, py, pz, xp, yp, f = p[:11]
    sf = tuple(p[11:15])
    energy, hc, re = p[15:18]
    u0 = np.ones((int(ny), int(nx)), np.complex128)
    u, U = oracle.plasma_apply_2d(u0, golden["plasma_ne"], golden["plasma_ni"], golden["plasma_te"],
                                  golden["plasma_zs"], sf, energy, (hc, re), dx, dy, wl, f, px, py, pz, xp, yp)
    assert rel_l2(u, golden["plasma_u"]) < 1e-13
    assert rel_l2(U, golden["plasma_U"]) < 1e-13


@pytest.mark.parametrize("integ", ["area_v1", "legacy_fastwave"])
def test_detectors(golden, oracle, integ):
    fn = oracle.detector_area_v1 if integ == "area_v1" else oracle.detector_legacy
    out = fn(golden[f"det_{integ}_small_in"], 0.7, 1.1, 1.3, 1.7, int(5.2 // 1.3), int(5.1 // 1.7), 8.0)
    np.testing.assert_allclose(out, golden[f"det_{integ}_small_out"], rtol=2e-14, atol=2e-14)
    out2 = fn(golden[f"det_{integ}_64_in"], 0.25e-6, 0.25e-6, 0.7e-6, 0.6e-6, int(15e-6 // 0.7e-6),
              int(14e-6 // 0.6e-6), 0.4)
    ref = golden[f"det_{integ}_64_out"]
    assert out2.shape == ref.shape
    assert rel_l2(out2, ref) < 1e-12


def test_run_simulation_chain(golden, oracle):
    """Point source -> gap -> 4-slice Sample -> final leg (skip_fft) -> area_v1 detector."""
    a0, a1, wl = golden["run_params"]
    dx = 0.5e-6
    f0, f1 = np.sin(a0) / wl, np.sin(a1) / wl
    u, U = oracle.point_source_2d(64, 64, dx, dx, 0.5, 1e-6, 0.0, wl, f0)
    db = np.array([0.0, 4.2e-6 + 1.9e-7j])
    u, U = oracle.sample_apply_2d(u, golden["run_grid"], db, dx, dx, wl, f1, 0.5e-6, 0.5e-6, 2e-6)
    u, U = oracle.propagate_2d(u, dx, dx, wl, 0.65 - (0.5 + 4 * 2e-6), f1, U=U, skip_fft=True)
    assert rel_l2(u, golden["run_u"]) < 1e-12
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        out = oracle.detector_area_v1(u, dx, dx, 1.5e-6, 1.25e-6, int(24e-6 // 1.5e-6), int(20e-6 // 1.25e-6), 0.65)
    assert rel_l2(out, golden["run_out"]) < 1e-12


def test_fastwave_fft_kats(oracle):
    """Hard-coded vectors of fast-wave/test/fwtest.cu:131-230 (numpy.fft.fft2 values)."""
    ones = np.ones((3, 3), np.complex128)
    exp = np.zeros((3, 3), np.complex128)
    exp[0, 0] = 9
    np.testing.assert_allclose(oracle.fft2(ones), exp, atol=1e-12)
    m = np.arange(1, 17, dtype=np.complex128).reshape(4, 4)
    exp4 = np.array([[136, -8 + 8j, -8, -8 - 8j], [-32 + 32j, 0, 0, 0], [-32, 0, 0, 0], [-32 - 32j, 0, 0, 0]])
    np.testing.assert_allclose(oracle.fft2(m), exp4, atol=1e-12)


def test_fresnel_plane(golden, oracle):
    nx, ny, dx, dy, dz, xs, ys, wl, f = golden["fp_params"]
    for name, dt in (("c128", np.complex128), ("c64", np.complex64)):
        u, U = oracle.fresnel_plane_2d(int(nx), int(ny), dx, dy, dz, xs, ys, wl, f, dt)
        tol = 1e-14 if dt == np.complex128 else 1e-6
        assert rel_l2(u, golden[f"fp_{name}_u"]) < tol
        assert rel_l2(U, golden[f"fp_{name}_U"]) < tol
