"""The C ABI's argument checks, which run before any CUDA call, so they need no GPU: each bad
argument returns its status code with a message in rs_last_error (thread-local), nothing exits,
and the Python layer maps the codes to the reference's exception types."""
import ctypes
import threading
from ctypes import byref, c_ulonglong, c_void_p

import pytest


@pytest.fixture(scope="module")
def L(rs):
    return rs._lib


def create(L, nx, ny, flags=0):
    h = c_void_p()
    st = L.lib().rs_plan_create(nx, ny, flags, byref(h))
    return st, L.lib().rs_last_error().decode()


def test_plan_create_rejects_bad_arguments(L):
    lib = L.lib()
    assert lib.rs_plan_create(16, 16, 0, None) == L.RS_EINVAL
    assert "out is NULL" in lib.rs_last_error().decode()
    assert create(L, 16, 16, 2) == (L.RS_EINVAL, "unknown plan flags 0x2")
    st, msg = create(L, 0, 16)
    assert st == L.RS_EINVAL and "nx and ny must be positive" in msg
    st, msg = create(L, 1024, 1024, L.RS_PLAN_FOURSTEP)
    assert st == L.RS_EUNSUPPORTED and "four-step plans need power-of-two axes" in msg
    st, msg = create(L, 7000, 7000)
    assert st == L.RS_EUNSUPPORTED and "axes must be powers of two" in msg
    assert lib.rs_plan_destroy(None) == L.RS_OK


def test_entry_points_reject_a_null_plan(L):
    lib = L.lib()
    p = c_void_p()
    assert lib.rs_fft2(None, p, p, None) == L.RS_EINVAL
    assert "plan is NULL" in lib.rs_last_error().decode()
    assert lib.rs_propagate(None, p, p, 1e-6, 1e-6, 1e-10, 0.1, 1e5, 0, None) == L.RS_EINVAL
    assert lib.rs_plan_is_fast(None) == 0 and lib.rs_plan_is_four_step(None) == 0
    assert lib.rs_launch_count(None) == L.RS_EINVAL
    n = c_ulonglong(123)
    assert lib.rs_launch_count(byref(n)) == L.RS_OK and n.value == L.launch_count()


def test_detector_noalloc_checks_its_geometry(L):
    lib = L.lib()
    buf = (ctypes.c_double * 4)()
    good = dict(dx=1e-6, dy=1e-6, ds_px=2e-6, ds_py=2e-6, detector_z=1.0, out_x=2, out_y=2, integrator=0,
                accumulate=0)
    cases = [({}, "NULL pointer argument", True),
             ({"out_x": 0}, "output must be non-empty", False),
             ({"dy": -1.0}, "spacings must be positive", False),
             ({"ds_px": float("nan")}, "spacings must be positive", False),
             ({"detector_z": 0.0}, "finite and non-zero", False)]
    for change, text, null_field in cases:
        g = L.DetectorGeom(**{**good, **change})
        u = None if null_field else ctypes.cast(buf, c_void_p)
        assert lib.rs_detector_noalloc(u, 4, 4, buf, byref(g), None) == L.RS_EINVAL
        assert text in lib.rs_last_error().decode()
    g = L.DetectorGeom(**good)
    assert lib.rs_detector_noalloc(ctypes.cast(buf, c_void_p), 0, 4, buf, byref(g), None) == L.RS_EINVAL


def test_last_error_is_per_thread(L):
    lib = L.lib()
    create(L, 0, 16)
    seen = {}

    def other():
        seen["before"] = lib.rs_last_error().decode()
        create(L, 16, 16, 2)
        seen["after"] = lib.rs_last_error().decode()

    t = threading.Thread(target=other)
    t.start()
    t.join()
    assert seen["before"] == "" and seen["after"] == "unknown plan flags 0x2"
    assert "nx and ny must be positive" in lib.rs_last_error().decode()


def test_status_codes_map_to_the_reference_exceptions(L):
    create(L, 0, 16)
    for code, exc in ((L.RS_EINVAL, ValueError), (L.RS_EUNSUPPORTED, NotImplementedError),
                      (L.RS_ENOMEM, MemoryError), (L.RS_ETIMEOUT, TimeoutError),
                      (L.RS_ECANCELLED, InterruptedError), (L.RS_ECUDA, RuntimeError)):
        with pytest.raises(exc, match="probe: nx and ny must be positive"):
            L.check(code, "probe")
    L.check(L.RS_OK, "probe")
