"""The C-ABI library builds, loads and exports every entry point include/rs_fresnel.h declares (no GPU calls)."""
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    text = (ROOT / "include" / "rs_fresnel.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(rs_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_boundary():
    syms = declared_symbols()
    for required in ("rs_plan_create", "rs_fft2", "rs_ifft2", "rs_propagate", "rs_apply_cutoff",
                     "rs_point_source", "rs_multislice_voxel", "rs_multislice_plasma", "rs_detector",
                     "rs_last_error"):
        assert required in syms


def test_library_exports_every_declared_symbol(rs):
    lib = rs._lib.lib()
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing
    assert lib.rs_version().startswith(b"rs_fresnel")


def test_python_binding_covers_the_header(rs):
    assert sorted(rs._lib.exported_symbols()) == declared_symbols()

