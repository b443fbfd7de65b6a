"""GB300-native (sm_103a) multislice Fresnel propagation behind big-wave's 2D Python API.

Modules mirror the reference layout: `propagation` (SimParams, propagate_2d, cutoff,
point-source init, detector), `optical_element` (Material, Sample), `plasma_sample`
(PlasmaSample), `source` (PointSource), `wavesim` (run_simulation), `vector` (GpuVector).
All numerics run in librs_fresnel.so (C ABI: include/rs_fresnel.h); importing this package
does not load it, the first call does (and raises if it cannot be built or loaded).
"""
from . import _build, _lib  # noqa: F401
from .vector import GpuVector  # noqa: F401
from .propagation import (  # noqa: F401
    SimParams,
    apply_frequency_cutoff_2d,
    convert_energy_wavelength,
    propagate_2d,
    propagate_analytically_2d,
    square_and_downsample_2d,
)
from .optical_element import Material, Sample, material_factor  # noqa: F401
from .plasma_sample import PlasmaSample  # noqa: F401
from .source import PointSource  # noqa: F401

__version__ = "0.1.0"


def build(force: bool = False) -> str:
    """Compile librs_fresnel.so for sm_103a (no-op when up to date) and return its path."""
    return str(_build.build(force=force))
