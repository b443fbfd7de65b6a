"""GPU drop-in for big-wave's PointSource in 2D (big-wave/source.py:44-113)."""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .propagation import SimParams, fresnel_plane_propagate_2d, grid_density_check_2d, point_source_propagate_2d


@dataclass
class PointSource:
    """Point source at (x, y, z); propagate_to initialises exp(2 pi i r/wl)/r at z_out, applies
    the circular frequency cutoff, and leaves U holding the cut-off spectrum."""

    x: float
    z: float
    y: float = 0.0

    def propagate_to(self, z_out: float, sim_params: SimParams, cutoff_freq: float, u, U, history) -> None:
        dz = z_out - self.z
        if not sim_params.is_2d:
            raise NotImplementedError("the GB300 PointSource implements the 2D path (ny > 1)")
        if sim_params.use_fresnel_scaling:
            # big-wave/source.py:62-95: the incident spherical phase is removed; the plane carries the
            # off-axis linear phase ramp and the 1/dz amplitude
            if sim_params.fresnel_effective_z <= 0 or sim_params.fresnel_magnification <= 0:
                raise ValueError("Fresnel detector geometry has not been configured")
            if dz <= 0:
                raise ValueError("Fresnel source-to-sample distance must be positive")
            if history is not None:
                raise ValueError("physical-z source history is not supported with Fresnel scaling")
            fresnel_plane_propagate_2d(u, U, dz, self.x, self.y, sim_params, cutoff_freq)
            return
        grid_density_check_2d(dz, self.x, sim_params.nx, sim_params.dx, self.y, sim_params.ny,
                              sim_params.get_dy(), sim_params.wl)
        point_source_propagate_2d(u, U, dz, self.x, self.y, sim_params, cutoff_freq)
        if history is not None:
            # analytic frames at z = k * history dz below z_out (big-wave/source.py:109-113)
            from .history import generate_analytic_history_2d
            zs = np.arange(0, z_out, history[1])[1:]
            generate_analytic_history_2d(history[0], zs, self.x, self.y, sim_params, cutoff_freq)
