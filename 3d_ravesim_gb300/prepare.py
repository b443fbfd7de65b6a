"""Preparing a multi-source simulation directory: big-wave's setup_simulation
(big-wave/multisim.py:520-1399) for the element and source types of the 2D GPU path.

A prepared directory is what `multisim.run_single_simulation` (here and in big-wave) runs, one
source at a time:

* ``config.yaml``: the input configuration with sim_params resolved (an integer chunk_size, nx,
  the runtime.big_wave backend settings), grid paths reduced to file names, and the elements cut
  at a ``save_and_exit`` marker;
* the element grids, copied beside it;
* ``computed.yaml``: the cutoff angle of every propagation leg (x, and y for diagnostics), the
  beam half-width at the detector, the energy range, the source points and how they were drawn,
  the Fresnel geometry, the requested and resolved runtime settings and the algorithm tags;
* ``<index:08>/subconfig.yaml`` per source: the point source, its energy, the delta/beta table
  of every material at that energy and the plasma elements' scattering factors.

The directory lives at ``save_dir/<year>/<month>/<YYYYmmdd_HHMMSSffffff>`` as in big-wave. The
delta/beta values and plasma factors come from this package's Chantler lookup (`chantler`, over
nist_lookup's xrayref.db); the random draws are big-wave's (`multisim.sample_source_points`).
Element types outside the path (gratings, precise samples) and ``vectors`` multisources raise
NotImplementedError from the parsers.
"""
from __future__ import annotations

import copy
import logging
import os
import shutil
import subprocess
from datetime import datetime
from pathlib import Path
from typing import Optional

import numpy as np

from . import chantler
from . import config as cfg
from .optical_element import Material, SaveAndExit, Sample
from .propagation import (DETECTOR_INTEGRATOR_VERSIONS, SimParams, compute_cutoff_angles, convert_energy_wavelength,
                          grid_density_check, grid_density_check_2d)

logger = logging.getLogger(__name__)
Z_TOLERANCE = 1e-8
ALGORITHM_VERSION = "big-wave-2d-p4-v1"


def _git_commit() -> str:
    """Revision of the checkout this package runs from, "unknown" outside a git checkout
    (the provenance entry of big-wave/multisim.py:73-86)."""
    try:
        out = subprocess.run(["git", "rev-parse", "HEAD"], cwd=Path(__file__).resolve().parent.parent, check=True,
                             capture_output=True, text=True, timeout=2)
        return out.stdout.strip() or "unknown"
    except (OSError, subprocess.SubprocessError):
        return "unknown"


# --------------------------------------------------------------------------- materials
def collect_all_materials(elements: list) -> list[Material]:
    """Materials of the voxel samples, each once, in order of first use
    (big-wave/optical_element.py:742-777; gratings are not on the 2D GPU path)."""
    found: list[Material] = []
    for el in elements:
        if isinstance(el, Sample):
            for mat in el.materials:
                if mat not in found:
                    found.append(mat)
    return found


def generate_deltabeta_table(materials: list[Material], energy: float) -> list:
    """[(material, delta + i beta)] at `energy` [eV] from the Chantler tables
    (big-wave/optical_element.py:780-795 over nist_lookup's xray_delta_beta)."""
    table = []
    for m in materials:
        delta, beta, _ = chantler.xray_delta_beta(m.mat, m.density, energy)
        table.append((m, delta + 1j * beta))
    return table


def deltabeta_table_to_tuples(table: list) -> list:
    """subconfig.yaml's form of a delta/beta table: [[name, density], [delta, beta]]
    (big-wave/multisim.py:522-532)."""
    return [((m.mat, m.density), (float(db.real), float(db.imag))) for m, db in table]


def plasma_optics_table_for_elements(elements_dct: list, energy: float) -> list:
    """Scattering factors of every plasma_sample element at `energy` (big-wave/plasma.py:269-308):
    {formula, f1bar, f2eff_bar, zbar, z2bar}; the compound average for a formula, else the bare
    element Z (formula None). Other element types have no entry."""
    table = []
    for el in elements_dct:
        if el.get("type") != "plasma_sample":
            continue
        formula = el.get("formula")
        if formula:
            values = chantler.compound_scattering_factors(formula, energy)
            formula = str(formula)
        else:
            z = int(el.get("Z", 0))
            if z <= 0:
                raise ValueError("plasma_sample requires 'formula' (multi-element) or a valid 'Z'")
            values = chantler.element_scattering_factors(z, energy)
            formula = None
        table.append({"formula": formula, **{k: float(v) for k, v in
                                             zip(("f1bar", "f2eff_bar", "zbar", "z2bar"), values)}})
    return table


# --------------------------------------------------------------------------- checks
def reduce_simulation_setup_for_save_and_exit(dct: dict, max_x_list: list[float]) -> float:
    """Cut the element list at the first save_and_exit marker, move the detector to its z and
    turn on save_final_u_vectors (big-wave/multisim.py:535-561). Returns the beam half-width at
    the (possibly moved) detector."""
    kept: list = []
    max_x = max_x_list[-1]
    for i, el in enumerate(dct["elements"]):
        if el["type"] != "save_and_exit":
            kept.append(el)
            continue
        max_x = max_x_list[i]
        dct["sim_params"]["z_detector"] = el["z_start"]
        if dct["save_final_u_vectors"]:
            logger.warning("save_final_u_vectors was activated on a config that contains a save_and_exit element. "
                           "Note that the vectors will be saved, but at the save_and_exit position instead of the "
                           "originally specified z_detector.")
        dct["save_final_u_vectors"] = True
        dct["elements"] = kept
        break
    return max_x


def check_simulation_inputs(params: SimParams, z_source: float, elements: list, cutoff_angles: list[float]) -> None:
    """Element order, phase-step counts, save_and_exit placement, detector position and the
    cutoff angles (big-wave/multisim.py:564-611); overlaps up to 1e-8 m are accepted."""
    assert len(cutoff_angles) == len(elements) + 1
    if elements:
        assert z_source <= elements[0].z_start, \
            "The source must not be at a greater z-coordinate than the first optical element"
    steps_seen: Optional[int] = None
    z = z_source
    for i, el in enumerate(elements):
        steps = len(el.x_positions)
        if steps > 1:
            assert steps_seen is None or steps_seen == steps, \
                "If multiple elements have phase stepping enabled, then all elements must have the same number of steps."
            steps_seen = steps
        el.check_valid()
        assert z <= el.z_start + Z_TOLERANCE, "Overlapping optical elements are not supported"
        z = el.z_start + el.get_thickness()
        if isinstance(el, SaveAndExit):
            if i == len(elements) - 1:
                assert params.z_detector == el.z_start, \
                    "A save_and_exit element at the end must have the same z coordinate as the detector"
            else:
                assert elements[i + 1].z_start == el.z_start, \
                    "A save_and_exit element must have the same z coordinate as the next optical element"
    assert z <= params.z_detector + Z_TOLERANCE, "Detector must be after the last optical element"
    for a, b in zip(cutoff_angles, cutoff_angles[1:]):
        assert a <= b, "cutoff angles must be increasing"
    for a in cutoff_angles:
        assert 0 <= a <= np.pi / 2, "cutoff angles must be between 0 and pi/2"


def fresnel_mode_name(params: SimParams) -> str:
    """"cone_beam_bpm", "thin" or "off" (big-wave/multisim.py:614-619)."""
    if params.use_cone_beam_bpm:
        return "cone_beam_bpm"
    return "thin" if params.use_fresnel_scaling else "off"


def validate_fresnel_mode(params: SimParams, elements: list, source_type: str) -> None:
    """Geometries the Fresnel modes cannot represent (big-wave/multisim.py:622-651)."""
    mode = fresnel_mode_name(params)
    if mode == "off":
        return
    if not params.is_2d:
        raise ValueError("Fresnel scaling is currently supported only in 2D mode")
    if source_type not in {"point", "points"}:
        raise ValueError("Fresnel scaling requires point sources")
    if not elements:
        raise ValueError("Fresnel scaling requires at least one optical element")
    unsupported = [type(el).__name__ for el in elements if type(el).__name__ not in {"Sample", "PlasmaSample"}]
    if unsupported:
        raise ValueError(f"Fresnel scaling supports only Sample/PlasmaSample elements, got {unsupported}")
    if mode == "thin" and len(elements) != 1:
        raise ValueError("Thin Fresnel scaling requires exactly one optical element; "
                         "use use_cone_beam_bpm=true for multislice or multiple-element propagation")


def compute_fresnel_cutoff_geometry(sim_params: SimParams, z_source: float, z_sample: float,
                                    x_source_range: tuple[float, float],
                                    y_source_range: tuple[float, float]) -> tuple[float, float, float, float]:
    """(x cutoff angle, y cutoff angle, magnification M, effective distance z_eff) of the Fresnel
    similarity frame (big-wave/multisim.py:654-687): with a = source-sample and b = sample-detector
    distances, M = (a + b)/a and z_eff = ab/(a + b); each angle is atan of the steepest source
    slope max|range|/a plus the slope to the effective detector's edge, size/(2 M z_eff)."""
    a = z_sample - z_source
    b = sim_params.z_detector - z_sample
    if a <= 0 or b <= 0:
        raise ValueError("Fresnel scaling requires z_source < z_sample < z_detector")
    m = (a + b) / a
    z_eff = a * b / (a + b)
    sx = max(map(abs, x_source_range)) / a + sim_params.get_detector_size_x() / (2.0 * m * z_eff)
    sy = max(map(abs, y_source_range)) / a + sim_params.get_detector_size_y() / (2.0 * m * z_eff)
    return float(np.arctan(sx)), float(np.arctan(sy)), float(m), float(z_eff)


def load_spectrum(path) -> tuple[np.ndarray, np.ndarray]:
    """(energy, pdf) datasets of a spectrum file (big-wave/multisim.py:690-692; HDF5)."""
    try:
        import h5py
    except ImportError as exc:
        raise RuntimeError("reading a multisource spectrum file needs h5py, which is not installed") from exc
    with h5py.File(path, "r") as f:
        return np.array(f["energy"]), np.array(f["pdf"])


def setup_sim_dir(save_dir: Path) -> Path:
    """save_dir/<year>/<month>/<YYYYmmdd_HHMMSSffffff>, created (big-wave/multisim.py:113-122)."""
    now = datetime.now()
    path = Path(save_dir) / now.strftime("%Y") / now.strftime("%m") / now.strftime("%Y%m%d_%H%M%S%f")
    os.makedirs(path)
    return path


# --------------------------------------------------------------------------- the setup
def _requested_runtime(dct: dict) -> dict:
    """runtime.big_wave as the user asked for it, before resolution (big-wave/multisim.py:750-790)."""
    runtime = copy.deepcopy(cfg.get_runtime_big_wave(dct))
    sim = copy.deepcopy(dct.get("sim_params", {}))
    disk_2d = bool(dct.get("use_disk_vector", False)) and int(sim.get("ny", 1)) > 1
    defaults = {"memory_budget_gb": cfg.DEFAULT_MEMORY_BUDGET_GB, "chunk_size": "auto",
                "fft2_backend": cfg.OOC_FFT2_BACKEND if disk_2d else cfg.DEFAULT_FFT2_BACKEND,
                "detector_integrator": cfg.DEFAULT_DETECTOR_INTEGRATOR,
                "save_debug_wavefields": cfg.DEFAULT_SAVE_DEBUG_WAVEFIELDS}
    return {k: runtime.get(k, sim.get(k, d)) for k, d in defaults.items()}


def _check_grid_2d_shape(p: SimParams) -> None:
    """N = nx ny, power-of-two axes and the large-field chunk rule (big-wave/multisim.py:803-820)."""
    if p.nx * p.ny != p.N:
        raise ValueError(f"N ({p.N}) must equal nx * ny ({p.nx} * {p.ny} = {p.nx * p.ny})")
    for name, n in (("nx", p.nx), ("ny", p.ny)):
        if not (n > 0 and (n & (n - 1)) == 0):
            raise ValueError(f"R1 requires {name} to be a power of two, got {n}")
    if p.N > cfg.MAX_SCIPY_FFT2_POINTS and p.chunk_size >= p.N:
        raise ValueError(f"2D large config must not use chunk_size >= N ({p.chunk_size} >= {p.N})")


def _check_grid_extent(p: SimParams, use_fresnel: bool) -> None:
    """The detector must fit the grid unless Fresnel scaling magnifies it (big-wave/multisim.py:833-847)."""
    if use_fresnel:
        logger.info("Fresnel scaling enabled, simulation FOV at sample plane does not need to cover physical "
                    f"detector ({p.N * p.dx * 1e3:.2f}mm vs {p.detector_size * 1e3:.1f}mm)")
        return
    assert p.N * p.dx >= p.detector_size, \
        f"Detector is bigger than simulation space ({p.detector_size} > {p.N * p.dx})."
    if p.is_2d:
        assert p.nx * p.dx >= p.get_detector_size_x(), "2D detector x-size exceeds simulation x-extent"
        assert p.ny * p.get_dy() >= p.get_detector_size_y(), "2D detector y-size exceeds simulation y-extent"


def _fresnel_sampling(p: SimParams, energy_range, x_range, z_source: float, m: float, z_eff: float) -> dict:
    """computed.yaml's audit of the Fresnel effective frame, with the check that the effective
    detector fits the wavefront grid (big-wave/multisim.py:1104-1177)."""
    wl = convert_energy_wavelength(energy_range[1])
    dx, dy = float(p.dx), float(p.get_dy())
    fov = (p.nx * dx, p.ny * dy)
    det = (p.get_detector_size_x() / m, p.get_detector_size_y() / m)
    px = (p.detector_pixel_size_x / m, p.detector_pixel_size_y / m)
    nyq = min(0.5 / dx, 0.5 / dy)
    aperture = float(np.arctan((p.get_detector_size_x() / 2.0 + max(map(abs, x_range))) / (p.z_detector - z_source)))
    if fov[0] < det[0] or fov[1] < det[1]:
        raise ValueError("Fresnel effective detector does not fit the wavefront grid: "
                         f"detector/M = ({det[0]:.6e}, {det[1]:.6e}) m vs "
                         f"wavefront FOV = ({fov[0]:.6e}, {fov[1]:.6e}) m")
    return {
        "units": "m",
        "mode": "fresnel_similarity_effective_frame_v1",
        "magnification": float(m),
        "effective_z": float(z_eff),
        "wavelength_m": float(wl),
        "wavefront_fov": [float(v) for v in fov],
        "detector_size_effective": [float(v) for v in det],
        "detector_pixel_effective": [float(v) for v in px],
        "detector_pixels_per_grid_point": [float(px[0] / dx), float(px[1] / dy)],
        "detector_fov_to_wavefront_fov": [float(det[0] / fov[0]), float(det[1] / fov[1])],
        "raw_grid_nyquist_frequency": float(nyq),
        "physical_aperture_angle_rad": float(aperture),
        "physical_aperture_frequency": float(np.sin(aperture) / wl),
        "raw_nyquist_check_applies": False,
        "raw_nyquist_ratio_reported_only": float(np.sqrt(2.0) * np.sin(aperture) / wl / nyq),
    }


def _check_circular_cutoff(p: SimParams, angles: list[float], energy_range) -> None:
    """The scalar cutoff kx^2 + ky^2 <= 2 f^2 reaches sqrt(2) f on an axis: it must stay below
    both axes' Nyquist frequencies (big-wave/multisim.py:1179-1198)."""
    wl = convert_energy_wavelength(energy_range[1])
    for axis, spacing in (("x", p.dx), ("y", p.get_dy())):
        for a in angles:
            f = np.sin(a) / wl
            if np.sqrt(2.0) * f > 0.5 / spacing:
                raise ValueError(f"2D {axis}-Nyquist cutoff exceeded: angle={a:.6f} rad, "
                                 f"max_freq={np.sqrt(2.0) * f:.6e}, nyquist={0.5 / spacing:.6e}")


def _algorithms_2d(p: SimParams) -> dict:
    """computed.yaml's algorithm tags of a 2D run (big-wave/multisim.py:1316-1385): the names big-wave
    records for its formats and operators, which a reader of the directory checks."""
    tile_rows = p.chunk_size // p.nx
    ooc = p.fft2_backend == cfg.OOC_FFT2_BACKEND
    return {
        "frequency_cutoff_2d": {"version": "circular_scalar_v1", "criterion": "kx^2 + ky^2 <= 2 * f^2",
                                "axis_max_frequency_factor": float(np.sqrt(2.0))},
        "local_operators_2d": {"version": "row_tile_v1", "tile_rows": tile_rows, "coordinate_storage": "axis_only"},
        "sample_grid_reader": {"version": "npy_memmap_tile_v1", "mmap_mode": "r"},
        "plasma_deltabeta": {"version": "vectorized_tile_v1", "chantler_cache_key": "element_and_energy"},
        "fft2": {"version": "bfpy_ooc_transactional_v1" if ooc else "scipy_in_memory_v1",
                 "backend": p.fft2_backend, "memory_budget_fraction": cfg.FFT2_MEMORY_BUDGET_FRACTION,
                 "passes": ["row_fft", "transpose_to_scratch", "column_fft", "transpose_to_output"],
                 "restart_manifest": ooc},
        "detector_2d": {"integrator": p.detector_integrator,
                        "version": DETECTOR_INTEGRATOR_VERSIONS[p.detector_integrator],
                        "streaming": True, "row_prefix_only": True,
                        "geometry_application": "fused_row_accumulation",
                        "fresnel_effective_geometry": p.use_fresnel_scaling,
                        "per_source_metadata": "detector_metadata.yaml"},
        "history_2d": {"version": "history_v2", "axis_order": ["z", "y", "x"], "streaming_format": "hdf5",
                       "legacy_reader": "y_x_z_to_z_y_x"},
        "run_checkpoint": {"version": "transactional_manifest_v1", "vectors": ["u", "U"],
                           "granularity": ["element", "sample_slice", "plasma_slice"],
                           "phase_snapshot_separate": True},
    }


def _element_grid_files(dct: dict, config_dir: Path) -> list[Path]:
    """Grid files to copy; the config keeps their base names (big-wave/multisim.py:1222-1236)."""
    keys = {"sample": ("grid_path",), "precise_sample": ("material_grid_path", "density_grid_path"),
            "plasma_sample": ("ne_grid_path", "ni_grid_path", "te_grid_path", "zstar_grid_path")}
    files = []
    for el in dct["elements"]:
        for key in keys.get(el["type"], ()):
            files.append(config_dir / el[key])
            el[key] = os.path.basename(el[key])
    return files


def setup_simulation(dct: dict, config_dir, save_dir) -> Path:
    """Create a simulation directory for the configuration `dct` under `save_dir` and return its
    path (big-wave/multisim.py:727-1399); grid paths are relative to `config_dir`.

    In order: resolve sim_params, check the grid, parse the elements, draw the source points and
    energies (``points`` multisource: checks of x/y/energy ranges and the source-to-sample Nyquist
    condition at the highest energy unless Fresnel scaling is on), compute the cutoff angles
    (the Fresnel similarity frame, or `compute_cutoff_angles` for x, y and the enclosing scalar
    cutoff in 2D), check the scalar cutoff against both Nyquist limits and the grid against the
    beam's width at the detector, cut at save_and_exit, check the element sequence, then write
    the directory."""
    logger.info("Setting up simulation")
    dct = copy.deepcopy(dct)
    requested = _requested_runtime(dct)
    config_dir, save_dir = Path(config_dir), Path(save_dir)

    dct["sim_params"] = cfg.resolve_sim_params(dct)
    p = cfg.parse_sim_params(dct["sim_params"])
    use_fresnel = p.use_fresnel_scaling
    if p.is_2d:
        _check_grid_2d_shape(p)
    elements = [cfg.parse_optical_element(el, config_dir) for el in dct["elements"]]
    if use_fresnel and not elements:
        raise ValueError("Fresnel scaling requires at least one optical element")
    _check_grid_extent(p, use_fresnel)
    materials = collect_all_materials(elements)

    multisource = dct["multisource"]
    validate_fresnel_mode(p, elements, str(multisource.get("type", "")))
    if multisource["type"] == "vectors":
        raise NotImplementedError("vector multisources (fields of a base simulation) are not part of the 2D GPU "
                                  "path")
    if multisource["type"] != "points":
        raise ValueError(f"Unknown multisource type {multisource['type']}.")

    from .multisim import generate_energies_from_spectrum, get_sub_dir, multisource_ranges, resolve_seed
    n_src, energy_range, x_range, y_range, z_source = multisource_ranges(multisource, p.is_2d)
    seed = resolve_seed(multisource)
    first_z = elements[0].z_start if elements else p.z_detector
    wl_short = convert_energy_wavelength(energy_range[1])
    if not use_fresnel:
        for xb in x_range:
            grid_density_check(first_z - z_source, xb, p.nx, p.dx, wl_short)
        if p.is_2d:
            for xb in x_range:
                for yb in y_range:
                    grid_density_check_2d(first_z - z_source, xb, p.nx, p.dx, yb, p.ny, p.get_dy(), wl_short)
    else:
        logger.info("Fresnel scaling enabled, skipping source→sample Nyquist check")

    rs, source_rs = np.random.RandomState(seed), np.random.RandomState(seed)
    if "spectrum" in multisource:
        spec_e, spec_i = load_spectrum(config_dir / multisource["spectrum"])
        energies = generate_energies_from_spectrum(spec_e, spec_i, rs, energy_range, n_src)
    else:
        energies = rs.rand(n_src) * (energy_range[1] - energy_range[0]) + energy_range[0]
    xs = source_rs.normal(loc=x_range[0] / 2 + x_range[1] / 2, scale=(x_range[1] - x_range[0]) / 2, size=n_src)
    ys = source_rs.normal(loc=(y_range[0] + y_range[1]) / 2, scale=(y_range[1] - y_range[0]) / 2, size=n_src)
    sub_dcts = [{"source": {"type": "point", "x": float(xs[i]), "y": float(ys[i]), "z": z_source},
                 "energy": float(energies[i]),
                 "deltabeta_table": deltabeta_table_to_tuples(generate_deltabeta_table(materials, energies[i])),
                 "plasma_optics_table": plasma_optics_table_for_elements(dct["elements"], energies[i])}
                for i in range(n_src)]
    source_points = [{"x": float(xs[i]), "y": float(ys[i]), "z": z_source, "energy": float(energies[i])}
                     for i in range(n_src)]
    max_x = max(abs(x_range[0]), abs(x_range[1]))
    max_y = max(abs(y_range[0]), abs(y_range[1]))

    z_distances = [el.z_start for el in elements]
    heights = [el.get_thickness() for el in elements]
    fresnel_m, fresnel_z_eff = 1.0, 0.0
    legs = len(elements) + 1
    if use_fresnel:
        cut_x, cut_y, fresnel_m, fresnel_z_eff = compute_fresnel_cutoff_geometry(
            p, z_source, float(elements[0].z_start), x_range, y_range)
        angles = [max(cut_x, cut_y)] * legs  # one scalar cutoff; the y angle is kept for the record
        angles_y = [cut_y] * legs
        max_x_list = [p.get_detector_size_x() / (2 * fresnel_m)] * legs
        logger.info("Fresnel cutoff: x=%.6g rad, y=%.6g rad, scalar=%.6g rad, z_eff=%.6g m",
                    cut_x, cut_y, angles[0], fresnel_z_eff)
    else:
        def cutoffs(size, spacing, width):
            return compute_cutoff_angles(detector_size=size, dx=spacing, energy_range=energy_range,
                                         z_source=z_source, z_distances=z_distances, element_heights=heights,
                                         z_detector=p.z_detector, max_x=width)
        angles, max_x_list = cutoffs(p.get_detector_size_x(), p.dx, max_x)
        if p.is_2d:
            # y on its own for the record; the scalar cutoff encloses both axes
            angles_y, max_y_list = cutoffs(p.get_detector_size_y(), p.get_dy(), max_y)
            angles, max_x_list = cutoffs(max(p.get_detector_size_x(), p.get_detector_size_y()),
                                         min(p.dx, p.get_dy()), max(max_x, max_y))
            max_y_list = list(max_x_list)
        else:
            angles_y, max_y_list = list(angles), list(max_x_list)

    fresnel_sampling = None
    if p.is_2d:
        if use_fresnel:
            fresnel_sampling = _fresnel_sampling(p, energy_range, x_range, z_source, fresnel_m, fresnel_z_eff)
        else:
            _check_circular_cutoff(p, angles, energy_range)

    if not use_fresnel:
        # a grid wide enough that no ray within the cutoffs reaches its edge
        need_x = int(np.ceil(max_x_list[-1] / p.dx) * 2)
        assert p.nx >= need_x, (f"Reflections at the boundary might occur: Nx={p.nx}, required_Nx={need_x}, "
                                f"max_x={max_x_list[-1]}, dx={p.dx}")
        if p.is_2d:
            need_y = int(np.ceil(max_y_list[-1] / p.get_dy()) * 2)
            assert p.ny >= need_y, (f"Reflections at the boundary might occur: ny={p.ny}, required_Ny={need_y}, "
                                    f"max_y={max_y_list[-1]}, dy={p.get_dy()}")

    grid_files = _element_grid_files(dct, config_dir)
    max_x = reduce_simulation_setup_for_save_and_exit(dct, max_x_list)
    check_simulation_inputs(p, z_source, elements, angles)

    sim_dir = setup_sim_dir(save_dir)
    for gf in grid_files:
        shutil.copyfile(gf, sim_dir / os.path.basename(gf))
    cfg.save(sim_dir / "config.yaml", dct)
    tile_rows = p.chunk_size // p.nx if p.is_2d else None
    resolved = {"memory_budget_gb": p.memory_budget_gb, "chunk_size": p.chunk_size, "tile_rows": tile_rows,
                "fft2_backend": p.fft2_backend, "detector_integrator": p.detector_integrator,
                "save_debug_wavefields": requested["save_debug_wavefields"]}
    cone = p.use_cone_beam_bpm
    computed = {
        "cutoff_angles": angles,
        "cutoff_angles_y": angles_y,
        "max_x": max_x,
        "energy_range": energy_range,
        "source_points": source_points,
        "source_sampling": {
            "units": "m",
            "distribution": "independent_gaussian_xy",
            "range_convention": "[mean - sigma, mean + sigma]; not hard bounds or FWHM",
            "seed": seed,
            "x_mean": (x_range[0] + x_range[1]) / 2,
            "x_sigma": (x_range[1] - x_range[0]) / 2,
            "y_mean": (y_range[0] + y_range[1]) / 2,
            "y_sigma": (y_range[1] - y_range[0]) / 2,
            "y_range_explicit": "y_range" in multisource,
        },
        "fresnel_mode": fresnel_mode_name(p),
        "fresnel_sampling": fresnel_sampling,
        "fresnel_geometry": {
            "version": "cone_beam_similarity_bpm_v1" if cone else ("thin_sample_similarity_v1" if use_fresnel
                                                                   else "off"),
            "reference_z": float(elements[0].z_start) if use_fresnel else None,
            "source_z": float(z_source) if use_fresnel else None,
            "magnification": float(fresnel_m),
            "effective_detector_distance": float(fresnel_z_eff),
            "material_coordinate_sampling": "local_scale_at_slice_midpoint" if cone else (
                "reference_plane" if use_fresnel else "physical_grid"),
            "propagation_step_mapping": "dz/(m_start*m_end)" if cone else (
                "single_z_eff_leg" if use_fresnel else "physical_dz"),
        },
        "runtime": {"big_wave": {"requested": requested, "resolved": resolved, **copy.deepcopy(resolved)}},
        "algorithms": _algorithms_2d(p) if p.is_2d else {},
        "provenance": {"algorithm_version": ALGORITHM_VERSION, "git_commit": _git_commit()},
    }
    cfg.save(sim_dir / "computed.yaml", computed)
    for i, sub in enumerate(sub_dcts):
        sub_dir = get_sub_dir(sim_dir, i)
        os.makedirs(sub_dir)
        cfg.save(sub_dir / "subconfig.yaml", sub)
    logger.info(f"Finished setting up simulation in {sim_dir}")
    return sim_dir
