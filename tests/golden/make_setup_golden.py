"""Generate the simulation directories under tests/golden/ that big-wave's own setup_simulation
(big-wave/multisim.py:727-1399) prepares, so the tests can check this package's source sampling,
its parsing of a prepared directory, and its own setup_simulation file by file:

* setup_ref/: 256 x 256, one voxel sample (W, Au), five point sources (uniform energies in
  15-30 keV, Gaussian source positions, seed 42);
* setup_ref_plasma/: 512 x 512 (nx from N / ny), a voxel sample then a plasma sample with a formula and one with a
  bare Z, chunk_size "auto" under a 2 GB runtime budget, c16, the detector directly behind the
  last element (the cutoff-angle rule for a last leg that is never propagated), three sources;
* setup_ref_fresnel/: 256 x 256 with use_fresnel_scaling and one voxel sample, the detector
  larger than the grid (the similarity frame), four sources;
* setup_ref_exit/: a voxel sample followed by a save_and_exit marker and a second sample (the
  element list cut at the marker, the detector moved to it), two sources;
* setup_errors.json: the exception type and message big-wave raises for each input of
  `setup_cases.error_cases` (non-power-of-two axis, detector larger than the grid, the source-to-sample
  and the cutoff Nyquist conditions, reflections at the boundary, thin Fresnel scaling with two elements, an unknown
  multisource, a bad y_range, overlapping elements, a non-integer chunk size);
* setup_rules.json: big-wave's compute_cutoff_angles on 60 seeded geometries and its
  resolve_sim_params on 40 seeded requests, with their outputs or exceptions.

big-wave needs two things this container does not have, which the script supplies:
* ruamel.yaml: config.load / config.save go through a stand-in backed by this package's
  yaml_io (so the YAML text is yaml_io's; the values are big-wave's);
* SQLAlchemy, under nist_lookup's database layer: the minimal stand-in of
  make_chantler_golden.py, so nist_lookup's own xray_delta_beta and big-wave's own plasma
  scattering factors run unmodified over nist_lookup's xrayref.db.

computed.yaml's provenance.git_commit (the reference checkout's revision) is replaced by
"reference" so the fixtures do not depend on the checkout. big-wave then runs source 0 of the
plasma, Fresnel and save_and_exit directories with its own run_single_simulation (NumPy, the
configured dtype); setup_runs.npz keeps their detector images and, for save_and_exit, every
fourth row and column of the field it saved.

    python tests/golden/make_setup_golden.py [/path/to/RAVE-SIM]
"""
from __future__ import annotations

import importlib
import json
import shutil
import sys
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
sys.path.insert(0, str(HERE.parents[1]))
from make_chantler_golden import _fake_sqlalchemy  # noqa: E402
from make_golden import import_reference  # noqa: E402
from setup_cases import CASES, RUN_CASES, error_cases, write_inputs  # noqa: E402

import numpy as np  # noqa: E402


def main(root: Path) -> None:
    _prop, oe, _ps, _src, _vec, _ws, ms = import_reference(root)
    import config as bw_config
    yio = importlib.import_module("3d_ravesim_gb300.yaml_io")

    class YamlStandIn:
        def __init__(self, typ=None):
            pass

        def indent(self, **kw):
            pass

        def load(self, path):
            return yio.load(path)

        def dump(self, dct, f):
            f.write(yio.dumps(dct))

    bw_config.YAML = YamlStandIn
    sys.modules.update(_fake_sqlalchemy())
    sys.modules.pop("nist_lookup.xraydb_plugin", None)  # the stub import_reference put there
    real = importlib.import_module("nist_lookup.xraydb_plugin")
    oe.xray_delta_beta = real.xray_delta_beta
    ms._git_commit = lambda: "reference"
    runs: dict = {}
    with tempfile.TemporaryDirectory() as tmp:
        tmp = Path(tmp)
        write_inputs(tmp)
        for name, make in CASES.items():
            sim = ms.setup_simulation(make(), tmp, tmp / f"out_{name}")
            out = HERE / name
            if out.exists():
                shutil.rmtree(out)
            shutil.copytree(sim, out)
            print("wrote", out)
            if name in RUN_CASES:
                # big-wave runs source 0 of the directory it prepared (its own NumPy path)
                ms.run_single_simulation(sim, 0, tmp / f"scratch_{name}")
                runs[f"{name}_detected"] = np.load(sim / "00000000" / "detected.npy")
                u_file = sim / "00000000" / "u_0000.npy"
                if u_file.exists():
                    n = CASES[name]()["sim_params"]
                    runs[f"{name}_u_sub"] = np.load(u_file).reshape(n["ny"], n["nx"])[::4, ::4].copy()
        # the inputs big-wave rejects: the exception type and message of each
        errors = {}
        for name, dct in error_cases().items():
            try:
                ms.setup_simulation(dct, tmp, tmp / f"err_{name}")
            except Exception as exc:  # noqa: BLE001 - every rejection is recorded as raised
                errors[name] = [type(exc).__name__, str(exc)]
            else:
                raise SystemExit(f"big-wave accepted the error case {name}")
    np.savez(HERE / "setup_runs.npz", **runs)
    print("wrote", HERE / "setup_runs.npz", sorted(runs))
    (HERE / "setup_errors.json").write_text(json.dumps(errors, indent=1) + "\n")
    print("wrote", HERE / "setup_errors.json")
    (HERE / "setup_rules.json").write_text(json.dumps(rule_cases(_prop, bw_config), indent=1) + "\n")
    print("wrote", HERE / "setup_rules.json")


def rule_cases(prop, bw_config) -> dict:
    """big-wave's compute_cutoff_angles (propagation.py:524-622) on seeded geometries, and its
    resolve_sim_params (config.py:230-315) on seeded sim_params / runtime requests: the inputs
    with the outputs, or the exception each raises."""
    rng = np.random.default_rng(11)
    cutoffs = []
    for i in range(60):
        n_el = int(rng.integers(0, 4))
        z_det = float(rng.uniform(0.5, 3.0))
        zs = sorted(float(v) for v in rng.uniform(0.05, z_det * 0.9, n_el))
        heights = [float(v) for v in rng.uniform(1e-6, 2e-3, n_el)]
        if n_el and i % 5 == 0:  # the detector right behind the last element
            z_det = zs[-1] + heights[-1] + float(rng.uniform(0, 5e-9))
        args = {"detector_size": float(rng.uniform(1e-5, 5e-3)), "dx": float(10 ** rng.uniform(-8.5, -7)),
                "energy_range": sorted(float(v) for v in rng.uniform(5e3, 5e4, 2)), "z_source": 0.0,
                "z_distances": zs, "element_heights": heights, "z_detector": z_det,
                "max_x": float(rng.uniform(0, 2e-4))}
        try:
            angles, widths = prop.compute_cutoff_angles(**{**args, "energy_range": tuple(args["energy_range"])})
            cutoffs.append({"args": args, "angles": [float(a) for a in angles], "widths": [float(w) for w in widths]})
        except Exception as exc:  # noqa: BLE001
            cutoffs.append({"args": args, "error": [type(exc).__name__, str(exc)]})
    resolves = []
    for i in range(40):
        ny = int(2 ** rng.integers(1, 12))
        nx = int(2 ** rng.integers(4, 14))
        sim = {"N": nx * ny, "ny": ny, "dx": 1e-7, "z_detector": 1.0, "detector_pixel_size_x": 1e-6,
               "detector_pixel_size_y": 1e-6}
        if i % 3:
            sim["nx"] = nx
        runtime = {}
        choice = int(rng.integers(0, 4))
        if choice == 0:
            sim["chunk_size"] = int(rng.integers(1, nx * ny * 2))
        elif choice == 1:
            runtime["chunk_size"] = "auto"
        if i % 4 == 0:
            runtime["memory_budget_gb"] = float(rng.choice([0.25, 0.5, 1.0, 2.0, 6.0, 64.0]))
        if i % 7 == 0:
            runtime["detector_integrator"] = "legacy_fastwave"
        dct = {"sim_params": sim, "dtype": str(rng.choice(["c8", "c16"]))}
        if runtime:
            dct["runtime"] = {"big_wave": runtime}
        try:
            resolves.append({"dct": dct, "out": bw_config.resolve_sim_params(dct)})
        except Exception as exc:  # noqa: BLE001
            resolves.append({"dct": dct, "error": [type(exc).__name__, str(exc)]})
    return {"compute_cutoff_angles": cutoffs, "resolve_sim_params": resolves}


if __name__ == "__main__":
    sys.path.insert(0, str(Path(__file__).resolve().parent))
    from _refroot import reference_root
    main(reference_root())
