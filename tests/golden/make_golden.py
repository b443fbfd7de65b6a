"""Generate tests/golden/bigwave_golden.npz by running big-wave itself on seeded inputs.

Run in a checkout that has the RAVE-SIM sources (pass its path, or set $RAVESIM_REFERENCE):
    python tests/golden/make_golden.py [/path/to/RAVE-SIM]
big-wave is imported with stub modules for its optional dependencies (bfpy, ruamel.yaml,
h5py, nist_lookup.xraydb_plugin), none of which the 2D in-memory path uses; `import config`
comes first because of big-wave's circular imports (examples/minimal_xpci/run.py:97-99).
The fixture holds every input and output, so the tests never need the reference.
"""
from __future__ import annotations

import sys
import types
from pathlib import Path

import numpy as np

OUT = Path(__file__).resolve().parent / "bigwave_golden.npz"


def import_reference(root: Path):
    paths = [str(root / "big-wave"), str(root / "nist_lookup"), str(root)]
    sys.path[:0] = paths
    bf = types.ModuleType("bfpy")
    bf.ChunkedEditor = object
    ru = types.ModuleType("ruamel")
    ry = types.ModuleType("ruamel.yaml")
    ryc = types.ModuleType("ruamel.yaml.comments")
    ry.YAML = object
    ryc.CommentedMap = dict
    ru.yaml = ry
    ry.comments = ryc
    xp = types.ModuleType("nist_lookup.xraydb_plugin")

    def _no_db(*a, **k):
        raise RuntimeError("Chantler lookups are not used by the golden cases")
    xp.xray_delta_beta = _no_db
    sys.modules.update({"bfpy": bf, "ruamel": ru, "ruamel.yaml": ry, "ruamel.yaml.comments": ryc,
                        "h5py": types.ModuleType("h5py"), "nist_lookup.xraydb_plugin": xp})
    import config  # noqa: F401  (must precede the others)
    import multisim
    import optical_element
    import plasma_sample
    import propagation
    import source
    import vector
    import wavesim
    return propagation, optical_element, plasma_sample, source, vector, wavesim, multisim


def cfield(rng, ny, nx, dtype):
    return (rng.normal(size=(ny, nx)) + 1j * rng.normal(size=(ny, nx))).astype(dtype)


def main(root: Path) -> None:
    prop, oe, ps, src, vec, ws, ms = import_reference(root)
    NV = vec.NumpyVector
    rng = np.random.default_rng(20261203)
    g: dict[str, np.ndarray] = {}

    # -- fft2 / ifft2 (vector.py:341-347) -------------------------------------------------
    for name, (ny, nx, dt) in {"c128_32x64": (32, 64, np.complex128), "c64_64x128": (64, 128, np.complex64)}.items():
        x = cfield(rng, ny, nx, dt)
        a, b = NV(x.reshape(-1).copy()), NV(np.zeros(nx * ny, dt))
        a.fft2(b, nx, ny)
        c = NV(np.zeros(nx * ny, dt))
        b.ifft2(c, nx, ny)
        g[f"fft2_{name}_in"], g[f"fft2_{name}_out"], g[f"fft2_{name}_inv"] = x, b.vec.reshape(ny, nx).copy(), c.vec.reshape(ny, nx).copy()

    # -- cutoff (propagation.py:298-326), active mask, rectangular spacing -----------------
    nx, ny, dx, dy = 64, 48, 1e-7, 1.3e-7
    x = cfield(rng, ny, nx, np.complex128)
    v = NV(x.reshape(-1).copy())
    prop.apply_frequency_cutoff_2d(v, 2.0e6, dx, dy, nx, ny, nx * 4)
    g["cutoff_in"], g["cutoff_out"] = x, v.vec.reshape(ny, nx)
    g["cutoff_params"] = np.array([nx, ny, dx, dy, 2.0e6])

    # -- propagate_2d (propagation.py:396-442), c128 and c64, plus skip_fft --------------
    wl8 = prop.convert_energy_wavelength(8000.0)
    for name, dt in {"c128": np.complex128, "c64": np.complex64}.items():
        x = cfield(rng, ny, nx, dt)
        u, U = NV(x.reshape(-1).copy()), NV(np.zeros(nx * ny, dt))
        prop.propagate_2d(u, U, dx, dy, wl8, 0.003, nx * 4, 2.0e6, nx, ny)
        g[f"prop_{name}_in"], g[f"prop_{name}_u"], g[f"prop_{name}_U"] = x, u.vec.reshape(ny, nx).copy(), U.vec.reshape(ny, nx).copy()
        prop.propagate_2d(u, U, dx, dy, wl8, 0.011, nx * 4, 2.5e6, nx, ny, skip_fft=True)
        g[f"prop_{name}_skip_u"], g[f"prop_{name}_skip_U"] = u.vec.reshape(ny, nx).copy(), U.vec.reshape(ny, nx).copy()
    g["prop_params"] = np.array([nx, ny, dx, dy, wl8, 0.003, 2.0e6, 0.011, 2.5e6])

    # -- point source (propagation.py:458-484; source.py:97-107) --------------------------
    p = prop.SimParams(N=40 * 28, nx=40, ny=28, dx=0.7e-6, dy=1.1e-6, z_detector=0.3, detector_size=28 * 1.1e-6,
                       detector_size_x=40 * 0.7e-6, detector_size_y=28 * 1.1e-6, detector_pixel_size_x=0.7e-6,
                       detector_pixel_size_y=1.1e-6, wl=1.3e-10, chunk_size=40 * 4)
    u = NV(np.zeros(p.N, np.complex128))
    prop.propagate_analytically_2d(u, 0.3, 1.2e-6, -2.4e-6, p)
    g["ps_analytic"] = u.vec.reshape(28, 40)
    g["ps_analytic_params"] = np.array([40, 28, 0.7e-6, 1.1e-6, 0.3, 1.2e-6, -2.4e-6, 1.3e-10])
    p2 = prop.SimParams(N=64 * 64, nx=64, ny=64, dx=1e-6, dy=1e-6, z_detector=1.0, detector_size=64e-6,
                        detector_pixel_size_x=1e-6, detector_pixel_size_y=1e-6,
                        wl=prop.convert_energy_wavelength(20000.0), chunk_size=64 * 8)
    for name, dt in {"c128": np.complex128, "c64": np.complex64}.items():
        u, U = NV(np.zeros(p2.N, dt)), NV(np.zeros(p2.N, dt))
        src.PointSource(x=3e-6, y=-2e-6, z=0.0).propagate_to(2.0, p2, 0.3e6, u, U, None)
        g[f"ps_prop_{name}_u"], g[f"ps_prop_{name}_U"] = u.vec.reshape(64, 64).copy(), U.vec.reshape(64, 64).copy()
    g["ps_prop_params"] = np.array([64, 64, 1e-6, 1e-6, 2.0, 3e-6, -2e-6, p2.wl, 0.3e6])

    # -- Fresnel-scaled source plane (source.py:62-95) -----------------------------------
    pf = prop.SimParams(N=64 * 48, nx=64, ny=48, dx=0.4e-6, dy=0.5e-6, z_detector=1.5, detector_size=64 * 0.4e-6,
                        detector_pixel_size_x=0.4e-6, detector_pixel_size_y=0.5e-6,
                        wl=prop.convert_energy_wavelength(30000.0), chunk_size=64 * 8, use_fresnel_scaling=True)
    pf.configure_fresnel_detector(0.0, 1.0)
    for name, dt in {"c128": np.complex128, "c64": np.complex64}.items():
        u, U = NV(np.zeros(pf.N, dt)), NV(np.zeros(pf.N, dt))
        src.PointSource(x=25e-6, y=-40e-6, z=0.0).propagate_to(1.0, pf, 0.8e6, u, U, None)
        g[f"fp_{name}_u"], g[f"fp_{name}_U"] = u.vec.reshape(48, 64).copy(), U.vec.reshape(48, 64).copy()
    g["fp_params"] = np.array([64, 48, 0.4e-6, 0.5e-6, 1.0, 25e-6, -40e-6, pf.wl, 0.8e6])

    # -- voxel Sample (optical_element.py:502-596): shell, bilinear (pitch != dx), offsets --
    nx = ny = 64
    dx = dy = 0.5e-6
    wl20 = prop.convert_energy_wavelength(20000.0)
    px, py, pz, nz = 0.7e-6, 0.6e-6, 1.5e-6, 6
    zz = (np.arange(nz) - (nz - 1) / 2.0)[:, None, None] * pz
    yy = (np.arange(60) - 30.0)[None, :, None] * py
    xx = (np.arange(52) - 26.0)[None, None, :] * px
    r = np.sqrt(xx ** 2 + yy ** 2 + zz ** 2)
    grid = ((r <= 14e-6) & (r >= 9e-6)).astype(np.uint32) + ((r < 5e-6)).astype(np.uint32) * 2
    db_list = np.array([0.0, 3.2e-6 + 2.1e-8j, 1.1e-6 + 4.0e-9j], dtype=np.complex128)
    for name, dt in {"c128": np.complex128, "c64": np.complex64}.items():
        pp = prop.SimParams(N=nx * ny, nx=nx, ny=ny, dx=dx, dy=dy, z_detector=0.1, detector_size=nx * dx,
                            detector_pixel_size_x=dx, detector_pixel_size_y=dy, wl=wl20, chunk_size=nx * 8)
        s = oe.Sample(z_start=0.05, pixel_size_x=px, pixel_size_z=pz, grid=grid,
                      materials=[oe.Material("A", 1.0), oe.Material("B", 1.0)],
                      x_positions=np.array([0.3e-6]), pixel_size_y=py, y_positions=np.array([-0.2e-6]))
        s.db_list = db_list
        u0 = (np.exp(1j * rng.uniform(0, 0.1, size=(ny, nx))) * (1 + 0.05 * rng.normal(size=(ny, nx)))).astype(dt)
        u, U = NV(u0.reshape(-1).copy()), NV(np.zeros(nx * ny, dt))
        s.apply(u, U, pp, 0.6 / dx, 0, None)
        g[f"sample_{name}_in"], g[f"sample_{name}_u"], g[f"sample_{name}_U"] = u0, u.vec.reshape(ny, nx).copy(), U.vec.reshape(ny, nx).copy()
    g["sample_grid"], g["sample_db"] = grid, db_list
    g["sample_params"] = np.array([nx, ny, dx, dy, wl20, px, py, pz, 0.3e-6, -0.2e-6, 0.6 / dx, 0.05])

    # -- PlasmaSample (plasma_sample.py:126-233) with injected Chantler scalars -----------
    shape = (3, 22, 26)
    ne = rng.uniform(0, 5e21, size=shape)
    ne[:, :3, :] = 0.0
    ni = ne / 3.5 * rng.uniform(0.8, 1.2, size=shape)
    te = rng.uniform(20, 500, size=shape)
    zs = rng.uniform(1.0, 3.5, size=shape)
    sf = (6.4, 0.013, 3.5, 18.5)
    nx, ny, dx = 32, 32, 0.6e-6
    pl = ps.PlasmaSample(z_start=0.02, pixel_size_x=0.8e-6, pixel_size_z=2e-6, ne_grid=ne, ni_grid=ni,
                         te_grid=te, zstar_grid=zs, Z=6, x_positions=np.array([0.1e-6]),
                         pixel_size_y=0.9e-6, y_positions=np.array([0.25e-6]))
    pl._scattering_factors = lambda energy: sf
    pp = prop.SimParams(N=nx * ny, nx=nx, ny=ny, dx=dx, dy=dx, z_detector=0.1, detector_size=nx * dx,
                        detector_pixel_size_x=dx, detector_pixel_size_y=dx, wl=wl8, chunk_size=nx * 4)
    u0 = np.ones((ny, nx), np.complex128)
    u, U = NV(u0.reshape(-1).copy()), NV(np.zeros(nx * ny, np.complex128))
    pl.apply(u, U, pp, 0.5 / dx, 0, None)
    from nist_lookup.physical_constants import PLANCK_HC, R_ELECTRON_CM
    g["plasma_ne"], g["plasma_ni"], g["plasma_te"], g["plasma_zs"] = ne, ni, te, zs
    g["plasma_u"], g["plasma_U"] = u.vec.reshape(ny, nx).copy(), U.vec.reshape(ny, nx).copy()
    g["plasma_params"] = np.array([nx, ny, dx, dx, wl8, 0.8e-6, 0.9e-6, 2e-6, 0.1e-6, 0.25e-6, 0.5 / dx,
                                   *sf, prop.convert_energy_wavelength(wl8), PLANCK_HC, R_ELECTRON_CM])

    # -- detectors (propagation.py:836-946, 995-1110), non-integer ratios ----------------
    for integ in ("area_v1", "legacy_fastwave"):
        pdet = prop.SimParams(N=11 * 7, nx=11, ny=7, dx=0.7, dy=1.1, z_detector=8.0, detector_size=5.2,
                              detector_size_x=5.2, detector_size_y=5.1, detector_pixel_size_x=1.3,
                              detector_pixel_size_y=1.7, wl=1e-10, chunk_size=22, detector_integrator=integ)
        f = cfield(rng, 7, 11, np.complex128)
        import warnings
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            out = prop.square_and_downsample_2d(NV(f.reshape(-1).copy()), pdet, 8.0)
        g[f"det_{integ}_small_in"], g[f"det_{integ}_small_out"] = f, out
        pdet2 = prop.SimParams(N=64 * 64, nx=64, ny=64, dx=0.25e-6, dy=0.25e-6, z_detector=0.4,
                               detector_size=15e-6, detector_size_x=15e-6, detector_size_y=14e-6,
                               detector_pixel_size_x=0.7e-6, detector_pixel_size_y=0.6e-6, wl=1e-10,
                               chunk_size=64 * 4, detector_integrator=integ)
        f2 = cfield(rng, 64, 64, np.complex64)
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            out2 = prop.square_and_downsample_2d(NV(f2.reshape(-1).copy()), pdet2, 0.4)
        g[f"det_{integ}_64_in"], g[f"det_{integ}_64_out"] = f2, out2

    # -- run_simulation (wavesim.py:89-409): point source -> gap -> Sample -> final leg ----
    nx = ny = 64
    pr = prop.SimParams(N=nx * ny, nx=nx, ny=ny, dx=0.5e-6, dy=0.5e-6, z_detector=0.65, detector_size=24e-6,
                        detector_size_x=24e-6, detector_size_y=20e-6, detector_pixel_size_x=1.5e-6,
                        detector_pixel_size_y=1.25e-6, wl=wl20, chunk_size=nx * 8)
    grid2 = np.zeros((4, 66, 66), np.uint32)
    yy2, xx2 = np.mgrid[0:66, 0:66]
    grid2[:, (yy2 - 33) ** 2 + (xx2 - 30) ** 2 < 100] = 1
    samp = oe.Sample(z_start=0.5, pixel_size_x=0.5e-6, pixel_size_z=2e-6, grid=grid2,
                     materials=[oe.Material("W", 19.3)], x_positions=np.array([0.0]),
                     pixel_size_y=0.5e-6, y_positions=np.array([0.0]))
    table = [(oe.Material("W", 19.3), np.complex128(4.2e-6 + 1.9e-7j))]
    u, U = NV(np.zeros(pr.N, np.complex128)), NV(np.zeros(pr.N, np.complex128))
    source_obj = src.PointSource(x=1e-6, y=0.0, z=0.0)
    angles = [0.6 * np.arcsin(pr.wl / (2 * pr.dx)), 0.7 * np.arcsin(pr.wl / (2 * pr.dx))]
    outs = ws.run_simulation(pr, source_obj, [samp], angles, u, U, table, Path("."), Path("."), False)
    g["run_out"] = outs[0]
    g["run_u"] = u.vec.reshape(ny, nx)
    g["run_grid"] = grid2
    g["run_params"] = np.array([*angles, wl20])

    # -- generate_energies_from_spectrum (multisim.py:695-724) ---------------------------
    e = np.arange(10, 51, dtype=np.float64) * 1e3
    inten = np.clip((45e3 - e) / e, 0, None) * np.exp(-np.linspace(6.9, 0.1, e.size))
    g["spectrum_e"], g["spectrum_i"] = e, inten
    g["spectrum_draw"] = ms.generate_energies_from_spectrum(e, inten, np.random.RandomState(11), (15e3, 40e3), 64)

    # big-wave mutates U.vec in place (modify_chunked), so every stored array is a copy
    np.savez_compressed(OUT, **{k: np.array(v, copy=True) for k, v in g.items()})
    print(f"wrote {OUT} ({OUT.stat().st_size / 1024:.0f} KiB, {len(g)} arrays)")


if __name__ == "__main__":
    sys.path.insert(0, str(Path(__file__).resolve().parent))
    from _refroot import reference_root
    main(reference_root())
