"""Generate tests/golden/plasma_db_golden.npz: big-wave's plasma_delta_beta_grid_multi
(big-wave/plasma.py:380-434) on seeded (n_e, n_i, T_e, Z*) tiles with the model's edge cases
(Z* above Z-bar, so q clips to 1; zero densities and temperatures; Z-bar = 0, where every ion
counts as bound; z2bar = 0, which turns the free-free term off) at two energies.

    python tests/golden/make_plasma_db_golden.py [/path/to/RAVE-SIM]
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parent))
from make_golden import import_reference  # noqa: E402

OUT = Path(__file__).resolve().parent / "plasma_db_golden.npz"
SCALARS = [(14.2, 0.031, 13.0, 169.0), (6.1, 0.0045, 6.0, 36.0), (29.5, 0.4, 0.0, 0.0), (14.2, 0.031, 13.0, 0.0)]
ENERGIES = [8000.0, 25000.0]


def tiles(rng, shape=(9, 11)):
    ne = 10.0 ** rng.uniform(19, 23, shape)
    ni = ne / rng.uniform(1, 14, shape)
    te = 10.0 ** rng.uniform(0, 3.5, shape)
    zstar = rng.uniform(0, 16, shape)
    ne[0, :3] = 0.0
    ni[1, :3] = 0.0
    te[2, :3] = 0.0
    zstar[3, :3] = 0.0
    zstar[4, :3] = 20.0
    return ne, ni, te, zstar


def main(root: Path) -> None:
    sys.path[:0] = [str(root / "big-wave")]
    import_reference(root)
    import plasma
    rng = np.random.default_rng(5)
    ne, ni, te, zstar = tiles(rng)
    out = {"ne": ne, "ni": ni, "te": te, "zstar": zstar, "scalars": np.array(SCALARS),
           "energies": np.array(ENERGIES)}
    for i, sc in enumerate(SCALARS):
        for j, e in enumerate(ENERGIES):
            d, b, a = plasma.plasma_delta_beta_grid_multi(ne, ni, te, zstar, *sc, e)
            out[f"delta_{i}_{j}"], out[f"beta_{i}_{j}"], out[f"atlen_{i}_{j}"] = d, b, a
    np.savez_compressed(OUT, **out)
    print("wrote", OUT)


if __name__ == "__main__":
    sys.path.insert(0, str(Path(__file__).resolve().parent))
    from _refroot import reference_root
    main(reference_root())
