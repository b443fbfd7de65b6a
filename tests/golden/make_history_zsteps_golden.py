"""Generate tests/golden/history_zsteps.json: big-wave's History z-step rule
(big-wave/history.py:370-378, _history_z_steps) on a spread of (dz, hist_dz) pairs: exact and
inexact multiples, a last step just above and just below half a step, dz below one step, and
seeded random pairs over six decades.

    python tests/golden/make_history_zsteps_golden.py [/path/to/RAVE-SIM]
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parent))
from make_golden import import_reference  # noqa: E402

OUT = Path(__file__).resolve().parent / "history_zsteps.json"


def cases() -> list:
    fixed = [(1.0, 0.1), (0.3, 0.1), (0.7, 0.1), (1.0, 0.3), (1.0, 0.4), (1.0, 0.5), (1.0, 0.6),
             (1.0, 1.0), (1.0, 2.0), (0.0, 0.1), (1e-9, 1e-3), (0.25, 0.1), (0.2500001, 0.1),
             (0.2499999, 0.1), (0.15, 0.1), (0.1500001, 0.1), (2.45, 0.7), (0.5, 1e-3), (0.9, 0.45)]
    rng = np.random.default_rng(11)
    rand = [(float(10.0 ** rng.uniform(-4, 1)), float(10.0 ** rng.uniform(-4, 0))) for _ in range(200)]
    return [list(c) for c in fixed] + [list(c) for c in rand if c[0] / c[1] < 300]


def main(root: Path) -> None:
    import_reference(root)
    import history
    out = [{"dz": dz, "hist_dz": h, "z": history._history_z_steps(dz, h).tolist()} for dz, h in cases()]
    OUT.write_text(json.dumps(out))
    print("wrote", OUT, len(out), "cases")


if __name__ == "__main__":
    sys.path.insert(0, str(Path(__file__).resolve().parent))
    from _refroot import reference_root
    main(reference_root())
