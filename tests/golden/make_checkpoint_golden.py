"""Generate tests/golden/checkpoint_ref/: a run checkpoint written by big-wave's own RunCheckpoint
(big-wave/checkpoint.py:83-208) for complex64 NumpyVectors, so the tests can check that this
package reads big-wave's checkpoints and writes the same format.

    python tests/golden/make_checkpoint_golden.py [/path/to/RAVE-SIM]
"""
from __future__ import annotations

import shutil
import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parent))
from make_golden import import_reference  # noqa: E402

OUT = Path(__file__).resolve().parent / "checkpoint_ref"
N = 64
FINGERPRINT = {"N": N, "nx": 8, "ny": 8, "dtype": np.dtype(np.complex64).str, "wavelength": 6.2e-11,
               "z_detector": 1.5, "source_index": 3}
STATE = {"current_z": 0.125, "element_index": 1, "slice_index": 10, "phase_step": 0, "u_fourier_valid": True,
         "stage": "element_slice"}


def main(root: Path) -> None:
    import_reference(root)
    import checkpoint
    import vector
    rng = np.random.default_rng(7)
    u = (rng.normal(size=N) + 1j * rng.normal(size=N)).astype(np.complex64)
    U = np.fft.fft(u).astype(np.complex64)
    if OUT.exists():
        shutil.rmtree(OUT)
    ck = checkpoint.RunCheckpoint(OUT, FINGERPRINT)
    ck.save(vector.NumpyVector(u.copy()), vector.NumpyVector(U.copy()), **STATE)
    np.save(OUT.parent / "checkpoint_ref_vectors.npy", np.stack([u, U]))
    print("wrote", OUT)


if __name__ == "__main__":
    sys.path.insert(0, str(Path(__file__).resolve().parent))
    from _refroot import reference_root
    main(reference_root())
