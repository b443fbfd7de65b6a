"""Cancel tokens read the way big-wave reads them in each step: history and checkpoints never call
the token (big-wave/history.py:33-43, big-wave/checkpoint.py:22-30); the detector calls a callable
token first (big-wave/propagation.py:669-679). tests/golden/cancel_tokens.json holds big-wave's own
answers for every token shape in tests/golden/token_cases.py."""
import importlib
import json
import sys
from pathlib import Path

import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLDEN))
from token_cases import CASES, outcome  # noqa: E402

EXPECTED = json.loads((GOLDEN / "cancel_tokens.json").read_text())


def _check(module: str):
    return importlib.import_module(f"3d_ravesim_gb300.{module}")._cancelled


@pytest.mark.parametrize("step,module", [("history", "history"), ("checkpoint", "checkpoint"),
                                         ("detector", "propagation")])
@pytest.mark.parametrize("case", sorted(CASES))
def test_token_answer_matches_bigwave(step, module, case):
    assert outcome(_check(module), CASES[case]()) == EXPECTED[step][case]


def test_progress_callback_that_is_also_an_event_cancels_a_checkpoint_save(tmp_path):
    """The object a run passes as both progress callback and cancel token is read through is_set
    by the checkpoint writer, never called with no arguments."""
    import torch
    ck = importlib.import_module("3d_ravesim_gb300.checkpoint")

    class Field:
        def __init__(self):
            self.vec = torch.zeros(64, dtype=torch.complex64)

    token = CASES["progress_callback_with_is_set"]()
    fp = {"N": 64, "nx": 8, "ny": 8, "dtype": "<c8", "wavelength": 6.2e-11, "z_detector": 1.5,
          "source_index": 0}
    with pytest.raises(InterruptedError):
        ck.RunCheckpoint(tmp_path, fp, cancel_token=token).save(
            Field(), Field(), current_z=0.0, element_index=0, slice_index=0, u_fourier_valid=False,
            stage="s")
