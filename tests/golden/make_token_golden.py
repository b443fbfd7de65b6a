"""Write tests/golden/cancel_tokens.json: big-wave's own answers to every token shape in
token_cases.py, from its history check (big-wave/history.py:33-43), its checkpoint check
(big-wave/checkpoint.py:22-30) and its detector check (big-wave/propagation.py:669-679).

    python tests/golden/make_token_golden.py /path/to/RAVE-SIM   (or set $RAVESIM_REFERENCE)
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

sys.path.insert(0, str(Path(__file__).resolve().parent))
from make_golden import import_reference  # noqa: E402
from token_cases import CASES, outcome  # noqa: E402

OUT = Path(__file__).resolve().parent / "cancel_tokens.json"


def main(root: Path) -> None:
    prop, *_ = import_reference(root)
    import checkpoint
    import history
    checks = {"history": history._cancelled, "checkpoint": checkpoint._cancelled,
              "detector": prop._detector_cancelled}
    out = {name: {case: outcome(fn, make()) for case, make in CASES.items()}
           for name, fn in checks.items()}
    OUT.write_text(json.dumps(out, indent=1, sort_keys=True) + "\n")
    print(json.dumps(out, indent=1, sort_keys=True))


if __name__ == "__main__":
    from _refroot import reference_root
    main(reference_root())
