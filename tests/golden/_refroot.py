"""Where the fixture generators find the RAVE-SIM sources they import or read."""
from __future__ import annotations

import os
import sys
from pathlib import Path

ENV = "RAVESIM_REFERENCE"


def reference_root() -> Path:
    """The RAVE-SIM checkout: the first command-line argument, else $RAVESIM_REFERENCE."""
    if len(sys.argv) > 1:
        return Path(sys.argv[1])
    if os.environ.get(ENV):
        return Path(os.environ[ENV])
    raise SystemExit(f"usage: python {Path(sys.argv[0]).name} /path/to/RAVE-SIM  (or set {ENV})")
