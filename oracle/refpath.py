"""Where the reference simulator's sources are (TEST INFRASTRUCTURE ONLY).

$EKGSIM_REFERENCE names the directory; without it a checkout called ``reference`` beside this
repository is used.  None when neither exists: the golden fixtures under tests/golden/ then pin
the oracle, and the recipes that compile or run the reference are skipped.
"""
from __future__ import annotations

import os
from typing import Optional

_REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def reference_dir() -> Optional[str]:
    d = os.environ.get("EKGSIM_REFERENCE") or os.path.join(os.path.dirname(_REPO), "reference")
    return d if os.path.isfile(os.path.join(d, "simlib", "simulator.cpp")) else None
