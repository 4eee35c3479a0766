"""Location of the reference checkout for the CPU tests and fixture scripts that read its
files (parameter sets, geometries, the RuNNer example, the analysis scripts): the
MDT_REFERENCE_ROOT environment variable, else a directory named ``reference`` beside this
repository's directory.  ``None`` when neither exists; the tests that need it then skip
(the GPU machines carry no reference checkout)."""
from __future__ import annotations

import os
from pathlib import Path


def reference_root() -> Path | None:
    env = os.environ.get("MDT_REFERENCE_ROOT")
    cand = Path(env) if env else Path(__file__).resolve().parent.parent.parent / "reference"
    return cand if cand.is_dir() else None
