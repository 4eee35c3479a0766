"""The C-ABI library builds for sm_103a, loads without a GPU and exports every symbol
include/mdt_gpu.h declares (no compute calls: this runs without a GPU)."""
import ctypes as ct
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols():
    txt = (ROOT / "include" / "mdt_gpu.h").read_text()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(mdt_[a-z0-9_]+)\s*\(", txt)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ("mdt_create", "mdt_calc_force", "mdt_md_steps", "mdt_propagate_1", "mdt_propagate_2"):
        assert s in syms


def test_library_exports_every_declared_symbol(built_lib):
    lib = ct.CDLL(str(built_lib))
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_python_binding_covers_header(built_lib):
    from md_tian2_gb300 import _lib
    assert set(declared_symbols()) <= set(_lib.SIGNATURES), set(declared_symbols()) - set(_lib.SIGNATURES)


def test_create_fails_loudly_without_gpu(built_lib):
    import pytest
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from md_tian2_gb300._lib import EngineError
    from md_tian2_gb300.engine import Engine
    with pytest.raises(EngineError):
        Engine(0)
