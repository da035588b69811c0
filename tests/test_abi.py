"""CPU: the C-ABI library loads and exports every symbol include/*.h declares.

No compute call is made here (there is no GPU in the CPU test run).
"""

import ctypes
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\b(pg_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_symbols()
    for required in ("pg_residues", "pg_schur_residues", "pg_binary_residues",
                     "pg_exact_permanent", "pg_last_error"):
        assert required in names


def test_library_exports_every_declared_symbol():
    from permgpu import _lib
    handle = ctypes.CDLL(str(_lib.LIB_PATH))
    missing = [n for n in declared_symbols() if not hasattr(handle, n)]
    assert not missing, missing


def test_ctypes_signatures_cover_header():
    from permgpu import _lib
    assert set(declared_symbols()) <= set(_lib.SIGNATURES)
