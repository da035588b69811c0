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


def test_exact_instantiations_match_their_generator(tmp_path):
    # exact_inst_*.cu and exact_dispatch.cu are written by gen_exact_inst.py;
    # regenerating into a scratch copy must reproduce them byte for byte
    import importlib.util
    import shutil
    from pathlib import Path
    csrc = Path(__file__).resolve().parents[1] / "rivin-perm_gb300" / "csrc"
    shutil.copy(csrc / "gen_exact_inst.py", tmp_path / "gen_exact_inst.py")
    spec = importlib.util.spec_from_file_location("gen_exact_inst", tmp_path / "gen_exact_inst.py")
    gen = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(gen)
    gen.main()
    generated = ("exact_inst_*.cu", "exact_dispatch.cu")
    made = sorted(p.name for pat in generated for p in tmp_path.glob(pat))
    assert made == sorted(p.name for pat in generated for p in csrc.glob(pat))
    for name in made:
        assert (tmp_path / name).read_text() == (csrc / name).read_text(), name
