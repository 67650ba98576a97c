"""The C-ABI libraries load and export every function their headers declare
(no compute calls: this runs without a GPU)."""
import ctypes
import pathlib
import re

import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]


def declared_functions(header: pathlib.Path):
    text = header.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(thmm_[a-z0-9_]+|oracle_[a-z0-9_]+)\s*\(", text)))


def test_product_library_exports_header(thmm):
    from parallel_tree_hmm_gb300 import _lib

    library = ctypes.CDLL(str(_lib.LIBRARY_PATH))
    names = declared_functions(ROOT / "include" / "thmm_gb300.h")
    assert len(names) >= 30
    missing = [name for name in names if not hasattr(library, name)]
    assert not missing, missing


def test_every_declared_entry_point_has_a_python_prototype(thmm):
    from parallel_tree_hmm_gb300 import _lib

    names = declared_functions(ROOT / "include" / "thmm_gb300.h")
    assert sorted(set(names) - set(_lib.PROTOTYPES)) == []


def test_oracle_library_exports_header():
    from oracle import bridge

    library = bridge.library()
    missing = [name for name in declared_functions(ROOT / "oracle" / "oracle.h")
               if not hasattr(library, name)]
    assert not missing, missing


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    from parallel_tree_hmm_gb300 import _lib

    monkeypatch.setattr(_lib, "LIBRARY_PATH", tmp_path / "absent.so")
    monkeypatch.setattr(_lib, "_LIB", None)
    with pytest.raises(RuntimeError, match="missing"):
        _lib.library()
