"""The C-ABI library loads and exports every function include/pcd.h declares
(no device calls: runs without a GPU)."""
import os
import re

from conftest import ROOT


def declared_functions():
    src = open(os.path.join(ROOT, "include", "pcd.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(pcd_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    from poisson_caustic_design_gb300 import _lib

    L = _lib.load()
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    # the ctypes table covers the same set
    assert set(names) <= set(_lib.SIGNATURES), set(names) - set(_lib.SIGNATURES)

