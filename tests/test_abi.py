"""The C-ABI library loads and exports every function include/nmg.h
declares (no GPU needed: nothing here calls into CUDA)."""
import ctypes
import os
import re

import nmesh_gb300 as ng

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "nmg.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(nmg_[A-Za-z0-9_]+)\s*\(", src)))


def test_header_declares_functions():
    names = declared_functions()
    assert "nmg_create" in names and "nmg_rk4_steps" in names and len(names) >= 25


def test_library_exports_all_declared_symbols():
    lib = ctypes.CDLL(ng._build.build())
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_error_paths_without_gpu():
    L = ng.lib()
    # null arguments are rejected before any CUDA call
    assert L.nmg_mesh_build(None, None) == 1
    assert L.nmg_set_state(None, None) == 1
    assert L.nmg_rhs(None, 0.0, None, None) == 1
    assert L.nmg_basis(1, None, None, None) == 1
