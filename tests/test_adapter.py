"""The nmesh-side adapter (nmesh_gb300/adapter/nmg_evolve.c) compiles
against the reference's own headers (only where the reference sources are
present; it is a binding for the reference, not part of the library)."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = "/root/reference"


def test_adapter_compiles_against_reference_headers():
    gen = os.path.join(ROOT, "oracle", "_ref", "gen")
    if not os.path.isdir(os.path.join(REF, "src")):
        pytest.skip("reference sources not present")
    if not os.path.isdir(gen):
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle", "ref"),
                        os.path.join(ROOT, "oracle", "_ref", "gen",
                                     "nmesh_automatic_initialize.c")],
                       check=True)
    res = subprocess.run(
        ["gcc", "-std=gnu99", "-fsyntax-only", "-Wall", "-Werror", "-I", gen,
         "-I", os.path.join(REF, "src", "main", "main"), "-I", os.path.join(ROOT, "include"),
         os.path.join(ROOT, "nmesh_gb300", "adapter", "nmg_evolve.c")],
        capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
