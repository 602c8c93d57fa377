"""The nmesh-side adapter (nmesh_gb300/adapter/nmg_evolve.c) compiles
against the reference's own headers with -Wall -Werror, and links into the
reference's own program together with libnmg.so with no undefined symbol
(only where the reference sources are present; it is a binding for the
reference, not part of the library)."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REFMAKE = os.path.join(ROOT, "oracle", "ref")


def _reference_dir():
    try:
        res = subprocess.run(["make", "-s", "-C", REFMAKE, "print-ref"], capture_output=True,
                             text=True)
    except OSError:  # no make on this machine
        return ""
    return res.stdout.strip() if res.returncode == 0 else ""


def test_adapter_links_into_the_reference_with_libnmg():
    ref = _reference_dir()
    if not ref or not os.path.isdir(os.path.join(ref, "src")):
        pytest.skip("reference sources not present")
    from nmesh_gb300 import build as nbuild
    nbuild.build()
    res = subprocess.run(["make", "-s", "-C", REFMAKE, "-j8", "adapter"], capture_output=True,
                         text=True)
    assert res.returncode == 0, res.stderr
    exe = os.path.join(ROOT, "oracle", "_ref", "nmesh_gpu")
    assert os.path.exists(exe)
    # the adapter's calls are bound to the library's entry points
    syms = subprocess.run(["nm", "-D", "--undefined-only", exe], capture_output=True,
                          text=True).stdout
    for name in ("nmg_mesh_from_desc", "nmg_create", "nmg_rk4_steps_host",
                 "nmg_evolve_steps_host", "nmg_set_evolve_method", "nmg_last_error"):
        assert name in syms, name
