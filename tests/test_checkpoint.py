"""Checkpoint files in the reference's variables.bin format (host side, no
GPU): element names, reading the reference's own checkpoint, byte-identical
writing, round trips with caller-given names, malformed files, and (where
the reference binary is built here) the reference restarting from a file
this library wrote."""
import os
import shutil
import subprocess
import tempfile

import numpy as np
import pytest

import nmesh_gb300 as ng
from helpers import GOLDEN, build_mesh, load, perm_to_mesh, to_mesh_order

CKPT_CASES = ["ckpt_box_l1_n4", "ckpt_cs7_l1_n3"]
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def ref_file(case):
    return os.path.join(GOLDEN, case + "_variables.bin")


def test_element_names_follow_the_octree():
    m = ng.Mesh.build(ng.MESH_BOX, n=3, luni=2, xc=(0, 0, 0), box_dout=1.0)
    names = m.names()
    assert len(set(names)) == m.nelem == 64
    pat, bbox = m.elements()
    for nm, b in zip(names, bbox):
        # digit bit d is set for the upper half in direction d, level by level
        digits = nm.split("_")[1]
        lo = np.array([b[0], b[2], b[4]])
        want = ""
        origin, size = np.array([-1.0] * 3), 2.0
        for _ in range(2):
            size /= 2
            upper = (lo >= origin + size - 1e-12).astype(int)
            want += str(upper[0] | upper[1] << 1 | upper[2] << 2)
            origin = origin + upper * size
        assert digits == want
    cs = ng.Mesh.build(ng.MESH_CUBEDSPHERES7, n=3, luni=0, cs_dc=1.0, cs_r0fac=20.0)
    assert cs.names() == [f"{p}_" for p in range(7)]


@pytest.mark.parametrize("case", CKPT_CASES)
def test_read_reference_checkpoint(case):
    d, meta = load(case)
    m = build_mesh(meta)
    u = ng.checkpoint_read_host(m, ref_file(case))
    assert np.array_equal(u, to_mesh_order(d["u_final"], perm_to_mesh(m, d)))


@pytest.mark.parametrize("case", CKPT_CASES)
def test_write_is_byte_identical(case, tmp_path):
    d, meta = load(case)
    m = build_mesh(meta)
    u = to_mesh_order(d["u_final"], perm_to_mesh(m, d))
    out = tmp_path / "variables.bin"
    ng.checkpoint_write_host(m, u, out)
    assert out.read_bytes() == open(ref_file(case), "rb").read()


def test_round_trip_with_given_names(tmp_path):
    d, meta = load("ckpt_cs7_l1_n3")
    m0 = build_mesh(meta)
    names = m0.names()
    # a described mesh has no names of its own: the caller passes them
    pat, bbox = m0.elements()
    m = ng.Mesh.from_arrays(bbox, np.ones(m0.nelem, np.int32), m0.coords(),
                            dXdx=m0.dXdx(), pat=pat)
    assert m.names() is None
    with pytest.raises(ng.NmgError):
        ng.checkpoint_write_host(m, np.zeros((m.nelem, 5, m.np)), tmp_path / "x.bin")
    rng = np.random.default_rng(5)
    u = rng.standard_normal((m.nelem, 5, m.np))
    ng.checkpoint_write_host(m, u, tmp_path / "v.bin", names=names)
    # the generated mesh reads it back by name, element for element
    assert np.array_equal(ng.checkpoint_read_host(m0, tmp_path / "v.bin"), u)
    # a reversed name table permutes the elements
    back = ng.checkpoint_read_host(m, tmp_path / "v.bin", names=names[::-1])
    assert np.array_equal(back, u[::-1])


def test_malformed_files_are_rejected(tmp_path):
    d, meta = load("ckpt_box_l1_n4")
    m = build_mesh(meta)
    raw = open(ref_file("ckpt_box_l1_n4"), "rb").read()
    cases = {
        "truncated": raw[: len(raw) // 2],
        "no_header": b"hello\n" + raw,
        "missing_var": raw.replace(b"scalarwave1_cz", b"scalarwave1_qq", 1),
        "missing_elem": raw.replace(b"{\n0_7\n", b"{\n0_6\n", 1),
        "unknown_elem": raw.replace(b"{\n0_7\n", b"{\n9_7\n", 1),
        # variable lines with explicit dimensions: negative, and a product
        # that wraps around 64 bits
        "negative_dims": raw.replace(b"{\n0_7\n64\n0\n", b"{\n0_7\n64\n0 -4 4 4\n", 1),
        "huge_dims": raw.replace(b"{\n0_7\n64\n0\n",
                                 b"{\n0_7\n64\n0 2147483647 2147483647 2147483647\n", 1),
    }
    for name, blob in cases.items():
        p = tmp_path / name
        p.write_bytes(blob)
        with pytest.raises(ng.NmgError):
            ng.checkpoint_read_host(m, p)
    with pytest.raises(ng.NmgError):
        ng.checkpoint_read_host(m, tmp_path / "does_not_exist")
    # a mesh of another order does not accept the file
    m5 = ng.Mesh.build(ng.MESH_BOX, n=5, luni=1, xc=(np.pi,) * 3, box_dout=np.pi)
    with pytest.raises(ng.NmgError):
        ng.checkpoint_read_host(m5, ref_file("ckpt_box_l1_n4"))


def test_reference_restarts_from_written_checkpoint(tmp_path):
    """The reference binary loads a variables.bin written here: a one-step
    run leaves its checkpoint directory, the file is replaced by a new
    state, and the restarted run's first dumped state is that state."""
    exe = os.path.join(ROOT, "oracle", "_ref", "nmesh")
    if not os.path.exists(exe):
        pytest.skip("reference binary not built (make -C oracle/ref)")
    import sys
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import make_golden as mg
    from oracle.refdump import read_dump
    case = "ckpt_box_l1_n4"
    d, meta = load(case)
    m = build_mesh(meta)
    prefix = str(tmp_path / "d")
    par = tmp_path / (case + ".par")
    par.write_text(mg.parfile(case, prefix))
    env = dict(os.environ, OMP_NUM_THREADS="1")
    subprocess.run([exe, str(par)], cwd=tmp_path, env=env, check=True, capture_output=True)
    rng = np.random.default_rng(9)
    u = rng.standard_normal((m.nelem, 5, m.np))
    ng.checkpoint_write_host(m, u, tmp_path / case / "checkpoint" / "variables.bin")
    par.write_text(mg.parfile(case, prefix).replace("iterations = 1", "iterations = 2"))
    res = subprocess.run([exe, str(par)], cwd=tmp_path, env=env, capture_output=True, text=True)
    assert res.returncode == 0, res.stdout[-2000:]
    assert "estarting from checkpoint" in res.stdout
    d0 = read_dump(prefix + "_rhs.bin", True)
    perm = perm_to_mesh(m, {"pat": d0["pat"], "bbox": d0["bbox"]})
    assert np.array_equal(d0["u"], u[perm])
