"""0d norms on the device (nmg_norms) against the reference's own
MeshVolumeIntegral / MeshExtremumLoc values of u0 (dumped by the reference
run) on a DG and a mixed DG / finite-volume mesh, and against numpy."""
import numpy as np
import pytest

import nmesh_gb300 as ng
from helpers import build_mesh, load, perm_to_mesh, to_mesh_order

pytestmark = pytest.mark.gpu

NAMES = ("pi", "cx", "cy", "cz", "phi")


@pytest.fixture(autouse=True)
def _gpu(cuda_ok):
    yield


@pytest.mark.parametrize("case", ["norms_cs7_l1_n5", "norms_mixcs7_l0_n6"])
@pytest.mark.parametrize("switchable", [False, True])
def test_norms_match_reference(case, switchable):
    d, meta = load(case)
    m = build_mesh(meta)
    perm = perm_to_mesh(m, d)
    ev = ng.Evolution(m, ng.BC_EXACT_PLANEWAVE, k=meta["k"], switchable=switchable)
    if switchable:
        ev.set_element_types(m.fv())
    ev.set_state(to_mesh_order(d["u0"], perm))
    res = ev.norms()
    ref = d["norms"]
    vol = ref[0]
    assert abs(res["volume"] - vol) <= 1e-13 * vol
    for l, name in enumerate(NAMES):
        volint, int2, lo, hi = ref[1 + 4 * l: 5 + 4 * l]
        r = res[name]
        assert abs(r["VolInt"] - volint) <= 1e-12 * np.sqrt(abs(int2) * vol)
        assert abs(r["rms"] - np.sqrt(abs(int2) / vol)) <= 1e-12 * np.sqrt(abs(int2) / vol)
        assert r["min"] == lo and r["max"] == hi
        assert r["maxAbs"] == max(abs(lo), abs(hi))
        assert abs(r["mean"] - volint / vol) <= 1e-12 * np.sqrt(abs(int2) / vol)


def test_norms_of_device_buffer():
    torch = pytest.importorskip("torch")
    m = ng.Mesh.build(ng.MESH_BOX, n=5, luni=1, xc=(0, 0, 0), box_dout=1.0)
    ev = ng.Evolution(m, ng.BC_OUTGOING)
    u = np.random.default_rng(0).standard_normal((m.nelem, 5, m.np))
    du = torch.from_numpy(u.ravel()).cuda()
    res = ev.norms(du.data_ptr())
    assert abs(res["volume"] - 8.0) <= 1e-13 * 8
    assert res["pi"]["min"] == u[:, 0].min() and res["phi"]["max"] == u[:, 4].max()
    x, w, _ = ng.basis(5)
    q = np.einsum("i,j,k->kji", w, w, w).ravel() / 8.0   # 1/det(dXb/dx) = (h/2)^3, h = 1
    assert abs(res["cx"]["VolInt"] - (u[:, 1] * q).sum()) <= 1e-13 * np.abs(u[:, 1]).sum()
