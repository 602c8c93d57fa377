"""The reference's default numerical flux (scalarwave1_numflux = upwind) on
the GPU: DG variants, finite-volume and mixed meshes against the reference's
own upwind runs, and the bit-exact finite-volume kernel against the oracle."""
import numpy as np
import pytest

import nmesh_gb300 as ng
from helpers import (PI, RTOL_RHS, RTOL_RK4, UPW_CASES, build_mesh, gaussian_pulses, load,
                     oracle_for, perm_to_mesh, rel_l2, to_mesh_order)

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _gpu(cuda_ok):
    yield


def _kernels(meta):
    if "fv" not in meta:
        return ["eo", "eof", "gather"]
    if meta["fv"].get("patches"):
        return [("eo", "fvx"), ("eof", "fv"), ("eo", "fvc:1:256")]
    return ["fvx", "fv", "fvc"]


@pytest.mark.parametrize("case", UPW_CASES)
def test_upwind_matches_reference(case):
    d, meta = load(case)
    m = build_mesh(meta)
    perm = perm_to_mesh(m, d)
    for kern in _kernels(meta):
        ev = ng.Evolution(m, ng.BC_EXACT_PLANEWAVE, k=meta["k"])
        ev.set_numflux("upwind")
        if "fv" in meta:
            ev.set_fv(meta["fv"]["rec"], meta["fv"]["extrap"])
        for kk in (kern if isinstance(kern, tuple) else (kern,)):
            ev.set_kernel(kk)
        r = ev.rhs(to_mesh_order(d["u0"], perm), 0.0)
        assert rel_l2(r[perm], d["r0"]) <= RTOL_RHS, kern
        u = ev.rk4_steps_host(to_mesh_order(d["u0"], perm), 0.0, meta["dt"], meta["steps"])
        assert rel_l2(u[perm], d["u_final"]) <= RTOL_RK4, kern
        ev.close()


@pytest.mark.parametrize("n,luni", [(4, 1), (7, 0)])
def test_upwind_outgoing_vs_oracle(n, luni):
    m = ng.Mesh.build(ng.MESH_CUBEDSPHERES7, n=n, luni=luni, cs_dc=1.0, cs_r0fac=20.0)
    u = gaussian_pulses(m.coords(), seed=n, rmin=1.0, rmax=6.0)
    u += 1e-2 * np.random.default_rng(n).standard_normal(u.shape)   # face jumps
    o = oracle_for(m, bc=1, numflux="upwind")
    ev = ng.Evolution(m, ng.BC_OUTGOING)
    ev.set_numflux("upwind")
    assert rel_l2(ev.rhs(u, 0.0), o.rhs(u, 0.0)) <= RTOL_RHS
    # LLF and upwind differ (tangential c jumps are not lifted by upwind)
    ev.set_numflux("LLF")
    assert rel_l2(ev.rhs(u, 0.0), o.rhs(u, 0.0)) > 1e-6
    ev.set_numflux("upwind")
    with pytest.raises(ng.NmgError):
        ev.rhs_vjp_device(ev.state_ptr, ev.state_ptr + 8)


def test_upwind_fv_periodic_bitexact():
    m = ng.Mesh.build(ng.MESH_BOX, n=7, luni=1, xc=(PI, PI, PI), box_dout=PI, periodic=True,
                      fv=True)
    xyz = m.coords()
    u = np.stack([np.sin(xyz[:, 0]), np.cos(xyz[:, 1]), np.sin(xyz[:, 2]),
                  np.cos(xyz[:, 0] + xyz[:, 2]), np.sin(xyz[:, 1])], 1)
    u += 0.1 * np.random.default_rng(0).standard_normal(u.shape)
    ev = ng.Evolution(m, ng.BC_OUTGOING)
    ev.set_fv("WENOm5_2", "dnfn_extrap1")
    ev.set_numflux("upwind")
    ev.set_kernel("fvx")
    o = oracle_for(m, bc=1, period=2 * PI, fv_rec="WENOm5_2", fv_extrap="dnfn_extrap1",
                   numflux="upwind")
    assert np.array_equal(ev.rhs(u, 0.0), o.rhs(u, 0.0))
