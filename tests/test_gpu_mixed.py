"""Mixed DG / finite-volume meshes on the GPU through the C ABI: DG elements
(LGL points) next to finite-volume elements (equally spaced points), with the
interface traces interpolated as the reference does (Lagrange from the DG
side, piecewise linear from the FV side).  One RK4 stage is three launches:
interface traces, the DG kernel (writing only DG elements), the FV kernel
(over the FV elements)."""
import numpy as np
import pytest

import nmesh_gb300 as ng
from helpers import (MIX_CASES, PI, RTOL_RHS, RTOL_RK4, build_mesh, gaussian_pulses, load,
                     oracle_for, perm_to_mesh, rel_l2, to_mesh_order)

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _gpu(cuda_ok):
    yield


COMBOS = [("eo", "fvx"), ("eof", "fv"), ("eo", "fvc"), ("gather", "fvx:1:512"), ("auto", None)]


def _set(ev, dg, fv):
    ev.set_kernel(dg)
    if fv:
        ev.set_kernel(fv)


@pytest.mark.parametrize("dg,fv", COMBOS)
@pytest.mark.parametrize("case", MIX_CASES)
def test_mixed_matches_reference(case, dg, fv):
    d, meta = load(case)
    m = build_mesh(meta)
    perm = perm_to_mesh(m, d)
    assert np.array_equal(m.fv()[perm], d["use_fv"])
    ev = ng.Evolution(m, ng.BC_EXACT_PLANEWAVE, k=meta["k"])
    ev.set_fv(meta["fv"]["rec"], meta["fv"]["extrap"])
    ev.set_fv_surface_interp(meta["fv"].get("surf", "linear"))
    _set(ev, dg, fv)
    r = ev.rhs(to_mesh_order(d["u0"], perm), 0.0)
    assert rel_l2(r[perm], d["r0"]) <= RTOL_RHS
    u = ev.rk4_steps_host(to_mesh_order(d["u0"], perm), 0.0, meta["dt"], meta["steps"])
    assert rel_l2(u[perm], d["u_final"]) <= RTOL_RK4


@pytest.mark.parametrize("patches", [[0], [0, 1, 3], [2, 4, 5, 6]])
@pytest.mark.parametrize("n,luni", [(4, 1), (7, 0), (9, 0)])
def test_mixed_cubed_spheres_outgoing_vs_oracle(n, luni, patches):
    m = ng.Mesh.build(ng.MESH_CUBEDSPHERES7, n=n, luni=luni, cs_dc=1.0, cs_r0fac=20.0,
                      fv=patches)
    u = gaussian_pulses(m.coords(), seed=n + luni, rmin=1.0, rmax=6.0)
    u += 1e-2 * np.random.default_rng(n).standard_normal(u.shape)
    rec, ex = "WENOm5_2", "dnfn_extrap1"
    o = oracle_for(m, bc=1, fv_rec=rec, fv_extrap=ex)
    ev = ng.Evolution(m, ng.BC_OUTGOING)
    ev.set_fv(rec, ex)
    ro = o.rhs(u, 0.0)
    assert rel_l2(ev.rhs(u, 0.0), ro) <= RTOL_RHS
    dt = 0.02 / n
    assert rel_l2(ev.rk4_steps_host(u, 0.0, dt, 2), o.rk4(u, dt, 2)) <= RTOL_RK4


def _mixed_box(n, luni, seed, frac=0.3):
    """Periodic box whose elements are finite-volume with probability frac:
    each element's coordinates from the all-DG or the all-FV mesh."""
    kw = dict(n=n, luni=luni, xc=(PI, PI, PI), box_dout=PI, periodic=True)
    mdg = ng.Mesh.build(ng.MESH_BOX, **kw)
    mfv = ng.Mesh.build(ng.MESH_BOX, fv=True, **kw)
    pat, bbox = mdg.elements()
    fv = (np.random.default_rng(seed).random(mdg.nelem) < frac).astype(np.int32)
    fv[0], fv[-1] = 1, 0
    xyz = np.where(fv[:, None, None] == 1, mfv.coords(), mdg.coords())
    m = ng.Mesh.from_arrays(bbox, np.zeros(mdg.nelem, np.int32), xyz, pat=pat,
                            period=(2 * PI,) * 3, fv=fv)
    return m, fv


@pytest.mark.parametrize("rec,ex", [("WENOm5_2", "dnfn_extrap1"), ("WENOm3_2", "no")])
@pytest.mark.parametrize("n,luni", [(5, 2), (7, 1), (8, 1)])
def test_mixed_periodic_box_random_pattern_vs_oracle(n, luni, rec, ex):
    m, fv = _mixed_box(n, luni, seed=10 * n + luni)
    assert m.fv().sum() == fv.sum()
    xyz = m.coords()
    arg = xyz[:, 0] + 2.0 * xyz[:, 1] - xyz[:, 2]
    u = np.stack([np.sin(arg), np.cos(arg), np.sin(2 * arg), np.cos(arg), np.sin(arg)], 1)
    u += 0.05 * np.random.default_rng(n).standard_normal(u.shape)
    o = oracle_for(m, bc=1, period=2 * PI, fv_rec=rec, fv_extrap=ex)
    ev = ng.Evolution(m, ng.BC_OUTGOING)
    ev.set_fv(rec, ex)
    for dg, fvk in (("eo", "fvx"), ("eof", "fv")):
        _set(ev, dg, fvk)
        assert rel_l2(ev.rhs(u, 0.0), o.rhs(u, 0.0)) <= RTOL_RHS
        dt = 0.02 * (2 * PI / 2 ** luni) / n
        l0 = ev.launches
        assert rel_l2(ev.rk4_steps_host(u, 0.0, dt, 3), o.rk4(u, dt, 3)) <= RTOL_RK4
        assert ev.launches - l0 == 3 * (4 * 3 + 1)   # per step: 4 stages x 3 launches + counter
    info = ev.kernel_info()
    assert "eof" in info and "+ fv:" in info


def test_mixed_single_steps_equal_graph_steps():
    m, fv = _mixed_box(6, 1, seed=3)
    u = np.random.default_rng(0).standard_normal((m.nelem, 5, m.np))
    ev = ng.Evolution(m, ng.BC_OUTGOING)
    ev.set_fv("WENOm5_2", "dnfn_extrap1")
    ug = ev.rk4_steps_host(u, 0.0, 0.01, 3)
    ev.set_state(u)
    for s in range(3):
        ev.rk4_step(0.01 * s, 0.01)
    assert np.array_equal(ev.get_state(), ug)


def test_parabolic_surface_interpolation_matches_oracle():
    """fv_surface_interp = parabolic on an outgoing mixed mesh, every DG
    variant, against the oracle; switching back to linear restores the
    linear traces."""
    m = ng.Mesh.build(ng.MESH_CUBEDSPHERES7, n=7, luni=1, cs_dc=1.0, cs_r0fac=20.0, fv=[0, 3])
    u = gaussian_pulses(m.coords(), seed=8, rmin=1.0, rmax=4.0)
    for surf in ("parabolic", "linear"):
        o = oracle_for(m, bc=1, fv_rec="WENOm5_2", fv_extrap="dnfn_extrap1",
                       fv_surface_interp=surf)
        ev = ng.Evolution(m, ng.BC_OUTGOING)
        ev.set_fv("WENOm5_2", "dnfn_extrap1")
        ev.set_fv_surface_interp("parabolic")
        ev.set_fv_surface_interp(surf)
        assert rel_l2(ev.rhs(u, 0.0), o.rhs(u, 0.0)) <= RTOL_RHS
        assert rel_l2(ev.rk4_steps_host(u, 0.0, 0.002, 2), o.rk4(u, 0.002, 2)) <= RTOL_RK4
    with pytest.raises(ng.NmgError):
        ng.Evolution(ng.Mesh.build(ng.MESH_BOX, n=5, luni=1), ng.BC_OUTGOING) \
            .set_fv_surface_interp("parabolic")
