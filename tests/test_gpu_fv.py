"""Finite-volume elements (the reference's fv_divf path with WENO midpoint
states and LLF) on the GPU through the C ABI, against the reference's own
all-FV outputs and against the oracle.

The FV kernel rounds every operation in the reference's order, so wherever
no exact-data outer face is involved (periodic box, outgoing-radiation
boundary) the GPU result must equal the oracle bit for bit; with exact-data
outer faces the plane wave's sin/cos come from a different math library
and the bar is relative L2 <= 1e-12."""
import numpy as np
import pytest

import nmesh_gb300 as ng
from helpers import (FV_CASES, MID_CASES, PI, RTOL_RHS, RTOL_RK4, build_mesh, gaussian_pulses,
                     load, oracle_for, perm_to_mesh, rel_l2, to_mesh_order)

pytestmark = pytest.mark.gpu

# "fvx": reference operation order, no FMA; "fv": FMA and one division per
# WENO reconstruction (within FP64 rounding); "fvc": "fv" with the face
# values reconstructed per cell (both faces from one set of indicators)
FV_EXACT = ["fvx:1:128", "fvx:1:256", "fvx:1:512"]
FV_FAST = ["fv:1:128", "fv:1:256", "fv:1:512", "fvc:1:128", "fvc:1:256", "fvc:1:512"]
FV_VARIANTS = FV_EXACT + FV_FAST


@pytest.fixture(autouse=True)
def _gpu(cuda_ok):
    yield


def _ev(m, meta, bc=ng.BC_EXACT_PLANEWAVE, k=None):
    ev = ng.Evolution(m, bc, k=k if k is not None else meta["k"])
    ev.set_fv(meta["fv"]["rec"], meta["fv"]["extrap"])
    return ev


@pytest.mark.parametrize("variant", FV_VARIANTS)
@pytest.mark.parametrize("case", FV_CASES)
def test_fv_rhs_matches_reference(case, variant):
    d, meta = load(case)
    m = build_mesh(meta)
    perm = perm_to_mesh(m, d)
    ev = _ev(m, meta)
    ev.set_kernel(variant)
    r = ev.rhs(to_mesh_order(d["u0"], perm), 0.0)
    assert rel_l2(r[perm], d["r0"]) <= RTOL_RHS
    assert np.abs(r[perm] - d["r0"]).max() <= 1e-11 * np.abs(d["r0"]).max()


@pytest.mark.parametrize("variant", ["fvx", "fv", "fvc", "auto"])
@pytest.mark.parametrize("case", FV_CASES)
def test_fv_rk4_matches_reference(case, variant):
    d, meta = load(case)
    m = build_mesh(meta)
    perm = perm_to_mesh(m, d)
    ev = _ev(m, meta)
    ev.set_kernel(variant)
    u = ev.rk4_steps_host(to_mesh_order(d["u0"], perm), 0.0, meta["dt"], meta["steps"])
    assert rel_l2(u[perm], d["u_final"]) <= RTOL_RK4


@pytest.mark.parametrize("case", FV_CASES)
def test_fv_rhs_vs_oracle_with_reference_data(case):
    """Same fixture inputs through the oracle: interior nodes of elements
    without outer faces see no sin/cos and agree bit for bit."""
    d, meta = load(case)
    m = build_mesh(meta)
    perm = perm_to_mesh(m, d)
    ev = _ev(m, meta)
    ev.set_kernel("fvx")
    u = to_mesh_order(d["u0"], perm)
    r = ev.rhs(u, 0.0)
    o = oracle_for(m, bc=0, k=meta["k"], fv_rec=meta["fv"]["rec"],
                   fv_extrap=meta["fv"]["extrap"])
    ro = o.rhs(u, 0.0)
    nb, _ = m.faces()
    inner = (nb >= 0).all(axis=1)
    if inner.any():
        assert np.array_equal(r[inner], ro[inner])
    assert rel_l2(r, ro) <= RTOL_RHS


REC_EXTRAP = [(rec, ex) for rec in ("1", "WENOm3_2", "WENOm5_2") for ex in ("no", "dnfn_extrap1")]


@pytest.mark.parametrize("rec,extrap", REC_EXTRAP)
@pytest.mark.parametrize("n,luni", [(2, 2), (3, 1), (5, 1), (7, 1), (13, 0)])
def test_fv_periodic_box_bitexact_vs_oracle(n, luni, rec, extrap):
    m = ng.Mesh.build(ng.MESH_BOX, n=n, luni=luni, xc=(PI, PI, PI), box_dout=PI,
                      periodic=True, fv=True)
    xyz = m.coords()
    rng = np.random.default_rng(100 * n + luni)
    arg = xyz[:, 0] + 2.0 * xyz[:, 1] - xyz[:, 2]
    u = np.stack([np.sin(arg), np.cos(arg), np.sin(2 * arg), np.cos(arg) ** 2, np.sin(arg)], 1)
    u += 0.2 * rng.standard_normal(u.shape)
    ev = ng.Evolution(m, ng.BC_OUTGOING)
    ev.set_fv(rec, extrap)
    ev.set_kernel("fvx")
    o = oracle_for(m, bc=1, period=2 * PI, fv_rec=rec, fv_extrap=extrap)
    ro = o.rhs(u, 0.0)
    assert np.array_equal(ev.rhs(u, 0.0), ro)
    dt = 0.05 * (2 * PI / 2 ** luni) / n
    uo = o.rk4(u, dt, 3)
    assert np.array_equal(ev.rk4_steps_host(u, 0.0, dt, 3), uo)
    for v in ("fv", "fvc"):
        ev.set_kernel(v)
        assert rel_l2(ev.rhs(u, 0.0), ro) <= RTOL_RHS
        assert rel_l2(ev.rk4_steps_host(u, 0.0, dt, 3), uo) <= RTOL_RK4


@pytest.mark.parametrize("rec,extrap", [("WENOm5_2", "dnfn_extrap1"), ("WENOm3_2", "no")])
@pytest.mark.parametrize("n,luni", [(4, 1), (7, 0), (9, 0)])
def test_fv_cubed_spheres_outgoing_bitexact_vs_oracle(n, luni, rec, extrap):
    m = ng.Mesh.build(ng.MESH_CUBEDSPHERES7, n=n, luni=luni, cs_dc=1.0, cs_r0fac=20.0, fv=True)
    u = gaussian_pulses(m.coords(), seed=n + 7 * luni, rmin=1.0, rmax=6.0)
    u += 1e-2 * np.random.default_rng(n).standard_normal(u.shape)
    ev = ng.Evolution(m, ng.BC_OUTGOING)
    ev.set_fv(rec, extrap)
    ev.set_kernel("fvx")
    o = oracle_for(m, bc=1, fv_rec=rec, fv_extrap=extrap)
    ro = o.rhs(u, 0.0)
    assert np.array_equal(ev.rhs(u, 0.0), ro)
    dt = 0.02 / n
    uo = o.rk4(u, dt, 2)
    assert np.array_equal(ev.rk4_steps_host(u, 0.0, dt, 2), uo)
    for v in ("fv", "fvc"):
        ev.set_kernel(v)
        assert rel_l2(ev.rhs(u, 0.0), ro) <= RTOL_RHS
        assert rel_l2(ev.rk4_steps_host(u, 0.0, dt, 2), uo) <= RTOL_RK4


def test_fv_variants_bitwise_identical_and_graph_steps():
    m = ng.Mesh.build(ng.MESH_CUBEDSPHERES7, n=7, luni=1, cs_dc=1.0, cs_r0fac=20.0, fv=True)
    u = gaussian_pulses(m.coords(), seed=3, rmin=1.0, rmax=6.0)
    ev = ng.Evolution(m, ng.BC_OUTGOING)
    ev.set_fv("WENOm5_2", "dnfn_extrap1")
    outs = []
    for v in FV_VARIANTS:
        ev.set_kernel(v)
        outs.append(ev.rk4_steps_host(u, 0.0, 0.002, 4))
    # the thread count does not change any thread's arithmetic
    for o in outs[1:3]:
        assert np.array_equal(o, outs[0])
    for o in outs[4:6]:
        assert np.array_equal(o, outs[3])
    for o in outs[7:9]:
        assert np.array_equal(o, outs[6])
    assert rel_l2(outs[3], outs[0]) <= RTOL_RK4
    assert rel_l2(outs[6], outs[0]) <= RTOL_RK4
    ev.set_kernel("fvx:1:256")
    # the single-step path equals the graph-captured multi-step path
    ev.set_state(u)
    t = 0.0
    for s in range(4):
        ev.rk4_step(t, 0.002)
        t += 0.002
    assert np.array_equal(ev.get_state(), outs[0])
    ev.set_kernel("auto")
    ev.rhs(u)
    assert "fvx" in ev.kernel_info() and "fv:1:256" in ev.kernel_info()


def test_fv_rejections():
    m = ng.Mesh.build(ng.MESH_BOX, n=5, luni=1, xc=(0, 0, 0), box_dout=1.0, fv=True)
    ev = ng.Evolution(m, ng.BC_OUTGOING)
    with pytest.raises(ng.NmgError):
        ev.rhs_vjp_device(ev.state_ptr, ev.state_ptr + 8)
    with pytest.raises(ng.NmgError):
        ng.Batch([m])
    with pytest.raises(ng.NmgError):
        ev.set_fv("WENOm5_2", "nonsense")
    big = ng.Mesh.build(ng.MESH_BOX, n=14, luni=0, xc=(0, 0, 0), box_dout=1.0, fv=True)
    with pytest.raises(ng.NmgError):
        ng.Evolution(big, ng.BC_OUTGOING)
    dg = ng.Mesh.build(ng.MESH_BOX, n=5, luni=1, xc=(0, 0, 0), box_dout=1.0)
    ev2 = ng.Evolution(dg, ng.BC_OUTGOING)
    with pytest.raises(ng.NmgError):
        ev2.set_fv("WENOm5_2", "no")


@pytest.mark.parametrize("variant", ["fvx", "fv"])
@pytest.mark.parametrize("case", MID_CASES)
def test_midpoint_data_matches_reference(case, variant):
    """coordinates_midpoint_data = yes against the reference's own runs."""
    d, meta = load(case)
    m = build_mesh(meta)
    perm = perm_to_mesh(m, d)
    ev = ng.Evolution(m, ng.BC_EXACT_PLANEWAVE, k=meta["k"])
    ev.set_fv(meta["fv"]["rec"], meta["fv"]["extrap"])
    if m.fv().min() == 0:
        ev.set_fv_surface_interp(meta["fv"].get("surf", "linear"))
    ev.set_fv_midpoint_data(True)
    ev.set_kernel(variant)
    if m.fv().min() == 0:
        ev.set_kernel("eo")      # the DG part fixed too (no autotuning)
    ev.set_evolve_method(meta.get("method", "RK4"))
    u0 = to_mesh_order(d["u0"], perm)
    assert rel_l2(ev.rhs(u0, 0.0)[perm], d["r0"]) <= RTOL_RHS
    u = ev.evolve_steps_host(u0, 0.0, meta["dt"], meta["steps"])
    assert rel_l2(u[perm], d["u_final"]) <= RTOL_RK4
    # switching it off gives the grid-point factors again
    ev.set_fv_midpoint_data(False)
    plain = ng.Evolution(m, ng.BC_EXACT_PLANEWAVE, k=meta["k"])
    plain.set_fv(meta["fv"]["rec"], meta["fv"]["extrap"])
    if m.fv().min() == 0:
        plain.set_fv_surface_interp(meta["fv"].get("surf", "linear"))
    plain.set_kernel(variant)
    if m.fv().min() == 0:
        plain.set_kernel("eo")
    assert np.array_equal(ev.rhs(u0, 0.0), plain.rhs(u0, 0.0))


@pytest.mark.parametrize("extrap,min_rate", [("dnfn_extrap1", 1.8), ("no", 0.9)])
def test_midpoint_data_constant_flux_converges(extrap, min_rate):
    """With the midpoint map the FV divergence of a constant flux on the
    curvilinear shells converges to zero (fv_tests, src/main/dg/fv_tests.c:
    second order with dnfn_extrap1, first order at the faces with "no")."""
    errs = []
    for luni in (1, 2):
        m = ng.Mesh.build(ng.MESH_CUBEDSPHERES7, n=7, luni=luni, cs_dc=1.0, cs_r0fac=4.0,
                          fv=True)
        u = np.zeros((m.nelem, 5, m.np))
        u[:, 0], u[:, 1], u[:, 2], u[:, 3] = 0.3, -0.5, 0.8, 0.2
        ev = ng.Evolution(m, ng.BC_OUTGOING)
        ev.set_fv("WENOm5_2", extrap)
        ev.set_fv_midpoint_data(True)
        r = ev.rhs(u, 0.0)
        nb, _ = m.faces()
        pat, _ = m.elements()
        inner = (nb >= 0).all(axis=1) & (pat > 0)
        errs.append(np.abs(r[inner, :4]).max())
    rate = np.log2(errs[0] / errs[1])
    assert rate > min_rate, (errs, rate)
