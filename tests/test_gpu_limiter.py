"""The reference's limiters (scalarwave1_limiter = MRS or minmodB,
nmg_set_limiter_ex) on the GPU: against the reference's own runs and
against the oracle."""
import numpy as np
import pytest

import nmesh_gb300 as ng
from helpers import (LIM_CASES, MMB_CASES, RTOL_RK4, build_mesh, gaussian_pulses,
                     limiter_kwargs, load, oracle_for, perm_to_mesh, rel_l2, to_mesh_order)

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _gpu(cuda_ok):
    yield


@pytest.mark.parametrize("path", ["host", "resident", "single"])
@pytest.mark.parametrize("case", LIM_CASES + MMB_CASES)
def test_limiter_matches_reference(case, path):
    d, meta = load(case)
    m = build_mesh(meta)
    perm = perm_to_mesh(m, d)
    ev = ng.Evolution(m, ng.BC_EXACT_PLANEWAVE, k=meta["k"])
    if "fv" in meta:
        ev.set_fv(meta["fv"]["rec"], meta["fv"]["extrap"])
    ev.set_limiter(**limiter_kwargs(meta))
    u0 = to_mesh_order(d["u0"], perm)
    dt, ns = meta["dt"], meta["steps"]
    if path == "host":
        u = ev.rk4_steps_host(u0, 0.0, dt, ns)
    elif path == "resident":
        ev.set_state(u0)
        ev.rk4_steps(0.0, dt, ns)
        u = ev.get_state()
    else:
        ev.set_state(u0)
        for s in range(ns):
            ev.rk4_step(s * dt, dt)
        u = ev.get_state()
    assert rel_l2(u[perm], d["u_final"]) <= RTOL_RK4


def test_limiter_flags_and_options_match_oracle():
    """Outgoing boundary, mixed DG/FV mesh (equally spaced quadrature on the
    FV elements), sspRK3 and Euler steps, and the per-element flags; with
    kind "none" the step is the plain one again."""
    m = ng.Mesh.build(ng.MESH_CUBEDSPHERES7, n=5, luni=1, cs_dc=1.0, cs_r0fac=20.0, fv=[0])
    u = gaussian_pulses(m.coords(), seed=5, rmin=1.0, rmax=4.0)
    u += 0.2 * np.random.default_rng(5).standard_normal(u.shape)
    o = oracle_for(m, bc=1, fv_rec="WENOm5_2", fv_extrap="dnfn_extrap1")
    ev = ng.Evolution(m, ng.BC_OUTGOING)
    ev.set_fv("WENOm5_2", "dnfn_extrap1")
    ev.set_limiter("MRS", 0.05)
    dt = 0.002
    got = ev.rk4_steps_host(u, 0.0, dt, 2)
    want = o.rk4_limited(u, dt, 2, alpha=0.05)
    assert rel_l2(got, want) <= RTOL_RK4
    # flags of the last limiter call: the new u of the step before limiting
    ev.set_state(u)
    ev.set_evolve_method("sspRK3")
    got3 = ev.evolve_steps_host(u, 0.0, dt, 1)
    ev.set_state(u)
    ev.evolve_steps(0.0, dt, 1)
    flags = ev.limited()
    assert np.array_equal(got3, ev.get_state())
    assert 0 < flags.sum() <= m.nelem
    ev.set_limiter("none")
    ev.set_evolve_method("RK4")
    assert rel_l2(ev.rk4_steps_host(u, 0.0, dt, 2), o.rk4(u, dt, 2)) <= RTOL_RK4
    with pytest.raises(ng.NmgError):
        ng.Evolution(m, ng.BC_OUTGOING).set_limiter("minmodB", 1.0, beta=-1.0)
    with pytest.raises(ng.NmgError):
        ng.Evolution(m, ng.BC_OUTGOING).set_limiter("MRS", -1.0)
    assert lib_set(ev, 3, 1.0, 0.5, 0) == 5          # NMG_EUNSUP: no such kind


def lib_set(ev, kind, alpha, beta, sb):
    return ng.lib().nmg_set_limiter_ex(ev._h, kind, alpha, beta, sb)


@pytest.mark.parametrize("scale_bound", [False, True])
@pytest.mark.parametrize("fv", [False, True])
def test_minmodb_options_and_flags_match_oracle(fv, scale_bound):
    """minmodB with the outgoing boundary (outer faces average 0), on a DG
    mesh and a mixed DG / finite-volume mesh (equally spaced analysis and
    synthesis on the FV elements), beta and scaleBound varied; the
    per-element flags of the last limiter call equal the oracle's, and a
    switch from MRS to minmodB on one context takes effect."""
    m = ng.Mesh.build(ng.MESH_CUBEDSPHERES7, n=5, luni=1, cs_dc=1.0, cs_r0fac=20.0,
                      fv=[0] if fv else None)
    u = gaussian_pulses(m.coords(), seed=7, rmin=1.0, rmax=4.0)
    u += 0.2 * np.random.default_rng(7).standard_normal(u.shape)
    okw = dict(bc=1)
    if fv:
        okw.update(fv_rec="WENOm5_2", fv_extrap="dnfn_extrap1")
    o = oracle_for(m, **okw)
    ev = ng.Evolution(m, ng.BC_OUTGOING)
    if fv:
        ev.set_fv("WENOm5_2", "dnfn_extrap1")
    ev.set_limiter("MRS", 0.05)
    kw = dict(kind="minmodB", alpha=2.0 if scale_bound else 0.3, beta=0.7,
              scale_bound=scale_bound)
    ev.set_limiter(**kw)
    dt = 0.002
    ev.set_state(u)
    ev.rk4_steps(0.0, dt, 1)
    want, flags = o.rk4_limited(u, dt, 1, flags=True, **kw)
    assert rel_l2(ev.get_state(), want) <= RTOL_RK4
    assert np.array_equal(ev.limited(), flags)
    assert 0 < flags.sum() < m.nelem
    ev.rk4_steps(dt, dt, 1)
    assert rel_l2(ev.get_state(), o.rk4_limited(u, dt, 2, **kw)) <= RTOL_RK4


def test_limiter_rejected_where_not_built():
    """The trouble flow and the adjoint refuse a context with the limiter on
    (the limiter is nonlinear; the trouble flow's own limiter calls are not
    built) instead of silently skipping it."""
    import torch
    m = ng.Mesh.build(ng.MESH_BOX, n=4, luni=1, xc=(0.0, 0.0, 0.0), box_dout=1.0, periodic=True)
    ev = ng.Evolution(m, ng.BC_OUTGOING, switchable=True)
    ev.set_fv("WENOm5_2", "dnfn_extrap1")
    ev.set_limiter("MRS", 1.0)
    ev.set_state(np.zeros(ev.shape))
    with pytest.raises(ng.NmgError):
        ev.rk4_step_trouble(0.0, 0.01, ng.TroubleParams())
    dg = ng.Evolution(m, ng.BC_OUTGOING)
    dg.set_limiter("MRS", 1.0)
    x = torch.zeros(dg.size, dtype=torch.float64, device="cuda")
    y = torch.zeros_like(x)
    with pytest.raises(ng.NmgError):
        dg.rhs_vjp_device(x.data_ptr(), y.data_ptr())
    dg.set_limiter("none")
    dg.rhs_vjp_device(x.data_ptr(), y.data_ptr())
