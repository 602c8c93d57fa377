"""The reference's other time integrators on the GPU (evolve_method = Euler
and sspRK3, nmg_set_evolve_method + nmg_evolve_steps): against the
reference's own runs and against the oracle."""
import numpy as np
import pytest

import nmesh_gb300 as ng
from helpers import (METHOD_CASES, RTOL_RK4, build_mesh, gaussian_pulses, load, oracle_for,
                     perm_to_mesh, rel_l2, to_mesh_order)

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _gpu(cuda_ok):
    yield


def _ev(m, meta, bc=ng.BC_EXACT_PLANEWAVE):
    ev = ng.Evolution(m, bc, k=meta["k"])
    if "fv" in meta:
        ev.set_fv(meta["fv"]["rec"], meta["fv"]["extrap"])
        if ev.mesh.fv().min() == 0:
            ev.set_fv_surface_interp(meta["fv"].get("surf", "linear"))
    ev.set_evolve_method(meta["method"])
    return ev


@pytest.mark.parametrize("case", METHOD_CASES)
def test_matches_reference(case):
    d, meta = load(case)
    m = build_mesh(meta)
    perm = perm_to_mesh(m, d)
    ev = _ev(m, meta)
    u = ev.evolve_steps_host(to_mesh_order(d["u0"], perm), 0.0, meta["dt"], meta["steps"])
    assert rel_l2(u[perm], d["u_final"]) <= RTOL_RK4


@pytest.mark.parametrize("variant", ["eo", "eof", "gather"])
@pytest.mark.parametrize("method", ["Euler", "sspRK3"])
def test_outgoing_pulses_match_oracle(method, variant):
    m = ng.Mesh.build(ng.MESH_CUBEDSPHERES7, n=6, luni=1, cs_dc=1.0, cs_r0fac=20.0)
    u = gaussian_pulses(m.coords(), seed=5, rmin=1.0, rmax=4.0)
    ev = ng.Evolution(m, ng.BC_OUTGOING)
    ev.set_kernel(variant)
    ev.set_evolve_method(method)
    dt = 0.003
    got = ev.evolve_steps_host(u, 0.0, dt, 4)
    want = oracle_for(m, bc=1).evolve(u, dt, 4, method=method)
    assert rel_l2(got, want) <= RTOL_RK4


def test_switching_methods_recaptures_step_graphs():
    """Resident steps of one context with the method changed between calls
    equal fresh contexts stepping the same sequence."""
    m = ng.Mesh.build(ng.MESH_BOX, n=5, luni=1, xc=(0, 0, 0), box_dout=1.0)
    u = np.random.default_rng(3).standard_normal((m.nelem, 5, m.np))
    ev = ng.Evolution(m, ng.BC_OUTGOING)
    ev.set_kernel("eo")
    ev.set_state(u)
    dt = 0.001
    ev.set_evolve_method("sspRK3")
    ev.evolve_steps(0.0, dt, 2)
    ev.set_evolve_method("RK4")
    ev.evolve_steps(2 * dt, dt, 2)
    ev.set_evolve_method("Euler")
    ev.evolve_steps(4 * dt, dt, 1)
    ref = u
    for meth, t0, k in (("sspRK3", 0.0, 2), ("RK4", 2 * dt, 2), ("Euler", 4 * dt, 1)):
        fresh = ng.Evolution(m, ng.BC_OUTGOING)
        fresh.set_kernel("eo")
        fresh.set_evolve_method(meth)
        ref = fresh.evolve_steps_host(ref, t0, dt, k)
    assert np.array_equal(ev.get_state(), ref)
    # the RK4 entry points keep RK4 whatever the method
    a = ng.Evolution(m, ng.BC_OUTGOING)
    a.set_kernel("eo")
    a.set_evolve_method("Euler")
    b = ng.Evolution(m, ng.BC_OUTGOING)
    b.set_kernel("eo")
    assert np.array_equal(a.rk4_steps_host(u, 0.0, dt, 2), b.rk4_steps_host(u, 0.0, dt, 2))
    with pytest.raises(KeyError):
        a.set_evolve_method("RK5")
