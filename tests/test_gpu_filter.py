"""The reference's exponential filter after every step (evolve_filter_all =
yes, nmg_set_filter) on the GPU: against the reference's own runs and
against the oracle."""
import numpy as np
import pytest

import nmesh_gb300 as ng
from helpers import (FILT_CASES, RTOL_RK4, build_mesh, gaussian_pulses, load, oracle_for,
                     perm_to_mesh, rel_l2, to_mesh_order)

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _gpu(cuda_ok):
    yield


@pytest.mark.parametrize("path", ["host", "resident", "single"])
@pytest.mark.parametrize("case", FILT_CASES)
def test_filter_matches_reference(case, path):
    d, meta = load(case)
    m = build_mesh(meta)
    perm = perm_to_mesh(m, d)
    ev = ng.Evolution(m, ng.BC_EXACT_PLANEWAVE, k=meta["k"])
    if "fv" in meta:
        ev.set_fv(meta["fv"]["rec"], meta["fv"]["extrap"])
    ev.set_filter(True)
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


@pytest.mark.parametrize("jpow,filter_fv,fv", [(1, True, [0, 2]), (0, True, [0, 2]),
                                               (1, False, [0, 2]), (1, True, True),
                                               (0, True, False)])
def test_filter_options_match_oracle(jpow, filter_fv, fv):
    m = ng.Mesh.build(ng.MESH_CUBEDSPHERES7, n=7, luni=1, cs_dc=1.0, cs_r0fac=20.0, fv=fv)
    u = gaussian_pulses(m.coords(), seed=4, rmin=1.0, rmax=4.0)
    u += 1e-2 * np.random.default_rng(4).standard_normal(u.shape)
    o = oracle_for(m, bc=1, fv_rec="WENOm5_2", fv_extrap="dnfn_extrap1")
    ev = ng.Evolution(m, ng.BC_OUTGOING)
    if fv is not False:
        ev.set_fv("WENOm5_2", "dnfn_extrap1")
    ev.set_filter(True, alp=30.0, s=8.0, dn=1, jpower=jpow, filter_fv=filter_fv)
    dt = 0.002
    got = ev.rk4_steps_host(u, 0.0, dt, 2)
    want = u
    for s in range(2):
        want = o.filter(o.rk4(want, dt, 1, t=s * dt), alp=30.0, s=8.0, dn=1, jpow=jpow,
                        filter_fv=filter_fv)
    assert rel_l2(got, want) <= RTOL_RK4
    # off again: plain RK4
    ev.set_filter(False)
    assert rel_l2(ev.rk4_steps_host(u, 0.0, dt, 2), o.rk4(u, dt, 2)) <= RTOL_RK4
