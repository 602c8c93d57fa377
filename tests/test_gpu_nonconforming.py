"""Non-conforming faces on the GPU: patches refined one level further than
their neighbours (the reference's amr_hrefine_p).  The traces of those faces
are interpolated from the neighbour faces each stage (hang_kernel), then the
DG kernels read them like any interface trace."""
import numpy as np
import pytest

import nmesh_gb300 as ng
from helpers import (NC_CASES, RTOL_RHS, RTOL_RK4, build_mesh, gaussian_pulses, load,
                     oracle_for, perm_to_mesh, rel_l2, to_mesh_order)

pytestmark = pytest.mark.gpu

VARIANTS = ["eo", "eof", "eofu", "gather"]


@pytest.fixture(autouse=True)
def _gpu(cuda_ok):
    yield


@pytest.mark.parametrize("variant", VARIANTS)
@pytest.mark.parametrize("case", NC_CASES)
def test_rhs_matches_reference(case, variant):
    d, meta = load(case)
    m = build_mesh(meta)
    perm = perm_to_mesh(m, d)
    ev = ng.Evolution(m, ng.BC_EXACT_PLANEWAVE, k=meta["k"])
    ev.set_numflux(meta.get("numflux", "LLF"))
    ev.set_kernel(variant)
    r = ev.rhs(to_mesh_order(d["u0"], perm), 0.0)
    assert rel_l2(r[perm], d["r0"]) <= RTOL_RHS


@pytest.mark.parametrize("case", NC_CASES)
def test_rk4_matches_reference(case):
    d, meta = load(case)
    m = build_mesh(meta)
    perm = perm_to_mesh(m, d)
    ev = ng.Evolution(m, ng.BC_EXACT_PLANEWAVE, k=meta["k"])
    ev.set_numflux(meta.get("numflux", "LLF"))
    u = ev.rk4_steps_host(to_mesh_order(d["u0"], perm), 0.0, meta["dt"], meta["steps"])
    assert rel_l2(u[perm], d["u_final"]) <= RTOL_RK4


def _pulse_case(n=7, luni=1, href=(0, 3), seed=3):
    m = ng.Mesh.build(ng.MESH_CUBEDSPHERES7, n=n, luni=luni, cs_dc=1.0, cs_r0fac=20.0,
                      hrefine=href)
    u = gaussian_pulses(m.coords(), seed=seed, rmin=1.0, rmax=4.0)
    u += 1e-3 * np.random.default_rng(seed).standard_normal(u.shape)
    return m, u


@pytest.mark.parametrize("variant", VARIANTS)
def test_outgoing_pulses_match_oracle(variant):
    m, u = _pulse_case()
    o = oracle_for(m, bc=1)
    ev = ng.Evolution(m, ng.BC_OUTGOING)
    ev.set_kernel(variant)
    dt = 0.002
    assert rel_l2(ev.rk4_steps_host(u, 0.0, dt, 5), o.rk4(u, dt, 5)) <= RTOL_RK4


def test_host_round_trip_equals_resident_steps():
    """The chunked final stage computes the traces once per stage; results
    equal resident stepping bit for bit."""
    m, u = _pulse_case(n=5, luni=1, href=(2, 5), seed=4)
    dt = 0.003
    a = ng.Evolution(m, ng.BC_OUTGOING)
    b = ng.Evolution(m, ng.BC_OUTGOING)
    a.set_kernel("eo")
    b.set_kernel("eo")
    ua = a.rk4_steps_host(u, 0.0, dt, 1)
    ua = a.rk4_steps_host(ua, dt, dt, 3)
    b.set_state(u)
    b.rk4_steps(0.0, dt, 4)
    assert np.array_equal(ua, b.get_state())


def test_unsupported_combinations_rejected():
    m, _ = _pulse_case(n=4, luni=0, href=(0,))
    with pytest.raises(ng.NmgError):
        ng.Evolution(m, ng.BC_OUTGOING, switchable=True)
    fvm = ng.Mesh.build(ng.MESH_CUBEDSPHERES7, n=5, luni=0, fv=[0], hrefine=(0,))
    with pytest.raises(ng.NmgError):
        ng.Evolution(fvm, ng.BC_OUTGOING)


@pytest.mark.parametrize("mode", [0, 1])
def test_batched_nonconforming(mode):
    """Batches carry the non-conforming lists (merged per order) and compute
    the traces before each stage; the persistent tile body is the
    eo:<epb>:256 variant, so the results equal single contexts bit for bit."""
    specs = [(5, 0, (0,)), (6, 1, (1, 4)), (5, 1, (0,)), (4, 1, ())]
    meshes, us = [], []
    for i, (n, luni, href) in enumerate(specs):
        m, u = _pulse_case(n=n, luni=luni, href=href, seed=10 + i)
        meshes.append(m)
        us.append(u)
    b = ng.Batch(meshes, ng.BC_OUTGOING)
    b.set_mode(mode)
    for p, u in enumerate(us):
        b.set_state(p, u)
    dt = 0.002
    b.rk4_steps(0.0, dt, 3)
    for p, (m, u) in enumerate(zip(meshes, us)):
        ev = ng.Evolution(m, ng.BC_OUTGOING)
        ev.set_kernel(f"eo:{max(1, 128 // (2 * m.n * m.n))}:256")
        ref = ev.rk4_steps_host(u, 0.0, dt, 3)
        got = b.get_state(p)
        if mode == 1:
            assert np.array_equal(got, ref), (p, rel_l2(got, ref))
        assert rel_l2(got, oracle_for(m, bc=1).rk4(u, dt, 3)) <= RTOL_RK4
