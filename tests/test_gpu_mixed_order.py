"""Problems whose parts have different orders (the reference's p-refinement
by patch, amr_prefine_p), stepped as one batched problem: the parts are
joined across their coinciding outer faces, whose exterior state is the
neighbour part's face plane interpolated at each node (set_ajsurf_vl's
interpolation branch, src/main/amr/surface.c:900-1460).  Checked against
the oracle's joined parts (oracle.nmo.LinkedOracle) within 1e-12."""
import numpy as np
import pytest

import nmesh_gb300 as ng
from helpers import RTOL_RK4, gaussian_pulses, oracle_for, rel_l2
from oracle import nmo

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _gpu(cuda_ok):
    yield


def _parts(groups, luni=1):
    """7 CubedSpheres split into parts: groups = [(patches, n), ...]."""
    return [ng.Mesh.build(ng.MESH_CUBEDSPHERES7, n=n, luni=luni, cs_dc=1.0, cs_r0fac=20.0,
                          patches=list(p)) for p, n in groups]


def _pulses(m, seed):
    u = gaussian_pulses(m.coords(), seed=seed, rmin=1.0, rmax=6.0)
    return u + 1e-3 * np.random.default_rng(seed).standard_normal(u.shape)


def test_parts_of_one_order_step_like_the_whole_mesh():
    """Split at one n, the joined parts give the unsplit context's steps
    (the interpolation at coincident points is the identity)."""
    full = ng.Mesh.build(ng.MESH_CUBEDSPHERES7, n=6, luni=1, cs_dc=1.0, cs_r0fac=20.0)
    parts = _parts([((0, 2, 4), 6), ((1, 3, 5, 6), 6)])
    P, B = full.elements()
    key = {(int(a),) + tuple(b): i for i, (a, b) in enumerate(zip(P, B))}
    idx = [np.array([key[(int(a),) + tuple(b)] for a, b in zip(*m.elements())]) for m in parts]
    u = _pulses(full, 3)
    ev = ng.Evolution(full, ng.BC_OUTGOING)
    ev.set_state(u)
    dt = 0.002
    ev.rk4_steps(0.0, dt, 3)
    want = ev.get_state()
    b = ng.Batch(parts, ng.BC_OUTGOING, problems=[0, 0])
    assert b.linked_faces > 0
    for p, ii in enumerate(idx):
        b.set_state(p, u[ii])
    b.rk4_steps(0.0, dt, 3)
    for p, ii in enumerate(idx):
        assert rel_l2(b.get_state(p), want[ii]) <= 1e-13


@pytest.mark.parametrize("groups", [
    [((0, 2, 4), 5), ((1, 3, 5, 6), 7)],
    [((0,), 8), ((1, 2), 4), ((3, 4, 5, 6), 6)],
])
def test_mixed_orders_match_the_oracle(groups):
    parts = _parts(groups)
    us = [_pulses(m, 10 + k) for k, m in enumerate(parts)]
    lo = nmo.LinkedOracle([oracle_for(m, bc=1) for m in parts], [m.coords() for m in parts])
    dt = 0.002
    b = ng.Batch(parts, ng.BC_OUTGOING, problems=[0] * len(parts))
    assert b.linked_faces == len(lo.links)
    for p, u in enumerate(us):
        b.set_state(p, u)
    b.rk4_steps(0.0, dt, 3)
    want = lo.rk4(us, dt, 3)
    for p in range(len(parts)):
        assert rel_l2(b.get_state(p), want[p]) <= RTOL_RK4, p
    # the persistent single launch and the per-order launches agree
    for mode in (1, 2):
        b2 = ng.Batch(parts, ng.BC_OUTGOING, problems=[0] * len(parts))
        b2.set_mode(mode)
        for p, u in enumerate(us):
            b2.set_state(p, u)
        b2.rk4_steps(0.0, dt, 3)
        for p in range(len(parts)):
            assert rel_l2(b2.get_state(p), want[p]) <= RTOL_RK4, (mode, p)
        b2.close()


def test_mixed_order_problem_among_independent_problems():
    """Problems stay independent: a box that shares coordinates with nothing
    and a second mixed-order problem at the same place as the first (but a
    different problem id) step as they do alone."""
    parts = _parts([((0, 2, 4), 5), ((1, 3, 5, 6), 7)])
    twin = _parts([((0, 2, 4), 5), ((1, 3, 5, 6), 7)])
    box = ng.Mesh.build(ng.MESH_BOX, n=4, luni=1, xc=(0.0, 0.0, 0.0), box_dout=1.0)
    meshes = parts + [box] + twin
    problems = [0, 0, 1, 2, 2]
    us = [_pulses(m, 20 + k) for k, m in enumerate(meshes)]
    dt = 0.002
    b = ng.Batch(meshes, ng.BC_OUTGOING, problems=problems)
    for p, u in enumerate(us):
        b.set_state(p, u)
    b.rk4_steps(0.0, dt, 2)
    lo = nmo.LinkedOracle([oracle_for(m, bc=1) for m in parts], [m.coords() for m in parts])
    want = lo.rk4(us[:2], dt, 2)
    for p in range(2):
        assert rel_l2(b.get_state(p), want[p]) <= RTOL_RK4
    lo2 = nmo.LinkedOracle([oracle_for(m, bc=1) for m in twin], [m.coords() for m in twin])
    want2 = lo2.rk4(us[3:], dt, 2)
    for p in range(2):
        assert rel_l2(b.get_state(3 + p), want2[p]) <= RTOL_RK4
    ob = oracle_for(box, bc=1)
    assert rel_l2(b.get_state(2), ob.rk4(us[2], dt, 2)) <= RTOL_RK4


def test_inner_cube_of_higher_order_matches_oracle():
    """The inner cube at n = 6 inside shells at n = 4 (a factor of 1.5 in
    points across every joined face), two RK4 steps."""
    parts = _parts([((0,), 6), ((1, 2, 3, 4, 5, 6), 4)], luni=1)
    us = [_pulses(m, 30 + k) for k, m in enumerate(parts)]
    lo = nmo.LinkedOracle([oracle_for(m, bc=1) for m in parts], [m.coords() for m in parts])
    dt = 0.003
    b = ng.Batch(parts, ng.BC_OUTGOING, problems=[0, 0])
    for p, u in enumerate(us):
        b.set_state(p, u)
    b.rk4_steps(0.0, dt, 2)
    want = lo.rk4(us, dt, 2)
    for p in range(2):
        assert rel_l2(b.get_state(p), want[p]) <= RTOL_RK4


def test_batches_of_different_orders_live_together():
    """A batch of low orders created after one of high orders leaves the
    first one steppable (the persistent kernel's shared-memory limit)."""
    hi = ng.Batch([ng.Mesh.build(ng.MESH_BOX, n=10, luni=1, xc=(0.0,) * 3, box_dout=1.0)],
                  ng.BC_OUTGOING)
    hi.set_mode(1)
    lo = ng.Batch([ng.Mesh.build(ng.MESH_BOX, n=3, luni=1, xc=(0.0,) * 3, box_dout=1.0)],
                  ng.BC_OUTGOING)
    lo.set_mode(1)
    lo.rk4_steps(0.0, 1e-3, 1)
    hi.rk4_steps(0.0, 1e-3, 1)
    lo.rk4_steps(1e-3, 1e-3, 1)
