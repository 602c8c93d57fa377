"""Batched execution of many independent problems of different orders and
sizes (nmg_batch_*, one persistent launch per RK4 stage) against the same
problems stepped one by one through their own contexts, and against the
oracle."""
import numpy as np
import pytest

import nmesh_gb300 as ng
from helpers import PI, RTOL_RK4, gaussian_pulses, oracle_for, rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _gpu(cuda_ok):
    yield


def _problems():
    specs = [("cs7", 9, 0), ("box", 5, 1), ("cs7", 4, 1), ("box", 5, 0), ("cs7", 6, 0),
             ("box", 3, 2), ("cs7", 10, 0), ("box", 7, 1)]
    meshes, us = [], []
    for i, (kind, n, luni) in enumerate(specs):
        if kind == "cs7":
            m = ng.Mesh.build(ng.MESH_CUBEDSPHERES7, n=n, luni=luni, cs_dc=1.0, cs_r0fac=20.0)
        else:
            m = ng.Mesh.build(ng.MESH_BOX, n=n, luni=luni, xc=(PI, PI, PI), box_dout=PI,
                              periodic=True)
        u = gaussian_pulses(m.coords(), seed=i, rmin=1.0, rmax=4.0)
        u += 1e-3 * np.random.default_rng(i).standard_normal(u.shape)
        meshes.append(m)
        us.append(u)
    return meshes, us


def _epb(n):
    return max(1, 128 // (2 * n * n))


def test_batched_equals_individual_contexts():
    meshes, us = _problems()
    b = ng.Batch(meshes, ng.BC_OUTGOING)
    b.set_mode(1)   # persistent single launch
    for p, u in enumerate(us):
        b.set_state(p, u)
    dt, nsteps = 0.001, 3
    b.rk4_steps(0.0, dt, nsteps)
    info = b.info()
    assert "grid" in info and "timings" in info
    for p, (m, u) in enumerate(zip(meshes, us)):
        ev = ng.Evolution(m, ng.BC_OUTGOING)
        ev.set_kernel(f"eo:{_epb(m.n)}:256")
        ref = ev.rk4_steps_host(u, 0.0, dt, nsteps)
        got = b.get_state(p)
        # the batched tile body is the eo:<epb>:256 variant: bitwise equal
        assert np.array_equal(got, ref), (p, rel_l2(got, ref))


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_batched_matches_oracle_and_continues(mode):
    meshes, us = _problems()
    b = ng.Batch(meshes, ng.BC_OUTGOING)
    b.set_mode(mode)
    for p, u in enumerate(us):
        b.set_state(p, u)
    dt = 0.001
    b.rk4_steps(0.0, dt, 2)
    b.rk4_steps(2 * dt, dt, 1)   # graphs are reused, buffers keep alternating
    for p in (0, 2, 6):
        o = oracle_for(meshes[p], bc=1)
        assert rel_l2(b.get_state(p), o.rk4(us[p], dt, 3)) <= RTOL_RK4


def test_batch_rejects_unsupported_orders():
    m = ng.Mesh.build(ng.MESH_CUBEDSPHERES7, n=11, luni=0)
    with pytest.raises(ng.NmgError):
        ng.Batch([m])
