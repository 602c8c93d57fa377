"""Known-answer and convergence checks of the GPU path, the counterparts of
the reference's own tests: the RHS of the exact plane wave against its time
derivative (scalarwave1_analyze's RHS errors, src/tests/scalarwave1/
scalarwave1.c:710-751), the temporal order of RK4, Euler and sspRK3
(evolve_test, src/main/evolve/evolve_test.c:11-136), and the finite-volume
divergence of a constant flux on curvilinear grids (fv_tests,
src/main/dg/fv_tests.c: second order in the interior)."""
import numpy as np
import pytest

import nmesh_gb300 as ng
from helpers import PI

pytestmark = pytest.mark.gpu

K = (0.7, -0.4, 0.3)


@pytest.fixture(autouse=True)
def _gpu(cuda_ok):
    yield


def plane_wave(xyz, t=0.0, k=K):
    """pi = -w cos(k.x - w t), c = k cos(k.x - w t), phi = sin(k.x - w t)
    (the exterior state of the exact-data boundary) and its time derivative."""
    k = np.asarray(k)
    w = np.sqrt(k @ k)
    arg = np.einsum("d,edn->en", k, xyz) - w * t
    u = np.stack([-w * np.cos(arg)] + [kk * np.cos(arg) for kk in k] + [np.sin(arg)], 1)
    du = np.stack([-w * w * np.sin(arg)] + [w * kk * np.sin(arg) for kk in k]
                  + [-w * np.cos(arg)], 1)
    return u, du


def test_rhs_converges_spectrally_to_the_time_derivative():
    errs = []
    for n in (4, 6, 8, 10):
        m = ng.Mesh.build(ng.MESH_BOX, n=n, luni=1, xc=(0, 0, 0), box_dout=1.0)
        u, du = plane_wave(m.coords())
        ev = ng.Evolution(m, ng.BC_EXACT_PLANEWAVE, k=K)
        r = ev.rhs(u, 0.0)
        errs.append(np.abs(r - du).max() / np.abs(du).max())
    # each two more points per direction gain at least a factor 30
    assert all(a > 30 * b for a, b in zip(errs, errs[1:])), errs
    assert errs[-1] < 1e-8, errs


@pytest.mark.parametrize("method,order", [("RK4", 4), ("sspRK3", 3), ("Euler", 1)])
def test_temporal_order(method, order):
    """Error at T against a 16x finer step: halving dt divides it by
    about 2^order."""
    m = ng.Mesh.build(ng.MESH_BOX, n=10, luni=1, xc=(PI, PI, PI), box_dout=PI)
    u0, _ = plane_wave(m.coords())
    T, dt0 = 0.4, 0.02

    def run(dt):
        ev = ng.Evolution(m, ng.BC_EXACT_PLANEWAVE, k=K)
        ev.set_evolve_method(method)
        return ev.evolve_steps_host(u0, 0.0, dt, int(round(T / dt)))

    ref = run(dt0 / 16)
    e1 = np.abs(run(dt0) - ref).max()
    e2 = np.abs(run(dt0 / 2) - ref).max()
    rate = np.log2(e1 / e2)
    assert abs(rate - order) < 0.5, (e1, e2, rate)


@pytest.mark.parametrize("extrap", ["dnfn_extrap1", "no"])
@pytest.mark.parametrize("rec", ["WENOm5_2", "WENOmZ_2", "WENOm3_2"])
def test_fv_divergence_of_a_constant_flux_vanishes_on_affine_elements(rec, extrap):
    """A constant state makes every flux constant: on a periodic box of
    finite-volume elements (constant metric, no outer faces) the divergence
    is zero to round-off.  (On the curvilinear shells the reference's
    default coordinates_midpoint_data = no takes the midpoint metric from
    the grid points, so there it is not zero; the GPU and the oracle give the
    same values, and the oracle is bit-exact to the reference there.)"""
    m = ng.Mesh.build(ng.MESH_BOX, n=7, luni=1, xc=(PI, PI, PI), box_dout=PI, periodic=True,
                      fv=True)
    u = np.zeros((m.nelem, 5, m.np))
    u[:, 0], u[:, 1], u[:, 2], u[:, 3], u[:, 4] = 0.3, -0.5, 0.8, 0.2, 1.0
    ev = ng.Evolution(m, ng.BC_OUTGOING)
    ev.set_fv(rec, extrap)
    r = ev.rhs(u, 0.0)
    assert np.abs(r[:, :4]).max() <= 1e-13
    assert np.array_equal(r[:, 4], u[:, 0])
