"""Hand-written adjoint of the RHS and of the RK4 step (no reference
counterpart): dot-product (tangent/adjoint) tests and the gradient of the
shell objective against central finite differences of the oracle's CPU
forward evolution (the bit-exact restatement of the reference RHS/RK4)."""
import numpy as np
import pytest

import nmesh_gb300 as ng
from helpers import PI, gaussian_pulses, oracle_for

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _gpu(cuda_ok):
    yield


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, np.float64)).cuda()


def _mesh(kind, n, luni):
    if kind == "cs7":
        return ng.Mesh.build(ng.MESH_CUBEDSPHERES7, n=n, luni=luni, cs_dc=1.0, cs_r0fac=20.0)
    if kind == "cs7h":   # inner cube one level finer (non-conforming faces)
        return ng.Mesh.build(ng.MESH_CUBEDSPHERES7, n=n, luni=luni, cs_dc=1.0, cs_r0fac=20.0,
                             hrefine=(0,))
    if kind == "boxs":   # nested spheres about the corner x = 0: jumps inside the patch
        return ng.Mesh.build(ng.MESH_BOX, n=n, luni=luni, xc=(PI, PI, PI), box_dout=PI,
                             sphere_levels=2, sphere_radius=2)
    return ng.Mesh.build(ng.MESH_BOX, n=n, luni=luni, xc=(PI, PI, PI), box_dout=PI,
                         periodic=True)


def _rel(a, b):
    return abs(a - b) / max(abs(a), abs(b), 1e-300)


@pytest.mark.parametrize("kind,n,luni,bc", [("cs7", 5, 1, ng.BC_OUTGOING),
                                            ("cs7", 9, 0, ng.BC_EXACT_PLANEWAVE),
                                            ("cs7", 4, 1, ng.BC_EXACT_PLANEWAVE),
                                            ("box", 6, 1, ng.BC_EXACT_PLANEWAVE),
                                            ("cs7h", 5, 0, ng.BC_OUTGOING),
                                            ("cs7h", 4, 1, ng.BC_EXACT_PLANEWAVE),
                                            ("boxs", 5, 1, ng.BC_OUTGOING)])
def test_rhs_vjp_dot_product(kind, n, luni, bc):
    import torch
    m = _mesh(kind, n, luni)
    ev = ng.Evolution(m, bc, k=(0.3, -0.2, 0.1))
    rng = np.random.default_rng(n)
    v = rng.standard_normal(ev.shape)
    w = rng.standard_normal(ev.shape)
    # linear part of the RHS: r(v) - r(0) removes the exterior data
    Lv = ev.rhs(v) - ev.rhs(np.zeros(ev.shape))
    wd, out = _dev(w), torch.zeros(ev.size, dtype=torch.float64, device="cuda")
    ev.rhs_vjp_device(wd.data_ptr(), out.data_ptr())
    torch.cuda.synchronize()
    LTw = out.cpu().numpy().reshape(ev.shape)
    assert _rel(np.vdot(w, Lv), np.vdot(LTw, v)) < 1e-12


@pytest.mark.parametrize("kind,n,luni", [("cs7", 5, 1), ("box", 4, 2), ("cs7h", 5, 0),
                                         ("boxs", 4, 1)])
def test_rk4_step_vjp_dot_product(kind, n, luni):
    import torch
    m = _mesh(kind, n, luni)
    ev = ng.Evolution(m, ng.BC_OUTGOING)
    rng = np.random.default_rng(1)
    v = rng.standard_normal(ev.shape)
    w = rng.standard_normal(ev.shape)
    dt = 0.02 / n ** 2
    ev.set_state(v)
    ev.rk4_step(0.0, dt)
    Pv = ev.get_state()
    wd = _dev(w)
    ev.rk4_step_vjp_device(wd.data_ptr(), 0.0, dt)
    torch.cuda.synchronize()
    PTw = wd.cpu().numpy().reshape(ev.shape)
    assert _rel(np.vdot(w, Pv), np.vdot(PTw, v)) < 1e-12


def _shell_weight(m, r0=3.0, r1=5.0):
    """Positive node weights on the shell r0 <= r <= r1 (LGL weight products)."""
    x, w, _ = ng.basis(m.n)
    wq = np.einsum("i,j,k->kji", w, w, w).ravel()
    r = np.linalg.norm(m.coords(), axis=1)
    return np.where((r >= r0) & (r <= r1), 1.0, 0.0) * wq[None, :]


def _oracle_J(o, u0, W, dt, nsteps):
    u = u0.copy()
    J = 0.0
    t = 0.0
    for s in range(nsteps):
        u = o.rk4(u, dt, 1, t=t)
        t += dt
        J += dt * float(np.sum(W * u[:, 4] ** 2))
    return J


@pytest.mark.parametrize("kind,nsteps,ckpt", [("cs7", 12, 5), ("cs7", 8, 1), ("cs7", 6, 6),
                                              ("cs7h", 6, 4)])
def test_gradient_matches_central_differences(kind, nsteps, ckpt):
    import torch
    m = _mesh(kind, 5, 1)
    ev = ng.Evolution(m, ng.BC_OUTGOING)
    u0 = gaussian_pulses(m.coords(), seed=7, rmin=2.0, rmax=5.0)
    W = _shell_weight(m)
    dt = 0.004
    ev.set_state(u0)
    Wd = _dev(W)
    g = torch.zeros(ev.size, dtype=torch.float64, device="cuda")
    J = ev.adjoint_gradient_device(Wd.data_ptr(), g.data_ptr(), 0.0, dt, nsteps, ckpt)
    grad = g.cpu().numpy().reshape(ev.shape)
    o = oracle_for(m, bc=1)
    J_cpu = _oracle_J(o, u0, W, dt, nsteps)
    assert _rel(J, J_cpu) < 1e-12
    rng = np.random.default_rng(nsteps)
    eps = 1e-6
    for _ in range(4):
        v = rng.standard_normal(ev.shape)
        v[:, 1:4] = 0.0   # directions in the initial psi (phi) and pi fields
        fd = (_oracle_J(o, u0 + eps * v, W, dt, nsteps) -
              _oracle_J(o, u0 - eps * v, W, dt, nsteps)) / (2 * eps)
        assert _rel(np.vdot(grad, v), fd) < 1e-6


def test_gradient_of_the_outer_shell_objective_16_directions():
    """The adjoint workload on a reduced mesh: 7 CubedSpheres at n = 9,
    level 1 (56 elements), J = sum_s dt sum W phi^2 over the shell
    17 <= r <= 19 (the outer shell r = 18), 50 RK4 steps with checkpoints
    every 10, against central differences (eps = 1e-6) of the oracle's
    forward run along 16 seeded directions in the initial psi and pi."""
    import torch
    m = _mesh("cs7", 9, 1)
    ev = ng.Evolution(m, ng.BC_OUTGOING)
    u0 = gaussian_pulses(m.coords(), seed=11, rmin=15.0, rmax=18.0)
    W = _shell_weight(m, 17.0, 19.0)
    dt = 0.25 * (2.0 / 2 ** 1) / 8 ** 2
    nsteps, ckpt = 50, 10
    ev.set_state(u0)
    Wd = _dev(W)
    g = torch.zeros(ev.size, dtype=torch.float64, device="cuda")
    J = ev.adjoint_gradient_device(Wd.data_ptr(), g.data_ptr(), 0.0, dt, nsteps, ckpt)
    grad = g.cpu().numpy().reshape(ev.shape)
    o = oracle_for(m, bc=1)
    assert J > 0 and _rel(J, _oracle_J(o, u0, W, dt, nsteps)) < 1e-12
    rng = np.random.default_rng(2016)
    eps = 1e-6
    worst = 0.0
    for _ in range(16):
        v = rng.standard_normal(ev.shape)
        v[:, 1:4] = 0.0
        fd = (_oracle_J(o, u0 + eps * v, W, dt, nsteps) -
              _oracle_J(o, u0 - eps * v, W, dt, nsteps)) / (2 * eps)
        worst = max(worst, _rel(np.vdot(grad, v), fd))
    print(f"\nworst relative gradient / central-difference mismatch over 16 directions: {worst:.2e}")
    assert worst < 1e-6
