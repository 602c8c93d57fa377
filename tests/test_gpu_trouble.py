"""DG <-> finite-volume element switching and trouble detection on the GPU
(switchable contexts), against the oracle: the state conversion between LGL
and equally spaced points, the RDMP / Persson indicators, and the RK4 step
that detects trouble, switches troubled elements to finite volume, redoes
the step and switches quiet elements back (the reference's
evolve_redo_troubled = step flow, restated in Python on oracle pieces)."""
import numpy as np
import pytest

import nmesh_gb300 as ng
from helpers import PI, RTOL_RHS, RTOL_RK4, oracle_for, rel_l2
from oracle import nmo

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(autouse=True)
def _gpu(cuda_ok):
    yield


def transfer_matrices(n):
    """P[p, j]: Lagrange weight of LGL point j at equally spaced point p;
    R = P^{-1}."""
    xl, _ = nmo.lgl(n)
    xu = nmo.uniform(n)
    wl = np.array([1.0 / np.prod([xl[i] - xl[j] for j in range(n) if j != i])
                   for i in range(n)])
    P = np.array([[np.prod([xu[p] - xl[q] for q in range(n) if q != j]) * wl[j]
                   for j in range(n)] for p in range(n)])
    return P, np.linalg.inv(P)


def convert(u, old, new, P, R):
    u = u.copy()
    n = round(u.shape[-1] ** (1 / 3))
    for e in range(u.shape[0]):
        if old[e] == new[e]:
            continue
        M = P if new[e] else R
        v = u[e].reshape(5, n, n, n)          # [field][k][j][i]
        u[e] = np.einsum("ai,bj,ck,fkji->fcba", M, M, M, v).reshape(5, -1)
    return u


class Setup:
    """Periodic box with both point-type geometries of every element."""

    def __init__(self, n, luni):
        kw = dict(n=n, luni=luni, xc=(PI, PI, PI), box_dout=PI, periodic=True)
        self.mdg = ng.Mesh.build(ng.MESH_BOX, **kw)
        self.mfv = ng.Mesh.build(ng.MESH_BOX, fv=True, **kw)
        self.n = n
        self.E = self.mdg.nelem
        self.P, self.R = transfer_matrices(n)

    def oracle(self, types, **kw):
        m = self.mesh(types)
        return oracle_for(m, bc=1, period=2 * PI, **kw)

    def mesh(self, types):
        pat, bbox = self.mdg.elements()
        xyz = np.where(types[:, None, None] == 1, self.mfv.coords(), self.mdg.coords())
        return ng.Mesh.from_arrays(bbox, np.zeros(self.E, np.int32), xyz, pat=pat,
                                   period=(2 * PI,) * 3, fv=types)


def test_switch_conversion_and_roundtrip():
    S = Setup(6, 1)
    ev = ng.Evolution(S.mdg, ng.BC_OUTGOING, switchable=True)
    u = np.random.default_rng(1).standard_normal((S.E, 5, 6 ** 3))
    ev.set_state(u)
    types = np.zeros(S.E, np.int32)
    types[[0, 3, 5]] = 1
    ev.set_element_types(types)
    assert np.array_equal(ev.element_types(), types)
    uf = ev.get_state()
    assert rel_l2(uf, convert(u, np.zeros(S.E, np.int32), types, S.P, S.R)) <= 1e-14
    ev.set_element_types(np.zeros(S.E, np.int32))
    assert rel_l2(ev.get_state(), u) <= 1e-12


@pytest.mark.parametrize("rec,ex", [("WENOm5_2", "dnfn_extrap1"), ("WENOm3_2", "no")])
def test_switchable_rhs_matches_mixed_oracle(rec, ex):
    S = Setup(7, 1)
    types = np.zeros(S.E, np.int32)
    types[[1, 2, 6]] = 1
    ev = ng.Evolution(S.mdg, ng.BC_OUTGOING, switchable=True)
    ev.set_fv(rec, ex)
    xyz = S.mesh(types).coords()
    arg = xyz[:, 0] + 2.0 * xyz[:, 1] - xyz[:, 2]
    u = np.stack([np.sin(arg), np.cos(arg), np.sin(2 * arg), np.cos(arg), np.sin(arg)], 1)
    ev.set_state(np.zeros_like(u))
    ev.set_element_types(types)
    o = S.oracle(types, fv_rec=rec, fv_extrap=ex)
    assert rel_l2(ev.rhs(u, 0.0), o.rhs(u, 0.0)) <= RTOL_RHS
    assert rel_l2(ev.rk4_steps_host(u, 0.0, 0.01, 2), o.rk4(u, 0.01, 2)) <= RTOL_RK4
    # an all-DG switchable context steps like a plain one
    ev.set_element_types(np.zeros(S.E, np.int32))
    plain = ng.Evolution(S.mdg, ng.BC_OUTGOING)
    ud = np.random.default_rng(2).standard_normal(u.shape)
    assert rel_l2(ev.rk4_steps_host(ud, 0.0, 0.01, 2),
                  plain.rk4_steps_host(ud, 0.0, 0.01, 2)) <= 1e-13


def test_trouble_indicators_match_oracle():
    S = Setup(6, 2)
    types = np.zeros(S.E, np.int32)
    types[::7] = 1
    xyz = S.mesh(types).coords()
    rng = np.random.default_rng(5)
    u_p = np.stack([np.sin(xyz[:, 0]), np.cos(xyz[:, 1]), np.sin(xyz[:, 2]),
                    np.cos(xyz[:, 0] + xyz[:, 1]), np.sin(xyz[:, 1] - xyz[:, 2])], 1)
    u = u_p + 1e-3 * rng.standard_normal(u_p.shape)
    bump = rng.random(S.E) < 0.2                     # elements pushed outside the bounds
    u[bump, 0] += 3.0 * (xyz[bump, 0] > xyz[bump, 0].mean(axis=1, keepdims=True))
    ev = ng.Evolution(S.mdg, ng.BC_OUTGOING, switchable=True)
    ev.set_element_types(types)
    o = S.oracle(types)
    du = torch.from_numpy(u.ravel()).cuda()
    dup = torch.from_numpy(u_p.ravel()).cuda()
    for kw in (dict(rdmp_delta0=1e-4, persson_max=1e300),
               dict(rdmp_delta0=1e10, persson_max=-2.0),
               dict(rdmp_delta0=1e-2, rdmp_epsilon=0.1, persson_max=-1.5)):
        fl, pe = ev.trouble_check_device(du.data_ptr(), dup.data_ptr(), ng.TroubleParams(**kw))
        flo, peo = o.trouble(u, u_p, deltafac=1.0, delta0=kw["rdmp_delta0"],
                             epsilon=kw.get("rdmp_epsilon", 1e-3),
                             persson_max=kw["persson_max"])
        assert np.array_equal(fl, flo)
        assert np.abs(pe - peo).max() <= 1e-10
    assert (fl == 1).any() and (fl == -1).any() and (fl == 0).any()


def _oracle_step(S, u, types, scores, t, dt, kw, notroubles):
    o = S.oracle(types, fv_rec="WENOm5_2", fv_extrap="dnfn_extrap1")
    u_p = u
    u = o.rk4(u_p, dt, 1, t)
    fl, _ = o.trouble(u, u_p, deltafac=1.0, delta0=kw["rdmp_delta0"], epsilon=1e-3,
                      persson_max=kw["persson_max"])
    for e in range(S.E):
        if fl[e] > 0:
            scores[e] = 1 if scores[e] <= 0 else scores[e] + 1
        elif fl[e] == 0:
            scores[e] = 0
        else:
            scores[e] = -1 if scores[e] >= 0 else scores[e] - 1
    g = scores.max() if scores.max() > 0 else scores.min()
    nfv = ndg = 0
    if g > 0:
        t2 = types.copy()
        t2[scores > 0] = 1
        nfv = int((t2 != types).sum())
        u_p = convert(u_p, types, t2, S.P, S.R)
        types = t2
        o = S.oracle(types, fv_rec="WENOm5_2", fv_extrap="dnfn_extrap1")
        u = o.rk4(u_p, dt, 1, t)
    if g > 0 or g <= -notroubles:
        t3 = types.copy()
        t3[(types == 1) & (scores <= -notroubles)] = 0
        ndg = int((t3 != types).sum())
        u = convert(u, types, t3, S.P, S.R)
        types = t3
    return u, types, scores, (nfv, ndg)


@pytest.mark.parametrize("filt", [False, True])
def test_rk4_step_trouble_matches_oracle_flow(filt):
    """With filt the exponential filter (evolve_filter_all) follows every
    step, on the element types the step ended with."""
    S = Setup(6, 2)
    xyz = S.mdg.coords()
    # a smooth wave in phi plus a ball of pi = 1: the ball's elements are
    # troubled (Persson's indicator above -1.8, smooth elements near -7)
    r = np.sqrt(np.sum((xyz - 4.0) ** 2, axis=1))
    u = np.zeros((S.E, 5, 6 ** 3))
    u[:, 4] = 0.1 * np.sin(xyz[:, 0] + xyz[:, 1])
    u[:, 0] = np.where(r < 1.0, 1.0, 0.0)
    kw = dict(rdmp_delta0=1e10, persson_max=-1.8)
    tp = ng.TroubleParams(rdmp_delta0=kw["rdmp_delta0"], persson_max=kw["persson_max"],
                          notroubles=2)
    ev = ng.Evolution(S.mdg, ng.BC_OUTGOING, switchable=True)
    ev.set_fv("WENOm5_2", "dnfn_extrap1")
    if filt:
        ev.set_filter(True, alp=36.0, s=4.0)
    ev.set_state(u)
    types = np.zeros(S.E, np.int32)
    scores = np.zeros(S.E, np.int64)
    uo = u.copy()
    dt, t = 0.02, 0.0
    seen = set()
    for step in range(6):
        sw = ev.rk4_step_trouble(t, dt, tp)
        uo, types, scores, swo = _oracle_step(S, uo, types, scores, t, dt, kw, 2)
        if filt:
            uo = S.oracle(types).filter(uo, alp=36.0, s=4.0)
        assert sw == swo, step
        seen.add(sw)
        assert np.array_equal(ev.element_types(), types)
        assert np.array_equal(ev.trouble_scores(), scores)
        assert rel_l2(ev.get_state(), uo) <= 1e-11
        t += dt
    assert any(s[0] > 0 for s in seen)          # troubled elements switched to FV
    assert any(s[1] > 0 for s in seen)          # quiet FV elements switched back


def _oracle_substep_step(S, u, types, scores, t, dt, kw, notroubles):
    """evolve_RK4_mesh with evolve_redo_troubled = substep, restated on
    oracle pieces: score after every substep; troubled elements take the
    substep back, the DG ones switch (u, u_p, w converted), r is recomputed
    on each with its neighbours in their old types and data, and the
    substep is applied again."""
    fvkw = dict(fv_rec="WENOm5_2", fv_extrap="dnfn_extrap1")
    cacc = [dt / 6, dt / 3, dt / 3, dt / 6]
    cw = [dt / 2, dt / 2, dt]
    ts = [t, t + dt / 2, t + dt / 2, t + dt]
    u_p, w = u.copy(), u.copy()
    nfv = 0
    for s in range(4):
        o = S.oracle(types, **fvkw)
        r = o.rhs(w, ts[s])
        u = (w if s == 0 else u) + cacc[s] * r
        fl, _ = o.trouble(u, u_p, deltafac=1.0, delta0=kw["rdmp_delta0"], epsilon=1e-3,
                          persson_max=kw["persson_max"], uscale=kw["uscale"])
        for e in range(S.E):
            if fl[e] > 0:
                scores[e] = 1 if scores[e] <= 0 else scores[e] + 1
            elif fl[e] == 0:
                scores[e] = 0
            else:
                scores[e] = -1 if scores[e] >= 0 else scores[e] - 1
        g = scores.max() if scores.max() > 0 else scores.min()
        if g > 0:
            T = np.flatnonzero(scores > 0)
            u[T] -= cacc[s] * r[T]
            t2 = types.copy()
            t2[T] = 1
            nfv += int((t2 != types).sum())
            u = convert(u, types, t2, S.P, S.R)
            u_p = convert(u_p, types, t2, S.P, S.R)
            w2 = convert(w, types, t2, S.P, S.R)
            for e in T:
                te = types.copy()
                te[e] = 1
                we = w.copy()
                we[e] = w2[e]
                r[e] = S.oracle(te, **fvkw).rhs(we, ts[s])[e]
            u[T] += cacc[s] * r[T]
            types, w = t2, w2
        if s < 3:
            w = u_p + cw[s] * r
    g = scores.max() if scores.max() > 0 else scores.min()
    ndg = 0
    if g > 0 or g <= -4 * notroubles:
        t3 = types.copy()
        t3[(types == 1) & (scores <= -4 * notroubles)] = 0
        ndg = int((t3 != types).sum())
        u = convert(u, types, t3, S.P, S.R)
        types = t3
    return u, types, scores, (nfv, ndg)


def test_rk4_step_trouble_substep_matches_oracle_flow():
    """The reference's default evolve_redo_troubled = substep.  The
    indicator's scale is fixed (persson_uscale): with c_0 from the data, a
    field that is still zero in an element is exactly zero in the oracle
    but round-off noise on the GPU, and noise has a large scale-free
    indicator; with a fixed scale the flags keep a margin of about 0.5 from
    the threshold throughout."""
    S = Setup(6, 2)
    xyz = S.mdg.coords()
    r = np.sqrt(np.sum((xyz - 4.0) ** 2, axis=1))
    u = np.zeros((S.E, 5, 6 ** 3))
    u[:, 4] = 0.1 * np.sin(xyz[:, 0] + xyz[:, 1])
    u[:, 0] = np.where(r < 1.0, 1.0, 0.0)
    kw = dict(rdmp_delta0=1e10, persson_max=-3.5, uscale=1.0)
    tp = ng.TroubleParams(rdmp_delta0=kw["rdmp_delta0"], persson_max=kw["persson_max"],
                          persson_uscale=kw["uscale"], notroubles=1, redo="substep")
    ev = ng.Evolution(S.mdg, ng.BC_OUTGOING, switchable=True)
    ev.set_fv("WENOm5_2", "dnfn_extrap1")
    ev.set_state(u)
    types = np.zeros(S.E, np.int32)
    scores = np.zeros(S.E, np.int64)
    uo = u.copy()
    dt, t = 0.02, 0.0
    seen = set()
    for step in range(4):
        sw = ev.rk4_step_trouble(t, dt, tp)
        uo, types, scores, swo = _oracle_substep_step(S, uo, types, scores, t, dt, kw, 1)
        assert sw == swo, step
        seen.add(sw)
        assert np.array_equal(ev.element_types(), types)
        assert np.array_equal(ev.trouble_scores(), scores)
        assert rel_l2(ev.get_state(), uo) <= 1e-11
        t += dt
    assert any(s[0] > 0 for s in seen)
    assert any(s[1] > 0 for s in seen)
