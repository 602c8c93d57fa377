"""The GRHD Cowling evolution on the GPU (include/nmg.h nmg_grhd_*) against
the oracle's restatement (oracle/nmo_grhd.c) on the same cubed shell:
right-hand side and RK4 steps on mixed DG / finite-volume meshes (relative
L2 <= 1e-12 over the DG and over the finite-volume states, 1e-11 per
field), the DG <-> finite-volume transfer, and the
known answers (a uniform state at rest keeps a zero DG right-hand side)."""
import numpy as np
import pytest

import nmesh_gb300 as ng
from helpers import grhd_blob, rel_l2
from oracle import nmo

pytestmark = pytest.mark.gpu

RTOL = 1e-12


@pytest.fixture(autouse=True)
def _gpu(cuda_ok):
    yield


def _case(n, nf, ndiv, fv_elems, mass=1.0, rec="WENOm5_2", seed=3, vel=(0.0, 0.0, 0.0)):
    E = 6 * ndiv ** 3
    fv = np.zeros(E, np.int32)
    fv[list(fv_elems)] = 1
    kw = dict(mass=mass, p_atm=1e-18, rho_atm=1e-10, tol=1e-15, maxits=100)
    o = nmo.GrhdOracle(n=n, nf=nf, ndiv=ndiv, fv=fv, rec=rec, **kw)
    pd, pf, ud, uf = grhd_blob(o, seed=seed, vel=vel)
    m = ng.Mesh.build(ng.MESH_CUBEDSHELL6, n=n, ndiv=ndiv, shell_rin=2.0, shell_rout=20.0)
    ev = ng.GrhdEvolution(m, nf=nf, rec=rec, **kw)
    ev.set_fv_elements(fv)
    ev.set_prim(pd, pf[fv == 1])
    return o, ev, fv, (ud, uf, pd, pf)


def _compare(fv, got_dg, got_fv, want_dg, want_fv, tol):
    """Relative L2 over all five fields of the DG elements and of the
    finite-volume elements within tol (as the scalar-wave tests measure a
    state), and per field within 10 tol: tau = psi^6 (rho h W^2 - p) - D
    cancels most of its digits against D (tau / D ~ eps ~ 1e-4 in the blob),
    so rounding differences of 1e-16 in the reconstructed primitives show
    in tau's right-hand side at ~1e-12."""
    dg = fv == 0
    assert rel_l2(got_dg[dg], want_dg[dg]) <= tol, "dg"
    if fv.any():
        assert rel_l2(got_fv, want_fv[fv == 1]) <= tol, "fv"
    for f in range(5):
        assert rel_l2(got_dg[dg][:, f], want_dg[dg][:, f]) <= 10 * tol, ("dg", f)
        if fv.any():
            assert rel_l2(got_fv[:, f], want_fv[fv == 1][:, f]) <= 10 * tol, ("fv", f)


@pytest.mark.parametrize("n,nf,rec", [(5, 9, "WENOm5_2"), (5, 10, "WENOm3_2"), (7, 13, "WENOm5_2"),
                                      (4, 8, "WENOmZ_2"), (8, 15, "WENOm5_2"), (9, 15, "WENOm5_2")])
def test_rhs_matches_oracle(n, nf, rec):
    o, ev, fv, (ud, uf, pd, pf) = _case(n, nf, 2, [1, 3, 10, 11, 20, 33, 47], rec=rec)
    u_dg, u_fv, _, _ = ev.get_state()
    _compare(fv, u_dg, u_fv, ud, uf, 1e-14)
    r_dg, r_fv = ev.rhs()
    want_dg, want_fv = o.rhs(ud, uf, pd, pf)
    _compare(fv, r_dg, r_fv, want_dg, want_fv, RTOL)


@pytest.mark.parametrize("n,nf", [(7, 13), (8, 15), (9, 15)])
def test_tensor_core_dg_kernel_matches_the_fp64_one(n, nf, monkeypatch):
    """At n = 7, 8, 9 the DG elements' divergence runs on the tensor cores
    (exact digit products, one FP64 rounding per line derivative); the FP64
    kernel (NMG_GRHD_DG=fp64) gives the same right-hand side and RK4 step
    within the oracle tolerance, and a blob moving across both kinds of
    element."""
    res = []
    for mode in ("fp64", None):
        if mode:
            monkeypatch.setenv("NMG_GRHD_DG", mode)
        else:
            monkeypatch.delenv("NMG_GRHD_DG", raising=False)
        o, ev, fv, _ = _case(n, nf, 2, [2, 5, 17, 30], vel=(0.04, 0.02, -0.03))
        r = ev.rhs()
        ev.rk4_steps(0.01, 2)
        res.append((fv, r, ev.get_state()))
        ev.close()
    (fv, ra, sa), (_, rb, sb) = res

    def full(compact):  # finite-volume rows back at their elements' places
        out = np.zeros((fv.size,) + compact.shape[1:])
        out[fv == 1] = compact
        return out

    _compare(fv, rb[0], rb[1], ra[0], full(ra[1]), RTOL)
    _compare(fv, sb[0], sb[1], sa[0], full(sa[1]), RTOL)


@pytest.mark.parametrize("mass", [1.0, 0.0])
def test_rk4_steps_match_oracle(mass):
    """Three RK4 steps with con2prim every stage, a moving blob crossing DG
    and finite-volume elements (nf = 2n - 1 points)."""
    o, ev, fv, (ud, uf, pd, pf) = _case(5, 9, 2, [0, 4, 9, 10, 22, 40], mass=mass,
                                         vel=(0.05, -0.03, 0.02))
    dt = 0.02
    ev.rk4_steps(dt, 3)
    got = ev.get_state()
    want = o.rk4(ud, uf, pd, pf, dt, 3)
    _compare(fv, got[0], got[1], want[0], want[1], RTOL)
    it, natm, launches = ev.stats()
    assert it > 0 and launches >= 3 * 4 * 3


def test_switch_transfers_the_state_like_the_oracle():
    """DG -> finite volume by P x P x P (Lagrange to 2n equally spaced
    points, the reference's PARENT_2n_P_UNIFORM), back by R = (P^T P)^-1 P^T;
    the round trip returns the DG state."""
    n, nf = 5, 10
    o, ev, fv, (ud, uf, pd, pf) = _case(n, nf, 2, [])
    u0 = ev.get_state()[0]
    P, R = o.transfer()
    sel = [2, 7, 30]
    fv2 = np.zeros(48, np.int32)
    fv2[sel] = 1
    ev.set_fv_elements(fv2)
    u_dg, u_fv, _, _ = ev.get_state()
    for k, e in enumerate(sel):
        want = o.apply3(P, u0[e])
        assert rel_l2(u_fv[k], want) <= 1e-14
    ev.set_fv_elements(np.zeros(48, np.int32))
    back = ev.get_state()[0]
    for e in sel:
        assert rel_l2(back[e], u0[e]) <= 1e-13
        assert rel_l2(back[e], o.apply3(R, o.apply3(P, u0[e]))) <= 1e-14
    others = np.setdiff1d(np.arange(48), sel)
    assert np.array_equal(back[others], u0[others])


def test_uniform_state_at_rest_keeps_a_zero_dg_rhs():
    n = 5
    m = ng.Mesh.build(ng.MESH_CUBEDSHELL6, n=n, ndiv=2, shell_rin=2.0, shell_rout=20.0)
    ev = ng.GrhdEvolution(m, mass=0.0, p_atm=1e-18)
    prim = np.zeros((48, 5, n ** 3))
    prim[:, 0], prim[:, 4] = 1.0, 0.01
    ev.set_prim(prim)
    r_dg, _ = ev.rhs()
    assert np.abs(r_dg).max() <= 1e-13
    ev.rk4_steps(0.05, 4)
    u, _, p, _ = ev.get_state()
    assert np.abs(p[:, 0] - 1.0).max() <= 1e-12 and np.abs(p[:, 1:4]).max() <= 1e-12


def test_bad_arguments_are_rejected():
    m = ng.Mesh.build(ng.MESH_CUBEDSPHERES7, n=5, luni=0, cs_dc=1.0, cs_r0fac=20.0)
    with pytest.raises(ng.NmgError):
        ng.GrhdEvolution(m)
    m = ng.Mesh.build(ng.MESH_CUBEDSHELL6, n=5, ndiv=1, shell_rin=2.0, shell_rout=20.0)
    with pytest.raises(ng.NmgError):
        ng.GrhdEvolution(m, nf=40)
    with pytest.raises(ng.NmgError):
        ng.GrhdEvolution(m, gamma=1.0)
    ev = ng.GrhdEvolution(m)
    with pytest.raises(ng.NmgError):
        ev.rk4_steps(-1.0, 1)


def test_twenty_steps_with_a_switch_midway_match_oracle():
    """Ten RK4 steps, elements switched to and from finite volume, ten more
    steps: the GPU state against the oracle's, which applies the same
    transfer (P x P x P to finite volume, R x R x R back)."""
    n, nf = 5, 10
    o, ev, fv, (ud, uf, pd, pf) = _case(n, nf, 2, [4, 9, 22], vel=(0.04, 0.02, -0.03))
    dt = 0.02
    ev.rk4_steps(dt, 10)
    ud, uf, pd, pf = o.rk4(ud, uf, pd, pf, dt, 10)
    got = ev.get_state()
    _compare(fv, got[0], got[1], ud, uf, RTOL)
    # switch: 4 back to DG, 30 and 31 to finite volume
    P, R = o.transfer()
    fv2 = fv.copy()
    fv2[4] = 0
    fv2[[30, 31]] = 1
    ev.set_fv_elements(fv2)
    ud[4], pd[4] = o.apply3(R, uf[4]), o.apply3(R, pf[4])
    for e in (30, 31):
        uf[e], pf[e] = o.apply3(P, ud[e]), o.apply3(P, pd[e])
    o.set_fv(fv2)
    ev.rk4_steps(dt, 10)
    ud, uf, pd, pf = o.rk4(ud, uf, pd, pf, dt, 10)
    got = ev.get_state()
    _compare(fv2, got[0], got[1], ud, uf, RTOL)


def test_trouble_indicator_and_switching_by_it():
    """Persson's indicator of D per element against the oracle's restatement
    (nmo_persson on the LGL values; finite-volume elements projected back by
    R x R x R first), then switching by the indicator with a margin."""
    n, nf = 5, 10
    o, ev, fv, (ud, uf, pd, pf) = _case(n, nf, 2, [3, 10, 33])
    ind = ev.trouble_indicators()
    _, R = o.transfer()
    want = np.array([nmo.persson(n, o.apply3(R, uf[e])[0] if fv[e] else ud[e, 0])
                     for e in range(48)])
    assert np.abs(ind - want).max() <= 1e-9
    thr = float(np.median(ind))
    to_fv, to_dg = ev.update_troubled(thr, back_margin=0.5)
    new = ev.fv_elements()
    exp = fv.copy()
    exp[(fv == 0) & (ind > thr)] = 1
    exp[(fv == 1) & (ind < thr - 0.5)] = 0
    assert np.array_equal(new, exp)
    assert to_fv == int(((fv == 0) & (ind > thr)).sum())
    assert to_dg == int(((fv == 1) & (ind < thr - 0.5)).sum())


def test_full_grhd_workload_against_oracle():
    """The benchmark's GRHD workload at its full size (6 x 12^3 elements at
    n = 7, the seeded 10 % on 13^3 finite-volume points, blob at r = 8,
    M = 1): the RHS and one RK4 step against the oracle from the same
    conserved state."""
    import bench
    n, nf, nd = 7, 13, 12
    E = 6 * nd ** 3
    flags = np.zeros(E, np.int32)
    flags[np.random.default_rng(34).choice(E, int(round(0.1 * E)), replace=False)] = 1
    kw = dict(mass=1.0, gamma=2.0, rho_atm=bench.GRHD_RHO_ATM,
              p_atm=bench.GRHD_K * bench.GRHD_RHO_ATM ** 2)
    o = nmo.GrhdOracle(n=n, nf=nf, ndiv=nd, fv=flags, **kw)
    pd = bench.grhd_initial_prim(o.xyz, seed=33)
    ud = np.stack([o.prim2con(pd[e], o.psi(o.xyz[e])) for e in range(E)])
    P, _ = o.transfer()
    uf = np.zeros((E, 5, nf ** 3))
    pf = np.zeros((E, 5, nf ** 3))
    for e in np.nonzero(flags)[0]:
        uf[e] = o.apply3(P, ud[e])
        pf[e] = o.apply3(P, pd[e])
    m = ng.Mesh.build(ng.MESH_CUBEDSHELL6, n=n, ndiv=nd, shell_rin=2.0, shell_rout=20.0)
    ev = ng.GrhdEvolution(m, nf=nf, **kw)
    ev.set_fv_elements(flags)
    ev.set_state(ud, uf[flags == 1], pd, pf[flags == 1])
    r_dg, r_fv = ev.rhs()
    w_dg, w_fv = o.rhs(ud, uf, pd, pf)
    _compare(flags, r_dg, r_fv, w_dg, w_fv, RTOL)
    ev.set_state(ud, uf[flags == 1], pd, pf[flags == 1])
    dt = 0.25 * (2.0 * (np.pi / 2.0) / nd) / (n - 1) ** 2
    ev.rk4_steps(dt, 1)
    got = ev.get_state()
    want = o.rk4(ud, uf, pd, pf, dt, 1)
    _compare(flags, got[0], got[1], want[0], want[1], RTOL)
    ev.close()
