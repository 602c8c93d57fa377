"""The oracle's GRHD Cowling evolution (oracle/nmo_grhd.c) on its own
cubed-shell mesh: known answers that need no GPU.  The reference has no
GRHD, so these pin the restatement by properties instead of vectors:
a uniform state at rest on a flat background has a zero DG right-hand side,
the finite-volume divergence of a uniform flow converges at second order,
the DG <-> finite-volume transfer inverts exactly, and the root finder
recovers the primitives."""
import numpy as np
import pytest

from helpers import grhd_blob
from oracle import nmo


def _uniform(o, rho=1.0, v=(0.0, 0.0, 0.0), p=0.01):
    (E, _, npd), (_, _, npf) = o.shapes
    out = []
    for npts, fvp in ((npd, False), (npf, True)):
        P = np.zeros((E, 5, npts))
        P[:, 0], P[:, 4] = rho, p
        P[:, 1], P[:, 2], P[:, 3] = v
        U = np.stack([o.prim2con(P[e], o.psi(o.points(e, fvp))) for e in range(E)])
        out += [P, U]
    return out


def test_dg_rhs_of_a_uniform_state_at_rest_is_zero():
    o = nmo.GrhdOracle(n=5, nf=9, ndiv=2, mass=0.0, p_atm=1e-18)
    pd, ud, pf, uf = _uniform(o)
    r_dg, _ = o.rhs(ud, uf, pd, pf)
    assert np.abs(r_dg).max() <= 1e-14


def test_finite_volume_free_stream_error_converges():
    """A uniform flow has the divergence of a constant flux: the point-wise
    metric of the curved shell leaves a residual on finite-volume elements
    (as the reference's default fin.-vol. metric does) that converges at
    second order inside the element (rms) and at first order on the half
    cells of its faces (max)."""
    errs_in, errs_face = [], []
    for nf in (6, 11):
        o = nmo.GrhdOracle(n=4, nf=nf, ndiv=2, mass=0.0, p_atm=1e-18,
                           fv=np.ones(48, np.int32))
        pd, ud, pf, uf = _uniform(o, v=(0.1, 0.05, 0.0))
        _, r_fv = o.rhs(ud, uf, pd, pf)
        idx = np.arange(nf ** 3)
        ijk = np.stack([idx % nf, (idx // nf) % nf, idx // (nf * nf)])
        inner = ((ijk > 0) & (ijk < nf - 1)).all(0)
        errs_in.append(np.sqrt((r_fv[:, :, inner] ** 2).mean()))
        errs_face.append(np.abs(r_fv[:, :, ~inner]).max())
    ratio = (11 - 1) / (6 - 1)
    assert np.log(errs_in[0] / errs_in[1]) / np.log(ratio) > 1.7, errs_in
    assert np.log(errs_face[0] / errs_face[1]) / np.log(ratio) > 0.9, errs_face


@pytest.mark.parametrize("n,nf", [(7, 14), (7, 13), (4, 8), (5, 5)])
def test_transfer_matrices_invert(n, nf):
    """R = (P^T P)^-1 P^T inverts P = LGL -> nf equally spaced points (the
    reference's UNI_to_no2LGLt with the pseudo-inverse), and P interpolates
    polynomials of degree n-1 exactly."""
    o = nmo.GrhdOracle(n=n, nf=nf, ndiv=1)
    P, R = o.transfer()
    assert np.abs(R @ P - np.eye(n)).max() <= 1e-13
    xl, _ = nmo.lgl(n)
    xu = nmo.uniform(nf)
    for k in range(n):
        assert np.abs(P @ xl ** k - xu ** k).max() <= 1e-13


def test_con2prim_recovers_the_blob_and_resets_the_atmosphere():
    fv = np.zeros(48, np.int32)
    fv[[5, 17]] = 1
    o = nmo.GrhdOracle(n=5, nf=9, ndiv=2, fv=fv, p_atm=1e-18)
    pd, pf, ud, uf = grhd_blob(o, seed=3)
    guess_d, guess_f = pd.copy(), pf.copy()
    guess_d[:, 4] *= 1.5
    guess_f[:, 4] *= 0.5
    natm, iters = o.con2prim(ud.copy(), uf.copy(), guess_d, guess_f)
    # points at the atmosphere density may round below it: atmosphere again
    at_atm = (pd[fv == 0, 0] < 2e-10).sum() + (pf[fv == 1, 0] < 2e-10).sum()
    assert natm <= at_atm and iters > 0
    dg = (fv == 0)[:, None] & (pd[:, 0] > 1e-7)
    for f in range(5):
        got, want = guess_d[:, f][dg], pd[:, f][dg]
        assert np.abs(got - want).max() <= 1e-12 * max(np.abs(want).max(), 1e-300)
    # below the atmosphere density: atmosphere, conserved variables reset
    ud2 = ud.copy()
    ud2[0, 0, :] = 0.5e-10
    natm, _ = o.con2prim(ud2, uf.copy(), pd.copy(), pf.copy())
    assert natm >= 1
