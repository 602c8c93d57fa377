"""The oracle (CPU restatement, oracle/nmo.c) against the reference's own
outputs: golden fixtures made by running the reference
(tests/golden/make_golden.py).  The restatement follows the reference's
operation order and must match it bit for bit."""
import numpy as np
import pytest

from helpers import (BIG_CASE, CASES, FILT_CASES, LIM_CASES, MMB_CASES, RTOL_FILT_ORACLE, FV_CASES, METHOD_CASES, METHOD_NEAR_CASES, MID_CASES,
                     MID_NEAR_CASES, MIX_CASES, MIX_NEAR_CASES, NC_CASES, RTOL_NC_ORACLE,
                     UPW_CASES, big_case_u0, build_mesh, limiter_kwargs, load, oracle_for, perm_to_mesh,
                     rel_l2, to_mesh_order)
from oracle import nmo


def _oracle_mesh(d, meta):
    n = int(d["n"][0, 0])
    curvi = (d["pat"] > 0).astype(np.int32) if meta["mesh"] == "cs7" else \
        np.zeros(len(d["pat"]), np.int32)
    fv = {}
    if "fv" in meta:
        nb, mix = nmo.match_faces(d["x"], n, fv=d["use_fv"])
        fv = dict(fv=d["use_fv"], fv_rec=meta["fv"]["rec"],
                  fv_extrap=meta["fv"]["extrap"], mixface=mix,
                  fv_surface_interp=meta["fv"].get("surf", "linear"))
    else:
        nb = nmo.match_faces(d["x"], n)
    if meta.get("hrefine") or meta.get("sphere"):
        nb, fv["hang"] = nmo.match_hanging(d["x"], n, d["pat"], d["bbox"], nb)
    return nmo.OracleMesh(d["bbox"], curvi, d["dXdx"], d["x"], nb, n, bc=0,
                          k=meta["k"], numflux=meta.get("numflux", "LLF"), **fv)


@pytest.mark.parametrize("case", CASES + FV_CASES)
def test_oracle_rhs_bitexact(case):
    d, meta = load(case)
    m = _oracle_mesh(d, meta)
    r = m.rhs(d["u0"], 0.0)
    assert np.array_equal(r, d["r0"])


@pytest.mark.parametrize("case", CASES + FV_CASES)
def test_oracle_rk4_bitexact(case):
    d, meta = load(case)
    m = _oracle_mesh(d, meta)
    u = m.rk4(d["u0"], meta["dt"], meta["steps"])
    assert np.array_equal(u, d["u_final"])


@pytest.mark.parametrize("case", [c for c in MIX_CASES + UPW_CASES if c not in MIX_NEAR_CASES])
def test_oracle_mixed_dg_fv_bitexact(case):
    """Mixed DG / finite-volume meshes (inner cube FV, shells DG): the
    interface traces are interpolated at the face points (Lagrange from the
    DG side, piecewise linear from the FV side) as the reference does."""
    d, meta = load(case)
    m = _oracle_mesh(d, meta)
    assert np.array_equal(m.rhs(d["u0"], 0.0), d["r0"])
    assert np.array_equal(m.rk4(d["u0"], meta["dt"], meta["steps"]), d["u_final"])


@pytest.mark.parametrize("case", METHOD_CASES)
def test_oracle_other_integrators_match_reference(case):
    """evolve_method = sspRK3 and Euler: bit for bit (a few ulp on the mixed
    even-n mesh, whose interface traces are a few ulp off)."""
    d, meta = load(case)
    m = _oracle_mesh(d, meta)
    u = m.evolve(d["u0"], meta["dt"], meta["steps"], method=meta["method"])
    if case in METHOD_NEAR_CASES:
        assert rel_l2(u, d["u_final"]) <= RTOL_NC_ORACLE
    else:
        assert np.array_equal(u, d["u_final"])


@pytest.mark.parametrize("case", MID_CASES)
def test_oracle_midpoint_data_matches_reference(case):
    """coordinates_midpoint_data = yes: the midpoint map values come from the
    product's mesh packer (nmg_mesh_get_midpoint_dXdx), the factors and
    normals from the oracle; bit for bit on all-FV meshes."""
    d, meta = load(case)
    m = build_mesh(meta)
    perm = perm_to_mesh(m, d)
    o = oracle_for(m, bc=0, k=meta["k"], fv_rec=meta["fv"]["rec"],
                   fv_extrap=meta["fv"]["extrap"],
                   fv_surface_interp=meta["fv"].get("surf", "linear"), midpoint_data=True)
    u0 = to_mesh_order(d["u0"], perm)
    r = o.rhs(u0)[perm]
    u = o.evolve(u0, meta["dt"], meta["steps"], method=meta.get("method", "RK4"))[perm]
    if case in MID_NEAR_CASES:
        assert rel_l2(r, d["r0"]) <= RTOL_NC_ORACLE
        assert rel_l2(u, d["u_final"]) <= RTOL_NC_ORACLE
    else:
        assert np.array_equal(r, d["r0"]) and np.array_equal(u, d["u_final"])


@pytest.mark.parametrize("case", MIX_NEAR_CASES)
def test_oracle_mixed_even_n_matches_reference(case):
    """Mixed DG / FV with FV patches 0, 2, 4, n = 6, WENO-Z: a few ulp."""
    d, meta = load(case)
    m = _oracle_mesh(d, meta)
    assert rel_l2(m.rhs(d["u0"], 0.0), d["r0"]) <= RTOL_NC_ORACLE
    assert rel_l2(m.rk4(d["u0"], meta["dt"], meta["steps"]), d["u_final"]) <= RTOL_NC_ORACLE


@pytest.mark.parametrize("case", NC_CASES)
def test_oracle_nonconforming_matches_reference(case):
    """Elements one level finer than their neighbours (patch-wise,
    amr_hrefine_p, and inside patches, amr_hrefine_sphere_levels): each
    node of a fine face interpolates the coarse face, each node of a coarse
    face averages the fine faces containing it.  The neighbour positions
    come from the element structure here and from inverse coordinate maps
    in the reference, so the match is to a few ulp (bitwise where both
    positions round alike)."""
    d, meta = load(case)
    m = _oracle_mesh(d, meta)
    assert rel_l2(m.rhs(d["u0"], 0.0), d["r0"]) <= RTOL_NC_ORACLE
    assert rel_l2(m.rk4(d["u0"], meta["dt"], meta["steps"]), d["u_final"]) <= RTOL_NC_ORACLE


def test_nonconforming_face_lists():
    """Structure of the non-conforming lists: inner cube refined once
    against six single-element shells, n = 5 (a node on the middle lines)."""
    d, meta = load("nc_cs7_l0_n5_h0")
    n = 5
    nb = nmo.match_faces(d["x"], n)
    nb2, (off, src, pos) = nmo.match_hanging(d["x"], n, d["pat"], d["bbox"], nb)
    hang = nb2[:, :, 0] == -3
    # 24 fine faces of the cube's outside, the 6 shells' inner faces
    assert hang[:8].sum() == 24 and hang[8:].sum() == 6
    assert (nb[hang] == -1).all() and (nb2[~hang] == nb[~hang]).all()
    cnt = np.diff(off).reshape(len(d["pat"]), 6, n * n)
    assert (cnt[:8][hang[:8]] == 1).all()
    coarse = cnt[8:][hang[8:]]          # [6, n*n]
    # interior nodes 1 source, middle-line nodes 2, the centre 4
    want = np.ones((n, n), int)
    want[2, :] = want[:, 2] = 2
    want[2, 2] = 4
    assert (coarse == want.ravel()[None, :]).all()
    assert np.abs(pos).max() <= 1 + 1e-14


def test_lgl_basis_properties():
    for n in range(2, 13):
        x, w = nmo.lgl(n)
        D = nmo.diffmat(n)
        assert abs(w.sum() - 2.0) < 1e-13
        assert np.all(np.diff(x) > 0)
        # D differentiates polynomials of degree n-1 exactly
        for p in range(n):
            assert np.allclose(D @ x ** p, p * x ** max(p - 1, 0) * (p > 0), atol=1e-10)
        # row sums vanish (negative-sum trick of the reference)
        assert np.abs(D.sum(axis=1)).max() < 1e-12


def test_outgoing_bc_absorbs_outgoing_characteristic():
    """With the outgoing BC a state whose incoming characteristic pi + c.n
    vanishes on the outer face gets no lift from the exterior jump in
    pi + c.n; here: the RHS is linear and homogeneous (r(0) = 0)."""
    d, meta = load("cs7_l0_n9")
    n = 9
    nb = nmo.match_faces(d["x"], n)
    m = nmo.OracleMesh(d["bbox"], (d["pat"] > 0).astype(np.int32), d["dXdx"], d["x"],
                       nb, n, bc=1)
    z = np.zeros_like(d["u0"])
    assert np.array_equal(m.rhs(z), z)
    u = d["u0"]
    r1 = m.rhs(u)
    r2 = m.rhs(2.0 * u)
    assert np.allclose(r2, 2.0 * r1, rtol=0, atol=1e-12 * np.abs(r1).max())


def test_periodic_plane_wave_is_smooth():
    """Periodic box: the RHS of the exact plane wave matches its time
    derivative to truncation accuracy (no boundary at all)."""
    import nmesh_gb300 as ng
    from helpers import PI
    mesh = ng.Mesh.build(ng.MESH_BOX, n=6, luni=2, xc=(PI, PI, PI), box_dout=PI,
                         periodic=True)
    xyz = mesh.coords()
    k = np.array([1.0, 1.0, 1.0])
    om = np.sqrt(3.0)
    arg = np.einsum("i,eip->ep", k, xyz)
    u = np.stack([-om * np.cos(arg), np.cos(arg), np.cos(arg), np.cos(arg), np.sin(arg)], 1)
    dudt = np.stack([-om * om * np.sin(arg), om * np.sin(arg), om * np.sin(arg),
                     om * np.sin(arg), -om * np.cos(arg)], 1)
    nb = nmo.match_faces(xyz, 6, period=2 * PI)
    assert (nb < 0).sum() == 0
    _, bbox = mesh.elements()
    m = nmo.OracleMesh(bbox, np.zeros(mesh.nelem, np.int32), mesh.dXdx(), xyz, nb, 6)
    r = m.rhs(u)
    assert np.abs(r - dudt).max() < 2e-3


def test_oracle_persson_matches_reference():
    """Persson's indicator of every field of every element of u0 against the
    reference's evolve_Persson_array_indicator (dumped by the reference run)."""
    d, meta = load("trbl_cs7_l1_n6")
    n = meta["n"]
    got = np.array([[nmo.persson(n, d["u0"][e, l]) for l in range(5)]
                    for e in range(len(d["pat"]))])
    assert np.array_equal(got, d["persson"])
    m = _oracle_mesh(d, meta)
    fl, pe = m.trouble(d["u0"], d["u0"])
    assert np.array_equal(pe, d["persson"])
    assert (fl == 0).all()                      # u == u_p: inside its own bounds
    fl, _ = m.trouble(d["u0"], d["u0"], persson_max=-2.0)
    assert np.array_equal(fl, (d["persson"] > -2.0).any(axis=1).astype(np.int32))


@pytest.mark.parametrize("case", FILT_CASES)
def test_oracle_filter_matches_reference(case):
    """evolve_filter_all = yes: RK4 step, then the exponential filter of
    every element (J-weighted on curvilinear elements, FV elements too)."""
    d, meta = load(case)
    m = build_mesh(meta)
    perm = perm_to_mesh(m, d)
    kw = {}
    if "fv" in meta:
        kw = dict(fv_rec=meta["fv"]["rec"], fv_extrap=meta["fv"]["extrap"])
    o = oracle_for(m, bc=0, k=meta["k"], **kw)
    u = to_mesh_order(d["u0"], perm)
    for s in range(meta["steps"]):
        u = o.filter(o.rk4(u, meta["dt"], 1, t=s * meta["dt"]))
    assert rel_l2(u[perm], d["u_final"]) <= RTOL_FILT_ORACLE


@pytest.mark.parametrize("case", LIM_CASES)
def test_oracle_mrs_limiter_matches_reference(case):
    """scalarwave1_limiter = MRS: w limited before every later RK4 stage and
    the new u after the step (limiter_MRS with limiter_alpha)."""
    d, meta = load(case)
    m = _oracle_mesh(d, meta)
    u = m.rk4_limited(d["u0"], meta["dt"], meta["steps"], alpha=meta["limiter"])
    assert rel_l2(u, d["u_final"]) <= RTOL_NC_ORACLE
    # without the limiter the run is far off: the limiter acts
    assert rel_l2(m.rk4(d["u0"], meta["dt"], meta["steps"]), d["u_final"]) > 1e-3


@pytest.mark.parametrize("case", MMB_CASES)
def test_oracle_minmodb_limiter_matches_reference(case):
    """scalarwave1_limiter = minmodB: the same stage placement as MRS, with
    limiter_minmodB's bounded minmod on the linear modes (limiter_alpha,
    limiter_beta, limiter_scaleBound), on DG, non-conforming and mixed
    DG / finite-volume meshes."""
    d, meta = load(case)
    m = _oracle_mesh(d, meta)
    kw = limiter_kwargs(meta)
    u = m.rk4_limited(d["u0"], meta["dt"], meta["steps"], **kw)
    assert rel_l2(u, d["u_final"]) <= RTOL_NC_ORACLE
    assert rel_l2(m.rk4(d["u0"], meta["dt"], meta["steps"]), d["u_final"]) > 1e-3
    # limited elements hold c000 plus linear modes only: limiting twice
    # changes nothing
    u1, f1 = m.limit_minmodb(d["u0"], kw["alpha"], kw["beta"], kw["scale_bound"])
    u2, f2 = m.limit_minmodb(u1, kw["alpha"], kw["beta"], kw["scale_bound"])
    assert f1.sum() > 0
    assert rel_l2(u2, u1) <= 1e-13


def _generated(meta, uniform=False):
    """The oracle's own mesh of a fixture's case and the permutation that
    takes fixture element i to generated element perm[i]."""
    n, L = meta["n"], meta["luni"]
    if meta["mesh"] == "box":
        g = nmo.generate_mesh(nmo.MESH_BOX, n, L, uniform=uniform, xc=(np.pi,) * 3,
                              box_dout=np.pi)
    else:
        g = nmo.generate_mesh(nmo.MESH_CUBEDSPHERES7, n, L, uniform=uniform)
    return g


def _perm(pat, bbox, d):
    key = {(int(a),) + tuple(b): i for i, (a, b) in enumerate(zip(pat, bbox))}
    return np.array([key[(int(a),) + tuple(b)] for a, b in zip(d["pat"], d["bbox"])])


@pytest.mark.parametrize("case", CASES + FV_CASES)
def test_oracle_mesh_generator_matches_reference_geometry(case):
    """The oracle's own mesh generator (oracle/nmo_mesh.c) gives the
    reference's element bboxes, coordinates and dX/dx bit for bit, and its
    C face matcher the coordinate-matching neighbour table."""
    d, meta = load(case)
    pat, bbox, curvi, xyz, dXdx = _generated(meta, uniform="fv" in meta)
    perm = _perm(pat, bbox, d)
    assert len(perm) == len(pat)
    assert np.array_equal(xyz[perm], d["x"])
    assert np.array_equal(dXdx[perm], d["dXdx"])
    if "fv" not in meta:
        assert np.array_equal(nmo.match_faces_conforming(d["x"], meta["n"]),
                              nmo.match_faces(d["x"], meta["n"]))


def test_oracle_benchmark_order_level2_fixture():
    """The benchmark's mesh family and order at level 2 (448 elements of 9^3
    nodes) on the oracle's own mesh: RHS and 10 RK4 steps equal the
    reference's run on the kept elements bit for bit, and the full norms."""
    d, meta = load(BIG_CASE)
    n = meta["n"]
    pat, bbox, curvi, xyz, dXdx = _generated(meta)
    perm = _perm(pat, bbox, d)
    u0 = to_mesh_order(big_case_u0(d, meta), perm)
    om = nmo.OracleMesh(bbox, curvi, dXdx, xyz, nmo.match_faces_conforming(xyz, n), n, bc=0,
                        k=meta["k"])
    sel = d["sel"]
    r = om.rhs(u0, 0.0)[perm]
    assert np.array_equal(r[sel], d["r0_sel"])
    assert np.linalg.norm(r.ravel()) == pytest.approx(float(d["r0_norm"]), rel=1e-15)
    u = om.rk4(u0, meta["dt"], meta["steps"])[perm]
    assert np.array_equal(u[sel], d["u_final_sel"])
    assert np.linalg.norm(u.ravel()) == pytest.approx(float(d["u_final_norm"]), rel=1e-15)
