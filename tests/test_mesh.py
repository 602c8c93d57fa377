"""Host-side mesh packer (nmesh_gb300/csrc/mesh.cpp): geometry against the
reference's own coordinates/metric, face table against the oracle's
independent coordinate matcher."""
import numpy as np
import pytest

import nmesh_gb300 as ng
from helpers import (CASES, DTAUTO_CASES, FV_CASES, MIX_CASES, NC_CASES, PI, build_mesh, load,
                     perm_to_mesh)
from oracle import nmo


@pytest.mark.parametrize("case", CASES + FV_CASES + MIX_CASES + NC_CASES)
def test_geometry_bitexact(case):
    """Coordinates and metric on LGL points (DG) and on equally spaced
    points (finite-volume meshes) equal the reference's."""
    d, meta = load(case)
    m = build_mesh(meta)
    perm = perm_to_mesh(m, d)
    assert np.array_equal(m.coords()[perm], d["x"])
    assert np.array_equal(m.dXdx()[perm], d["dXdx"])
    if "fv" in meta:
        assert np.array_equal(m.fv()[perm], d["use_fv"])


def test_uniform_points_match_oracle():
    import ctypes
    for n in range(1, 20):
        x = np.zeros(n)
        assert ng.lib().nmg_uniform_points(n, x.ctypes.data_as(ctypes.c_void_p)) == 0
        assert np.array_equal(x, nmo.uniform(n))


def test_mixed_dg_fv_face_table():
    """Inner cube finite-volume, shells DG: exactly the faces between the two
    point types carry the mixed bit (64), with the orientation found from the
    corners; the element-by-element description reproduces the table."""
    m = ng.Mesh.build(ng.MESH_CUBEDSPHERES7, n=5, luni=1, cs_dc=1.0, cs_r0fac=20.0, fv=[0])
    pat, bbox = m.elements()
    fv = m.fv()
    assert np.array_equal(fv, (pat == 0).astype(np.int32))
    nb, code = m.faces()
    for e in range(m.nelem):
        for f in range(6):
            if nb[e, f] < 0:
                assert code[e, f] == 0
                continue
            assert bool(code[e, f] & 64) == (fv[e] != fv[nb[e, f]])
    assert (code & 64).any()
    m2 = ng.Mesh.from_arrays(bbox, (pat > 0).astype(np.int32), m.coords(), dXdx=m.dXdx(),
                             pat=pat, fv=fv)
    assert np.array_equal(m2.fv(), fv)
    nb2, code2 = m2.faces()
    assert np.array_equal(nb, nb2) and np.array_equal(code, code2)
    # the oracle's own matcher finds the same mixed faces and orientations
    nbo, mix = nmo.match_faces(m.coords(), 5, fv=fv)
    for e in range(m.nelem):
        for f in range(6):
            if code[e, f] & 64:
                assert (nbo[e, f] == -2).all()
                assert tuple(mix[e, f]) == (nb[e, f], code[e, f] & 7, (code[e, f] >> 3) & 7)


def _faces_from_nbnode(nbnode, n):
    """(neighbour element, face, orientation) implied by a node table."""
    npt = n ** 3
    E = nbnode.shape[0]
    out = {}
    for e in range(E):
        for f in range(6):
            t = nbnode[e, f]
            if t[0] < 0:
                continue
            out[(e, f)] = tuple(int(v) for v in t)
    return out


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("periodic", [False, True])
def test_face_table_matches_oracle_matcher(case, periodic):
    d, meta = load(case)
    if periodic and meta["mesh"] != "box":
        pytest.skip("periodic only for the box")
    m = build_mesh(meta, periodic=periodic)
    n = m.n
    nb, code = m.faces()
    ref = nmo.match_faces(m.coords(), n, period=2 * PI if periodic else None)
    npt = n ** 3
    for e in range(m.nelem):
        for f in range(6):
            if nb[e, f] < 0:
                assert (ref[e, f] < 0).all()
                continue
            f2, o = code[e, f] & 7, code[e, f] >> 3
            for b in range(n):
                for a in range(n):
                    s, fa, fb = o & 1, (o >> 1) & 1, (o >> 2) & 1
                    aa, bb = (b, a) if s else (a, b)
                    aa = n - 1 - aa if fa else aa
                    bb = n - 1 - bb if fb else bb
                    idx = nmo.face_plane_index(n, f2)[aa + n * bb]
                    assert ref[e, f, a + n * b] == nb[e, f] * npt + idx


def test_desc_roundtrip_with_explicit_node_table():
    d, meta = load("cs7_l1_n4")
    m = build_mesh(meta)
    pat, bbox = m.elements()
    xyz = m.coords()
    J = m.dXdx()
    curvi = (pat > 0).astype(np.int32)
    ref = nmo.match_faces(xyz, m.n)
    m2 = ng.Mesh.from_arrays(bbox, curvi, xyz, J, nbnode=ref, pat=pat)
    m3 = ng.Mesh.from_arrays(bbox, curvi, xyz, J, pat=pat)
    for mm in (m2, m3):
        nb2, code2 = mm.faces()
        nb1, code1 = m.faces()
        assert np.array_equal(nb1, nb2) and np.array_equal(code1, code2)


@pytest.mark.parametrize("case", NC_CASES)
def test_nonconforming_lists_match_oracle(case):
    """The packer's non-conforming face lists equal the oracle's (found
    independently from bboxes and node coordinates): the same sources per
    face node and the same positions on the source faces."""
    d, meta = load(case)
    m = build_mesh(meta)
    n, nn = m.n, m.n * m.n
    nbm, code = m.faces()
    hface, hoff, hsrc, hpos = m.hanging()
    assert len(hface) == int(((code & 128) != 0).sum()) > 0
    pat, bbox = m.elements()
    nb = nmo.match_faces(m.coords(), n)
    nb2, (off, src, pos) = nmo.match_hanging(m.coords(), n, pat, bbox, nb)
    assert (nb2[:, :, 0] == -3).sum() == len(hface)
    for h, (e, f) in enumerate(hface):
        assert nb2[e, f, 0] == -3
        for jk in range(nn):
            a0, a1 = hoff[h * nn + jk], hoff[h * nn + jk + 1]
            q = (e * 6 + f) * nn + jk
            b0, b1 = off[q], off[q + 1]
            mine = sorted(zip(map(tuple, hsrc[a0:a1]), map(tuple, hpos[a0:a1])))
            theirs = sorted(zip(map(tuple, src[b0:b1]), map(tuple, pos[b0:b1])))
            assert [s_ for s_, _ in mine] == [s_ for s_, _ in theirs]
            assert np.allclose([p_ for _, p_ in mine], [p_ for _, p_ in theirs],
                               rtol=0, atol=1e-14)
    # element names carry each element's own level: the halvings of its
    # patch's extent, and the names are the fixture's
    names = m.names()
    lo = {p_: bbox[pat == p_, 0].min() for p_ in set(pat.tolist())}
    hi = {p_: bbox[pat == p_, 1].max() for p_ in set(pat.tolist())}
    for e in range(m.nelem):
        lev = len(names[e].split("_")[1])
        ext = (hi[pat[e]] - lo[pat[e]]) / (bbox[e, 1] - bbox[e, 0])
        assert 2 ** lev == round(ext)
        if "hrefine" in meta:
            assert lev == meta["luni"] + (str(pat[e]) in meta["hrefine"].split())


def test_nonconforming_concat_keeps_lists():
    a = build_mesh(load("nc_cs7_l0_n5_h0")[1])
    b = build_mesh(load("nc_cs7_l1_n5_h02")[1])
    c = ng.Mesh.concat([a, b])
    ha, hb, hc = a.hanging(), b.hanging(), c.hanging()
    assert len(hc[0]) == len(ha[0]) + len(hb[0])
    assert np.array_equal(hc[0][len(ha[0]):, 0], hb[0][:, 0] + a.nelem)
    assert np.array_equal(hc[2][len(ha[2]):, 0], hb[2][:, 0] + a.nelem)
    assert np.array_equal(hc[3], np.concatenate([ha[3], hb[3]]))
    assert np.array_equal(np.diff(hc[1]), np.concatenate([np.diff(ha[1]), np.diff(hb[1])]))


@pytest.mark.parametrize("case", DTAUTO_CASES)
def test_auto_dt_equals_the_references(case):
    """dt = auto: the smallest corner spacing times dtfac (uniform_dtfac
    where that spacing lies on equally spaced points), bit for bit."""
    d, meta = load(case)
    assert build_mesh(meta).auto_dt() == d["dt_ref"][0]


def test_mesh_errors():
    with pytest.raises(ng.NmgError):
        ng.Mesh.build(ng.MESH_BOX, n=1)
    with pytest.raises(ng.NmgError):
        ng.Mesh.build(99, n=4)
    with pytest.raises(ng.NmgError):
        ng.Mesh.build(ng.MESH_CUBEDSPHERES7, n=4, cs_r0fac=1.0)
    # a partial neighbour table is rejected
    d, meta = load("box_l1_n5")
    m = build_mesh(meta)
    pat, bbox = m.elements()
    xyz = m.coords()
    ref = nmo.match_faces(xyz, m.n)
    e, f = np.argwhere(ref[:, :, 0] >= 0)[0]
    ref[e, f, 3] = -1
    with pytest.raises(ng.NmgError):
        ng.Mesh.from_arrays(bbox, np.zeros(len(pat), np.int32), xyz, nbnode=ref)


def test_config2_mesh_counts():
    """The cubed-sphere workload: 7 patches x 16^3 elements at n = 9."""
    m = ng.Mesh.build(ng.MESH_CUBEDSPHERES7, n=3, luni=4, cs_dc=1.0, cs_r0fac=20.0)
    assert m.nelem == 7 * 16 ** 3
    nb, _ = m.faces()
    assert (nb < 0).sum() == 6 * 16 * 16   # only the outer sphere is outer
    r = np.linalg.norm(m.coords(), axis=1)
    assert abs(r.max() - 20.0) < 1e-12 and abs(r.min() - 0.0) < 1e-12 or r.min() >= 0


@pytest.mark.parametrize("luni", [0, 1])
def test_periodic_self_neighbour_face_table(luni):
    """A periodic box with one element per direction is its own neighbour on
    every face; the in-face node map must be the identity shifted by a
    period, not a position collision of wrapped corners."""
    m = ng.Mesh.build(ng.MESH_BOX, n=4, luni=luni, xc=(PI, PI, PI), box_dout=PI,
                      periodic=True)
    nb, code = m.faces()
    assert (nb >= 0).all()
    ref = nmo.match_faces(m.coords(), 4, period=2 * PI)
    npt = 64
    for e in range(m.nelem):
        for f in range(6):
            f2, o = code[e, f] & 7, code[e, f] >> 3
            assert f2 == (f ^ 1) and o == 0
            idx = nmo.face_plane_index(4, f2)
            assert np.array_equal(ref[e, f], nb[e, f] * npt + idx)


@pytest.mark.parametrize("case", NC_CASES)
def test_described_mesh_finds_nonconforming_faces(case):
    """A mesh given element by element (what the nmesh adapter packs from a
    tMesh: patch, bbox, x, dXdx) gets each element's level from its bbox
    and the same face table and non-conforming lists as the generated mesh."""
    d, meta = load(case)
    m = build_mesh(meta)
    pat, bbox = m.elements()
    curvi = (pat > 0).astype(np.int32) if meta["mesh"] == "cs7" else np.zeros(len(pat), np.int32)
    md = ng.Mesh.from_arrays(bbox, curvi, m.coords(), m.dXdx(), pat=pat)
    for a, b in zip(m.faces() + m.hanging(), md.faces() + md.hanging()):
        assert np.array_equal(a, b)


def test_level_jump_of_two_rejected():
    """Two nested spheres of radius 2 and 4 on a level-1 cubed-sphere mesh
    put level-3 cube elements against level-1 shells: not built, and the
    build says so instead of leaving those faces outer."""
    with pytest.raises(ng.NmgError, match="level jump"):
        ng.Mesh.build(ng.MESH_CUBEDSPHERES7, n=4, luni=1, cs_dc=1.0, cs_r0fac=20.0,
                      sphere_levels=2, sphere_radius=2)


def test_patch_parts_cover_the_mesh():
    """Meshes of patch subsets (patch_mask) hold exactly the elements of
    those patches with the whole mesh's geometry; the faces between parts
    become outer faces of each part."""
    full = ng.Mesh.build(ng.MESH_CUBEDSPHERES7, n=4, luni=1, cs_dc=1.0, cs_r0fac=20.0)
    a = ng.Mesh.build(ng.MESH_CUBEDSPHERES7, n=4, luni=1, cs_dc=1.0, cs_r0fac=20.0,
                      patches=[0, 2, 4])
    b = ng.Mesh.build(ng.MESH_CUBEDSPHERES7, n=4, luni=1, cs_dc=1.0, cs_r0fac=20.0,
                      patches=[1, 3, 5, 6])
    assert a.nelem + b.nelem == full.nelem
    P, B = full.elements()
    key = {(int(p),) + tuple(bb): i for i, (p, bb) in enumerate(zip(P, B))}
    outer_full = (full.faces()[0] < 0).sum()
    outer_parts = 0
    for part, pats in ((a, {0, 2, 4}), (b, {1, 3, 5, 6})):
        pp, bb = part.elements()
        assert set(int(p) for p in pp) == pats
        idx = np.array([key[(int(p),) + tuple(x)] for p, x in zip(pp, bb)])
        assert np.array_equal(part.coords(), full.coords()[idx])
        assert np.array_equal(part.dXdx(), full.dXdx()[idx])
        outer_parts += (part.faces()[0] < 0).sum()
    assert outer_parts > outer_full
    with pytest.raises(ng.NmgError):
        ng.Mesh.build(ng.MESH_BOX, n=4, luni=1, xc=(0.0,) * 3, box_dout=1.0, patches=[3])
