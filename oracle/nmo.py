"""ORACLE (test infrastructure only): ctypes binding of oracle/nmo.c, the
plain-C restatement of the reference's scalarwave1 DG right-hand side and
RK4 step, plus the coordinate-matching face connectivity it consumes.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
this module; the product path never imports it.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libnmo.so")
# the restated RHS / steps / GRHD pieces, and the oracle's own mesh generator
SOURCES = ["nmo.c", "nmo_mesh.c", "nmo_grhd.c"]


def build(verbose=False):
    """Compile oracle/nmo.c into oracle/_build/libnmo.so (gcc, OpenMP,
    -ffp-contract=off so that x86-64 and aarch64 results agree bitwise)."""
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(HERE, f) for f in SOURCES]
    if os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(s) for s in srcs):
        return LIB
    cmd = ["gcc", "-O2", "-std=gnu99", "-fopenmp", "-ffp-contract=off",
           "-fPIC", "-shared", "-o", LIB + ".tmp"] + srcs + ["-lm"]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


class _Mesh(ctypes.Structure):
    _fields_ = [("nelem", ctypes.c_int), ("n", ctypes.c_int),
                ("bbox", ctypes.c_void_p), ("curvi", ctypes.c_void_p),
                ("dXdx", ctypes.c_void_p), ("xyz", ctypes.c_void_p),
                ("nbnode", ctypes.c_void_p), ("bc", ctypes.c_int),
                ("k", ctypes.c_double * 3), ("fv", ctypes.c_void_p),
                ("fv_rec", ctypes.c_int), ("fv_extrap", ctypes.c_int),
                ("fv_w3ratio", ctypes.c_double), ("mixface", ctypes.c_void_p),
                ("numflux", ctypes.c_int), ("hang_off", ctypes.c_void_p),
                ("hang_src", ctypes.c_void_p), ("hang_pos", ctypes.c_void_p),
                ("surf_interp", ctypes.c_int), ("dXdxm", ctypes.c_void_p),
                ("ext", ctypes.c_void_p)]

# reconstruction modes (reference par fv_rec) and div(f) extrapolation
# modes (par fv_divf_extrap) understood by the oracle
FV_REC = {"1": 0, "WENOm3_2": 1, "WENOm5_2": 2, "WENOmZ_2": 3}
FV_EXTRAP = {"no": 0, "dnfn_extrap1": 1}


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        for name in ("nmo_rhs", "nmo_rk4"):
            getattr(_lib, name).restype = ctypes.c_int
    return _lib


def persson(n, u, u_scale=-1.0):
    """Persson's modal indicator of one field u[n^3] on LGL points
    (reference evolve_Persson_array_indicator, trouble.c:505)."""
    f = lib().nmo_persson
    f.restype = ctypes.c_double
    u = np.ascontiguousarray(u, np.float64)
    return f(ctypes.c_int(n), u.ctypes.data_as(ctypes.c_void_p), ctypes.c_double(u_scale))


def uniform(n):
    """Equally spaced points on [-1,1] (reference Legendre.c:626)."""
    x = np.zeros(n)
    lib().nmo_uniform(ctypes.c_int(n), x.ctypes.data_as(ctypes.c_void_p))
    return x


def lgl(n):
    """LGL nodes and weights on [-1,1] (reference Legendre.c:149)."""
    x = np.zeros(n)
    w = np.zeros(n)
    lib().nmo_lgl(ctypes.c_int(n), x.ctypes.data_as(ctypes.c_void_p),
                  w.ctypes.data_as(ctypes.c_void_p))
    return x, w


def diffmat(n):
    """D[i, j] = l_j'(x_i) at the LGL nodes (reference Lagrange.c:126)."""
    x, _ = lgl(n)
    D = np.zeros((n, n))
    lib().nmo_diffmat(ctypes.c_int(n), x.ctypes.data_as(ctypes.c_void_p),
                      D.ctypes.data_as(ctypes.c_void_p))
    return D


MESH_BOX, MESH_SHELL6, MESH_CUBEDSPHERES7 = 1, 6, 7


def generate_mesh(kind, n, luni, uniform=False, xc=(0.0, 0.0, 0.0), box_dout=1.0, cs_dc=1.0,
                  cs_r0fac=20.0, r_in=2.0, r_out=20.0, ndiv=0):
    """The oracle's own uniform mesh (oracle/nmo_mesh.c): a box
    (MESH_BOX: centre xc, half edge box_dout), the 7-patch cubed spheres
    (MESH_CUBEDSPHERES7: cube of half edge cs_dc, outer radius cs_r0fac cs_dc)
    or 6 cubed-sphere shells between radii r_in and r_out (MESH_SHELL6), at
    level luni (or, ndiv > 0, ndiv^3 equal elements per patch) with n LGL
    (or equally spaced) points per direction.
    Returns (pat [E], bbox [E,6], curvi [E], xyz [E,3,np], dXdx [E,9,np])."""
    f = lib().nmo_mesh_count
    f.restype = ctypes.c_int64
    E = int(f(ctypes.c_int(kind), ctypes.c_int(luni)))
    if E < 0:
        raise ValueError("unknown mesh kind or level")
    if ndiv > 0:
        E = E // 8 ** luni * ndiv ** 3
    prm = {MESH_BOX: (xc[0], xc[1], xc[2], box_dout),
           MESH_CUBEDSPHERES7: (cs_dc, cs_r0fac, 0.0, 0.0),
           MESH_SHELL6: (r_in, r_out, 0.0, 0.0)}[kind]
    npt = n ** 3
    pat = np.zeros(E, np.int32)
    bbox = np.zeros((E, 6))
    curvi = np.zeros(E, np.int32)
    xyz = np.zeros((E, 3, npt))
    dXdx = np.zeros((E, 9, npt))
    rc = lib().nmo_mesh_generate(ctypes.c_int(kind), ctypes.c_int(n), ctypes.c_int(luni),
                                 ctypes.c_int(ndiv), (ctypes.c_double * 4)(*prm), ctypes.c_int(int(uniform)),
                                 pat.ctypes.data_as(ctypes.c_void_p),
                                 bbox.ctypes.data_as(ctypes.c_void_p),
                                 curvi.ctypes.data_as(ctypes.c_void_p),
                                 xyz.ctypes.data_as(ctypes.c_void_p),
                                 dXdx.ctypes.data_as(ctypes.c_void_p))
    if rc:
        raise RuntimeError("nmo_mesh_generate failed")
    return pat, bbox, curvi, xyz, dXdx


def match_faces_conforming(xyz, n, period=None):
    """Neighbour table nbnode[E, 6, n*n] of a conforming mesh, as
    match_faces, computed in C (oracle/nmo_mesh.c: nmo_match_faces)."""
    xyz = np.ascontiguousarray(xyz, np.float64)
    E = xyz.shape[0]
    nb = np.empty((E, 6, n * n), np.int64)
    per = None if period is None else (ctypes.c_double * 3)(*([float(period)] * 3))
    rc = lib().nmo_match_faces(ctypes.c_int64(E), ctypes.c_int(n),
                               xyz.ctypes.data_as(ctypes.c_void_p), per,
                               nb.ctypes.data_as(ctypes.c_void_p), None, None)
    if rc:
        raise ValueError("nmo_match_faces: faces do not match conformingly")
    return nb


def face_table(xyz, n, period=None):
    """Face table of a conforming mesh: nb[E, 6] neighbour element (-1
    outer) and code[E, 6] = neighbour face | orientation << 3."""
    xyz = np.ascontiguousarray(xyz, np.float64)
    E = xyz.shape[0]
    nbn = np.empty((E, 6, n * n), np.int64)
    nb = np.empty((E, 6), np.int32)
    code = np.empty((E, 6), np.int32)
    per = None if period is None else (ctypes.c_double * 3)(*([float(period)] * 3))
    rc = lib().nmo_match_faces(ctypes.c_int64(E), ctypes.c_int(n),
                               xyz.ctypes.data_as(ctypes.c_void_p), per,
                               nbn.ctypes.data_as(ctypes.c_void_p),
                               nb.ctypes.data_as(ctypes.c_void_p),
                               code.ctypes.data_as(ctypes.c_void_p))
    if rc:
        raise ValueError("nmo_match_faces: faces do not match conformingly")
    return nb, code


def face_plane_index(n, f):
    """Volume indices (i + n*(j + n*k)) of the face-f plane, ordered by the
    in-plane index JK = a + n*b (reference Ind_n_norm / forplaneN)."""
    d, p = f // 2, (f % 2) * (n - 1)
    a, b = np.meshgrid(np.arange(n), np.arange(n), indexing="xy")
    a = a.ravel()
    b = b.ravel()
    if d == 0:
        i, j, k = np.full_like(a, p), a, b
    elif d == 1:
        i, j, k = a, np.full_like(a, p), b
    else:
        i, j, k = a, b, np.full_like(a, p)
    return i + n * (j + n * k)


def match_faces(xyz, n, period=None, tol=1e-9, fv=None):
    """Neighbour table for the oracle by matching face-node coordinates.

    xyz: [E, 3, np].  Two element faces are neighbours when their four
    corners coincide (compared modulo `period` on every axis when given,
    which makes a box periodic).  Returns nbnode[E, 6, n*n] with
    e'*np + ijk' of the coincident node of the neighbour, or -1 on outer
    faces (the reference copies coincident neighbour points,
    src/main/amr/surface.c:799-900).  With per-element point types `fv`
    (1: equally spaced points), a face whose neighbour has the other point
    type is marked -2 and (nbnode, mixface) is returned, mixface[E, 6, 3] =
    (neighbour element, neighbour face, orientation o) where in-plane node
    (a, b) lies at the neighbour's in-plane position (a', b') = (s ? b : a,
    s ? a : b), reversed per axis by bits 1 and 2 of o (s = bit 0)."""
    E = xyz.shape[0]
    npt = n ** 3
    planes = [face_plane_index(n, f) for f in range(6)]
    corners = [0, n - 1, n * (n - 1), n * n - 1]   # (a, b) = (0,0),(n-1,0),(0,n-1),(n-1,n-1)

    def wrap(p):
        q = np.array(p, dtype=float)
        if period is not None:
            q = np.mod(q, period)
            q = np.where(np.abs(q - period) < 1e-7, 0.0, q)
        return q

    def pkey(q):
        return tuple(np.round(q / tol).astype(np.int64))

    def orient(o, a, b):
        aa, bb = (b, a) if o & 1 else (a, b)
        return (n - 1 - aa if o & 2 else aa), (n - 1 - bb if o & 4 else bb)

    faces = {}
    for e in range(E):
        for f in range(6):
            raw = xyz[e][:, planes[f]].T              # [n*n, 3]
            # a face never straddles a period: average the corners, then wrap
            cen = raw[corners].mean(axis=0)
            faces.setdefault(pkey(wrap(cen)), []).append((e, f, raw, cen))
    nb = np.full((E, 6, n * n), -1, np.int64)
    mixface = np.zeros((E, 6, 3), np.int32)
    mixed = False
    for fkey, lst in faces.items():
        if len(lst) == 1:
            continue
        if len(lst) != 2:
            raise ValueError("non-conforming face match")
        for (e, f, P, c1), (e2, f2, P2, c2) in (lst, lst[::-1]):
            # whole periods between the two faces (zero without a period)
            shift = np.zeros(3)
            if period is not None:
                shift = np.round((c2 - c1) / period) * period
            if fv is not None and bool(fv[e]) != bool(fv[e2]):
                found = None
                for o in range(8):
                    ok = True
                    for a, b in ((0, 0), (n - 1, 0), (0, n - 1), (n - 1, n - 1)):
                        aa, bb = orient(o, a, b)
                        if pkey(P[a + n * b]) != pkey(P2[aa + n * bb] - shift):
                            ok = False
                    if ok:
                        found = o
                        break
                if found is None:
                    raise ValueError("mixed face: corners do not match")
                nb[e, f, :] = -2
                mixface[e, f] = (e2, f2, found)
                mixed = True
                continue
            where = {pkey(q - shift): planes[f2][i] for i, q in enumerate(P2)}
            for jk in range(n * n):
                nb[e, f, jk] = e2 * npt + where[pkey(P[jk])]
    if fv is not None:
        return nb, (mixface if mixed else None)
    return nb


def match_hanging(xyz, n, pat, bbox, nbnode, tol=1e-9):
    """Non-conforming faces of a mesh whose elements sit at different levels
    (the reference's amr_hrefine_p and amr_hrefine_sphere_levels).

    Faces left outer (-1) by match_faces are tested: a face that lies on its
    parent element's face is the quarter of a coarser element's face when
    the parent face's corners (carried by the four siblings on it) are that
    face's corners.  Elements are located by their bbox within the patch
    (level and integer position), the orientation between the parent face
    and the coarse face from the corners.  Each node of a fine face takes
    the coarse face at its position; each node of a coarse face averages
    the fine faces that contain it (set_ajsurf_vl,
    src/main/amr/surface.c:1160-1340).  Returns (nbnode with -3 on those
    faces, (hang_off, hang_src, hang_pos)) or (nbnode, None)."""
    E = xyz.shape[0]
    nn = n * n
    planes = [face_plane_index(n, f) for f in range(6)]
    corners = [0, n - 1, n * (n - 1), n * n - 1]
    x = lgl(n)[0]
    nbnode = np.array(nbnode, copy=True)

    def pkey(q):
        return tuple(np.round(np.asarray(q) / tol).astype(np.int64))

    # level and integer position of each element in its patch
    ext = {}
    for e in range(E):
        lo, hi = ext.get(int(pat[e]), (bbox[e, 0::2].copy(), bbox[e, 1::2].copy()))
        ext[int(pat[e])] = (np.minimum(lo, bbox[e, 0::2]), np.maximum(hi, bbox[e, 1::2]))
    lev = np.zeros(E, np.int64)
    pos = np.zeros((E, 3), np.int64)
    where = {}
    for e in range(E):
        lo, hi = ext[int(pat[e])]
        h = bbox[e, 1::2] - bbox[e, 0::2]
        lev[e] = int(round(np.log2((hi[0] - lo[0]) / h[0])))
        pos[e] = np.round((bbox[e, 0::2] - lo) / h).astype(np.int64)
        where[(int(pat[e]), int(lev[e])) + tuple(pos[e])] = e
    # centre keys of the faces still outer
    free = {}
    for e in range(E):
        for f in range(6):
            if nbnode[e, f, 0] == -1:
                free.setdefault(pkey(xyz[e][:, planes[f][corners]].mean(axis=1)), []).append((e, f))

    def orient(o, a, b):
        aa, bb = (b, a) if o & 1 else (a, b)
        return (n - 1 - aa if o & 2 else aa), (n - 1 - bb if o & 4 else bb)

    pairs = []   # (fine e, f, coarse e2, f2, A, B, o)
    for e in range(E):
        for f in range(6):
            if nbnode[e, f, 0] != -1 or lev[e] < 1:
                continue
            d, s = f // 2, f % 2
            d1, d2 = (1, 2) if d == 0 else ((0, 2) if d == 1 else (0, 1))
            if pos[e, d] % 2 != s:
                continue
            cpts = []
            for t in range(4):
                q = pos[e].copy()
                q[d1] = (q[d1] & ~1) | (t & 1)
                q[d2] = (q[d2] & ~1) | (t >> 1)
                # the sibling, or (refined further) its descendant at the corner
                lv = int(lev[e])
                bits = np.zeros(3, np.int64)
                bits[d], bits[d1], bits[d2] = s, t & 1, t >> 1
                while (int(pat[e]), lv) + tuple(q) not in where:
                    q, lv = 2 * q + bits, lv + 1
                sib = where[(int(pat[e]), lv) + tuple(q)]
                cpts.append(xyz[sib][:, planes[f][corners[t]]])
            cand = [g for g in free.get(pkey(np.mean(cpts, axis=0)), [])
                    if lev[g[0]] == lev[e] - 1]
            if not cand:
                continue
            e2, f2 = cand[0]
            found = None
            for o in range(8):
                ok = True
                for t in range(4):
                    a2, b2 = orient(o, (t & 1) * (n - 1), (t >> 1) * (n - 1))
                    ok = ok and pkey(cpts[t]) == pkey(xyz[e2][:, planes[f2][a2 + n * b2]])
                if ok:
                    found = o
                    break
            if found is None:
                raise ValueError("non-conforming face: corners do not match")
            pairs.append((e, f, e2, f2, int(pos[e, d1] & 1), int(pos[e, d2] & 1), found))
    if not pairs:
        return nbnode, None
    lists = {}
    for (e, f, e2, f2, A, B, o) in pairs:
        sw, fa, fb = o & 1, (o >> 1) & 1, (o >> 2) & 1
        L = []
        for b in range(n):
            for a in range(n):
                pa, pb = (x[a] + (2 * A - 1)) * 0.5, (x[b] + (2 * B - 1)) * 0.5
                u, v = (pb, pa) if sw else (pa, pb)
                L.append([(e2, f2, -u if fa else u, -v if fb else v)])
        lists[(e, f)] = L
    coarse = {}
    for P in pairs:
        coarse.setdefault((P[2], P[3]), []).append(P)
    for (e2, f2), ps in coarse.items():
        ps = sorted(ps, key=lambda P: P[4] + 2 * P[5])
        o = ps[0][6]
        sw, fa, fb = o & 1, (o >> 1) & 1, (o >> 2) & 1
        L = []
        for b2 in range(n):
            for a2 in range(n):
                u, v = (-x[a2] if fa else x[a2]), (-x[b2] if fb else x[b2])
                pa, pb = (v, u) if sw else (u, v)
                lst = []
                for (e, f, _, _, A, B, _) in ps:
                    ina = pa >= -1e-10 if A else pa <= 1e-10
                    inb = pb >= -1e-10 if B else pb <= 1e-10
                    if ina and inb:
                        lst.append((e, f, 2 * pa - (2 * A - 1), 2 * pb - (2 * B - 1)))
                L.append(lst)
        lists[(e2, f2)] = L
    off = np.zeros(E * 6 * nn + 1, np.int32)
    src, hp = [], []
    cnt = np.zeros(E * 6 * nn, np.int32)
    for (e, f), L in lists.items():
        nbnode[e, f, :] = -3
        for jk, lst in enumerate(L):
            cnt[(e * 6 + f) * nn + jk] = len(lst)
    off[1:] = np.cumsum(cnt)
    src = np.zeros((int(off[-1]), 2), np.int32)
    hp = np.zeros((int(off[-1]), 2))
    for (e, f), L in lists.items():
        for jk, lst in enumerate(L):
            q = off[(e * 6 + f) * nn + jk]
            for i, (es, fs, u, v) in enumerate(lst):
                src[q + i] = (es, fs)
                hp[q + i] = (u, v)
    return nbnode, (off, src, hp)


class OracleMesh:
    """Arrays describing a mesh for the oracle, kept alive with the struct."""

    def __init__(self, bbox, curvi, dXdx, xyz, nbnode, n, bc=0,
                 k=(1.0, 1.0, 1.0), fv=None, fv_rec="WENOm5_2",
                 fv_extrap="dnfn_extrap1", fv_w3ratio=2.0, mixface=None, numflux="LLF",
                 hang=None, fv_surface_interp="linear", dXdxm=None):
        """fv: per-element finite-volume flags (None: all DG); fv_rec and
        fv_extrap name the reference's fv_rec / fv_divf_extrap modes;
        mixface: faces between the two point types (see match_faces);
        numflux: "LLF" or "upwind" (the reference's scalarwave1_numflux);
        hang: non-conforming face lists (see match_hanging)."""
        self.n = int(n)
        self.bbox = np.ascontiguousarray(bbox, np.float64)
        self.curvi = np.ascontiguousarray(curvi, np.int32)
        self.dXdx = np.ascontiguousarray(dXdx, np.float64)
        self.xyz = np.ascontiguousarray(xyz, np.float64)
        self.nbnode = np.ascontiguousarray(nbnode, np.int64)
        self.nelem = self.bbox.shape[0]
        self.fv = None if fv is None else np.ascontiguousarray(fv, np.int32)
        self.mixface = None if mixface is None else np.ascontiguousarray(mixface, np.int32)
        self.hang = None if hang is None else tuple(np.ascontiguousarray(a) for a in hang)
        self.dXdxm = None if dXdxm is None else np.ascontiguousarray(dXdxm, np.float64)
        self.s = _Mesh(self.nelem, self.n, self.bbox.ctypes.data,
                       self.curvi.ctypes.data, self.dXdx.ctypes.data,
                       self.xyz.ctypes.data, self.nbnode.ctypes.data, int(bc),
                       (ctypes.c_double * 3)(*k),
                       None if self.fv is None else self.fv.ctypes.data,
                       FV_REC[fv_rec], FV_EXTRAP[fv_extrap], float(fv_w3ratio),
                       None if self.mixface is None else self.mixface.ctypes.data,
                       1 if numflux == "upwind" else 0,
                       *((None,) * 3 if self.hang is None else
                         tuple(a.ctypes.data for a in self.hang)),
                       {"linear": 0, "parabolic": 1}[fv_surface_interp],
                       None if self.dXdxm is None else self.dXdxm.ctypes.data, None)
        self.ext = None

    def set_ext(self, ext):
        """Exterior states [E, 6, n*n, 5] of the face nodes marked -4."""
        self.ext = np.ascontiguousarray(ext, np.float64)
        self.s.ext = self.ext.ctypes.data

    def rhs(self, w, t=0.0):
        w = np.ascontiguousarray(w, np.float64)
        r = np.zeros_like(w)
        rc = lib().nmo_rhs(ctypes.byref(self.s), ctypes.c_double(t),
                           w.ctypes.data_as(ctypes.c_void_p),
                           r.ctypes.data_as(ctypes.c_void_p))
        if rc:
            raise RuntimeError(f"nmo_rhs failed ({rc})")
        return r

    def trouble(self, u, u_p, deltafac=1.0, delta0=1e-4, epsilon=1e-3, persson_max=1e300,
                uscale=-1.0):
        """Trouble flags [E] (DG troubled 1 / fine 0, FV troubled 0 / fine -1)
        and Persson indicators [E, 5] of state u against the previous u_p."""
        u = np.ascontiguousarray(u, np.float64)
        u_p = np.ascontiguousarray(u_p, np.float64)
        fl = np.zeros(self.nelem, np.int32)
        pe = np.zeros((self.nelem, 5))
        rc = lib().nmo_trouble(ctypes.byref(self.s), u.ctypes.data_as(ctypes.c_void_p),
                               u_p.ctypes.data_as(ctypes.c_void_p), ctypes.c_double(deltafac),
                               ctypes.c_double(delta0), ctypes.c_double(epsilon),
                               ctypes.c_double(persson_max), ctypes.c_double(uscale),
                               fl.ctypes.data_as(ctypes.c_void_p),
                               pe.ctypes.data_as(ctypes.c_void_p))
        if rc:
            raise RuntimeError(f"nmo_trouble failed ({rc})")
        return fl, pe

    def evolve(self, u, dt, nsteps, t=0.0, method="RK4"):
        """nsteps steps of the reference's evolve_method RK4, Euler or sspRK3."""
        u = np.array(u, np.float64, copy=True, order="C")
        rc = lib().nmo_evolve(ctypes.byref(self.s), ctypes.c_int({"RK4": 0, "Euler": 1,
                                                                   "sspRK3": 2}[method]),
                              ctypes.c_double(t), ctypes.c_double(dt), ctypes.c_int(nsteps),
                              u.ctypes.data_as(ctypes.c_void_p))
        if rc:
            raise RuntimeError(f"nmo_evolve failed ({rc})")
        return u

    def limit_mrs(self, u, alpha=5.0):
        """The reference's MRS limiter of every element (limiter_MRS);
        returns (limited u, per-element flag theta < 1)."""
        u = np.array(u, np.float64, copy=True, order="C")
        flags = np.zeros(self.s.nelem, np.int32)
        rc = lib().nmo_limiter_mrs(ctypes.byref(self.s), u.ctypes.data_as(ctypes.c_void_p),
                                   ctypes.c_double(alpha), flags.ctypes.data_as(ctypes.c_void_p))
        if rc:
            raise RuntimeError(f"nmo_limiter_mrs failed ({rc})")
        return u, flags

    def limit_minmodb(self, u, alpha=5.0, beta=0.5, scale_bound=False):
        """The reference's minmodB limiter of every element (limiter_minmodB
        with limiter_alpha, limiter_beta, limiter_scaleBound); returns
        (limited u, per-element flag: some field limited)."""
        u = np.array(u, np.float64, copy=True, order="C")
        flags = np.zeros(self.s.nelem, np.int32)
        rc = lib().nmo_limiter_minmodb(ctypes.byref(self.s), u.ctypes.data_as(ctypes.c_void_p),
                                       ctypes.c_double(alpha), ctypes.c_double(beta),
                                       ctypes.c_int(int(bool(scale_bound))),
                                       flags.ctypes.data_as(ctypes.c_void_p))
        if rc:
            raise RuntimeError(f"nmo_limiter_minmodb failed ({rc})")
        return u, flags

    def limit(self, u, kind="MRS", alpha=5.0, beta=0.5, scale_bound=False):
        """scalarwave1_limiter kind ("MRS" or "minmodB") on every element."""
        if kind == "MRS":
            return self.limit_mrs(u, alpha)
        return self.limit_minmodb(u, alpha, beta, scale_bound)

    def rk4_limited(self, u, dt, nsteps, alpha=5.0, t=0.0, kind="MRS", beta=0.5,
                    scale_bound=False, flags=False):
        """RK4 steps as nmo_rk4 takes them, with the limiter (MRS or
        minmodB) on w before every later stage and on the new u
        (evolve_RK4_mesh with scalarwave1_limiter set,
        src/main/evolve/RungeKutta.c:19-82).  flags: also return the
        per-element flags of the last limiter call."""
        u = np.array(u, np.float64, copy=True)
        c = (dt / 6., dt / 3., dt / 3., dt / 6.)
        a = (dt / 2., dt / 2., dt)
        te = np.longdouble(0.)
        for _ in range(nsteps):
            ts0 = float(np.longdouble(t) + te)
            ts = (ts0, ts0 + 0.5 * dt, ts0 + 0.5 * dt, ts0 + dt)
            u_p = u.copy()
            w = u.copy()
            for s in range(4):
                r = self.rhs(w, ts[s])
                u = u + c[s] * r
                if s < 3:
                    w = 1. * u_p + a[s] * r
                    w = self.limit(w, kind, alpha, beta, scale_bound)[0]
            u, last = self.limit(u, kind, alpha, beta, scale_bound)
            te += np.longdouble(dt)
        return (u, last) if flags else u

    def filter(self, u, alp=36.0, s=32.0, dn=0, jpow=1, filter_fv=True):
        """The reference's exponential filter of every element (evolve_filter_all)."""
        u = np.array(u, np.float64, copy=True, order="C")
        rc = lib().nmo_filter(ctypes.byref(self.s), u.ctypes.data_as(ctypes.c_void_p),
                              ctypes.c_double(alp), ctypes.c_double(s), ctypes.c_int(dn),
                              ctypes.c_int(jpow), ctypes.c_int(int(bool(filter_fv))))
        if rc:
            raise RuntimeError(f"nmo_filter failed ({rc})")
        return u

    def rk4(self, u, dt, nsteps, t=0.0):
        u = np.array(u, np.float64, copy=True, order="C")
        rc = lib().nmo_rk4(ctypes.byref(self.s), ctypes.c_double(t),
                           ctypes.c_double(dt), ctypes.c_int(nsteps),
                           u.ctypes.data_as(ctypes.c_void_p))
        if rc:
            raise RuntimeError(f"nmo_rk4 failed ({rc})")
        return u


# ---- GRHD (restated; the root finder follows the reference's newton1d_brak)
class _Grhd(ctypes.Structure):
    _fields_ = [("gamma", ctypes.c_double), ("rho_atm", ctypes.c_double),
                ("p_atm", ctypes.c_double), ("tol", ctypes.c_double), ("maxits", ctypes.c_int)]


FDF = ctypes.CFUNCTYPE(None, ctypes.c_double, ctypes.c_void_p,
                       ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double))


def newton1d_brak(fdf, x0, x1, x2, maxits=100, xacc=1e-14, lib_=None):
    """Restated newton1d_brak (or, with lib_, the same-signature function of
    another library such as the reference's own): returns (rc, root)."""
    L = lib_ or lib()
    fn = L.nmo_newton1d_brak if lib_ is None else L.newton1d_brak
    fn.restype = ctypes.c_int
    x = ctypes.c_double(x0)
    cb = FDF(lambda xx, par, f, df: fdf(xx, f, df))
    if lib_ is None:
        rc = fn(ctypes.byref(x), cb, ctypes.c_double(x1), ctypes.c_double(x2), None,
                ctypes.c_int(maxits), ctypes.c_double(xacc))
    else:   # the reference's signature has a trailing print flag
        rc = fn(ctypes.byref(x), cb, ctypes.c_double(x1), ctypes.c_double(x2), None,
                ctypes.c_int(maxits), ctypes.c_double(xacc), ctypes.c_int(0))
    return rc, x.value


def grhd_prim2con(prim, psi=None, gamma=2.0, rho_atm=1e-12, p_atm=1e-14, tol=1e-15, maxits=100):
    prim = np.ascontiguousarray(prim, np.float64)
    npts = prim.shape[1]
    cons = np.zeros_like(prim)
    g = _Grhd(gamma, rho_atm, p_atm, tol, maxits)
    ps = None if psi is None else np.ascontiguousarray(psi, np.float64)
    lib().nmo_grhd_prim2con(ctypes.byref(g), ctypes.c_int64(npts),
                            None if ps is None else ps.ctypes.data_as(ctypes.c_void_p),
                            prim.ctypes.data_as(ctypes.c_void_p),
                            cons.ctypes.data_as(ctypes.c_void_p))
    return cons


def grhd_con2prim(cons, prim_guess, psi=None, gamma=2.0, rho_atm=1e-12, p_atm=1e-14,
                  tol=1e-15, maxits=100):
    """Returns (prim, cons after atmosphere resets, status)."""
    cons = np.array(cons, np.float64, copy=True, order="C")
    prim = np.array(prim_guess, np.float64, copy=True, order="C")
    npts = cons.shape[1]
    st = np.zeros(npts, np.int32)
    g = _Grhd(gamma, rho_atm, p_atm, tol, maxits)
    ps = None if psi is None else np.ascontiguousarray(psi, np.float64)
    lib().nmo_grhd_con2prim(ctypes.byref(g), ctypes.c_int64(npts),
                            None if ps is None else ps.ctypes.data_as(ctypes.c_void_p),
                            cons.ctypes.data_as(ctypes.c_void_p),
                            prim.ctypes.data_as(ctypes.c_void_p),
                            st.ctypes.data_as(ctypes.c_void_p))
    return prim, cons, st


def grhd_fluxes(prim, d, alpha=None, psi=None, gamma=2.0):
    prim = np.ascontiguousarray(prim, np.float64)
    npts = prim.shape[1]
    flux = np.zeros_like(prim)
    lam = np.zeros((2, npts))
    g = _Grhd(gamma, 1e-12, 1e-14, 1e-15, 100)
    a = None if alpha is None else np.ascontiguousarray(alpha, np.float64)
    ps = None if psi is None else np.ascontiguousarray(psi, np.float64)
    lib().nmo_grhd_fluxes(ctypes.byref(g), ctypes.c_int64(npts), ctypes.c_int(d),
                          None if a is None else a.ctypes.data_as(ctypes.c_void_p),
                          None if ps is None else ps.ctypes.data_as(ctypes.c_void_p),
                          prim.ctypes.data_as(ctypes.c_void_p),
                          flux.ctypes.data_as(ctypes.c_void_p),
                          lam.ctypes.data_as(ctypes.c_void_p))
    return flux, lam


def grhd_sources(prim, alpha, psi, dalpha, dpsi, gamma=2.0):
    prim = np.ascontiguousarray(prim, np.float64)
    npts = prim.shape[1]
    src = np.zeros_like(prim)
    g = _Grhd(gamma, 1e-12, 1e-14, 1e-15, 100)
    arrs = [np.ascontiguousarray(x, np.float64) for x in (alpha, psi, dalpha, dpsi)]
    lib().nmo_grhd_sources(ctypes.byref(g), ctypes.c_int64(npts),
                           *[x.ctypes.data_as(ctypes.c_void_p) for x in arrs],
                           prim.ctypes.data_as(ctypes.c_void_p),
                           src.ctypes.data_as(ctypes.c_void_p))
    return src


class _GrMesh(ctypes.Structure):
    _fields_ = [("nelem", ctypes.c_int), ("n", ctypes.c_int), ("nf", ctypes.c_int),
                ("mesh_type", ctypes.c_int), ("prm", ctypes.c_double * 4),
                ("pat", ctypes.c_void_p), ("bbox", ctypes.c_void_p), ("xyz", ctypes.c_void_p),
                ("dXdx", ctypes.c_void_p), ("nb", ctypes.c_void_p), ("code", ctypes.c_void_p),
                ("fv", ctypes.c_void_p), ("g", _Grhd), ("mass", ctypes.c_double),
                ("rec", ctypes.c_int)]


class GrhdOracle:
    """The GRHD Cowling evolution restated in C (oracle/nmo_grhd.c) on the
    oracle's own cubed-shell mesh (oracle/nmo_mesh.c): six CubedShell
    patches between r_in and r_out, ndiv^3 elements each, n LGL points per
    direction on DG elements and nf equally spaced points on the
    finite-volume elements fv[e] = 1.

    States are kept per point type for every element, [E, 5, n^3] and
    [E, 5, nf^3]; only the DG rows of DG elements and the FV rows of FV
    elements are used.  prim_* hold the root finder's starting guesses."""

    def __init__(self, n, nf, ndiv, r_in=2.0, r_out=20.0, fv=None, mass=1.0, gamma=2.0,
                 rho_atm=1e-10, p_atm=1e-16, tol=1e-15, maxits=100, rec="WENOm5_2"):
        self.n, self.nf = int(n), int(nf)
        self.prm = (float(r_in), float(r_out), 0.0, 0.0)
        self.pat, self.bbox, curvi, self.xyz, self.dXdx = generate_mesh(
            MESH_SHELL6, self.n, 0, r_in=r_in, r_out=r_out, ndiv=ndiv)
        self.nelem = len(self.pat)
        self.nb, self.code = face_table(self.xyz, self.n)
        self.fv = np.zeros(self.nelem, np.int32) if fv is None else \
            np.ascontiguousarray(fv, np.int32)
        self.g = _Grhd(gamma, rho_atm, p_atm, tol, maxits)
        self.mass, self.rec = float(mass), FV_REC[rec]
        self._sync()

    def _sync(self):
        self.s = _GrMesh(self.nelem, self.n, self.nf, MESH_SHELL6, (ctypes.c_double * 4)(*self.prm),
                         self.pat.ctypes.data, self.bbox.ctypes.data, self.xyz.ctypes.data,
                         self.dXdx.ctypes.data, self.nb.ctypes.data, self.code.ctypes.data,
                         self.fv.ctypes.data, self.g, self.mass, self.rec)

    @property
    def shapes(self):
        return (self.nelem, 5, self.n ** 3), (self.nelem, 5, self.nf ** 3)

    def points(self, e, fvpts):
        """Cartesian coordinates [3, npts] of element e's LGL nodes or
        equally spaced points."""
        npts = (self.nf if fvpts else self.n) ** 3
        out = np.zeros((3, npts))
        lib().nmo_gr_points(ctypes.byref(self.s), ctypes.c_int(int(e)), ctypes.c_int(int(fvpts)),
                            out.ctypes.data_as(ctypes.c_void_p))
        return out

    def background(self, xyz):
        """alpha, psi, d alpha [3], d psi [3] at points xyz [3, npts]."""
        out = np.zeros((8, xyz.shape[1]))
        bg = (ctypes.c_double * 8)()
        f = lib().nmo_gr_background
        f.restype = None
        for q in range(xyz.shape[1]):
            f(ctypes.c_double(self.mass), (ctypes.c_double * 3)(*xyz[:, q]), bg)
            out[:, q] = list(bg)
        return out

    def psi(self, xyz):
        """psi = 1 + M/(2r) at points xyz [3, npts] (as the background)."""
        r = np.sqrt(xyz[0] * xyz[0] + xyz[1] * xyz[1] + xyz[2] * xyz[2])
        return 1. + 0.5 * self.mass / r

    def set_fv(self, fv):
        self.fv = np.ascontiguousarray(fv, np.int32)
        self._sync()

    def prim2con(self, prim, psi):
        prim = np.ascontiguousarray(prim, np.float64)
        cons = np.zeros_like(prim)
        psi = np.ascontiguousarray(psi, np.float64)
        lib().nmo_grhd_prim2con(ctypes.byref(self.g), ctypes.c_int64(prim.shape[-1]),
                                psi.ctypes.data_as(ctypes.c_void_p),
                                prim.ctypes.data_as(ctypes.c_void_p),
                                cons.ctypes.data_as(ctypes.c_void_p))
        return cons

    def con2prim(self, u_dg, u_fv, prim_dg, prim_fv):
        """In place; returns (atmosphere points, root-finder iterations)."""
        it = ctypes.c_int64(0)
        f = lib().nmo_gr_con2prim
        f.restype = ctypes.c_int64
        natm = f(ctypes.byref(self.s), *(a.ctypes.data_as(ctypes.c_void_p)
                                         for a in (u_dg, u_fv, prim_dg, prim_fv)),
                 ctypes.byref(it))
        return int(natm), int(it.value)

    def rhs(self, u_dg, u_fv, prim_dg, prim_fv):
        """(r_dg, r_fv) of copies of the states after their con2prim."""
        w_dg, w_fv = u_dg.copy(), u_fv.copy()
        p_dg, p_fv = prim_dg.copy(), prim_fv.copy()
        self.con2prim(w_dg, w_fv, p_dg, p_fv)
        r_dg, r_fv = np.zeros_like(w_dg), np.zeros_like(w_fv)
        rc = lib().nmo_gr_rhs(ctypes.byref(self.s), *(a.ctypes.data_as(ctypes.c_void_p) for a in
                                                      (w_dg, w_fv, p_dg, p_fv, r_dg, r_fv)))
        if rc:
            raise RuntimeError("nmo_gr_rhs failed")
        return r_dg, r_fv

    def rk4(self, u_dg, u_fv, prim_dg, prim_fv, dt, nsteps):
        """nsteps RK4 steps of copies; returns (u_dg, u_fv, prim_dg, prim_fv)."""
        out = [np.array(a, np.float64, copy=True, order="C")
               for a in (u_dg, u_fv, prim_dg, prim_fv)]
        rc = lib().nmo_gr_rk4(ctypes.byref(self.s), ctypes.c_double(dt), ctypes.c_int(nsteps),
                              *(a.ctypes.data_as(ctypes.c_void_p) for a in out))
        if rc:
            raise RuntimeError("nmo_gr_rk4 failed")
        return tuple(out)

    def transfer(self):
        """(P [nf, n], R [n, nf]): LGL -> equally spaced and back."""
        P = np.zeros((self.nf, self.n))
        R = np.zeros((self.n, self.nf))
        lib().nmo_gr_transfer(ctypes.c_int(self.n), ctypes.c_int(self.nf),
                              P.ctypes.data_as(ctypes.c_void_p), R.ctypes.data_as(ctypes.c_void_p))
        return P, R

    def apply3(self, A, v):
        """(A x A x A) v for every field of one element: v [5, ni^3]."""
        no, ni = A.shape
        A = np.ascontiguousarray(A)
        out = np.zeros((v.shape[0], no ** 3))
        for f in range(v.shape[0]):
            src = np.ascontiguousarray(v[f])
            dst = np.zeros(no ** 3)
            lib().nmo_gr_apply3(ctypes.c_int(ni), ctypes.c_int(no), A.ctypes.data_as(ctypes.c_void_p),
                                src.ctypes.data_as(ctypes.c_void_p), dst.ctypes.data_as(ctypes.c_void_p))
            out[f] = dst
        return out



class LinkedOracle:
    """Parts of one problem, each an OracleMesh with its own n (the
    reference's p-refinement by patch, amr_prefine_p), joined across their
    coinciding outer faces: a face node's exterior state is the other
    part's face plane interpolated at the node's position, Lagrange in both
    in-plane directions (set_ajsurf_vl's interpolation branch,
    src/main/amr/surface.c:900-1460)."""

    def __init__(self, parts, xyzs):
        """parts: OracleMesh of each part; xyzs: their coordinates [E,3,np]."""
        self.parts = list(parts)
        self.links = []   # (part, e, f, src part, e2, f2, o)
        keyof = {}
        h, tol = 1e-6, 1e-9
        corners = []
        for i, (om, xyz) in enumerate(zip(self.parts, xyzs)):
            n = om.n
            nbn = om.nbnode.reshape(om.nelem, 6, n * n)
            for e in range(om.nelem):
                for f in range(6):
                    if nbn[e, f, 0] != -1:
                        continue
                    pl = face_plane_index(n, f)
                    c = xyz[e][:, pl[[0, n - 1, n * (n - 1), n * n - 1]]].T
                    k = tuple(np.round(c.mean(0) / h).astype(np.int64))
                    keyof.setdefault(k, []).append((i, e, f, c))
        for lst in keyof.values():
            for (i, e, f, c) in lst:
                for (j, e2, f2, c2) in lst:
                    if i == j:
                        continue
                    for o in range(8):
                        ok = True
                        for t in range(4):
                            ca, cb = t & 1, t >> 1
                            aa, bb = (cb, ca) if o & 1 else (ca, cb)
                            aa = 1 - aa if o & 2 else aa
                            bb = 1 - bb if o & 4 else bb
                            if np.abs(c[t] - c2[aa + 2 * bb]).max() > tol:
                                ok = False
                                break
                        if ok:
                            self.links.append((i, e, f, j, e2, f2, o))
                            break
        for (i, e, f, j, e2, f2, o) in self.links:
            om = self.parts[i]
            om.nbnode.reshape(om.nelem, 6, om.n * om.n)[e, f, :] = -4
        self.exts = [np.zeros((om.nelem, 6, om.n * om.n, 5)) for om in self.parts]
        for om, ext in zip(self.parts, self.exts):
            om.set_ext(ext)

    @staticmethod
    def _bary(n):
        x, _ = lgl(n)
        b = np.array([1.0 / np.prod([x[i] - x[j] for j in range(n) if j != i]) for i in range(n)])
        return x, b

    def _fill(self, us):
        for ext in self.exts:
            ext[:] = 0.0
        for (i, e, f, j, e2, f2, o) in self.links:
            nt, ns = self.parts[i].n, self.parts[j].n
            xt, _ = lgl(nt)
            xs, bs = self._bary(ns)
            pl = face_plane_index(ns, f2)
            W = us[j][e2][:, pl].reshape(5, ns, ns)   # [field][b][a]
            for b_ in range(nt):
                for a_ in range(nt):
                    u, v = (xt[b_], xt[a_]) if o & 1 else (xt[a_], xt[b_])
                    u = -u if o & 2 else u
                    v = -v if o & 4 else v
                    la = np.array([bs[k] * np.prod([u - xs[q] for q in range(ns) if q != k])
                                   for k in range(ns)])
                    lb = np.array([bs[k] * np.prod([v - xs[q] for q in range(ns) if q != k])
                                   for k in range(ns)])
                    self.exts[i][e, f, a_ + nt * b_] = np.einsum("fba,a,b->f", W, la, lb)

    def rhs(self, us, t=0.0):
        self._fill(us)
        return [om.rhs(u, t) for om, u in zip(self.parts, us)]

    def rk4(self, us, dt, nsteps, t=0.0):
        """Classic RK4 steps of all parts together (evolve_RK4_mesh)."""
        us = [np.array(u, np.float64, copy=True) for u in us]
        c = (dt / 6., dt / 3., dt / 3., dt / 6.)
        a = (dt / 2., dt / 2., dt)
        te = np.longdouble(0.)
        for _ in range(nsteps):
            ts0 = float(np.longdouble(t) + te)
            ts = (ts0, ts0 + 0.5 * dt, ts0 + 0.5 * dt, ts0 + dt)
            up = [u.copy() for u in us]
            w = [u.copy() for u in us]
            for s in range(4):
                r = self.rhs(w, ts[s])
                for k in range(len(us)):
                    us[k] = us[k] + c[s] * r[k]
                    if s < 3:
                        w[k] = up[k] + a[s] * r[k]
            te += np.longdouble(dt)
        return us
