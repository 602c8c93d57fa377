"""Shared helpers of the tests: golden fixtures, element permutations,
seeded inputs."""
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
PI = 3.141592653589793
CASES = ["box_l1_n5", "box_l2_n4", "cs7_l0_n9", "cs7_l1_n5", "cs7_l1_n4"]
# the benchmark's mesh family and order at level 2 (slim fixture: u0 is the
# dump module's seeded noise, regenerated by dump_noise; r0 and u_final kept
# on a sample of the elements)
BIG_CASE = "cs7_l2_n9_noise"
# all-finite-volume fixtures (uniform points, WENO at the midpoints)
FV_CASES = ["fvbox_l1_n7_w5no", "fvbox_l1_n7_w5dnfn", "fvbox_l2_n5_w3dnfn",
            "fvbox_l0_n13_w5dnfn", "fvcs7_l0_n7_w5dnfn", "fvcs7_l0_n6_w5no",
            "fvcs7_l0_n7_wZdnfn", "fvbox_l1_n8_wZno"]
# mixed fixtures: inner cube finite-volume, cubed-sphere shells DG
MIX_CASES = ["mixcs7_l0_n7_w5dnfn", "mixcs7_l1_n5_w3no", "mixcs7_l1_n6_wZdnfn",
             "mixcs7_l0_n7_w5parab"]
# mixed fixtures where the oracle is a few ulp off the reference: the
# interface positions come from the point sets here and from coordinate
# conversions (X -> the neighbour's Xb) in the reference; they round
# differently on the equally spaced points of even n
MIX_NEAR_CASES = ["mixcs7_l1_n6_wZdnfn"]
# the reference's default upwind flux (DG, mixed, finite volume)
UPW_CASES = ["upw_cs7_l1_n5", "upw_box_l1_n6", "upw_mixcs7_l0_n7_w5dnfn", "upw_fvbox_l1_n7_w5no"]
# the reference's other time integrators (evolve_method = sspRK3, Euler);
# the mixed one is a few ulp off in the oracle like MIX_NEAR_CASES
METHOD_CASES = ["ssp3_cs7_l1_n5", "eul_box_l1_n5", "ssp3_mixcs7_l1_n6_wZdnfn",
                "ssp3_mixcs7_l0_n7_wZparab"]
METHOD_NEAR_CASES = ["ssp3_mixcs7_l1_n6_wZdnfn", "ssp3_mixcs7_l0_n7_wZparab"]
# evolve_filter_all = yes (exponential modal filter after every step); the
# oracle's matrix products sum in another order than the reference's
# mm_array routines, so it matches these to
FILT_CASES = ["filt_cs7_l1_n6", "filt_mixcs7_l0_n7"]
# scalarwave1_limiter = MRS (limiter_alpha in meta["limiter"])
LIM_CASES = ["lim_box_l1_n5_a0.01", "lim_cs7_l1_n4_a0.05", "lim_nc_cs7_l0_n5_h0_a0.02"]
# scalarwave1_limiter = minmodB (limiter_alpha, limiter_beta in meta["beta"],
# limiter_scaleBound = yes where meta["scalebound"])
MMB_CASES = ["mmb_box_l1_n5_a0.05", "mmb_cs7_l1_n4_a0.2_b0.8", "mmb_nc_cs7_l0_n5_h0_a0.1_sb",
             "mmb_mixcs7_l0_n7_w5dnfn_a0.1"]


def limiter_kwargs(meta):
    """The limiter parameters of a limiter fixture (MRS or minmodB)."""
    return dict(kind=meta.get("limname", "MRS"), alpha=meta["limiter"],
                beta=meta.get("beta", 0.5), scale_bound=bool(meta.get("scalebound", False)))
RTOL_FILT_ORACLE = 1e-13
# dt = auto (the reference's dtfac * hmin; uniform_dtfac on FV elements)
DTAUTO_CASES = ["dtauto_cs7_l1_n5", "dtauto_box_l2_n6", "dtauto_mixcs7_l0_n7"]
# coordinates_midpoint_data = yes (FV midpoint factors and normals from the
# map at the midpoints); the mixed one is a few ulp off in the oracle
MID_CASES = ["fvcs7_l0_n7_w5dnfn_mid", "fvcs7_l1_n6_w3no_mid", "ssp3_mixcs7_l0_n7_wZparab_mid"]
MID_NEAR_CASES = ["ssp3_mixcs7_l0_n7_wZparab_mid"]
# non-conforming faces: patches refined one level further (amr_hrefine_p)
NC_CASES = ["nc_cs7_l0_n5_h0", "nc_cs7_l0_n4_h1", "nc_cs7_l1_n5_h02", "nc_upw_cs7_l0_n6_h35",
            "sph_box_l1_n5_s2r2", "sph_box_l2_n4_s1r3", "sph_cs7_l1_n4_s1r6"]
# the oracle's non-conforming (and even-n DG/FV interface) traces take the
# neighbour positions from the element structure, the reference from its
# coordinate maps: equal to a few ulp of the position, so the oracle matches
# those fixtures to
RTOL_NC_ORACLE = 1e-14

# relative L2 tolerance of the CUDA path against the reference / oracle for
# one RHS evaluation and for a few RK4 steps (FP64; FMA contraction and a
# different summation order only)
RTOL_RHS = 1e-12
RTOL_RK4 = 1e-12


def load(case):
    d = np.load(os.path.join(GOLDEN, case + ".npz"))
    meta = json.loads(str(d["meta"]))
    return d, meta


def build_mesh(meta, periodic=False):
    import nmesh_gb300 as ng
    href = [int(p) for p in meta.get("hrefine", "").split()]
    sph = meta.get("sphere", (0, 10))
    fv = "fv" in meta
    if fv and "patches" in meta["fv"]:
        fv = [int(p) for p in meta["fv"]["patches"].split()]
    if meta["mesh"] == "box":
        return ng.Mesh.build(ng.MESH_BOX, n=meta["n"], luni=meta["luni"],
                             xc=(PI, PI, PI), box_dout=PI, periodic=periodic, fv=fv,
                             sphere_levels=sph[0], sphere_radius=sph[1])
    return ng.Mesh.build(ng.MESH_CUBEDSPHERES7, n=meta["n"], luni=meta["luni"],
                         cs_dc=1.0, cs_r0fac=20.0, fv=fv, hrefine=href,
                         sphere_levels=sph[0], sphere_radius=sph[1])


def perm_to_mesh(mesh, d):
    """Index array p such that mesh element p[i] is fixture element i."""
    pat, bbox = mesh.elements()
    key = {(int(a),) + tuple(b): i for i, (a, b) in enumerate(zip(pat, bbox))}
    return np.array([key[(int(a),) + tuple(b)] for a, b in zip(d["pat"], d["bbox"])])


def to_mesh_order(arr, perm):
    out = np.empty_like(arr)
    out[perm] = arr
    return out


def rel_l2(a, b):
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


def oracle_for(mesh, bc=0, k=(1.0, 1.0, 1.0), period=None, fv_rec="WENOm3_2",
               fv_extrap="dnfn_extrap1", fv_w3ratio=2.0, numflux="LLF",
               fv_surface_interp="linear", midpoint_data=False):
    """Oracle mesh built from the product mesh's geometry, with its own
    coordinate-matching neighbour table (and the mesh's finite-volume flags
    with the given fin.-vol. options)."""
    from oracle import nmo
    pat, bbox = mesh.elements()
    xyz = mesh.coords()
    dXdx = mesh.dXdx()
    curvi = np.array([0 if np.allclose(dXdx[e], np.repeat(np.eye(3).ravel()[:, None],
                                                          mesh.np, 1)) else 1
                      for e in range(mesh.nelem)], np.int32)
    fv = mesh.fv()
    mix = hang = None
    if fv.any():
        nb, mix = nmo.match_faces(xyz, mesh.n, period=period, fv=fv)
    else:
        nb = nmo.match_faces(xyz, mesh.n, period=period)
    if (mesh.faces()[1] & 128).any():
        nb, hang = nmo.match_hanging(xyz, mesh.n, pat, bbox, nb)
    return nmo.OracleMesh(bbox, curvi, dXdx, xyz, nb, mesh.n, bc=bc, k=k,
                          fv=fv if fv.any() else None, fv_rec=fv_rec,
                          fv_extrap=fv_extrap, fv_w3ratio=fv_w3ratio, mixface=mix,
                          numflux=numflux, hang=hang, fv_surface_interp=fv_surface_interp,
                          dXdxm=mesh.midpoint_dXdx() if midpoint_data else None)


def gaussian_pulses(xyz, seed, npulse=8, rmin=3.0, rmax=10.0, wmin=0.5, wmax=2.0,
                    amin=0.1, amax=1.0):
    """Seeded sum of Gaussian pulses in pi (and consistent c = grad psi of the
    same profile), phi = psi; xyz: [E,3,np] -> u [E,5,np]."""
    rng = np.random.default_rng(seed)
    E, _, npt = xyz.shape
    u = np.zeros((E, 5, npt))
    for _ in range(npulse):
        r = rng.uniform(rmin, rmax)
        v = rng.normal(size=3)
        v /= np.linalg.norm(v)
        c = r * v
        w = rng.uniform(wmin, wmax)
        a = rng.uniform(amin, amax)
        dx = xyz - c[None, :, None]
        g = a * np.exp(-np.sum(dx * dx, axis=1) / (w * w))
        u[:, 4] += g
        u[:, 1:4] += -2.0 * dx / (w * w) * g[:, None, :]
        u[:, 0] += 0.0
    return u


def dump_noise(seed, eps, nelem, npt):
    """The reference-side dump module's initial perturbation with amplitude 0
    for the plane wave: u[e, f, ijk] = eps * hash(seed * 1000003 + (e << 24) +
    (f << 20) + ijk), hash a splitmix64 finaliser mapped to [-1, 1)
    (oracle/ref/nmgdump/nmgdump.c: nmgdump_hash, nmgdump_perturb); bit for
    bit, e in the reference's element order."""
    e = np.arange(nelem, dtype=np.uint64)[:, None, None]
    f = np.arange(5, dtype=np.uint64)[None, :, None]
    q = np.arange(npt, dtype=np.uint64)[None, None, :]
    a = np.uint64(seed) * np.uint64(1000003) + (e << np.uint64(24)) + \
        (f << np.uint64(20)) + q
    a = a + np.uint64(0x9E3779B97F4A7C15)
    a = (a ^ (a >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    a = (a ^ (a >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    a = a ^ (a >> np.uint64(31))
    h = (a >> np.uint64(11)).astype(np.float64) * (2.0 / 9007199254740992.0) - 1.0
    return eps * h


def big_case_u0(d, meta):
    """u0 of the slim fixture in the reference's element order."""
    n = meta["n"]
    return dump_noise(meta["seed"], meta["eps"], len(d["pat"]), n ** 3)


def grhd_blob(o, seed, rho0=1e-3, K=100.0, center=(8.0, 0.0, 0.0), width=2.0, pert=0.01,
              vel=(0.0, 0.0, 0.0)):
    """Seeded Gaussian density blob on the GRHD oracle's mesh `o`
    (oracle.nmo.GrhdOracle): rho = rho_atm + rho0 exp(-|x - c|^2 / width^2)
    (1 + pert U(-1, 1)), polytropic p = K rho^2, velocity `vel`; on every
    element's LGL nodes and equally spaced points.  Returns (prim_dg [E, 5,
    n^3], prim_fv [E, 5, nf^3], u_dg, u_fv) (conserved via the oracle)."""
    rng = np.random.default_rng(seed)
    (E, _, npd), (_, _, npf) = o.shapes
    out = [np.zeros((E, 5, npd)), np.zeros((E, 5, npf))]
    cons = [np.zeros((E, 5, npd)), np.zeros((E, 5, npf))]
    c = np.asarray(center, float)[:, None]
    for e in range(E):
        for k, fvp in enumerate((False, True)):
            x = o.points(e, fvp)
            r2 = ((x - c) ** 2).sum(0)
            rho = o.g.rho_atm + rho0 * np.exp(-r2 / width ** 2) * \
                (1.0 + pert * rng.uniform(-1.0, 1.0, x.shape[1]))
            P = out[k][e]
            P[0] = rho
            P[1], P[2], P[3] = vel
            P[4] = K * rho * rho
            cons[k][e] = o.prim2con(P, o.psi(x))
    return out[0], out[1], cons[0], cons[1]
