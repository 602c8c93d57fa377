"""nmesh_gb300 -- GB300-native nmesh evolution path (scalarwave1 DG RHS,
LLF face flux + lift, RK4), FP64, behind the C ABI of include/nmg.h.

This module is a thin ctypes binding of nmesh_gb300/_build/libnmg.so.  It
mirrors the reference's interface for the path: a mesh is made from the
reference's amr_* parameters (src/main/amr/mesh.c:181), `rhs` replaces
evolve_setrhs_mesh (src/main/evolve/evolve.c:182) and `rk4_step(s)` replace
evolve_RK4_mesh (src/main/evolve/RungeKutta.c:19).  There is no CPU
fallback: every call goes to the CUDA library and raises if it is missing
or fails.
"""
import ctypes
import os

import numpy as np

from . import build as _build

NFIELDS = 5
FIELDS = ("pi", "cx", "cy", "cz", "phi")
MESH_BOX = 1
MESH_CUBEDSPHERES7 = 7
MESH_CUBEDSHELL6 = 6
BC_EXACT_PLANEWAVE = 0
BC_OUTGOING = 1
# finite-volume reconstruction (reference par fv_rec) and div(f) completion
# on face points (par fv_divf_extrap)
EVOLVE_METHOD = {"RK4": 0, "Euler": 1, "sspRK3": 2}
FV_REC = {"1": 0, "WENOm3_2": 1, "WENOm5_2": 2, "WENOmZ_2": 3}
FV_EXTRAP = {"no": 0, "dnfn_extrap1": 1}

_c_dp = ctypes.POINTER(ctypes.c_double)
_lib = None


class NmgError(RuntimeError):
    pass


class _MeshParams(ctypes.Structure):
    _fields_ = [("mesh_type", ctypes.c_int32), ("n", ctypes.c_int32),
                ("luni", ctypes.c_int32), ("periodic", ctypes.c_int32),
                ("xc", ctypes.c_double * 3), ("box_dout", ctypes.c_double),
                ("cs_dc", ctypes.c_double), ("cs_r0fac", ctypes.c_double),
                ("fv", ctypes.c_int32), ("hrefine", ctypes.c_int32),
                ("sphere_levels", ctypes.c_int32), ("sphere_radius", ctypes.c_double),
                ("ndiv", ctypes.c_int32), ("shell_rin", ctypes.c_double),
                ("shell_rout", ctypes.c_double), ("patch_mask", ctypes.c_int32)]


class TroubleParams(ctypes.Structure):
    """Trouble detection parameters (include/nmg.h nmg_trouble_params)."""
    _fields_ = [("rdmp_deltafac", ctypes.c_double), ("rdmp_delta0", ctypes.c_double),
                ("rdmp_epsilon", ctypes.c_double), ("persson_max", ctypes.c_double),
                ("persson_uscale", ctypes.c_double), ("notroubles", ctypes.c_int32),
                ("redo", ctypes.c_int32)]

    def __init__(self, rdmp_deltafac=1.0, rdmp_delta0=1e-4, rdmp_epsilon=1e-3,
                 persson_max=1e300, persson_uscale=-1.0, notroubles=11, redo="step"):
        """redo: "step" or "substep" (the reference's evolve_redo_troubled)."""
        super().__init__(rdmp_deltafac, rdmp_delta0, rdmp_epsilon, persson_max,
                         persson_uscale, notroubles, {"step": 0, "substep": 1}[redo])


class GrhdParams(ctypes.Structure):
    """Ideal-gas GRHD conversion parameters (include/nmg.h nmg_grhd_params)."""
    _fields_ = [("gamma", ctypes.c_double), ("rho_atm", ctypes.c_double),
                ("p_atm", ctypes.c_double), ("tol", ctypes.c_double),
                ("maxits", ctypes.c_int32)]

    def __init__(self, gamma=2.0, rho_atm=1e-12, p_atm=1e-14, tol=1e-15, maxits=100):
        super().__init__(gamma, rho_atm, p_atm, tol, maxits)


def grhd_prim2con_device(params, npts, psi_ptr, prim_ptr, cons_ptr, stream=0):
    """Conserved (D, S_i, tau) from primitives (rho, v^i, p) on device SoA
    arrays [5][npts] (ints are device pointers; psi_ptr 0: flat)."""
    rc = lib().nmg_grhd_prim2con(ctypes.byref(params), int(npts),
                                 ctypes.c_void_p(psi_ptr or None), ctypes.c_void_p(prim_ptr),
                                 ctypes.c_void_p(cons_ptr), ctypes.c_void_p(stream or None))
    if rc:
        raise NmgError(f"nmg_grhd_prim2con failed ({rc})")


def grhd_con2prim_device(params, npts, psi_ptr, cons_ptr, prim_ptr, status_ptr, stream=0):
    """Primitives from conserved variables (atmosphere where needed); see
    include/nmg.h nmg_grhd_con2prim."""
    rc = lib().nmg_grhd_con2prim(ctypes.byref(params), int(npts),
                                 ctypes.c_void_p(psi_ptr or None), ctypes.c_void_p(cons_ptr),
                                 ctypes.c_void_p(prim_ptr), ctypes.c_void_p(status_ptr),
                                 ctypes.c_void_p(stream or None))
    if rc:
        raise NmgError(f"nmg_grhd_con2prim failed ({rc})")


def grhd_fluxes_device(params, npts, d, alpha_ptr, psi_ptr, prim_ptr, flux_ptr, lam_ptr,
                       stream=0):
    """Valencia fluxes along d and characteristic speeds (include/nmg.h)."""
    rc = lib().nmg_grhd_fluxes(ctypes.byref(params), int(npts), int(d),
                               ctypes.c_void_p(alpha_ptr or None), ctypes.c_void_p(psi_ptr or None),
                               ctypes.c_void_p(prim_ptr), ctypes.c_void_p(flux_ptr),
                               ctypes.c_void_p(lam_ptr), ctypes.c_void_p(stream or None))
    if rc:
        raise NmgError(f"nmg_grhd_fluxes failed ({rc})")


def grhd_sources_device(params, npts, alpha_ptr, psi_ptr, dalpha_ptr, dpsi_ptr, prim_ptr,
                        src_ptr, stream=0):
    """Cowling source terms (include/nmg.h)."""
    rc = lib().nmg_grhd_sources(ctypes.byref(params), int(npts), ctypes.c_void_p(alpha_ptr),
                                ctypes.c_void_p(psi_ptr), ctypes.c_void_p(dalpha_ptr),
                                ctypes.c_void_p(dpsi_ptr), ctypes.c_void_p(prim_ptr),
                                ctypes.c_void_p(src_ptr), ctypes.c_void_p(stream or None))
    if rc:
        raise NmgError(f"nmg_grhd_sources failed ({rc})")


class _MeshDesc(ctypes.Structure):
    _fields_ = [("nelem", ctypes.c_int32), ("n", ctypes.c_int32),
                ("pat", ctypes.c_void_p), ("bbox", ctypes.c_void_p),
                ("curvi", ctypes.c_void_p), ("xyz", ctypes.c_void_p),
                ("dXdx", ctypes.c_void_p), ("nbnode", ctypes.c_void_p),
                ("period", ctypes.c_double * 3), ("fv", ctypes.c_void_p)]


def library_path():
    return _build.LIB


def lib(build_if_missing=True):
    """Load libnmg.so (building it first if it is missing or stale)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.build() if build_if_missing else _build.LIB
    if not os.path.exists(path):
        raise NmgError(f"native library missing: {path}")
    L = ctypes.CDLL(path)
    vp, i32, i64, f64 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_double
    sig = {
        "nmg_mesh_build": (ctypes.c_int, [vp, vp]),
        "nmg_mesh_from_desc": (ctypes.c_int, [vp, vp]),
        "nmg_mesh_nelem": (i64, [vp]),
        "nmg_mesh_n": (i32, [vp]),
        "nmg_mesh_get_elements": (ctypes.c_int, [vp, vp, vp]),
        "nmg_mesh_get_coords": (ctypes.c_int, [vp, vp]),
        "nmg_mesh_get_dXdx": (ctypes.c_int, [vp, vp]),
        "nmg_mesh_get_faces": (ctypes.c_int, [vp, vp, vp]),
        "nmg_basis": (ctypes.c_int, [i32, vp, vp, vp]),
        "nmg_mesh_free": (None, [vp]),
        "nmg_mesh_last_error": (ctypes.c_char_p, []),
        "nmg_create": (ctypes.c_int, [vp, i32, vp, vp]),
        "nmg_destroy": (None, [vp]),
        "nmg_last_error": (ctypes.c_char_p, [vp]),
        "nmg_state_size": (i64, [vp]),
        "nmg_set_state": (ctypes.c_int, [vp, vp]),
        "nmg_get_state": (ctypes.c_int, [vp, vp]),
        "nmg_state_device_ptr": (vp, [vp]),
        "nmg_rhs": (ctypes.c_int, [vp, f64, vp, vp]),
        "nmg_rhs_host": (ctypes.c_int, [vp, f64, vp, vp]),
        "nmg_rk4_step": (ctypes.c_int, [vp, f64, f64]),
        "nmg_rk4_steps": (ctypes.c_int, [vp, f64, f64, i32]),
        "nmg_rk4_steps_host": (ctypes.c_int, [vp, f64, f64, i32, vp]),
        "nmg_kernel_launches": (i64, [vp]),
        "nmg_stream": (vp, [vp]),
        "nmg_fp64_peak": (ctypes.c_int, [vp]),
        "nmg_fp64_dmma_peak": (ctypes.c_int, [vp]),
        "nmg_set_kernel": (ctypes.c_int, [vp, ctypes.c_char_p]),
        "nmg_rk4_step_noalloc": (ctypes.c_int, [vp, f64, f64, vp, vp]),
        "nmg_mesh_concat": (ctypes.c_int, [vp, i32, vp]),
        "nmg_batch_create": (ctypes.c_int, [vp, i32, i32, vp, vp]),
        "nmg_batch_create_linked": (ctypes.c_int, [vp, i32, vp, i32, vp, vp]),
        "nmg_batch_linked_faces": (i64, [vp]),
        "nmg_batch_destroy": (None, [vp]),
        "nmg_batch_last_error": (ctypes.c_char_p, [vp]),
        "nmg_batch_problem_size": (i64, [vp, i32]),
        "nmg_batch_set_state": (ctypes.c_int, [vp, i32, vp]),
        "nmg_batch_get_state": (ctypes.c_int, [vp, i32, vp]),
        "nmg_rk4_steps_batched": (ctypes.c_int, [vp, f64, f64, i32]),
        "nmg_batch_info": (ctypes.c_int, [vp, vp, i32]),
        "nmg_batch_stream": (vp, [vp]),
        "nmg_batch_set_mode": (ctypes.c_int, [vp, i32]),
        "nmg_rhs_vjp": (ctypes.c_int, [vp, f64, vp, vp, vp]),
        "nmg_rk4_step_vjp": (ctypes.c_int, [vp, f64, f64, vp, vp]),
        "nmg_adjoint_gradient": (ctypes.c_int, [vp, f64, f64, i32, i32, vp, vp, vp]),
        "nmg_kernel_info": (ctypes.c_int, [vp, vp, i32]),
        "nmg_mesh_get_fv": (ctypes.c_int, [vp, vp]),
        "nmg_uniform_points": (ctypes.c_int, [i32, vp]),
        "nmg_set_fv": (ctypes.c_int, [vp, i32, i32, f64]),
        "nmg_create_switchable": (ctypes.c_int, [vp, i32, vp, vp]),
        "nmg_set_element_types": (ctypes.c_int, [vp, vp]),
        "nmg_get_element_types": (ctypes.c_int, [vp, vp]),
        "nmg_trouble_check": (ctypes.c_int, [vp, vp, vp, vp, vp, vp]),
        "nmg_rk4_step_trouble": (ctypes.c_int, [vp, f64, f64, vp, vp]),
        "nmg_get_trouble_scores": (ctypes.c_int, [vp, vp]),
        "nmg_norms": (ctypes.c_int, [vp, vp, vp]),
        "nmg_set_numflux": (ctypes.c_int, [vp, i32]),
        "nmg_set_evolve_method": (ctypes.c_int, [vp, i32]),
        "nmg_set_fv_surface_interp": (ctypes.c_int, [vp, i32]),
        "nmg_set_fv_midpoint_data": (ctypes.c_int, [vp, i32]),
        "nmg_set_filter": (ctypes.c_int, [vp, i32, f64, f64, i32, i32, i32]),
        "nmg_set_limiter": (ctypes.c_int, [vp, i32, f64]),
        "nmg_set_limiter_ex": (ctypes.c_int, [vp, i32, f64, f64, i32]),
        "nmg_get_limited": (ctypes.c_int, [vp, vp]),
        "nmg_mesh_get_midpoint_dXdx": (ctypes.c_int, [vp, vp]),
        "nmg_mesh_auto_dt": (ctypes.c_int, [vp, f64, f64, vp]),
        "nmg_evolve_steps": (ctypes.c_int, [vp, f64, f64, i32]),
        "nmg_evolve_steps_host": (ctypes.c_int, [vp, f64, f64, i32, vp]),
        "nmg_checkpoint_write": (ctypes.c_int, [vp, vp, ctypes.c_char_p, vp]),
        "nmg_checkpoint_read": (ctypes.c_int, [vp, vp, ctypes.c_char_p, vp]),
        "nmg_checkpoint_write_host": (ctypes.c_int, [vp, vp, ctypes.c_char_p, vp]),
        "nmg_checkpoint_read_host": (ctypes.c_int, [vp, ctypes.c_char_p, vp, vp]),
        "nmg_checkpoint_last_error": (ctypes.c_char_p, []),
        "nmg_mesh_element_name": (ctypes.c_char_p, [vp, i64]),
        "nmg_mesh_get_hanging": (ctypes.c_int, [vp, vp, vp, vp, vp, vp, vp]),
        "nmg_grhd_prim2con": (ctypes.c_int, [vp, i64, vp, vp, vp, vp]),
        "nmg_grhd_con2prim": (ctypes.c_int, [vp, i64, vp, vp, vp, vp, vp]),
        "nmg_grhd_fluxes": (ctypes.c_int, [vp, i64, i32, vp, vp, vp, vp, vp, vp]),
        "nmg_grhd_sources": (ctypes.c_int, [vp, i64, vp, vp, vp, vp, vp, vp, vp]),
        "nmg_grhd_create": (ctypes.c_int, [vp, vp, vp]),
        "nmg_grhd_destroy": (None, [vp]),
        "nmg_grhd_last_error": (ctypes.c_char_p, [vp]),
        "nmg_grhd_sizes": (ctypes.c_int, [vp, vp, vp, vp]),
        "nmg_grhd_set_fv_elements": (ctypes.c_int, [vp, vp]),
        "nmg_grhd_get_fv_elements": (ctypes.c_int, [vp, vp]),
        "nmg_grhd_fv_count": (i64, [vp]),
        "nmg_grhd_set_prim": (ctypes.c_int, [vp, vp, vp]),
        "nmg_grhd_set_state": (ctypes.c_int, [vp, vp, vp, vp, vp]),
        "nmg_grhd_get_state": (ctypes.c_int, [vp, vp, vp, vp, vp]),
        "nmg_grhd_rhs": (ctypes.c_int, [vp, vp, vp]),
        "nmg_grhd_rk4_steps": (ctypes.c_int, [vp, f64, i32]),
        "nmg_grhd_stats": (ctypes.c_int, [vp, vp, vp, vp]),
        "nmg_grhd_reset_stats": (ctypes.c_int, [vp]),
        "nmg_grhd_stream": (vp, [vp]),
        "nmg_grhd_profile_step": (ctypes.c_int, [vp, f64, vp]),
        "nmg_grhd_trouble_indicators": (ctypes.c_int, [vp, vp]),
        "nmg_grhd_update_troubled": (ctypes.c_int, [vp, f64, f64, vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def fp64_peak_gflops():
    """Measured FP64 FMA throughput of the current GPU (GFLOP/s)."""
    v = ctypes.c_double(0.0)
    if lib().nmg_fp64_peak(ctypes.byref(v)):
        raise NmgError("nmg_fp64_peak failed")
    return v.value


def fp64_dmma_peak_gflops():
    """Measured FP64 tensor-core (DMMA) throughput of the current GPU (GFLOP/s)."""
    v = ctypes.c_double(0.0)
    if lib().nmg_fp64_dmma_peak(ctypes.byref(v)):
        raise NmgError("nmg_fp64_dmma_peak failed")
    return v.value


def basis(n):
    """LGL nodes x, weights w and D[i, j] = l_j'(x_i) (Legendre.c/Lagrange.c)."""
    x, w, D = np.zeros(n), np.zeros(n), np.zeros((n, n))
    if lib().nmg_basis(n, _ptr(x), _ptr(w), _ptr(D)):
        raise NmgError(lib().nmg_mesh_last_error().decode())
    return x, w, D


class Mesh:
    """Host-side packed mesh (geometry, metric, face table)."""

    def __init__(self, handle):
        self._h = ctypes.c_void_p(handle)
        self.nelem = int(lib().nmg_mesh_nelem(self._h))
        self.n = int(lib().nmg_mesh_n(self._h))
        self.np = self.n ** 3

    @classmethod
    def build(cls, mesh_type=MESH_BOX, n=5, luni=0, xc=(0.0, 0.0, 0.0),
              box_dout=1.0, cs_dc=1.0, cs_r0fac=20.0, periodic=False, fv=False,
              hrefine=(), sphere_levels=0, sphere_radius=10.0, ndiv=0, shell_rin=2.0,
              shell_rout=20.0, patches=None):
        """Mesh from the reference's parameters: amr_mesh_type (1 BoxMesh /
        7 CubedSpheres), amr_n0..2 = n, amr_luni, amr_mesh_xc,
        amr_BoxMesh_dout, amr_CubedSphere_dc, amr_CubedSphere_r0fac;
        fv=True puts every patch in amr_uniform_p and amr_fv_p, a list of
        patch indices puts those patches there; hrefine lists the patches
        of amr_hrefine_p (refined one level further); sphere_levels and
        sphere_radius are amr_hrefine_sphere_levels / _radius (elements
        whose centre lies within radius 2^(levels-1-i) of x = 0 are refined
        in pass i).  MESH_CUBEDSHELL6: six cubed-sphere patches between the
        spheres of radius shell_rin and shell_rout; ndiv > 0 splits every
        patch into ndiv^3 equal elements instead of 2^luni per direction.
        patches: build only these patches (a part of the mesh)."""
        pmask = 0
        for p_ in (patches or ()):
            pmask |= 1 << int(p_)
        hmask = 0
        for p_ in hrefine:
            hmask |= 1 << int(p_)
        if fv is True:
            mask = -1
        elif not fv:
            mask = 0
        else:
            mask = 0
            for p_ in fv:
                mask |= 1 << int(p_)
        p = _MeshParams(int(mesh_type), int(n), int(luni), int(bool(periodic)),
                        (ctypes.c_double * 3)(*xc), float(box_dout),
                        float(cs_dc), float(cs_r0fac), int(mask), hmask,
                        int(sphere_levels), float(sphere_radius), int(ndiv), float(shell_rin),
                        float(shell_rout), pmask)
        h = ctypes.c_void_p()
        rc = lib().nmg_mesh_build(ctypes.byref(p), ctypes.byref(h))
        if rc:
            raise NmgError(f"nmg_mesh_build: {lib().nmg_mesh_last_error().decode()}")
        return cls(h.value)

    @classmethod
    def from_arrays(cls, bbox, curvi, xyz, dXdx=None, nbnode=None, pat=None,
                    period=(0.0, 0.0, 0.0), fv=None):
        """Mesh from per-element arrays (what an nmesh adapter packs)."""
        bbox = np.ascontiguousarray(bbox, np.float64)
        E = bbox.shape[0]
        xyz = np.ascontiguousarray(xyz, np.float64)
        n = int(round(xyz.shape[-1] ** (1.0 / 3.0)))
        keep = [bbox, np.ascontiguousarray(curvi, np.int32), xyz]
        dX = None if dXdx is None else np.ascontiguousarray(dXdx, np.float64)
        nb = None if nbnode is None else np.ascontiguousarray(nbnode, np.int64)
        pt = None if pat is None else np.ascontiguousarray(pat, np.int32)
        fva = None if fv is None else np.ascontiguousarray(fv, np.int32)
        d = _MeshDesc(E, n, None if pt is None else pt.ctypes.data, bbox.ctypes.data,
                      keep[1].ctypes.data, xyz.ctypes.data,
                      None if dX is None else dX.ctypes.data,
                      None if nb is None else nb.ctypes.data,
                      (ctypes.c_double * 3)(*period),
                      None if fva is None else fva.ctypes.data)
        h = ctypes.c_void_p()
        rc = lib().nmg_mesh_from_desc(ctypes.byref(d), ctypes.byref(h))
        if rc:
            raise NmgError(f"nmg_mesh_from_desc: {lib().nmg_mesh_last_error().decode()}")
        return cls(h.value)

    def elements(self):
        pat = np.zeros(self.nelem, np.int32)
        bbox = np.zeros((self.nelem, 6))
        lib().nmg_mesh_get_elements(self._h, _ptr(pat), _ptr(bbox))
        return pat, bbox

    def coords(self):
        x = np.zeros((self.nelem, 3, self.np))
        lib().nmg_mesh_get_coords(self._h, _ptr(x))
        return x

    def dXdx(self):
        x = np.zeros((self.nelem, 9, self.np))
        lib().nmg_mesh_get_dXdx(self._h, _ptr(x))
        return x

    def fv(self):
        """Per-element finite-volume flags."""
        f = np.zeros(self.nelem, np.int32)
        lib().nmg_mesh_get_fv(self._h, _ptr(f))
        return f

    def names(self):
        """The reference's element names "<patch>_<octree digits>" (None for
        a mesh built from arrays)."""
        out = [lib().nmg_mesh_element_name(self._h, e) for e in range(self.nelem)]
        return None if any(x is None for x in out) else [x.decode() for x in out]

    @classmethod
    def concat(cls, meshes):
        """One mesh of several of the same n, elements renumbered in order
        (nmg_mesh_concat)."""
        arr = (ctypes.c_void_p * len(meshes))(*[m_._h for m_ in meshes])
        h = ctypes.c_void_p()
        if lib().nmg_mesh_concat(arr, len(meshes), ctypes.byref(h)):
            raise NmgError(f"nmg_mesh_concat: {lib().nmg_mesh_last_error().decode()}")
        return cls(h.value)

    def auto_dt(self, dtfac=0.25, uniform_dtfac=0.125):
        """The reference's dt = auto for this mesh."""
        v = ctypes.c_double()
        if lib().nmg_mesh_auto_dt(self._h, float(dtfac), float(uniform_dtfac), ctypes.byref(v)):
            raise NmgError(lib().nmg_mesh_last_error().decode())
        return v.value

    def midpoint_dXdx(self):
        """dX^a/dx^i [E, 3, 9, np] at the midpoints right of each node in
        each direction (coordinates_midpoint_data)."""
        out = np.zeros((self.nelem, 3, 9, self.np))
        if lib().nmg_mesh_get_midpoint_dXdx(self._h, _ptr(out)):
            raise NmgError(lib().nmg_mesh_last_error().decode())
        return out

    def hanging(self):
        """Non-conforming faces: (hface [H,2], hoff [H*n*n+1], hsrc [C,2],
        hpos [C,2]) — per face node the contributions averaged into its trace."""
        H, C = ctypes.c_int64(), ctypes.c_int64()
        lib().nmg_mesh_get_hanging(self._h, ctypes.byref(H), ctypes.byref(C), None, None, None,
                                   None)
        hface = np.zeros((H.value, 2), np.int32)
        hoff = np.zeros(H.value * self.n * self.n + 1 if H.value else 0, np.int32)
        hsrc = np.zeros((C.value, 2), np.int32)
        hpos = np.zeros((C.value, 2))
        lib().nmg_mesh_get_hanging(self._h, ctypes.byref(H), ctypes.byref(C), _ptr(hface),
                                   _ptr(hoff), _ptr(hsrc), _ptr(hpos))
        return hface, hoff, hsrc, hpos

    def faces(self):
        nb = np.zeros((self.nelem, 6), np.int32)
        code = np.zeros((self.nelem, 6), np.int32)
        lib().nmg_mesh_get_faces(self._h, _ptr(nb), _ptr(code))
        return nb, code

    def close(self):
        if self._h:
            lib().nmg_mesh_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _names_arg(names):
    if names is None:
        return None, None
    arr = (ctypes.c_char_p * len(names))(*[str(x).encode() for x in names])
    return ctypes.cast(arr, ctypes.c_void_p), arr


def checkpoint_write_host(mesh, u, path, names=None):
    """Write host state u [E,5,np] as the reference's checkpoint variables.bin."""
    u = np.ascontiguousarray(u, np.float64)
    p, keep = _names_arg(names)
    if lib().nmg_checkpoint_write_host(mesh._h, _ptr(u), str(path).encode(), p):
        raise NmgError(lib().nmg_checkpoint_last_error().decode())


def checkpoint_read_host(mesh, path, names=None):
    """Read the reference's checkpoint variables.bin into a host state."""
    u = np.zeros((mesh.nelem, NFIELDS, mesh.np))
    p, keep = _names_arg(names)
    if lib().nmg_checkpoint_read_host(mesh._h, str(path).encode(), _ptr(u), p):
        raise NmgError(lib().nmg_checkpoint_last_error().decode())
    return u


class Evolution:
    """Device context: mesh data and RK4 state resident in HBM."""

    def __init__(self, mesh, bc=BC_EXACT_PLANEWAVE, k=(1.0, 1.0, 1.0), switchable=False):
        """switchable=True: elements can change between DG and finite volume
        (nmg_create_switchable)."""
        self.mesh = mesh
        kk = np.ascontiguousarray(k, np.float64)
        h = ctypes.c_void_p()
        create = lib().nmg_create_switchable if switchable else lib().nmg_create
        rc = create(mesh._h, int(bc), _ptr(kk), ctypes.byref(h))
        self._h = h
        if rc:
            msg = lib().nmg_last_error(h).decode() if h.value else ""
            self.close()
            raise NmgError(f"nmg_create failed ({rc}): {msg}")
        self.size = int(lib().nmg_state_size(self._h))
        self.shape = (mesh.nelem, NFIELDS, mesh.np)

    def _check(self, rc, what):
        if rc:
            raise NmgError(f"{what} failed ({rc}): {lib().nmg_last_error(self._h).decode()}")

    def set_state(self, u):
        u = np.ascontiguousarray(u, np.float64)
        assert u.size == self.size
        self._check(lib().nmg_set_state(self._h, _ptr(u)), "nmg_set_state")

    def get_state(self):
        u = np.zeros(self.shape)
        self._check(lib().nmg_get_state(self._h, _ptr(u)), "nmg_get_state")
        return u

    def rhs(self, w, t=0.0):
        """r = RHS(w, t) for a host array w (copied to HBM and back)."""
        w = np.ascontiguousarray(w, np.float64)
        assert w.size == self.size
        r = np.zeros(self.shape)
        self._check(lib().nmg_rhs_host(self._h, float(t), _ptr(w), _ptr(r)), "nmg_rhs_host")
        return r

    def rhs_device(self, w_ptr, r_ptr, t=0.0):
        """r = RHS(w, t) on device pointers (ints), on the context stream."""
        self._check(lib().nmg_rhs(self._h, float(t), ctypes.c_void_p(w_ptr),
                                  ctypes.c_void_p(r_ptr)), "nmg_rhs")

    def rk4_step(self, t, dt):
        self._check(lib().nmg_rk4_step(self._h, float(t), float(dt)), "nmg_rk4_step")

    def rk4_steps(self, t, dt, nsteps):
        self._check(lib().nmg_rk4_steps(self._h, float(t), float(dt), int(nsteps)),
                    "nmg_rk4_steps")

    def rk4_steps_host(self, u, t, dt, nsteps, inplace=False):
        """nsteps RK4 steps of host state u (copied to HBM and back); with
        inplace=True u (C-contiguous float64, e.g. pinned) is updated."""
        if not (inplace and isinstance(u, np.ndarray) and u.dtype == np.float64
                and u.flags.c_contiguous):
            u = np.array(u, np.float64, copy=True, order="C")
        assert u.size == self.size
        self._check(lib().nmg_rk4_steps_host(self._h, float(t), float(dt), int(nsteps),
                                             _ptr(u)), "nmg_rk4_steps_host")
        return u

    # ---- adjoint ----
    def rhs_vjp_device(self, rbar_ptr, wbar_ptr, t=0.0):
        """wbar = (dRHS/dw)^T rbar on device pointers (ints)."""
        self._check(lib().nmg_rhs_vjp(self._h, float(t), None, ctypes.c_void_p(rbar_ptr),
                                      ctypes.c_void_p(wbar_ptr)), "nmg_rhs_vjp")

    def rk4_step_vjp_device(self, ubar_ptr, t, dt):
        """ubar <- (du_{n+1}/du_n)^T ubar in place on a device pointer."""
        self._check(lib().nmg_rk4_step_vjp(self._h, float(t), float(dt), None,
                                           ctypes.c_void_p(ubar_ptr)), "nmg_rk4_step_vjp")

    def adjoint_gradient_device(self, weight_ptr, grad_ptr, t0, dt, nsteps, ckpt_every):
        """J and dJ/du0 for u0 = the current state (see include/nmg.h)."""
        J = ctypes.c_double(0.0)
        self._check(lib().nmg_adjoint_gradient(self._h, float(t0), float(dt), int(nsteps),
                                               int(ckpt_every), ctypes.c_void_p(weight_ptr),
                                               ctypes.byref(J), ctypes.c_void_p(grad_ptr)),
                    "nmg_adjoint_gradient")
        return J.value

    def set_numflux(self, kind="LLF"):
        """Numerical flux: "LLF" or "upwind" (reference par scalarwave1_numflux)."""
        k = {"LLF": 0, "upwind": 1}.get(kind)
        if k is None:
            raise NmgError(f"nmg_set_numflux: unknown numerical flux {kind!r}")
        self._check(lib().nmg_set_numflux(self._h, k), "nmg_set_numflux")

    def set_fv(self, rec="WENOm3_2", extrap="dnfn_extrap1", w3ratio=2.0):
        """Finite-volume options (reference pars fv_rec, fv_divf_extrap,
        fv_WENOm3_opt_weightratio)."""
        if rec not in FV_REC or extrap not in FV_EXTRAP:
            raise NmgError(f"nmg_set_fv: unknown fv_rec {rec!r} or fv_divf_extrap {extrap!r}")
        self._check(lib().nmg_set_fv(self._h, FV_REC[rec], FV_EXTRAP[extrap],
                                     float(w3ratio)), "nmg_set_fv")

    def norms(self, u_ptr=0):
        """0d norms of the resident state (or of device state u_ptr): dict
        with 'volume' and per field name (VolInt, mean, rms, min, max,
        maxAbs) (the reference's output0d quantities)."""
        out = np.zeros(1 + 6 * NFIELDS)
        self._check(lib().nmg_norms(self._h, ctypes.c_void_p(u_ptr or None), _ptr(out)),
                    "nmg_norms")
        res = {"volume": out[0]}
        for l, name in enumerate(FIELDS):
            res[name] = dict(zip(("VolInt", "mean", "rms", "min", "max", "maxAbs"),
                                 out[1 + 6 * l: 7 + 6 * l]))
        return res

    def set_fv_surface_interp(self, mode="linear"):
        """Traces of finite-volume neighbours on DG faces: "linear" or
        "parabolic" (the reference's fv_surface_interp)."""
        self._check(lib().nmg_set_fv_surface_interp(self._h, {"linear": 0,
                                                              "parabolic": 1}[mode]),
                    "nmg_set_fv_surface_interp")

    def set_filter(self, on=True, alp=36.0, s=32.0, dn=0, jpower=1, filter_fv=True):
        """The reference's evolve_filter_all = yes (exponential modal filter
        after every step; defaults as the reference's parameters)."""
        self._check(lib().nmg_set_filter(self._h, int(bool(on)), float(alp), float(s), int(dn),
                                         int(jpower), int(bool(filter_fv))), "nmg_set_filter")

    def set_limiter(self, kind="MRS", alpha=5.0, beta=0.5, scale_bound=False):
        """The reference's scalarwave1_limiter ("none", "MRS" or "minmodB")
        with limiter_alpha (default 5), limiter_beta (minmodB, default 0.5)
        and limiter_scaleBound (minmodB, default no)."""
        k = {"none": 0, "MRS": 1, "minmodB": 2}[kind]
        self._check(lib().nmg_set_limiter_ex(self._h, k, float(alpha), float(beta),
                                             int(bool(scale_bound))), "nmg_set_limiter_ex")

    def limited(self):
        """Per element 1 if the last limiter call limited it."""
        out = np.zeros(self.shape[0], np.int32)
        self._check(lib().nmg_get_limited(self._h, _ptr(out)), "nmg_get_limited")
        return out

    def set_fv_midpoint_data(self, on=True):
        """The reference's coordinates_midpoint_data = yes: FV midpoint flux
        factors and normals from the map at the midpoints."""
        self._check(lib().nmg_set_fv_midpoint_data(self._h, int(bool(on))),
                    "nmg_set_fv_midpoint_data")

    def set_evolve_method(self, method="RK4"):
        """The reference's evolve_method ("RK4", "Euler", "sspRK3") used by
        evolve_steps / evolve_steps_host."""
        self._check(lib().nmg_set_evolve_method(self._h, EVOLVE_METHOD[method]),
                    "nmg_set_evolve_method")

    def evolve_steps(self, t, dt, nsteps):
        self._check(lib().nmg_evolve_steps(self._h, float(t), float(dt), int(nsteps)),
                    "nmg_evolve_steps")

    def evolve_steps_host(self, u, t, dt, nsteps):
        u = np.array(u, np.float64, copy=True, order="C")
        assert u.size == self.size
        self._check(lib().nmg_evolve_steps_host(self._h, float(t), float(dt), int(nsteps),
                                                _ptr(u)), "nmg_evolve_steps_host")
        return u

    def checkpoint_write(self, path, names=None):
        """Resident state -> the reference's checkpoint variables.bin."""
        p, keep = _names_arg(names)
        if lib().nmg_checkpoint_write(self._h, self.mesh._h, str(path).encode(), p):
            raise NmgError(lib().nmg_checkpoint_last_error().decode())

    def checkpoint_read(self, path, names=None):
        """Resident state <- the reference's checkpoint variables.bin."""
        p, keep = _names_arg(names)
        if lib().nmg_checkpoint_read(self._h, self.mesh._h, str(path).encode(), p):
            raise NmgError(lib().nmg_checkpoint_last_error().decode())

    # ---- DG <-> finite-volume switching ----
    def set_element_types(self, fv):
        """Switch element types (1: finite volume) converting the state."""
        f = np.ascontiguousarray(fv, np.int32)
        self._check(lib().nmg_set_element_types(self._h, _ptr(f)), "nmg_set_element_types")

    def element_types(self):
        f = np.zeros(self.mesh.nelem, np.int32)
        self._check(lib().nmg_get_element_types(self._h, _ptr(f)), "nmg_get_element_types")
        return f

    def trouble_check_device(self, u_ptr, u_p_ptr, params=None):
        """Trouble flags and Persson indicators of device state u_ptr against
        u_p_ptr (ints)."""
        tp = params or TroubleParams()
        fl = np.zeros(self.mesh.nelem, np.int32)
        pe = np.zeros((self.mesh.nelem, NFIELDS))
        self._check(lib().nmg_trouble_check(self._h, ctypes.c_void_p(u_ptr),
                                            ctypes.c_void_p(u_p_ptr), ctypes.byref(tp),
                                            _ptr(fl), _ptr(pe)), "nmg_trouble_check")
        return fl, pe

    def rk4_step_trouble(self, t, dt, params=None):
        """One RK4 step with trouble detection and element switching; returns
        (elements switched to FV, elements switched back to DG)."""
        tp = params or TroubleParams()
        sw = np.zeros(2, np.int32)
        self._check(lib().nmg_rk4_step_trouble(self._h, float(t), float(dt), ctypes.byref(tp),
                                               _ptr(sw)), "nmg_rk4_step_trouble")
        return int(sw[0]), int(sw[1])

    def trouble_scores(self):
        s_ = np.zeros(self.mesh.nelem, np.int32)
        self._check(lib().nmg_get_trouble_scores(self._h, _ptr(s_)), "nmg_get_trouble_scores")
        return s_

    def set_kernel(self, spec="auto"):
        """Force a stage-kernel variant ("eo", "gather", "tc",
        "<name>:<epb>:<threads>"), choose the transposed kernel of the
        adjoint ("vjp": FP64, "tcvjp": tensor cores, the default at
        n = 7..9), or re-enable the autotuner ("auto")."""
        self._check(lib().nmg_set_kernel(self._h, spec.encode()), "nmg_set_kernel")

    def kernel_info(self):
        buf = ctypes.create_string_buffer(4096)
        self._check(lib().nmg_kernel_info(self._h, ctypes.cast(buf, ctypes.c_void_p), 4096),
                    "nmg_kernel_info")
        return buf.value.decode()

    @property
    def launches(self):
        return int(lib().nmg_kernel_launches(self._h))

    @property
    def stream(self):
        return int(lib().nmg_stream(self._h) or 0)

    @property
    def state_ptr(self):
        return int(lib().nmg_state_device_ptr(self._h) or 0)

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().nmg_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Many independent problems stepped together (nmg_batch_*)."""

    def __init__(self, meshes, bc=BC_OUTGOING, k=(1.0, 1.0, 1.0), problems=None):
        """problems: per mesh a problem id; meshes of one problem are parts
        joined across their coinciding outer faces (their n may differ)."""
        self.meshes = list(meshes)
        arr = (ctypes.c_void_p * len(self.meshes))(*[m._h.value for m in self.meshes])
        kk = np.ascontiguousarray(k, np.float64)
        h = ctypes.c_void_p()
        if problems is None:
            rc = lib().nmg_batch_create(arr, len(self.meshes), int(bc), _ptr(kk), ctypes.byref(h))
        else:
            pr = np.ascontiguousarray(problems, np.int32)
            rc = lib().nmg_batch_create_linked(arr, len(self.meshes), _ptr(pr), int(bc), _ptr(kk),
                                               ctypes.byref(h))
        self._h = h
        if rc:
            msg = lib().nmg_batch_last_error(h).decode() if h.value else ""
            self.close()
            raise NmgError(f"nmg_batch_create failed ({rc}): {msg}")

    def _check(self, rc, what):
        if rc:
            raise NmgError(f"{what} failed ({rc}): {lib().nmg_batch_last_error(self._h).decode()}")

    def shape(self, p):
        m = self.meshes[p]
        return (m.nelem, NFIELDS, m.np)

    def set_state(self, p, u):
        u = np.ascontiguousarray(u, np.float64)
        assert u.size == lib().nmg_batch_problem_size(self._h, p)
        self._check(lib().nmg_batch_set_state(self._h, p, _ptr(u)), "nmg_batch_set_state")

    def get_state(self, p):
        u = np.zeros(self.shape(p))
        self._check(lib().nmg_batch_get_state(self._h, p, _ptr(u)), "nmg_batch_get_state")
        return u

    def rk4_steps(self, t, dt, nsteps):
        self._check(lib().nmg_rk4_steps_batched(self._h, float(t), float(dt), int(nsteps)),
                    "nmg_rk4_steps_batched")

    @property
    def linked_faces(self):
        return int(lib().nmg_batch_linked_faces(self._h))

    def set_mode(self, mode):
        """0 autotune, 1 persistent single launch, 2 one launch per order."""
        self._check(lib().nmg_batch_set_mode(self._h, int(mode)), "nmg_batch_set_mode")

    def info(self):
        buf = ctypes.create_string_buffer(8192)
        lib().nmg_batch_info(self._h, ctypes.cast(buf, ctypes.c_void_p), 8192)
        return buf.value.decode()

    @property
    def stream(self):
        return int(lib().nmg_batch_stream(self._h) or 0)

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().nmg_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _GrhdEvolveParams(ctypes.Structure):
    _fields_ = [("eos", GrhdParams), ("mass", ctypes.c_double), ("nf", ctypes.c_int32),
                ("rec", ctypes.c_int32)]


class GrhdEvolution:
    """GRHD in the Cowling approximation on a cubed-shell mesh
    (include/nmg.h nmg_grhd_*): DG elements on the mesh's LGL points,
    finite-volume elements on nf equally spaced points.  States on the host
    are (u_dg [E, 5, n^3], u_fv [nfv, 5, nf^3]) with the finite-volume rows
    in ascending element order."""

    def __init__(self, mesh, mass=1.0, gamma=2.0, rho_atm=1e-10, p_atm=1e-16, tol=1e-15,
                 maxits=100, nf=0, rec="WENOm5_2"):
        self.mesh = mesh
        p = _GrhdEvolveParams(GrhdParams(gamma, rho_atm, p_atm, tol, maxits), float(mass),
                              int(nf), FV_REC[rec])
        h = ctypes.c_void_p()
        rc = lib().nmg_grhd_create(mesh._h, ctypes.byref(p), ctypes.byref(h))
        self._h = h
        if rc:
            msg = lib().nmg_grhd_last_error(h).decode() if h.value else ""
            self.close()
            raise NmgError(f"nmg_grhd_create failed ({rc}): {msg}")
        n, nf_, E = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int64()
        lib().nmg_grhd_sizes(self._h, ctypes.byref(n), ctypes.byref(nf_), ctypes.byref(E))
        self.n, self.nf, self.nelem = n.value, nf_.value, E.value

    def _check(self, rc, what):
        if rc:
            raise NmgError(f"{what} failed ({rc}): {lib().nmg_grhd_last_error(self._h).decode()}")

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            lib().nmg_grhd_destroy(self._h)
        self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def nfv(self):
        return int(lib().nmg_grhd_fv_count(self._h))

    @property
    def stream(self):
        return lib().nmg_grhd_stream(self._h)

    def set_fv_elements(self, fv):
        fv = np.ascontiguousarray(fv, np.int32)
        self._check(lib().nmg_grhd_set_fv_elements(self._h, _ptr(fv)), "nmg_grhd_set_fv_elements")

    def trouble_indicators(self):
        """Persson's indicator of D per element (log10)."""
        ind = np.zeros(self.nelem)
        self._check(lib().nmg_grhd_trouble_indicators(self._h, _ptr(ind)),
                    "nmg_grhd_trouble_indicators")
        return ind

    def update_troubled(self, persson_max, back_margin=1.0):
        """Switch by the indicator; returns (to finite volume, to DG)."""
        sw = np.zeros(2, np.int32)
        self._check(lib().nmg_grhd_update_troubled(self._h, float(persson_max),
                                                   float(back_margin), _ptr(sw)),
                    "nmg_grhd_update_troubled")
        return int(sw[0]), int(sw[1])

    def fv_elements(self):
        fv = np.zeros(self.nelem, np.int32)
        self._check(lib().nmg_grhd_get_fv_elements(self._h, _ptr(fv)), "nmg_grhd_get_fv_elements")
        return fv

    def _shapes(self):
        return (self.nelem, 5, self.n ** 3), (self.nfv, 5, self.nf ** 3)

    def set_prim(self, prim_dg, prim_fv=None):
        sd, sf = self._shapes()
        pd = np.ascontiguousarray(np.broadcast_to(prim_dg, sd), np.float64)
        pf = np.ascontiguousarray(np.zeros(sf) if prim_fv is None else prim_fv, np.float64)
        self._check(lib().nmg_grhd_set_prim(self._h, _ptr(pd), _ptr(pf)), "nmg_grhd_set_prim")

    def set_state(self, u_dg, u_fv, prim_dg=None, prim_fv=None):
        sd, sf = self._shapes()
        arr = [np.ascontiguousarray(a, np.float64) if a is not None else None
               for a in (u_dg, u_fv, prim_dg, prim_fv)]
        ptrs = [_ptr(a) if a is not None else None for a in arr]
        self._check(lib().nmg_grhd_set_state(self._h, *ptrs), "nmg_grhd_set_state")

    def get_state(self):
        """(u_dg, u_fv, prim_dg, prim_fv)"""
        sd, sf = self._shapes()
        out = [np.zeros(sd), np.zeros(sf), np.zeros(sd), np.zeros(sf)]
        self._check(lib().nmg_grhd_get_state(self._h, *(_ptr(a) for a in out)),
                    "nmg_grhd_get_state")
        return tuple(out)

    def rhs(self):
        sd, sf = self._shapes()
        r_dg, r_fv = np.zeros(sd), np.zeros(sf)
        self._check(lib().nmg_grhd_rhs(self._h, _ptr(r_dg), _ptr(r_fv)), "nmg_grhd_rhs")
        return r_dg, r_fv

    def rk4_steps(self, dt, nsteps):
        self._check(lib().nmg_grhd_rk4_steps(self._h, float(dt), int(nsteps)),
                    "nmg_grhd_rk4_steps")

    def stats(self):
        """(con2prim iterations, atmosphere points, kernel launches)"""
        a, b, c = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        self._check(lib().nmg_grhd_stats(self._h, ctypes.byref(a), ctypes.byref(b),
                                         ctypes.byref(c)), "nmg_grhd_stats")
        return a.value, b.value, c.value

    def reset_stats(self):
        self._check(lib().nmg_grhd_reset_stats(self._h), "nmg_grhd_reset_stats")

    def profile_step(self, dt):
        """One RK4 step timed per kernel class: dict of milliseconds."""
        ms = np.zeros(4)
        self._check(lib().nmg_grhd_profile_step(self._h, float(dt), _ptr(ms)),
                    "nmg_grhd_profile_step")
        return dict(zip(("con2prim", "traces", "dg", "fv"), ms.tolist()))
