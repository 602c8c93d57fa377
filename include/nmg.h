/* nmg.h -- C ABI of the GB300-native nmesh evolution path (scalarwave1 DG
 * right-hand side, LLF face flux + lift, RK4 stage update), FP64 throughout.
 *
 * The reference plugs evolution in per element (EvoFuncPtr =
 * int (*)(tElm*, tEvoVars*), src/main/main/lists.h:20) inside OpenMP loops;
 * a GPU needs the whole mesh at once, so this boundary is taken at the mesh
 * level: one context owns the device mirror of every element and face of a
 * static mesh, and each call replaces one reference call over all elements.
 *
 * Conventions
 *  - All functions return 0 on success and a nonzero NMG_E* code otherwise
 *    (the reference's bin convention: 0 = fine); nmg_last_error() then
 *    describes the failure.  Nothing here exits or aborts.
 *  - State arrays are FP64, element-contiguous structure of arrays
 *    [element][field][node], node = i + n*(j + n*k) (the reference's Ind_n,
 *    src/main/amr/nmesh_amr_loops.h:279), fields in the reference's vlu order
 *    (pi, cx, cy, cz, phi) (src/tests/scalarwave1/scalarwave1.c:669-672).
 *  - One CUDA stream per context; a context is not re-entrant.
 */
#ifndef NMG_H
#define NMG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NMG_NFIELDS 5

/* error codes */
#define NMG_OK 0
#define NMG_EINVAL 1   /* bad argument */
#define NMG_ECUDA 2    /* CUDA runtime error */
#define NMG_EMESH 3    /* mesh is not conforming / cannot be packed */
#define NMG_ENOMEM 4   /* host or device allocation failed */
#define NMG_EUNSUP 5   /* unsupported configuration (e.g. n out of range) */

/* mesh types, as the reference's amr_mesh_type (src/main/amr/mesh.c:181) */
#define NMG_MESH_BOX 1           /* "1 BoxMesh": one Cartesian box patch */
#define NMG_MESH_CUBEDSPHERES7 7 /* "7 CubedSpheres": box + 6 cubed spheres */
#define NMG_MESH_CUBEDSHELL6 6   /* 6 cubed-sphere patches between two spheres
                                    (the reference's CubedShell map,
                                    src/main/coordinates/coordtrans_CubedSphere.c:
                                    84-92,236-245, with constant radii) */

/* outer-boundary treatment */
#define NMG_BC_EXACT_PLANEWAVE 0 /* exterior state = exact plane wave
                                    (scalarwave1.c:182-204) */
#define NMG_BC_OUTGOING 1        /* outgoing radiation: no incoming
                                    characteristic (no reference counterpart) */

/* numerical flux, the reference's par scalarwave1_numflux
 * (src/tests/scalarwave1/scalarwave1.c:701-704; its default is upwind) */
#define NMG_NUMFLUX_LLF 0    /* "LLF": numflux1d_LLF (src/main/dg/numflux1d.c:85) */
#define NMG_NUMFLUX_UPWIND 1 /* scalarwave1_numflux1d_upwind (scalarwave1.c:323) */

/* finite-volume reconstruction at the midpoints, the reference's par fv_rec
 * (src/main/dg/dg.c:286-330, rec1d.c) */
#define NMG_FV_REC_1 0        /* "1": first order (rec1d_p_1 / rec1d_m_1) */
#define NMG_FV_REC_WENOM3_2 1 /* "WENOm3_2" (reference default) */
#define NMG_FV_REC_WENOM5_2 2 /* "WENOm5_2": WENO5 inside, WENOm3_2 near ends */
#define NMG_FV_REC_WENOMZ_2 3 /* "WENOmZ_2": WENO-Z inside, WENOm3_2 near ends
                                 (rec1d_p/m_WENOmZ_2, rec1d.c:1627-1796) */
/* how div(f) is completed on face points, the reference's par fv_divf_extrap
 * (src/main/dg/dg.c:341-361) */
#define NMG_FV_EXTRAP_NO 0    /* "no": face fluxes weighted by 1/|distXb| */
#define NMG_FV_EXTRAP_DNFN1 1 /* "dnfn_extrap1" (reference default) */

typedef struct nmg_mesh nmg_mesh; /* host-side packed mesh */
typedef struct nmg_ctx nmg_ctx;   /* device context; owns all device memory */

/* Parameters of a generated mesh, named after the reference's parameters
 * (src/main/amr/mesh.c:181-250,350-445,447-622). */
typedef struct nmg_mesh_params {
  int32_t mesh_type;  /* NMG_MESH_BOX or NMG_MESH_CUBEDSPHERES7 */
  int32_t n;          /* LGL nodes per direction (amr_n0 = amr_n1 = amr_n2) */
  int32_t luni;       /* uniform refinement level (amr_luni) */
  int32_t periodic;   /* box only: opposite outer faces are neighbours */
  double xc[3];       /* amr_mesh_xc */
  double box_dout;    /* amr_BoxMesh_dout: half edge of the box */
  double cs_dc;       /* amr_CubedSphere_dc: half edge of the inner cube */
  double cs_r0fac;    /* amr_CubedSphere_r0fac: outer radius / dc */
  int32_t fv;         /* bit p set: the elements of patch p are
                         finite-volume elements on equally spaced points
                         (amr_uniform_p and amr_fv_p list patch p,
                         src/main/amr/mesh.c:35-83); -1: every patch; 0: DG */
  int32_t hrefine;    /* bit p set: patch p is refined one level further
                         (amr_hrefine_p, src/main/amr/mesh.c:269-284); its
                         faces against other patches are non-conforming */
  int32_t sphere_levels; /* amr_hrefine_sphere_levels: nested spheres about
                            x = 0 in which elements are refined further
                            (hrefine_sphere_loadbalance, src/main/amr/
                            refine.c:1087-1100); 0: none */
  double sphere_radius;  /* amr_hrefine_sphere_radius: innermost radius (the
                            reference reads it as an integer) */
  int32_t ndiv;          /* > 0: every patch split into ndiv^3 equal elements
                            (instead of 2^luni per direction); 0: luni */
  double shell_rin, shell_rout; /* NMG_MESH_CUBEDSHELL6: inner and outer radius */
  int32_t patch_mask;    /* bit p set: build only the elements of patch p
                            (0: every patch); faces towards the patches left
                            out are outer faces of this mesh.  Parts of one
                            mesh with different n are joined again by
                            nmg_batch_create_linked (p-refinement by patch,
                            the reference's amr_prefine_p) */
} nmg_mesh_params;

/* A mesh given element by element, e.g. packed from the reference's tMesh
 * by an adapter (elm->bbox, elm->n, pat->dXYZ_dxyz != NULL, the x/y/z and
 * dXdx variables of coordinates_init_node, src/main/coordinates/
 * coordinates.c:133-224). */
typedef struct nmg_mesh_desc {
  int32_t nelem;
  int32_t n;              /* LGL nodes per direction, same in all elements */
  const int32_t *pat;     /* [nelem] patch index (informational) */
  const double *bbox;     /* [nelem][6] element bbox in patch coordinates */
  const int32_t *curvi;   /* [nelem] 1 if the patch map is not Cartesian */
  const double *xyz;      /* [nelem][3][n^3] Cartesian coordinates */
  const double *dXdx;     /* [nelem][9][n^3] dX^a/dx^i, a-major; read for
                             curvi elements only; may be NULL if none */
  const int64_t *nbnode;  /* [nelem][6][n*n] global index e'*n^3+ijk' of the
                             coincident node across each face node, -1 on
                             outer faces; NULL: matched from coordinates */
  double period[3];       /* >0: coordinates compared modulo period when
                             matching (periodic box); 0 otherwise */
  const int32_t *fv;      /* [nelem] node->dat->info->use_fv (elements on
                             equally spaced points), or NULL: all DG.  Faces
                             between a DG and a finite-volume element are
                             found from coordinates (nbnode must be NULL
                             then) and get interpolated traces. */
} nmg_mesh_desc;

/* ---- host mesh ---------------------------------------------------------- */
int nmg_mesh_build(const nmg_mesh_params *p, nmg_mesh **out);
int nmg_mesh_from_desc(const nmg_mesh_desc *d, nmg_mesh **out);
int64_t nmg_mesh_nelem(const nmg_mesh *m);
int32_t nmg_mesh_n(const nmg_mesh *m);
/* copies out [nelem] patch indices and [nelem][6] bboxes */
int nmg_mesh_get_elements(const nmg_mesh *m, int32_t *pat, double *bbox);
/* copies out [nelem][3][n^3] Cartesian coordinates */
int nmg_mesh_get_coords(const nmg_mesh *m, double *xyz);
/* copies out [nelem][9][n^3] dX^a/dx^i (identity on Cartesian elements) */
int nmg_mesh_get_dXdx(const nmg_mesh *m, double *dXdx);
/* copies out the face table: [nelem][6] neighbour element (-1 outer) and
   [nelem][6] code = neighbour face | orientation << 3 */
int nmg_mesh_get_faces(const nmg_mesh *m, int32_t *nb, int32_t *code);
/* copies out [nelem] finite-volume flags (1: element on uniform points) */
int nmg_mesh_get_fv(const nmg_mesh *m, int32_t *fv);
/* LGL nodes and weights on [-1,1] and D[i*n+j] = l_j'(x_i)
   (src/main/basis/Legendre.c:149-213, Lagrange.c:126-147) */
int nmg_basis(int32_t n, double *x, double *w, double *D);
/* Non-conforming faces of the mesh (patches at different levels): counts,
 * and if the arrays are given, per face (element, face) [nface][2], per face
 * node the offsets of its contributions [nface*n*n + 1], per contribution
 * the source (element, face) [ncontrib][2] and the node's position on the
 * source face in its in-plane coordinates [ncontrib][2].  A face node's
 * trace is the average of its contributions (set_ajsurf_vl,
 * src/main/amr/surface.c:799-1360). */
int nmg_mesh_get_hanging(const nmg_mesh *m, int64_t *nface, int64_t *ncontrib, int32_t *hface,
                         int32_t *hoff, int32_t *hsrc, double *hpos);
/* [nelem][3][9][n^3]: dX^a/dx^i at the midpoints between the equally spaced
 * points (coordinates_midpoint_data, src/main/coordinates/coordinates.c:
 * 283-375): block d at node (i,j,k) holds the value at the midpoint to the
 * right of that node in direction d (last plane unused); generated meshes */
int nmg_mesh_get_midpoint_dXdx(const nmg_mesh *m, double *dXdxm);
/* the reference's dt = auto (dtfac, default 0.25, and uniform_dtfac, default
 * 0.125 on finite-volume elements, times the smallest corner spacing;
 * src/main/amr/storage.c:1305-1385, src/main/coordinates/utilities.c:
 * 972-1300) */
int nmg_mesh_auto_dt(const nmg_mesh *m, double dtfac, double uniform_dtfac, double *dt);
/* equally spaced points on [-1,1] (uniform_x, src/main/basis/Legendre.c:626) */
int nmg_uniform_points(int32_t n, double *x);
void nmg_mesh_free(nmg_mesh *m);
const char *nmg_mesh_last_error(void);

/* ---- device context ----------------------------------------------------- */
/* Uploads the mesh (metric, face factors, face table) and allocates the RK4
 * state (u, u accumulator, two stage buffers) on the current CUDA device.
 * bc_kind: NMG_BC_*; k: plane-wave vector for NMG_BC_EXACT_PLANEWAVE. */
int nmg_create(const nmg_mesh *m, int32_t bc_kind, const double k[3],
               nmg_ctx **out);
void nmg_destroy(nmg_ctx *c);
const char *nmg_last_error(const nmg_ctx *c);
int64_t nmg_state_size(const nmg_ctx *c); /* doubles per state */

/* u <-> host ([element][field][node] FP64); a copy to/from HBM */
int nmg_set_state(nmg_ctx *c, const double *host_u);
int nmg_get_state(nmg_ctx *c, double *host_u);
/* device pointer of the resident state u (for zero-copy use) */
double *nmg_state_device_ptr(nmg_ctx *c);

/* A context whose elements can switch between DG (LGL points) and finite
 * volume (equally spaced points) while it runs: both geometries of every
 * element are kept, and every RK4 stage runs the interface-trace, DG and
 * finite-volume kernels.  The mesh must be generated (nmg_mesh_build) or
 * have Cartesian elements only. */
int nmg_create_switchable(const nmg_mesh *m, int32_t bc_kind, const double k[3],
                          nmg_ctx **out);
/* switch element types (fv[e] = 1: finite volume) and convert the resident
 * state of the switched elements: LGL -> equally spaced points by Lagrange
 * interpolation, back by its inverse (the reference's p-refinement between
 * P_LGL and P_UNIFORM, src/main/basis/gridpoints.c:158-317) */
int nmg_set_element_types(nmg_ctx *c, const int32_t *fv);
int nmg_get_element_types(nmg_ctx *c, int32_t *fv);

/* Trouble detection for the scalar wave: an element is troubled when a
 * field leaves the relaxed discrete maximum principle bounds of the previous
 * state over the element and its face neighbours (evolve_RDMP_trouble,
 * src/main/evolve/trouble.c:438-503) or, on a DG element, when Persson's
 * modal indicator of a field exceeds persson_max
 * (evolve_Persson_array_indicator, trouble.c:505-564). */
typedef struct nmg_trouble_params {
  double rdmp_deltafac, rdmp_delta0, rdmp_epsilon;  /* evolve_RDMP_trouble args */
  double persson_max;      /* log10 indicator threshold (large: off) */
  double persson_uscale;   /* u_scale of the indicator (< 0: keep c_0) */
  int32_t notroubles;      /* quiet steps before switching back to DG
                              (NOTROUBLES = 11, src/main/evolve/evolve.h:60) */
  int32_t redo;            /* NMG_REDO_STEP or NMG_REDO_SUBSTEP (the
                              parameter evolve_redo_troubled) */
} nmg_trouble_params;
/* evolve_redo_troubled = step: detect after the whole RK4 step, go back to
 * u_p, switch, redo the step; = substep (the reference's default): detect
 * after every RK4 substep and redo that substep on the troubled elements
 * (evolve_trouble_redo_u_step_mesh, src/main/evolve/RungeKutta.c:19-80,
 * 221-330); quiet elements then switch back after notroubles * 4 substeps
 * (evolve_notroubles, RungeKutta.c:206-211) */
#define NMG_REDO_STEP 0
#define NMG_REDO_SUBSTEP 1
/* flags[e]: DG troubled 1, DG fine 0, FV troubled 0, FV fine -1 (the
 * reference's TROUBLE return convention, trouble.c:17-26) for state u_dev
 * against u_p_dev; persson[E][5] (may be NULL): the indicators (0 on FV) */
int nmg_trouble_check(nmg_ctx *c, const double *u_dev, const double *u_p_dev,
                      const nmg_trouble_params *tp, int32_t *flags, double *persson);
/* One RK4 step of the resident state with trouble detection and element
 * switching (evolve_mesh, src/main/evolve/evolve.c:74-140, with
 * evolve_redo_troubled = tp->redo: the whole step redone, or each troubled
 * substep redone on the troubled elements); switched[0] = elements switched
 * to FV, switched[1] = elements switched back to DG */
int nmg_rk4_step_trouble(nmg_ctx *c, double t, double dt, const nmg_trouble_params *tp,
                         int32_t *switched);
int nmg_get_trouble_scores(nmg_ctx *c, int32_t *scores);

/* 0d norms of a state on the device (the ingredients of output0d_mesh_vl,
 * src/utility/output/output0d.c:44-176, with the volume integrals of
 * MeshVolumeIntegral / NodeVolumeIntegral, src/main/main/norms.c:10-28,
 * src/main/coordinates/integrals.c:12-60): out[0] = volume, then per field
 * (pi, cx, cy, cz, phi) VolInt, mean, rms, min, max, maxAbs (31 doubles).
 * u_dev NULL: the resident state.  Only the 31 numbers leave the GPU. */
int nmg_norms(nmg_ctx *c, const double *u_dev, double *out);

/* ---- other time integrators of the reference ----------------------------
 * The reference's evolve_method = Euler or sspRK3 (evolve_Euler_mesh,
 * evolve_sspRK3_mesh, src/main/evolve/RungeKutta.c:84-200) besides RK4:
 * nmg_set_evolve_method picks the integrator of nmg_evolve_steps(_host),
 * which step the resident state like nmg_rk4_steps (graph-captured steps,
 * step times accumulated as evolve_mesh does).  The nmg_rk4_* entry points
 * always use RK4. */
#define NMG_EVOLVE_RK4 0
#define NMG_EVOLVE_EULER 1
#define NMG_EVOLVE_SSPRK3 2
int nmg_set_evolve_method(nmg_ctx *c, int32_t method);
int nmg_evolve_steps(nmg_ctx *c, double t, double dt, int32_t nsteps);
int nmg_evolve_steps_host(nmg_ctx *c, double t, double dt, int32_t nsteps, double *host_u);

/* ---- checkpoints in the reference's variable file format ---------------
 * The state as the reference's checkpoint "variables.bin"
 * (checkpoint_save_EvoVars / checkpoint_load_Vars,
 * src/main/checkpoint/checkpoint_save.c:335-470, checkpoint_load.c:397),
 * matched by element name ("<patch>_<octree digits>", known for generated
 * meshes; names[e] given otherwise, NULL for a generated mesh) and variable
 * name (scalarwave1_pi, _cx, _cy, _cz, _phi).  A GPU run restarts from a
 * reference checkpoint with nmg_checkpoint_read, and the reference restarts
 * from a checkpoint directory whose variables.bin nmg_checkpoint_write
 * produced (its CRC.txt vars entry then no longer matches: a warning). */
int nmg_checkpoint_write(nmg_ctx *c, const nmg_mesh *m, const char *path,
                         const char *const *names);
int nmg_checkpoint_read(nmg_ctx *c, const nmg_mesh *m, const char *path,
                        const char *const *names);
/* the same with a host state [element][field][node] */
int nmg_checkpoint_write_host(const nmg_mesh *m, const double *u, const char *path,
                              const char *const *names);
int nmg_checkpoint_read_host(const nmg_mesh *m, const char *path, double *u,
                             const char *const *names);
const char *nmg_checkpoint_last_error(void);
/* the reference's name of mesh element e (NULL for a described mesh) */
const char *nmg_mesh_element_name(const nmg_mesh *m, int64_t e);

/* ---- GRHD: pointwise conservative <-> primitive conversion ---------------
 * Ideal gas on a conformally flat 3-metric gamma_ij = psi^4 delta_ij; no
 * counterpart in the reference (its GRHD is external), except the root
 * finder newton1d_brak (src/utility/numerics/newton1d_brak.c:20-121).
 * Arrays are device SoA [5][npts]: conserved (D, S_1, S_2, S_3, tau)
 * densitized by psi^6, primitives (rho, v^1, v^2, v^3, p); psi may be NULL
 * (flat).  con2prim uses prim[4] as the starting pressure, writes status
 * (iterations >= 0, or < 0 where the atmosphere was set and the conserved
 * variables reset), and runs on `stream` (a cudaStream_t, NULL: default). */
typedef struct nmg_grhd_params {
  double gamma;    /* adiabatic index of p = (gamma - 1) rho eps */
  double rho_atm;  /* atmosphere density (floor of D / psi^6) */
  double p_atm;    /* atmosphere pressure */
  double tol;      /* relative pressure accuracy of the root finder */
  int32_t maxits;  /* iteration limit of the root finder */
} nmg_grhd_params;
int nmg_grhd_prim2con(const nmg_grhd_params *g, int64_t npts, const double *psi_dev,
                      const double *prim_dev, double *cons_dev, void *stream);
int nmg_grhd_con2prim(const nmg_grhd_params *g, int64_t npts, const double *psi_dev,
                      double *cons_dev, double *prim_dev, int32_t *status_dev, void *stream);
/* Valencia fluxes along direction dir of the densitized conserved variables
 * (flux [5][npts]) and the characteristic speeds (lam [2][npts]: lambda_-,
 * lambda_+) on the static background ds^2 = -alpha^2 dt^2 + psi^4 dx^2
 * (alpha, psi may be NULL: 1) */
int nmg_grhd_fluxes(const nmg_grhd_params *g, int64_t npts, int32_t dir, const double *alpha_dev,
                    const double *psi_dev, const double *prim_dev, double *flux_dev,
                    double *lam_dev, void *stream);
/* Cowling source terms [5][npts] (0 for D) from alpha, psi and their
 * gradients dalpha, dpsi [3][npts] */
int nmg_grhd_sources(const nmg_grhd_params *g, int64_t npts, const double *alpha_dev,
                     const double *psi_dev, const double *dalpha_dev, const double *dpsi_dev,
                     const double *prim_dev, double *src_dev, void *stream);

/* ---- GRHD evolution in the Cowling approximation ------------------------
 * No counterpart in the reference (its GRHD is external; parity unpinned,
 * checked against the oracle's restatement).  Densitized conserved fields
 * (D, S_1, S_2, S_3, tau) on a fixed isotropic Schwarzschild background of
 * mass `mass` (psi = 1 + M/(2r), alpha = (1 - M/(2r))/(1 + M/(2r)), zero
 * shift; mass 0: flat), on an NMG_MESH_CUBEDSHELL6 mesh.  DG elements use
 * the mesh's n LGL points: strong-form divergence with the chain rule
 * (src/main/coordinates/derivs.c:102-181,756-815), LLF face flux and lift
 * (src/main/dg/numflux1d.c:85-112, src/main/dg/dg.c:30-151), Cowling
 * sources.  Elements in finite-volume mode use nf equally spaced points
 * (nf = 0: 2n, the reference's PARENT_2n_P_UNIFORM, src/main/amr/refine.h:
 * 32): primitives reconstructed at the midpoints (rec, NMG_FV_REC_*,
 * src/main/dg/rec1d.c), LLF midpoint fluxes, conservative differences.
 * Every stage runs con2prim (newton1d_brak, atmosphere floors) on its input.
 * Outer faces (r_in, r_out) copy the interior state.  Host layouts: DG
 * [nelem][5][n^3], finite volume [nfv][5][nf^3] for the finite-volume
 * elements in ascending order.  At n = 7, 8, 9 the DG elements' line
 * derivatives run on the tensor cores (exact digit products); the
 * environment variable NMG_GRHD_DG=fp64, read at creation, keeps them in
 * FP64. */
typedef struct nmg_grhd_evolve_params {
  nmg_grhd_params eos;
  double mass;   /* background mass M (>= 0) */
  int32_t nf;    /* finite-volume points per direction (0: 2n; 4..16) */
  int32_t rec;   /* NMG_FV_REC_* midpoint reconstruction */
} nmg_grhd_evolve_params;
typedef struct nmg_grhd_ctx nmg_grhd_ctx;
int nmg_grhd_create(const nmg_mesh *m, const nmg_grhd_evolve_params *p, nmg_grhd_ctx **out);
void nmg_grhd_destroy(nmg_grhd_ctx *c);
const char *nmg_grhd_last_error(const nmg_grhd_ctx *c);
int nmg_grhd_sizes(const nmg_grhd_ctx *c, int32_t *n, int32_t *nf, int64_t *nelem);
/* element modes (fv[e] = 1: finite volume) with the state transferred
 * (trouble.c:162-183, gridpoints.c:158-200): to finite volume by Lagrange
 * interpolation P from the LGL points to the nf equally spaced points in
 * each direction, back by the pseudo-inverse R = (P^T P)^-1 P^T */
int nmg_grhd_set_fv_elements(nmg_grhd_ctx *c, const int32_t *fv);
int nmg_grhd_get_fv_elements(nmg_grhd_ctx *c, int32_t *fv);
/* Persson's modal indicator of D per element (evolve_Persson_array_indicator,
 * src/main/evolve/trouble.c:505-564): log10 of the share of the squared
 * normalised Legendre coefficients in the highest modes, on the LGL points
 * (a finite-volume element's state projected back by R x R x R first);
 * ind[nelem] on the host */
int nmg_grhd_trouble_indicators(nmg_grhd_ctx *c, double *ind);
/* DG elements whose indicator exceeds persson_max switch to finite volume,
 * finite-volume elements whose indicator fell below persson_max -
 * back_margin switch back (the state transferred as nmg_grhd_set_fv_elements
 * does); switched[0] / [1] (may be NULL): elements switched to FV / to DG */
int nmg_grhd_update_troubled(nmg_grhd_ctx *c, double persson_max, double back_margin,
                             int32_t *switched);
int64_t nmg_grhd_fv_count(const nmg_grhd_ctx *c);
/* state from primitives (rho, v^1, v^2, v^3, p) (U = prim2con; the
 * primitives are also the root finder's starting guesses) */
int nmg_grhd_set_prim(nmg_grhd_ctx *c, const double *prim_dg, const double *prim_fv);
/* conserved state in/out, with the primitives (guesses; may be NULL) */
int nmg_grhd_set_state(nmg_grhd_ctx *c, const double *u_dg, const double *u_fv,
                       const double *prim_dg, const double *prim_fv);
int nmg_grhd_get_state(nmg_grhd_ctx *c, double *u_dg, double *u_fv, double *prim_dg,
                       double *prim_fv);
/* r = RHS of the resident state after its con2prim (which, as in the first
 * stage of a step, may reset atmosphere points of the state) */
int nmg_grhd_rhs(nmg_grhd_ctx *c, double *r_dg, double *r_fv);
/* nsteps RK4 steps (RungeKutta.c:19-82), graph-captured */
int nmg_grhd_rk4_steps(nmg_grhd_ctx *c, double dt, int32_t nsteps);
/* root-finder iterations and atmosphere points summed over every con2prim
 * since the last reset, and the kernels launched */
int nmg_grhd_stats(nmg_grhd_ctx *c, int64_t *c2p_iterations, int64_t *atmosphere_points,
                   int64_t *launches);
int nmg_grhd_reset_stats(nmg_grhd_ctx *c);
/* one RK4 step, launched stage by stage with CUDA events around each kernel
 * class: ms[0] con2prim, ms[1] DG / finite-volume traces, ms[2] DG
 * elements, ms[3] finite-volume elements (milliseconds, summed over the
 * four stages) */
int nmg_grhd_profile_step(nmg_grhd_ctx *c, double dt, double *ms);
void *nmg_grhd_stream(nmg_grhd_ctx *c);

/* numerical flux of a context (default NMG_NUMFLUX_LLF, what the workloads
 * use); the adjoint entry points support LLF only */
int nmg_set_numflux(nmg_ctx *c, int32_t kind);

/* Finite-volume options of a context whose mesh is finite-volume: the
 * reference's DG globals fv_rec, fv_divf_extrap and
 * fv_WENOm3_opt_weightratio (src/main/dg/dg.c:286-400; defaults WENOm3_2,
 * dnfn_extrap1, 2).  NMG_EUNSUP on a DG context. */
int nmg_set_fv(nmg_ctx *c, int32_t rec, int32_t extrap, double w3ratio);
/* traces of finite-volume neighbours on DG faces, the reference's par
 * fv_surface_interp (src/main/dg/dg.c:369-379, basis_pw_linear /
 * basis_pw_parab in set_ajsurf_vl, src/main/amr/surface.c:1200-1240) */
#define NMG_FV_SURF_LINEAR 0    /* "linear" (reference default) */
#define NMG_FV_SURF_PARABOLIC 1 /* "parabolic" */
int nmg_set_fv_surface_interp(nmg_ctx *c, int32_t mode);
/* the reference's par coordinates_midpoint_data = yes (on != 0): the
 * finite-volume flux factors J sqrtgdiag of the midpoints and the normals of
 * the midpoint fluxes come from the map at the midpoints (fv.c:384-411,
 * coordinates.c:283-437) instead of the grid points; generated meshes */
int nmg_set_fv_midpoint_data(nmg_ctx *c, int32_t on);
/* the reference's evolve_filter_all = yes: after every step each field of
 * every element is filtered, u -> J^-p F(J^p u) with the exponential modal
 * filter c_ijk -> c_ijk f_i f_j f_k, f_k = exp(-alp (k/(n-1-dn))^s)
 * (expfilter_var, src/main/basis/filter.c:15-96; pars evolve_filter_alp,
 * _s, _dn, basis_expfilter_JacobianPower = p (0 or 1), basis_filter_fv;
 * evolve_filter_evosys_mesh, src/main/evolve/evolve.c:656-700).  on = 0
 * switches it off.  Applied by the step entry points (nmg_rk4_step(s),
 * nmg_evolve_steps, the host round trips, nmg_rk4_step_trouble,
 * nmg_rk4_step_noalloc); not by the adjoint and the batches. */
/* The reference's scalarwave1_limiter (src/tests/scalarwave1/scalarwave1.c:
 * 687-697) with limiter_alpha, limiter_beta and limiter_scaleBound, applied
 * as evolve_limiter_mesh does: to w before every later stage, RungeKutta.c:
 * 45-67,161,173, and to the new u after the step, evolve.c:143-144.
 *   MRS (limdata_MRS / limiter_MRS, src/main/limiter/limiter.c:61-204): per
 * element theta = min(1, min over fields of phi((M - wbar) / (wM - wbar)),
 * phi(y) = min(y/1.1, 1) (0 for y < 0), with M the neighbours' extrema
 * widened to wbar +- alpha h^1.5) and u <- wbar + theta (u - wbar).
 *   minmodB (limdata_c000_100_010_001 / limiter_minmodB, limiter.c:201-380):
 * per element and field the normalised-Legendre coefficients c000, c100,
 * c010, c001; the face averages w0[f] (mean c000 of the neighbours across
 * face f, 0 on outer faces); slopes limited by minmod3B(c100, beta/sqrt3
 * (c000 - w0[0]), beta/sqrt3 (w0[1] - c000), bound) (likewise in y, z) with
 * bound = alpha h (times the mean |w0[f]| if scale_bound); a field whose
 * slopes move by more than 1e-10 becomes c000 plus the limited linear modes.
 * kind: NMG_LIMITER_NONE, NMG_LIMITER_MRS or NMG_LIMITER_MINMODB;
 * nmg_set_limiter takes beta = 0.5 and scale_bound = 0 (the reference's
 * defaults).  Applied by nmg_rk4_step(s), nmg_evolve_steps, the host round
 * trips and nmg_rk4_step_noalloc; the trouble flow and the adjoint reject a
 * context with the limiter on (NMG_EUNSUP).
 * nmg_get_limited: per element 1 if the last limiter call limited it. */
#define NMG_LIMITER_NONE 0
#define NMG_LIMITER_MRS 1
#define NMG_LIMITER_MINMODB 2
int nmg_set_limiter(nmg_ctx *c, int32_t kind, double alpha);
int nmg_set_limiter_ex(nmg_ctx *c, int32_t kind, double alpha, double beta,
                       int32_t scale_bound);
int nmg_get_limited(nmg_ctx *c, int32_t *limited);

int nmg_set_filter(nmg_ctx *c, int32_t on, double alp, double s, int32_t dn, int32_t jpower,
                   int32_t filter_fv);

/* r = RHS(w, t) with w, r device pointers of nmg_state_size() doubles.
 * Replaces evolve_setrhs_mesh (src/main/evolve/evolve.c:182-232) for the
 * scalarwave1 VOLRHS+SURFRHS bins. */
int nmg_rhs(nmg_ctx *c, double t, const double *w_dev, double *r_dev);
/* same with host buffers: copies w in, computes, copies r out */
int nmg_rhs_host(nmg_ctx *c, double t, const double *w_host, double *r_host);

/* One classic RK4 step of the resident state u from t to t+dt
 * (evolve_RK4_mesh, src/main/evolve/RungeKutta.c:19-82). */
int nmg_rk4_step(nmg_ctx *c, double t, double dt);
/* nsteps RK4 steps; step s starts at the time accumulated as the reference's
 * evolve_mesh does (src/main/main/main.c:610-626).  The 4*nsteps stage
 * launches are captured once into a CUDA graph and replayed. */
int nmg_rk4_steps(nmg_ctx *c, double t, double dt, int32_t nsteps);
/* host round trip: set u from host, nsteps RK4 steps, copy u back */
int nmg_rk4_steps_host(nmg_ctx *c, double t, double dt, int32_t nsteps,
                       double *host_u);

/* ---- batched execution of many independent problems --------------------- */
/* The reference runs one mesh per process; these run many independent
 * problems (each its own mesh and order n in [2,10]) together.  Problems of
 * the same order are merged into one mesh (nmg_mesh_concat); one persistent
 * kernel launch per RK4 stage walks the element tiles of all orders
 * (runtime dispatch to the order's kernel body, highest order first), and
 * one RK4 step (4 launches + a step counter) is captured in a CUDA graph.
 * The persistent grid size is chosen by timing (autotuner).  All problems
 * share t, dt and the boundary kind. */
typedef struct nmg_batch nmg_batch;
int nmg_mesh_concat(const nmg_mesh *const *meshes, int32_t count, nmg_mesh **out);
int nmg_batch_create(const nmg_mesh *const *meshes, int32_t count, int32_t bc_kind,
                     const double k[3], nmg_batch **out);
/* The same, with meshes that are parts of one problem: meshes with equal
 * problem[i] are joined across their coinciding outer faces (all four
 * corners coincide; the parts may have different n, each face between them
 * is then p-nonconforming).  A face node's exterior state is the
 * neighbour part's face plane interpolated at the node's position (Lagrange
 * in both in-plane directions), as set_ajsurf_vl's interpolation branch
 * does (src/main/amr/surface.c:900-1460), filled by one launch per stage for
 * every such face of the batch.  States stay per part (mesh index). */
int nmg_batch_create_linked(const nmg_mesh *const *meshes, int32_t count, const int32_t *problem,
                            int32_t bc_kind, const double k[3], nmg_batch **out);
/* number of faces joined across parts (each side counted) */
int64_t nmg_batch_linked_faces(const nmg_batch *b);
void nmg_batch_destroy(nmg_batch *b);
const char *nmg_batch_last_error(const nmg_batch *b);
int64_t nmg_batch_problem_size(const nmg_batch *b, int32_t p); /* doubles of problem p */
int nmg_batch_set_state(nmg_batch *b, int32_t p, const double *host_u);
int nmg_batch_get_state(nmg_batch *b, int32_t p, double *host_u);
/* nsteps RK4 steps of every problem (== evolve_RK4_mesh on each mesh) */
int nmg_rk4_steps_batched(nmg_batch *b, double t, double dt, int32_t nsteps);
int nmg_batch_info(nmg_batch *b, char *buf, int32_t len);
/* 0: the autotuner chooses (default); 1: persistent single launch only;
   2: one launch per order (each with its order's tuned kernel variant) */
int nmg_batch_set_mode(nmg_batch *b, int32_t mode);
void *nmg_batch_stream(nmg_batch *b);

/* ---- adjoint (vector-Jacobian products) --------------------------------- */
/* The reference has no adjoint; these are the hand-written transposes of
 * the RHS and of the RK4 step above.  The scalar-wave RHS is linear in w, so
 * wbar = (dRHS/dw)^T rbar does not depend on w (w_dev may be NULL) and the
 * exterior plane-wave data (constant in w) drops out.  Non-conforming faces
 * are transposed too (their lists are built on the first adjoint call);
 * finite-volume contexts are rejected (NMG_EUNSUP).
 *   nmg_rhs_vjp:       wbar_dev = J^T rbar_dev (device buffers, distinct)
 *   nmg_rk4_step_vjp:  ubar_dev <- (du_{n+1}/du_n)^T ubar_dev, in place; the
 *                      step Jacobian is the RK4 polynomial of dt L, so this is
 *                      an RK4 step of the transposed operator (u_n unused).
 *   nmg_adjoint_gradient: for u0 = the context's current state,
 *                      J = sum_{s=1..nsteps} dt sum_nodes W phi(t_s)^2
 *                      (weight_dev: [nelem][n^3] doubles) and grad_dev =
 *                      dJ/du0 (nmg_state_size() doubles), by the discrete
 *                      adjoint of the trajectory with u checkpointed every
 *                      ckpt_every steps and recomputed segment by segment in
 *                      the reverse sweep (device memory for nsteps/ckpt_every
 *                      + max(ckpt_every,2) + 2 states is allocated per call). */
int nmg_rhs_vjp(nmg_ctx *c, double t, const double *w_dev, const double *rbar_dev,
                double *wbar_dev);
int nmg_rk4_step_vjp(nmg_ctx *c, double t, double dt, const double *u_n_dev, double *ubar_dev);
int nmg_adjoint_gradient(nmg_ctx *c, double t0, double dt, int32_t nsteps, int32_t ckpt_every,
                         const double *weight_dev, double *J, double *grad_dev);

/* ---- allocation-free step ----------------------------------------------- */
/* No counterpart in the reference.  For callers that cannot call cudaMalloc
 * while they step (device memory owned by their own pool or a framework
 * allocator, regions where the memory footprint must not grow): one RK4
 * step from u_in_dev to u_out_dev (distinct device buffers of
 * nmg_state_size() doubles) that allocates nothing.  Its two stage buffers
 * live in one static device array of 2 x NMG_NOALLOC_MAX_STATE doubles
 * (32 MiB) that every GPU loading this library holds until exit; larger
 * states are rejected with NMG_EINVAL.  The first call on a device looks up
 * that array (cudaGetSymbolAddress) and should come before any stream
 * capture.  All calls share the array: calls that overlap on the GPU race.
 * Nothing in it needs to start at zero.  The step is nmg_rk4_step's,
 * including the context's limiter and filter.  The context's device must be
 * current (NMG_EINVAL otherwise).  Waits for the step to finish. */
#define NMG_NOALLOC_MAX_STATE 2097152
int nmg_rk4_step_noalloc(nmg_ctx *c, double t, double dt, const double *u_in_dev,
                         double *u_out_dev);

/* ---- kernel selection (autotuner) --------------------------------------- */
/* The first RHS/RK4 call of a context times every compiled variant of the
 * stage kernel ("eo": even-odd line derivatives, "eof"/"eofu": with the face
 * lift in the line passes, "gather": node-parallel dot products, "tc" at
 * n = 7, 8, 9: line derivatives on the tensor cores as exact integer digit
 * products) and tile shape (elements and threads per CTA) on the context's
 * mesh and keeps the fastest.  spec = "auto" re-tunes; a name such as "eo",
 * "gather" or "tc", or "<name>:<elements per CTA>:<threads>", forces a
 * variant (the environment variable NMG_KERNEL does the same for new
 * contexts).  "vjp" and "tcvjp" choose the transposed kernel of the adjoint
 * entry points (FP64 line transforms, or the tensor-core digit products,
 * the default where compiled: n = 7, 8, 9). */
int nmg_set_kernel(nmg_ctx *c, const char *spec);
/* selected variant, candidates and tuning timings as text */
int nmg_kernel_info(nmg_ctx *c, char *buf, int32_t len);

/* ---- measurement helpers ------------------------------------------------ */
/* kernels launched by this context so far */
int64_t nmg_kernel_launches(const nmg_ctx *c);
/* the CUDA stream of the context (cudaStream_t) */
void *nmg_stream(nmg_ctx *c);
/* measured FP64 FMA throughput of the current device in GFLOP/s (the roof
   of this FP64 path on GB300); runs a ~10 ms probe kernel */
int nmg_fp64_peak(double *gflops);
/* measured FP64 tensor-core throughput (mma.sync m8n8k4 f64, DMMA) of the
   current device in GFLOP/s: the other FP64 roof, reported beside the FMA
   one (on GB300 both share one FP64 rate) */
int nmg_fp64_dmma_peak(double *gflops);

#ifdef __cplusplus
}
#endif
#endif /* NMG_H */
