/* nmg_evolve.c -- nmesh-side adapter for the GB300 evolution path.
 *
 * A maintainer adds this file as an nmesh module (a directory under
 * src/projects/ with the usual nmesh_<name>.c / Makefile, linked with
 * -lnmg -lcudart) and a three-line case to evolve_myln's method switch
 * (src/main/evolve/evolve.c:45-61):
 *
 *     else if(Getv(evolve_method, "RK4gpu"))
 *       Evolve_mesh = evolve_RK4gpu_mesh;
 *
 * (and likewise "sspRK3gpu" / "Eulergpu" for evolve_sspRK3gpu_mesh and
 * evolve_Eulergpu_mesh, the GPU forms of evolve_sspRK3_mesh and
 * evolve_Euler_mesh)
 *
 * evolve_RK4gpu_mesh has the signature and the time semantics of
 * evolve_RK4_mesh (src/main/evolve/RungeKutta.c:19-82): on the first call it
 * packs the mesh (element bboxes, Cartesian/curvilinear flag, x/y/z and
 * dXdx of coordinates_init_node) into an nmg mesh and creates the device
 * context; every call copies u of scalarwave1 into the context, takes one
 * RK4 step on the GPU and copies u back (a code that keeps u resident would
 * call nmg_rk4_steps and nmg_get_state only when an output bin needs u).
 * Nonzero nmg return codes become errorexit at this boundary only.
 */
#include "nmesh.h"
#include "nmg.h"

static nmg_mesh *nmg_evolve_mesh = NULL;
static nmg_ctx *nmg_evolve_ctx = NULL;
static double *nmg_evolve_u = NULL;

/* scalarwave1 evolved variables in the order of its vlu */
static void nmg_evolve_var_indices(tMesh *mesh, int iu[5])
{
  iu[0] = Ind("scalarwave1_pi");
  iu[1] = Ind("scalarwave1_cx");
  iu[2] = iu[1] + 1;
  iu[3] = iu[1] + 2;
  iu[4] = Ind("scalarwave1_phi");
}

static void nmg_evolve_check(int rc, const char *what)
{
  if(rc)
  {
    printf("%s failed (%d): %s\n", what, rc,
           nmg_evolve_ctx ? nmg_last_error(nmg_evolve_ctx) : nmg_mesh_last_error());
    errorexit("nmg_evolve: GPU evolution failed");
  }
}

/* pack the static mesh once (elements with the same n in all directions) */
static void nmg_evolve_setup(tMesh *mesh)
{
  int E = (int)mesh->nmyelm;
  int n = mesh->myelm[0]->n[0];
  int np = n * n * n;
  int ix = Ind("x"), idXdx = Ind("dXdx");
  nmg_mesh_desc d;
  int32_t *pat = malloc(sizeof(int32_t) * E);
  int32_t *curvi = malloc(sizeof(int32_t) * E);
  double *bbox = malloc(sizeof(double) * 6 * E);
  double *xyz = malloc(sizeof(double) * 3 * np * (size_t)E);
  double *dXdx = malloc(sizeof(double) * 9 * np * (size_t)E);
  double k[3] = {0., 0., 0.};
  int e, c;

  if(!pat || !curvi || !bbox || !xyz || !dXdx) errorexit("nmg_evolve: out of memory");
  for(e = 0; e < E; e++)
  {
    tElm *elm = mesh->myelm[e];
    if(elm->n[0] != n || elm->n[1] != n || elm->n[2] != n)
      errorexit("nmg_evolve: all elements need the same n in all directions");
    pat[e] = elm->pat->p;
    curvi[e] = (elm->pat->dXYZ_dxyz != NULL);
    memcpy(bbox + 6 * e, elm->bbox, 6 * sizeof(double));
    for(c = 0; c < 3; c++)
      memcpy(xyz + ((size_t)e * 3 + c) * np, Vard_(elm, ix + c), np * sizeof(double));
    for(c = 0; c < 9; c++)
      memcpy(dXdx + ((size_t)e * 9 + c) * np, Vard_(elm, idXdx + c), np * sizeof(double));
  }
  memset(&d, 0, sizeof(d));
  d.nelem = E;
  d.n = n;
  d.pat = pat;
  d.bbox = bbox;
  d.curvi = curvi;
  d.xyz = xyz;
  d.dXdx = dXdx;
  d.nbnode = NULL; /* coincident face nodes are matched from x,y,z */
  nmg_evolve_check(nmg_mesh_from_desc(&d, &nmg_evolve_mesh), "nmg_mesh_from_desc");
  sscanf(Gets(Par("scalarwave1_k")), "%lg %lg %lg", &k[0], &k[1], &k[2]);
  nmg_evolve_check(nmg_create(nmg_evolve_mesh, NMG_BC_EXACT_PLANEWAVE, k,
                              &nmg_evolve_ctx), "nmg_create");
  nmg_evolve_u = malloc(sizeof(double) * 5 * np * (size_t)E);
  if(!nmg_evolve_u) errorexit("nmg_evolve: out of memory");
  free(pat); free(curvi); free(bbox); free(xyz); free(dXdx);
}

/* one step of u of scalarwave1 through the context: method -1 is RK4
   (nmg_rk4_steps_host), otherwise an NMG_EVOLVE_* integrator */
static void nmg_evolve_step(tMesh *mesh, int method)
{
  int E, np, e, f, iu[5];
  double t = mesh->time, dt = mesh->dt;

  /* the reference limits w inside its own RK stages (RungeKutta.c:45-67)
     and u again in evolve_mesh (evolve.c:144), which keeps running here:
     the GPU stages would have to limit w only, so a limiter is refused */
  if(!Getv(Par("scalarwave1_limiter"), "none"))
    errorexit("nmg_evolve: use scalarwave1_limiter = none, or keep u resident and call "
              "nmg_set_limiter");
  if(!nmg_evolve_ctx) nmg_evolve_setup(mesh);
  E = (int)mesh->nmyelm;
  np = mesh->myelm[0]->np;
  nmg_evolve_var_indices(mesh, iu);
  for(e = 0; e < E; e++)
    for(f = 0; f < 5; f++)
      memcpy(nmg_evolve_u + ((size_t)e * 5 + f) * np, Vard_(mesh->myelm[e], iu[f]),
             np * sizeof(double));
  if(method < 0)
    nmg_evolve_check(nmg_rk4_steps_host(nmg_evolve_ctx, t, dt, 1, nmg_evolve_u),
                     "nmg_rk4_steps_host");
  else
  {
    nmg_evolve_check(nmg_set_evolve_method(nmg_evolve_ctx, method), "nmg_set_evolve_method");
    nmg_evolve_check(nmg_evolve_steps_host(nmg_evolve_ctx, t, dt, 1, nmg_evolve_u),
                     "nmg_evolve_steps_host");
  }
  for(e = 0; e < E; e++)
    for(f = 0; f < 5; f++)
      memcpy(Vard_(mesh->myelm[e], iu[f]), nmg_evolve_u + ((size_t)e * 5 + f) * np,
             np * sizeof(double));
  mesh->time = t + dt; /* as RungeKutta.c:76 */
}

/* same signatures and time semantics as evolve_RK4_mesh, evolve_sspRK3_mesh
   and evolve_Euler_mesh (src/main/evolve/RungeKutta.c:19-200) */
void evolve_RK4gpu_mesh(tMesh *mesh) { nmg_evolve_step(mesh, -1); }
void evolve_sspRK3gpu_mesh(tMesh *mesh) { nmg_evolve_step(mesh, NMG_EVOLVE_SSPRK3); }
void evolve_Eulergpu_mesh(tMesh *mesh) { nmg_evolve_step(mesh, NMG_EVOLVE_EULER); }
