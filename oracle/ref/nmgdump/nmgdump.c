/* nmgdump.c -- test-side add-on module that is compiled together with the
   unmodified reference sources (see oracle/ref/Makefile).  It only uses the
   reference's public module interface (AddFun/AddPar/Vard/formyelms) and
   changes no reference numerics.

   It writes raw FP64 dumps that pin the oracle and the CUDA path:
     POST_INITIALDATA: optionally scales the plane-wave data by an amplitude
                       and adds a seeded element-local perturbation, so that
                       face values of neighbouring elements differ;
     PRE_EVOLVE (first call): r = RHS(u, t0) through the reference's own
                       evolve_setrhs_mesh (src/main/evolve/evolve.c:182), then
                       dumps geometry, u and r ("<prefix>_rhs.bin");
     FINALIZE:         dumps u after the evolution ("<prefix>_final.bin").

   Record layout (little endian, all counts int32, all reals float64):
     header: magic 'NMGD', version 2, nelem, then per element:
       int32 pat, int32 n[3], int32 use_fv, float64 bbox[6],
       float64 x[np], y[np], z[np]            (Cartesian coordinates)
       float64 dXdx[9][np]                    (dX^a/dx^i, a-major)
       float64 sqrtgdiag[3][np]
       float64 det_dXbdx[np]
       float64 u[5][np]  (pi, cx, cy, cz, phi)
       float64 r[5][np]  (only in the *_rhs.bin file)
   where np = n0*n1*n2 and arrays are i-fastest (Ind_n). */

#include "nmesh.h"
#include "evolve.h"

/* defined in src/main/evolve/trouble.c, not declared in a header */
double evolve_Persson_array_indicator(tArray *u, double u_scale,
                                      int pt_typ[3], int ncoeffs[3]);

static int nmgdump_rhs_done = 0;

/* small counter-based hash -> uniform in [-1,1) */
static double nmgdump_hash(unsigned long long a)
{
  a += 0x9E3779B97F4A7C15ULL;
  a = (a ^ (a >> 30)) * 0xBF58476D1CE4E5B9ULL;
  a = (a ^ (a >> 27)) * 0x94D049BB133111EBULL;
  a = a ^ (a >> 31);
  return (double)(a >> 11) * (2.0 / 9007199254740992.0) - 1.0;
}

static void nmgdump_vl_indices(tMesh *mesh, int iu[5])
{
  iu[0] = Ind("scalarwave1_pi");
  iu[1] = Ind("scalarwave1_cx");
  iu[2] = iu[1] + 1;
  iu[3] = iu[1] + 2;
  iu[4] = Ind("scalarwave1_phi");
}

int nmgdump_perturb(tMesh *mesh)
{
  double amp = Getd(Par("nmgdump_amp"));
  double eps = Getd(Par("nmgdump_perturb"));
  unsigned long long seed = (unsigned long long)Geti(Par("nmgdump_seed"));
  int iu[5];
  int e;

  nmgdump_vl_indices(mesh, iu);
  for(e = 0; e < mesh->nmyelm; e++)
  {
    tElm *elm = mesh->myelm[e];
    int f, ijk;
    for(f = 0; f < 5; f++)
    {
      double *u = Vard(elm, iu[f]);
      for(ijk = 0; ijk < elm->np; ijk++)
      {
        unsigned long long key = seed * 1000003ULL
                               + ((unsigned long long)e << 24)
                               + ((unsigned long long)f << 20)
                               + (unsigned long long)ijk;
        u[ijk] = amp * u[ijk] + eps * nmgdump_hash(key);
      }
    }
  }
  return 0;
}

static void nmgdump_write(tMesh *mesh, const char *suffix, int with_r)
{
  char fname[4096];
  FILE *fp;
  int iu[5], ir[5];
  int ix = Ind("x");
  int idXdx = Ind("dXdx");
  int isqg = Ind("sqrtgdiagx");
  int idet = Ind("det_dXbdx");
  int hdr[3] = { 0x44474D4E, 2, (int)mesh->nmyelm };
  int e, c;

  nmgdump_vl_indices(mesh, iu);
  ir[0] = Ind("scalarwave1_pi_r");
  ir[1] = Ind("scalarwave1_cx_r");
  ir[2] = ir[1] + 1;
  ir[3] = ir[1] + 2;
  ir[4] = Ind("scalarwave1_phi_r");

  snprintf(fname, sizeof(fname), "%s_%s.bin", Gets(Par("nmgdump_prefix")),
           suffix);
  fp = fopen(fname, "wb");
  if(!fp) errorexits("cannot open %s", fname);
  fwrite(hdr, sizeof(int), 3, fp);
  for(e = 0; e < mesh->nmyelm; e++)
  {
    tElm *elm = mesh->myelm[e];
    int pat = elm->pat->p;
    int np = elm->np;
    int use_fv = elm->dat->info->use_fv;
    fwrite(&pat, sizeof(int), 1, fp);
    fwrite(elm->n, sizeof(int), 3, fp);
    fwrite(&use_fv, sizeof(int), 1, fp);
    fwrite(elm->bbox, sizeof(double), 6, fp);
    for(c = 0; c < 3; c++) fwrite(Vard(elm, ix + c), sizeof(double), np, fp);
    for(c = 0; c < 9; c++) fwrite(Vard(elm, idXdx + c), sizeof(double), np, fp);
    for(c = 0; c < 3; c++) fwrite(Vard(elm, isqg + c), sizeof(double), np, fp);
    fwrite(Vard(elm, idet), sizeof(double), np, fp);
    for(c = 0; c < 5; c++) fwrite(Vard(elm, iu[c]), sizeof(double), np, fp);
    if(with_r)
      for(c = 0; c < 5; c++) fwrite(Vard(elm, ir[c]), sizeof(double), np, fp);
  }
  fclose(fp);
  printf("nmgdump: wrote %s (%d elements)\n", fname, (int)mesh->nmyelm);
}

/* r = RHS(u, t) once, before the first step, via the reference's own
   evolve_setrhs_mesh with w = u */
/* Persson's modal indicator of each field of each element (the reference's
   evolve_Persson_array_indicator, u_scale < 0, all coefficients):
   "<prefix>_persson.bin" = int32 nelem, then float64 [nelem][5] */
static void nmgdump_persson(tMesh *mesh)
{
  char fname[4096];
  FILE *fp;
  int iu[5];
  int ne = (int)mesh->nmyelm, e, c;

  nmgdump_vl_indices(mesh, iu);
  snprintf(fname, sizeof(fname), "%s_persson.bin", Gets(Par("nmgdump_prefix")));
  fp = fopen(fname, "wb");
  if(!fp) errorexits("cannot open %s", fname);
  fwrite(&ne, sizeof(int), 1, fp);
  for(e = 0; e < ne; e++)
  {
    tElm *elm = mesh->myelm[e];
    for(c = 0; c < 5; c++)
    {
      double se = evolve_Persson_array_indicator(VarA(elm, iu[c]), -1.,
                                                 elm->pt_typ, elm->n);
      fwrite(&se, sizeof(double), 1, fp);
    }
  }
  fclose(fp);
}

/* the reference's 0d norms of each field of u0 (output0d_mesh_vl's
   ingredients): "<prefix>_norms.bin" = float64 Vol, then per field
   VolInt, Int(v^2), min, max */
static void nmgdump_norms(tMesh *mesh)
{
  char fname[4096], nodeloc[105];
  FILE *fp;
  int iu[5], c, p, ijk;
  double X[3], x[3], v;

  nmgdump_vl_indices(mesh, iu);
  snprintf(fname, sizeof(fname), "%s_norms.bin", Gets(Par("nmgdump_prefix")));
  fp = fopen(fname, "wb");
  if(!fp) errorexits("cannot open %s", fname);
  v = MeshVolumeIntegral(mesh, NULL, Ind("X"), 0.0, 0);
  fwrite(&v, sizeof(double), 1, fp);
  for(c = 0; c < 5; c++)
  {
    v = MeshVolumeIntegral(mesh, NULL, iu[c], 1., 0);
    fwrite(&v, sizeof(double), 1, fp);
    v = MeshVolumeIntegral(mesh, NULL, iu[c], 2., 0);
    fwrite(&v, sizeof(double), 1, fp);
    v = MeshExtremumLoc(mesh, NULL, iu[c], 0, &p, nodeloc, &ijk, X, x);
    fwrite(&v, sizeof(double), 1, fp);
    v = MeshExtremumLoc(mesh, NULL, iu[c], 1, &p, nodeloc, &ijk, X, x);
    fwrite(&v, sizeof(double), 1, fp);
  }
  fclose(fp);
}

int nmgdump_rhs(tMesh *mesh)
{
  tEvoSys *evosys = mesh->evosys;
  int i;

  if(nmgdump_rhs_done) return 0;
  nmgdump_rhs_done = 1;

  evolve_init_evosys(mesh);
  forList(evosys->u, i)
    vlcopy(NULL, ListEntry(evosys->w, i), ListEntry(evosys->u, i));
  evolve_setrhs_mesh(mesh, evosys->rhs, evosys->w);
  nmgdump_write(mesh, "rhs", 1);
  {
    /* the time step of the run (dt = auto: the reference's dtfac * hmin) */
    char fn[1000];
    FILE *fp;
    snprintf(fn, sizeof fn, "%s_dt.bin", Gets(Par("nmgdump_prefix")));
    fp = fopen(fn, "wb");
    if(fp) { fwrite(&mesh->dt, sizeof(double), 1, fp); fclose(fp); }
  }
  if(Getb(Par("nmgdump_persson"))) nmgdump_persson(mesh);
  if(Getb(Par("nmgdump_norms"))) nmgdump_norms(mesh);
  return 0;
}

int nmgdump_final(tMesh *mesh)
{
  nmgdump_write(mesh, "final", 0);
  return 0;
}

int nmesh_nmgdump(tMesh *mesh)
{
  if(!Getv(Par("physics"), "nmgdump")) return 0;

  printf("Adding nmgdump\n");

  AddFun(POST_INITIALDATA, nmgdump_perturb);
  AddFun(PRE_EVOLVE, nmgdump_rhs);
  AddFun(FINALIZE, nmgdump_final);

  AddPar("nmgdump_prefix", "nmgdump", "path prefix of the dump files");
  AddPar("nmgdump_amp", "1", "factor applied to the initial plane wave");
  AddPar("nmgdump_perturb", "0", "amplitude of the seeded perturbation");
  AddPar("nmgdump_seed", "1", "seed of the perturbation");
  AddPar("nmgdump_persson", "no", "also dump Persson's indicator of u0 [no,yes]");
  AddPar("nmgdump_norms", "no", "also dump the 0d norms of u0 [no,yes]");
  return 0;
}
