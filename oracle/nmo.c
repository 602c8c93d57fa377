/* nmo.c -- ORACLE (test infrastructure only; never part of the product path).
 *
 * A plain-C CPU restatement of nmesh's scalarwave1 evolution right-hand side
 * (DG volume derivative + LLF surface flux + lift) and of its classic RK4
 * step.  It follows the reference's operation order so that, compiled with
 * -ffp-contract=off, it reproduces the reference's FP64 results bit for bit
 * on the same inputs.  Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg load it, as the checker / the timed CPU implementation.
 *
 * Reference functions restated here (paths within nmeshsource/nmesh):
 *   LGL nodes/weights    src/main/basis/Legendre.c:59-98,149-213
 *   Lagrange weights     src/main/basis/Lagrange.c:15-27
 *   D matrix             src/main/basis/Lagrange.c:126-147
 *   directional matmul   src/main/amr/array.c:36-45,100-120,194-304
 *   Cartesian partials   src/main/coordinates/derivs.c:102-181
 *   divergence           src/main/coordinates/derivs.c:756-815
 *   fluxes / eigenvals   src/tests/scalarwave1/scalarwave1.c:39-59,62-134
 *   volume RHS           src/tests/scalarwave1/scalarwave1.c:242-284
 *   face fluxes          src/tests/scalarwave1/scalarwave1.c:139-209
 *   exact plane wave     src/tests/scalarwave1/scalarwave1.c:503-524
 *   LLF                  src/main/dg/numflux1d.c:85-112
 *   upwind flux          src/tests/scalarwave1/scalarwave1.c:323-499
 *   surface flux + lift  src/main/dg/dg.c:30-151
 *   node normals         src/main/coordinates/utilities.c:48-88
 *   sqrtgdiag            src/main/coordinates/coordinates.c:728-800
 *   vladdto_onfaces      src/main/main/variables.c:1044-1066
 *   RK4                  src/main/evolve/RungeKutta.c:19-82
 *
 * Finite-volume elements (fv_divf with use_only_right_flux, LLF at the
 * midpoints, WENO reconstruction; coordinates_midpoint_data = no):
 *   uniform points       src/main/basis/Legendre.c:626-660,701-719
 *   midpoints, dists     src/main/coordinates/get_coords.c:509-518,1702-1865
 *   det(dXb/dx)          src/main/coordinates/coordinates.c:174-223,
 *                        src/main/coordinates/utilities.c:199-211
 *   fv_divf              src/main/dg/fv.c:115-624
 *   WENO3 / WENOm3_2     src/main/dg/rec1d.c:16-27,121-227,880-1030
 *   WENO5 / WENOm5_2     src/main/dg/rec1d.c:1186-1368
 *   dnfn extrapolation   src/main/dg/rec1d.c:542-628
 *   midpoint states      src/tests/scalarwave1/scalarwave1.c:761-802
 *   fin.-vol. surface    src/main/dg/dg.c:58-70,81-90 (oow = 1/|distXb|,
 *                        F = f*)
 *   root finder          src/utility/numerics/newton1d_brak.c:20-121 (GRHD
 *                        con2prim; the GRHD physics itself has no
 *                        reference counterpart: parity unpinned)
 *   trouble indicators   src/main/evolve/trouble.c:438-564 (RDMP, Persson),
 *                        src/main/basis/Legendre.c:14-38,277-310 (modal
 *                        analysis matrix)
 *   DG / FV interfaces   src/main/amr/surface.c:1080-1250 (neighbour trace
 *                        interpolated onto the face points: Lagrange from a
 *                        DG neighbour, piecewise linear from a fin.-vol.
 *                        one), src/main/basis/interpolate.c:53-100,296-360,
 *                        src/main/basis/Lagrange.c:15-27,151-159
 *
 * Extensions without a reference counterpart (restated, parity unpinned):
 *   BC kind 1: outgoing-radiation outer boundary (characteristic upwinding
 *              of the first-order wave system: incoming characteristic
 *              pi + c.n set to zero in the exterior state);
 *   periodic faces are plain face connections in the neighbour table.
 *
 * Data layout: state arrays are [element][field][node], node = i + n*(j + n*k),
 * fields (pi, cx, cy, cz, phi) as in the reference's vlu (scalarwave1.c:669).
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define NF 5

typedef struct nmo_mesh {
  int nelem;
  int n;                    /* LGL nodes per direction */
  const double *bbox;       /* [e][6] element bbox in patch coordinates */
  const int32_t *curvi;     /* [e] 1 if the patch map is not Cartesian */
  const double *dXdx;       /* [e][9][np] dX^a/dx^i (a-major); may be NULL if no curvi */
  const double *xyz;        /* [e][3][np] Cartesian coordinates */
  const int64_t *nbnode;    /* [e][6][n*n] global index e'*np+ijk' of the
                               coincident node across the face, -1 = outer,
                               -2 = neighbour with the other point type */
  int bc;                   /* outer faces: 0 exact plane wave, 1 outgoing */
  double k[3];              /* plane-wave vector for bc 0 */
  /* finite-volume elements (fv.c); fv == NULL: all elements are DG */
  const int32_t *fv;        /* [e] 1: fin.-vol. element on uniform points */
  int fv_rec;               /* NMO_REC_* reconstruction (par fv_rec) */
  int fv_extrap;            /* 0: fv_divf_extrap = no, 1: dnfn_extrap1 */
  double fv_w3ratio;        /* par fv_WENOm3_opt_weightratio (default 2) */
  const int32_t *mixface;   /* [e][6][3] (e', f', orientation) of the faces
                               marked -2 in nbnode; NULL if none */
  int numflux;              /* 0: LLF, 1: upwind (par scalarwave1_numflux) */
  /* non-conforming faces (nbnode -3): per face node (e, f, JK) the
     contributions hang_off[q] .. hang_off[q+1]-1, q = (e*6+f)*n*n + JK,
     each a neighbour face (hang_src: e', f') and the node's position on it
     (hang_pos: in-plane coordinates in [-1,1]); NULL if none */
  const int32_t *hang_off;  /* [e*6*n*n + 1] */
  const int32_t *hang_src;  /* [c][2] */
  const double *hang_pos;   /* [c][2] */
  int surf_interp;          /* traces from FV neighbours: 0 piecewise linear,
                               1 piecewise parabolic (par fv_surface_interp) */
  const double *dXdxm;      /* [e][3][9][np] dX^a/dx^i at the midpoint right of
                               each node in each direction (par
                               coordinates_midpoint_data = yes), or NULL */
  const double *ext;        /* [e][6][n*n][5] exterior states of the face
                               nodes marked -4 in nbnode (faces joined to a
                               part of the problem held elsewhere), or NULL */
} nmo_mesh;

/* points of both point types: LGL (DG) with their Lagrange weights, and
   equally spaced (finite volume) */
typedef struct nmo_pts {
  double xl[64], wl[64], xu[64];
} nmo_pts;

enum { NMO_REC_1 = 0, NMO_REC_WENOM3_2 = 1, NMO_REC_WENOM5_2 = 2, NMO_REC_WENOMZ_2 = 3 };

/* ------------------------------------------------------------------ */
/* basis: LGL points, weights and differentiation matrix               */
/* ------------------------------------------------------------------ */
static void legendre_P_dP_Q_dQ(int l, double x, double *P, double *dP,
                               double *Q, double *dQ)
{
  double P0 = 1., P1 = x, dP0 = 0., dP1 = 1., Pk = 0., dPk = 0.;
  int k;
  if (l == 0) { *P = 1.; *dP = 0.; return; }
  if (l == 1) { *P = x; *dP = 1.; return; }
  for (k = 2; k <= l + 1; k++) {
    Pk = (P1 * x * (2 * k - 1) - P0 * (k - 1)) / k;
    dPk = P1 * (2 * k - 1) + dP0;
    if (k >= l + 1) break;
    P0 = P1; P1 = Pk; dP0 = dP1; dP1 = dPk;
  }
  *P = P1; *dP = dP1; *Q = Pk - P0; *dQ = dPk - dP0;
}

void nmo_lgl(int npoints, double *x, double *w)
{
  const double PI = 3.14159265358979323846264338327950;
  int N = npoints - 1, i, j;
  double P, dP, Q, dQ, y, dy;
  if (N == 0) { x[0] = 0.; w[0] = 2.; return; }
  x[0] = -1.; x[N] = 1.;
  w[0] = 2.0 / (N * (N + 1.0)); w[N] = w[0];
  if (N == 1) return;
  for (j = 1; j <= N / 2; j++) {
    if (j == N / 2.0) {
      y = 0.;
    } else {
      y = -cos(PI * (j + 0.25) / N - 3 / (8 * N * PI * (j + 0.25)));
      for (i = 0; i < 100; i++) {
        legendre_P_dP_Q_dQ(N, y, &P, &dP, &Q, &dQ);
        dy = -Q / dQ;
        y += dy;
        if (fabs(dy) < fabs(1e-15 * y)) break;
      }
    }
    x[N - j] = -y;
    x[j] = y;
    legendre_P_dP_Q_dQ(N, y, &P, &dP, &Q, &dQ);
    w[j] = 2.0 / ((N * (N + 1)) * P * P);
    w[N - j] = w[j];
  }
}

/* D[i*n + j] = d l_j / dx (x_i) */
void nmo_diffmat(int n, const double *x, double *D)
{
  double wi[64];
  int i, j, m;
  for (i = 0; i < n; i++) {
    double denom = 1.;
    for (m = 0; m < n; m++) if (m != i) denom *= (x[i] - x[m]);
    wi[i] = 1. / denom;
  }
  for (i = 0; i < n; i++) {
    double Dii = 0;
    for (j = 0; j < n; j++) {
      if (i != j) {
        double Dij = (wi[j] / wi[i]) / (x[i] - x[j]);
        Dii -= Dij;
        D[i * n + j] = Dij;
      }
    }
    D[i * n + i] = Dii;
  }
}

/* ------------------------------------------------------------------ */
/* RHS                                                                 */
/* ------------------------------------------------------------------ */
static void planewave(const double k[3], const double xyz[3], double t,
                      double u[5])
{
  double om = sqrt(k[0] * k[0] + k[1] * k[1] + k[2] * k[2]);
  double arg = k[0] * xyz[0] + k[1] * xyz[1] + k[2] * xyz[2] - om * t;
  double s = sin(arg), c = cos(arg);
  u[4] = s;
  u[0] = -om * c;
  u[1] = k[0] * c;
  u[2] = k[1] * c;
  u[3] = k[2] * c;
}

static void flux1d(double *f, const double norm[3], const double *u)
{
  f[0] = -(u[1] * norm[0] + u[2] * norm[1] + u[3] * norm[2]);
  f[1] = -u[0] * norm[0];
  f[2] = -u[0] * norm[1];
  f[3] = -u[0] * norm[2];
  f[4] = 0.;
}

/* numflux1d_LLF with the scalar-wave eigenvalues (1,-1,0,0,0) on both
   sides: amax = 1 */
static void llf(const double *ui, const double *ua, const double *fi,
                const double *fa, double *fnum)
{
  const double lam[5] = {1.0, -1.0, 0.0, 0.0, 0.0};
  double apl = 0., ami = 0., amax;
  int l;
  for (l = 0; l < NF; l++) {
    apl = fmax(apl, lam[l]);
    ami = fmin(ami, lam[l]);
  }
  apl = fabs(apl); ami = fabs(ami);
  amax = fmax(ami, apl);
  for (l = 0; l < NF; l++)
    fnum[l] = 0.5 * (fa[l] + fi[l] - amax * (ua[l] - ui[l]));
}

/* Upwind flux of the first-order wave (scalarwave1_numflux1d_upwind):
   f* = R diag(lam+) R^-1 u_in + R diag(lam-) R^-1 u_adj over (pi, c) with
   the characteristic matrices R, R^-1 of the face normal (three forms,
   chosen by which normal component is nonzero), evaluated as matrix
   products in that order; f*_phi = 0.  Eigenvalues (1, -1, 0, 0). */
static void upwind(const double *ui, const double *ua, const double nrm[3], double *fnum)
{
  const double lam[4] = {1.0, -1.0, 0.0, 0.0};
  const double nx = nrm[0], ny = nrm[1], nz = nrm[2];
  double lp[4][4], ln[4][4], ip[4][4], in_[4][4], sp[4][4], sn[4][4], fi[4], fa[4];
  double R[4][4], Ri[4][4];
  int l, m, q;
  for (l = 0; l < 4; l++) {
    for (m = 0; m < 4; m++) lp[l][m] = ln[l][m] = ip[l][m] = in_[l][m] = sp[l][m] = sn[l][m] = 0.;
    fi[l] = fa[l] = 0.;
  }
  for (l = 0; l < 4; l++) {
    if (lam[l] > 0.) lp[l][l] = lam[l];
    else ln[l][l] = lam[l];
  }
  if (nz != 0) {
    double A[4][4] = {{1.0, 1.0, 0.0, 0.0}, {-nx, nx, 0.0, nz}, {-ny, ny, nz, 0.0},
                      {-nz, nz, -ny, -nx}};
    double B[4][4] = {{1.0 / 2.0, -nx / 2.0, -ny / 2.0, -nz / 2.0},
                      {1.0 / 2.0, nx / 2.0, ny / 2.0, nz / 2.0},
                      {0.0, -(nx * ny) / nz, (nx * nx + nz * nz) / nz, -ny},
                      {0.0, (ny * ny + nz * nz) / nz, -(nx * ny) / nz, -nx}};
    memcpy(R, A, sizeof R);
    memcpy(Ri, B, sizeof Ri);
  } else if (nx != 0) {
    double A[4][4] = {{1.0, 1.0, 0.0, 0.0}, {-nx, nx, -nz, -ny}, {-ny, ny, 0.0, nx},
                      {-nz, nz, nx, 0.0}};
    double B[4][4] = {{1.0 / 2.0, -nx / 2.0, -ny / 2.0, -nz / 2.0},
                      {1.0 / 2.0, nx / 2.0, ny / 2.0, nz / 2.0},
                      {0.0, -nz, -(ny * nz) / nx, (nx * nx + ny * ny) / nx},
                      {0.0, -ny, (nx * nx + nz * nz) / nx, -(ny * nz) / nx}};
    memcpy(R, A, sizeof R);
    memcpy(Ri, B, sizeof Ri);
  } else {
    double A[4][4] = {{1.0, 1.0, 0.0, 0.0}, {-nx, nx, 0.0, ny}, {-ny, ny, -nz, -nx},
                      {-nz, nz, ny, 0.0}};
    double B[4][4] = {{1.0 / 2.0, -nx / 2.0, -ny / 2.0, -nz / 2.0},
                      {1.0 / 2.0, nx / 2.0, ny / 2.0, nz / 2.0},
                      {0.0, -(nx * nz) / ny, -nz, (nx * nx + ny * ny) / ny},
                      {0.0, (ny * ny + nz * nz) / ny, -nx, -(nx * nz) / ny}};
    memcpy(R, A, sizeof R);
    memcpy(Ri, B, sizeof Ri);
  }
  for (l = 0; l < 4; l++)
    for (m = 0; m < 4; m++)
      for (q = 0; q < 4; q++) {
        ip[l][m] += lp[l][q] * Ri[q][m];
        in_[l][m] += ln[l][q] * Ri[q][m];
      }
  for (l = 0; l < 4; l++)
    for (m = 0; m < 4; m++)
      for (q = 0; q < 4; q++) {
        sp[l][m] += R[l][q] * ip[q][m];
        sn[l][m] += R[l][q] * in_[q][m];
      }
  for (l = 0; l < 4; l++)
    for (m = 0; m < 4; m++) {
      fi[l] += sp[l][m] * ui[m];
      fa[l] += sn[l][m] * ua[m];
    }
  for (l = 0; l < 4; l++) fnum[l] = fi[l] + fa[l];
  fnum[4] = 0.;
}

/* out = D_dir applied to in along direction dir (array.c MM_SET_AB order) */
static void deriv_dir(int n, const double *D, int dir, const double *in,
                      double *out)
{
  /* stride of direction dir and the sum over l in ascending order */
  const int st = (dir == 0) ? 1 : (dir == 1) ? n : n * n;
  int i, j, k, l;
  for (k = 0; k < n; k++)
    for (j = 0; j < n; j++)
      for (i = 0; i < n; i++) {
        const int ii = (dir == 0) ? i : (dir == 1) ? j : k;
        const int ijk = i + n * (j + n * k);
        const double *line = in + ijk - ii * st;
        const double *Drow = D + ii * n;
        double sum = 0.0;
        for (l = 0; l < n; l++) sum += Drow[l] * line[l * st];
        out[ijk] = sum;
      }
}

/* d/dx^m of U for all m (array_cart_partials): du[m][.] */
static void cart_partials(const nmo_mesh *m, int e, const double *D,
                          const double *U, double *dU, double *du)
{
  int n = m->n, np = n * n * n, a, mm, ind;
  const double *bb = m->bbox + 6 * e;
  double dXbdX[3];
  for (a = 0; a < 3; a++) dXbdX[a] = 2. / (bb[2 * a + 1] - bb[2 * a]);
  for (a = 0; a < 3; a++) deriv_dir(n, D, a, U, dU + a * np);
  for (ind = 0; ind < np; ind++)
    for (a = 0; a < 3; a++) dU[a * np + ind] *= dXbdX[a];
  if (m->curvi[e]) {
    const double *X = m->dXdx + (size_t)e * 9 * np;
    for (ind = 0; ind < np; ind++) {
      double dw[3];
      for (mm = 0; mm < 3; mm++) {
        dw[mm] = 0.;
        for (a = 0; a < 3; a++) dw[mm] += X[(a * 3 + mm) * np + ind] * dU[a * np + ind];
      }
      for (mm = 0; mm < 3; mm++) du[mm * np + ind] = dw[mm];
    }
  } else {
    memcpy(du, dU, sizeof(double) * 3 * np);
  }
}

/* divU = d_i U^i with U^i in Ux, Uy, Uz (cart_divergence, add=0) */
static void cart_divergence(const nmo_mesh *m, int e, const double *D,
                            const double *Ux, const double *Uy,
                            const double *Uz, double *divU, double *tmp)
{
  int np = m->n * m->n * m->n, i;
  double *dU = tmp, *du = tmp + 3 * np;
  cart_partials(m, e, D, Ux, dU, du);
  for (i = 0; i < np; i++) divU[i] = du[i];
  cart_partials(m, e, D, Uy, dU, du);
  for (i = 0; i < np; i++) divU[i] += du[np + i];
  cart_partials(m, e, D, Uz, dU, du);
  for (i = 0; i < np; i++) divU[i] += du[2 * np + i];
}

/* normal of face f at node ijk (node_normal_from_idXdx_at_ijk) */
static void node_normal(const nmo_mesh *m, int e, int f, int ijk, double nrm[3])
{
  int np = m->n * m->n * m->n, dir = f / 2, sig = 2 * (f % 2) - 1;
  double smag;
  if (m->curvi[e]) {
    const double *X = m->dXdx + (size_t)e * 9 * np;
    nrm[0] = X[(dir * 3 + 0) * np + ijk];
    nrm[1] = X[(dir * 3 + 1) * np + ijk];
    nrm[2] = X[(dir * 3 + 2) * np + ijk];
  } else {
    nrm[0] = nrm[1] = nrm[2] = 0.;
    nrm[dir] = 1.;
  }
  smag = sig * sqrt(nrm[0] * nrm[0] + nrm[1] * nrm[1] + nrm[2] * nrm[2]);
  if (smag == 0.0) smag = sig;
  nrm[0] /= smag; nrm[1] /= smag; nrm[2] /= smag;
}

/* sqrt(g^{dir dir}) in Xb coords at ijk for a flat 3-metric */
static double sqrtgdiag(const nmo_mesh *m, int e, int dir, int ijk)
{
  int np = m->n * m->n * m->n, l;
  const double *bb = m->bbox + 6 * e;
  double dXbdX = 2. / (bb[2 * dir + 1] - bb[2 * dir]);
  double g = 0.0;
  if (m->curvi[e]) {
    const double *X = m->dXdx + (size_t)e * 9 * np;
    for (l = 0; l < 3; l++) g += X[(dir * 3 + l) * np + ijk] * X[(dir * 3 + l) * np + ijk];
  } else {
    g = 1.0;
  }
  return dXbdX * sqrt(g);
}

/* volume index of in-plane point (a, b) on face f (forplaneN order) */
static int face_node(int n, int f, int a, int b)
{
  int dir = f / 2, p = (f % 2) * (n - 1);
  if (dir == 0) return p + n * (a + n * b);
  if (dir == 1) return a + n * (p + n * b);
  return a + n * (b + n * p);
}

/* LLF flux f* through face f at face node ijk (in-plane index JK) of element
   e: inner state from w, outer state from the coincident neighbour node or
   the boundary condition (scalarwave1_fluxes_pt + numflux1d_LLF).  Returns
   the inner flux fi and f*. */
/* piecewise linear basis function k at x (basis_pw_linear) */
static double pw_linear(int k, double x, int np, const double *xp)
{
  if (np <= 1) return 1.;
  if (x < xp[1]) {
    if (k == 0) return (x - xp[1]) / (xp[0] - xp[1]);
    if (k == 1) return (x - xp[0]) / (xp[1] - xp[0]);
    return 0.;
  }
  if (x >= xp[np - 2]) {
    int n0 = np - 2, n1 = np - 1, l = k - n0;
    if (l == 0) return (x - xp[n1]) / (xp[n0] - xp[n1]);
    if (l == 1) return (x - xp[n0]) / (xp[n1] - xp[n0]);
    return 0.;
  }
  if (k < np - 1 && x >= xp[k] && x < xp[k + 1]) return (x - xp[k + 1]) / (xp[k] - xp[k + 1]);
  if (k > 0 && x >= xp[k - 1] && x < xp[k]) return (x - xp[k - 1]) / (xp[k] - xp[k - 1]);
  return 0.;
}

/* piecewise-parabolic basis function k of the points xp at x
   (basis_pw_parab, src/main/basis/interpolate.c:106-224) */
static double pw_parab(int k, double x, int np, const double *xp)
{
  int m, m1, m2;
  double xml, xmr, xmll, xmrr;
  if (np < 3) return pw_linear(k, x, np, xp);
  if (np == 3) {
    if (k == 0) return (x - xp[1]) * (x - xp[2]) / ((xp[0] - xp[1]) * (xp[0] - xp[2]));
    if (k == 1) return (x - xp[0]) * (x - xp[2]) / ((xp[1] - xp[0]) * (xp[1] - xp[2]));
    if (k == 2) return (x - xp[0]) * (x - xp[1]) / ((xp[2] - xp[0]) * (xp[2] - xp[1]));
    return 0.;
  }
  xmr = 0.5 * (xp[0] + xp[1]);
  if (x < xmr) {
    if (k == 0) return (x - xp[1]) * (x - xp[2]) / ((xp[0] - xp[1]) * (xp[0] - xp[2]));
    if (k == 1) return (x - xp[0]) * (x - xp[2]) / ((xp[1] - xp[0]) * (xp[1] - xp[2]));
    if (k == 2) return (x - xp[0]) * (x - xp[1]) / ((xp[2] - xp[0]) * (xp[2] - xp[1]));
    return 0.;
  }
  xml = 0.5 * (xp[np - 2] + xp[np - 1]);
  if (x >= xml) {
    int n0 = np - 3, n1 = np - 2, n2 = np - 1, l = k - n0;
    if (l == 0) return (x - xp[n1]) * (x - xp[n2]) / ((xp[n0] - xp[n1]) * (xp[n0] - xp[n2]));
    if (l == 1) return (x - xp[n0]) * (x - xp[n2]) / ((xp[n1] - xp[n0]) * (xp[n1] - xp[n2]));
    if (l == 2) return (x - xp[n0]) * (x - xp[n1]) / ((xp[n2] - xp[n0]) * (xp[n2] - xp[n1]));
    return 0.;
  }
  if (k <= 0) {
    m = 0;
    xmr = 0.5 * (xp[m] + xp[m + 1]);
    xml = xp[m] - (xmr - xp[m]);
    xmll = xml - (xmr - xml);
    xmrr = 0.5 * (xp[m + 1] + xp[m + 2]);
    m1 = 1;
    m2 = 2;
  } else if (k < np - 1) {
    m = k;
    xml = 0.5 * (xp[m] + xp[m - 1]);
    xmr = 0.5 * (xp[m] + xp[m + 1]);
    if (k < np - 2) xmrr = 0.5 * (xp[m + 1] + xp[m + 2]);
    else xmrr = xmr + (xmr - xml);
    if (k >= 2) xmll = 0.5 * (xp[m - 1] + xp[m - 2]);
    else xmll = xml - (xmr - xml);
    m1 = k - 1;
    m2 = k + 1;
  } else {
    m = np - 1;
    xml = 0.5 * (xp[m - 1] + xp[m]);
    xmr = xp[m] + (xp[m] - xml);
    xmll = 0.5 * (xp[m - 2] + xp[m - 1]);
    xmrr = xmr + (xmr - xml);
    m1 = m - 2;
    m2 = m - 1;
  }
  if (x >= xml && x < xmr)
    return (x - xp[m1]) * (x - xp[m2]) / ((xp[m] - xp[m1]) * (xp[m] - xp[m2]));
  if (x >= xmll && x < xml)
    return (x - xp[m - 2]) * (x - xp[m - 1]) / ((xp[m] - xp[m - 2]) * (xp[m] - xp[m - 1]));
  if (x >= xmr && x < xmrr)
    return (x - xp[m + 1]) * (x - xp[m + 2]) / ((xp[m] - xp[m + 1]) * (xp[m] - xp[m + 2]));
  return 0.;
}

/* Lagrange basis function k at x (Lagrange_of_x) */
static double lagrange_of_x(int k, double x, int np, const double *xp, const double *wl)
{
  double prod = 1.;
  int q;
  for (q = 0; q < np; q++) if (q != k) prod *= (x - xp[q]);
  return prod * wl[k];
}

/* Exterior state at face node (a, b) of face f of element e whose neighbour
   (e2, f2, orientation o) has the other point type: the neighbour's face
   plane interpolated to this node (basis_array_interp2d). */
static void mixed_trace(const nmo_mesh *m, const nmo_pts *P, int e, int f, int a, int b,
                        const double *w, double ua[5])
{
  int n = m->n, np = n * n * n, l, j, k;
  const int32_t *mf = m->mixface + ((size_t)e * 6 + f) * 3;
  int e2 = mf[0], f2 = mf[1], o = mf[2];
  int sw = o & 1, fa = (o >> 1) & 1, fb = (o >> 2) & 1;
  int aa = sw ? b : a, bb = sw ? a : b;
  const double *xme = m->fv[e] ? P->xu : P->xl;
  int nbfv = m->fv[e2] != 0;
  double c1, c2, B1[64], B2[64];
  aa = fa ? n - 1 - aa : aa;
  bb = fb ? n - 1 - bb : bb;
  c1 = xme[aa];
  c2 = xme[bb];
  for (k = 0; k < n; k++) {
    if (nbfv && m->surf_interp == 1) {
      B1[k] = pw_parab(k, c1, n, P->xu);
      B2[k] = pw_parab(k, c2, n, P->xu);
    } else {
      B1[k] = nbfv ? pw_linear(k, c1, n, P->xu) : lagrange_of_x(k, c1, n, P->xl, P->wl);
      B2[k] = nbfv ? pw_linear(k, c2, n, P->xu) : lagrange_of_x(k, c2, n, P->xl, P->wl);
    }
  }
  for (l = 0; l < NF; l++) {
    const double *v = w + ((size_t)e2 * NF + l) * np;
    double sum = 0.;
    for (k = 0; k < n; k++)
      for (j = 0; j < n; j++) sum += v[face_node(n, f2, j, k)] * B1[j] * B2[k];
    ua[l] = sum;
  }
}

/* Exterior state at face node JK of a non-conforming face: each neighbour
   face that contains the node interpolated there (basis_interp2d_toIpoints
   with Lagrange_of_x), then the average over those neighbours
   (set_ajsurf_vl, src/main/amr/surface.c:1160-1340). */
static void hang_trace(const nmo_mesh *m, const nmo_pts *P, int e, int f, int JK,
                       const double *w, double ua[5])
{
  int n = m->n, np = n * n * n, l, j, k, c;
  size_t q = ((size_t)e * 6 + f) * n * n + JK;
  int c0 = m->hang_off[q], c1 = m->hang_off[q + 1], cnt = c1 - c0;
  for (l = 0; l < NF; l++) ua[l] = 0.;
  for (c = c0; c < c1; c++) {
    int e2 = m->hang_src[2 * c], f2 = m->hang_src[2 * c + 1];
    double B1[64], B2[64];
    for (k = 0; k < n; k++) {
      B1[k] = lagrange_of_x(k, m->hang_pos[2 * c], n, P->xl, P->wl);
      B2[k] = lagrange_of_x(k, m->hang_pos[2 * c + 1], n, P->xl, P->wl);
    }
    for (l = 0; l < NF; l++) {
      const double *v = w + ((size_t)e2 * NF + l) * np;
      double sum = 0.;
      for (k = 0; k < n; k++)
        for (j = 0; j < n; j++) sum += v[face_node(n, f2, j, k)] * B1[j] * B2[k];
      ua[l] += sum;
    }
  }
  if (cnt > 1)
    for (l = 0; l < NF; l++) ua[l] /= cnt;
}

static void face_fnum(const nmo_mesh *m, const nmo_pts *P, int e, int f, int ijk, int JK,
                      double t, const double *w, double fi[5], double fnum[5])
{
  int n = m->n, np = n * n * n, l;
  const double *we = w + (size_t)e * NF * np;
  double norm[3], ui[5], ua[5], fa[5];
  int64_t nb = m->nbnode[((size_t)e * 6 + f) * n * n + JK];
  node_normal(m, e, f, ijk, norm);
  for (l = 0; l < NF; l++) ui[l] = we[l * np + ijk];
  if (nb >= 0) {
    int64_t en = nb / np, in = nb % np;
    for (l = 0; l < NF; l++) ua[l] = w[(size_t)en * NF * np + l * np + in];
  } else if (nb == -2) {
    mixed_trace(m, P, e, f, JK % n, JK / n, w, ua);
  } else if (nb == -3) {
    hang_trace(m, P, e, f, JK, w, ua);
  } else if (nb == -4) {
    const double *X = m->ext + (((size_t)e * 6 + f) * n * n + JK) * NF;
    for (l = 0; l < NF; l++) ua[l] = X[l];
  } else if (m->bc == 0) {
    const double *X = m->xyz + (size_t)e * 3 * np;
    double xyz[3] = {X[ijk], X[np + ijk], X[2 * np + ijk]};
    planewave(m->k, xyz, t, ua);
  } else {
    /* outgoing radiation: exterior state with zero incoming
       characteristic pi + c.n, copy of the outgoing characteristic
       pi - c.n and of the tangential c */
    double cn = ui[1] * norm[0] + ui[2] * norm[1] + ui[3] * norm[2];
    double wout = ui[0] - cn;
    double pie = 0.5 * wout, cne = -0.5 * wout;
    ua[0] = pie;
    for (l = 0; l < 3; l++) ua[1 + l] = ui[1 + l] + (cne - cn) * norm[l];
    ua[4] = ui[4];
  }
  flux1d(fi, norm, ui);
  flux1d(fa, norm, ua);
  if (m->numflux == 1) upwind(ui, ua, norm, fnum);
  else llf(ui, ua, fi, fa, fnum);
}

/* RHS of one element: r[e] = RHS(w) at time t.  tmp holds 18*np doubles. */
static void rhs_elem(const nmo_mesh *m, const nmo_pts *P, const double *D,
                     const double *wq, double t, const double *w, double *r, int e,
                     double *tmp)
{
  int n = m->n, np = n * n * n, i, j, k, f, l;
  const double *we = w + (size_t)e * NF * np;
  double *re = r + (size_t)e * NF * np;
  const double *pi = we, *cx = we + np, *cy = we + 2 * np, *cz = we + 3 * np;
  double *fl = tmp;            /* 3 flux arrays */
  double *divf = tmp + 3 * np; /* 4 div arrays: pi, cx, cy, cz */
  double *work = tmp + 7 * np; /* 6 np for cart_partials */
  double *zero = tmp + 13 * np;
  double *fpx = fl, *fpy = fl + np, *fpz = fl + 2 * np;

  /* flux arrays f_pi^i = -c_i (scalarwave1_f_divf) */
  for (i = 0; i < np; i++) {
    double u[5] = {pi[i], cx[i], cy[i], cz[i], we[4 * np + i]};
    double ff[5], no[3] = {1., 0., 0.};
    flux1d(ff, no, u); fpx[i] = ff[0];
    no[0] = 0; no[1] = 1.;
    flux1d(ff, no, u); fpy[i] = ff[0];
    no[1] = 0.; no[2] = 1.;
    flux1d(ff, no, u); fpz[i] = ff[0];
  }
  cart_divergence(m, e, D, fpx, fpy, fpz, divf, work);
  /* f_{c_j}^i = -pi delta^i_j: the off-diagonal flux arrays are (signed)
     zeros whose derivatives are zero */
  for (j = 0; j < 3; j++) {
    double *fc[3];
    for (i = 0; i < 3; i++) fc[i] = zero;
    for (i = 0; i < np; i++) fl[i] = -pi[i] * 1.0;
    fc[j] = fl;
    for (i = 0; i < np; i++) zero[i] = 0.;
    cart_divergence(m, e, D, fc[0], fc[1], fc[2], divf + (1 + j) * np, work);
  }

  /* volume RHS (scalarwave1_vol_rhs_u) */
  for (k = 0; k < n; k++)
    for (j = 0; j < n; j++)
      for (i = 0; i < n; i++) {
        int ijk = i + n * (j + n * k);
        int onface = (i == 0 || i == n - 1 || j == 0 || j == n - 1 ||
                      k == 0 || k == n - 1);
        double interior = !onface;
        re[4 * np + ijk] = pi[ijk];
        for (l = 0; l < 4; l++) re[l * np + ijk] = -divf[l * np + ijk] * interior;
      }

  /* surface fluxes (dg_add_surface_fluxes_sign_fvflag, sign=+1, sqrtgdiag) */
  for (f = 0; f < 6; f++) {
    int dir = f / 2, p = (f % 2) * (n - 1), a, b;
    double oow = 1. / wq[p];
    for (b = 0; b < n; b++)
      for (a = 0; a < n; a++) {
        int ijk = face_node(n, f, a, b), JK = a + n * b;
        double fi[5], fnum[5], gd_ow;
        face_fnum(m, P, e, f, ijk, JK, t, w, fi, fnum);
        gd_ow = sqrtgdiag(m, e, dir, ijk) * oow;
        for (l = 0; l < 4; l++) {
          double F = (fnum[l] - fi[l] * 1.0) * 1.0;
          divf[l * np + ijk] += F * gd_ow;
        }
      }
  }

  /* vladdto_onfaces(r, -1, divf) */
  for (k = 0; k < n; k++)
    for (j = 0; j < n; j++)
      for (i = 0; i < n; i++)
        if (i == 0 || i == n - 1 || j == 0 || j == n - 1 || k == 0 || k == n - 1) {
          int ijk = i + n * (j + n * k);
          for (l = 0; l < 4; l++) re[l * np + ijk] += -1. * divf[l * np + ijk];
        }
}

/* ------------------------------------------------------------------ */
/* finite-volume elements                                              */
/* ------------------------------------------------------------------ */
/* equally spaced points on [-1, 1] (uniform_x) */
void nmo_uniform(int npoints, double *x)
{
  int N = npoints - 1, j;
  double y, h;
  if (N == 0) { x[0] = 0.; return; }
  x[0] = -1.; x[N] = 1.;
  if (N == 1) return;
  h = 2. / N;
  for (j = 1; j <= N / 2; j++) {
    if (j == N / 2.0) y = 0.;
    else y = -1. + j * h;
    x[N - j] = -y;
    x[j] = +y;
  }
}

/* WENO3 towards midpoint im from the left (rec1d_p_WENO3, u_scale = 1) */
static double weno3_p(const double *u, int im, double o0, double o1,
                      double l00, double l01, double l10, double l11)
{
  double u_im1 = u[im - 1], u_i = u[im], u_ip1 = u[im + 1];
  double d1 = u_i - u_im1, d2 = u_ip1 - u_i;
  double b1 = d1 * d1 + 1e-6 * 1.0, b2 = d2 * d2 + 1e-6 * 1.0;
  double ob1 = o0 / (b1 * b1), ob2 = o1 / (b2 * b2);
  double sum = ob1 + ob2;
  double w1 = ob1 / sum, w2 = ob2 / sum;
  double u1 = l00 * u_im1 + l01 * u_i, u2 = l10 * u_i + l11 * u_ip1;
  return w1 * u1 + w2 * u2;
}

/* WENO3 towards midpoint im from the right (rec1d_m_WENO3) */
static double weno3_m(const double *u, int im, double o0, double o1,
                      double l00, double l01, double l10, double l11)
{
  double u_i = u[im], u_ip1 = u[im + 1], u_ip2 = u[im + 2];
  double d1 = u_ip1 - u_i, d2 = u_ip2 - u_ip1;
  double b1 = d1 * d1 + 1e-6 * 1.0, b2 = d2 * d2 + 1e-6 * 1.0;
  double ob1 = o0 / (b1 * b1), ob2 = o1 / (b2 * b2);
  double sum = ob1 + ob2;
  double w1 = ob1 / sum, w2 = ob2 / sum;
  double u1 = l00 * u_i + l01 * u_ip1, u2 = l10 * u_ip1 + l11 * u_ip2;
  return w1 * u1 + w2 * u2;
}

#define C1312 (1.083333333333333333333333)
/* WENO5 with uniform weights (rec1d_p_WENO5_uniform) */
static double weno5_p(const double *u, int im)
{
  const double oo6 = 1 / 6.;
  double u_im2 = u[im - 2], u_im1 = u[im - 1], u_i = u[im];
  double u_ip1 = u[im + 1], u_ip2 = u[im + 2];
  double b01 = u_im2 - 2. * u_im1 + u_i, b02 = u_im2 - 4. * u_im1 + 3. * u_i;
  double b11 = u_im1 - 2. * u_i + u_ip1, b12 = u_im1 - u_ip1;
  double b21 = u_i - 2. * u_ip1 + u_ip2, b22 = 3. * u_i - 4. * u_ip1 + u_ip2;
  double b0 = C1312 * b01 * b01 + 0.25 * b02 * b02;
  double b1 = C1312 * b11 * b11 + 0.25 * b12 * b12;
  double b2 = C1312 * b21 * b21 + 0.25 * b22 * b22;
  double e0 = b0 + 1e-40 * 1.0, e1 = b1 + 1e-40 * 1.0, e2 = b2 + 1e-40 * 1.0;
  double o0 = 1. / (e0 * e0), o1 = 6. / (e1 * e1), o2 = 3. / (e2 * e2);
  double oos = 1. / (o0 + o1 + o2);
  double w0 = o0 * oos, w1 = o1 * oos, w2 = o2 * oos;
  double q0 = (2. * oo6) * u_im2 + (-7. * oo6) * u_im1 + (11. * oo6) * u_i;
  double q1 = (-oo6) * u_im1 + (5. * oo6) * u_i + (2. * oo6) * u_ip1;
  double q2 = (2. * oo6) * u_i + (5. * oo6) * u_ip1 + (-oo6) * u_ip2;
  return w0 * q0 + w1 * q1 + w2 * q2;
}

/* rec1d_m_WENO5_uniform */
static double weno5_m(const double *u, int im)
{
  const double oo6 = 1 / 6.;
  double u_im1 = u[im - 1], u_i = u[im], u_ip1 = u[im + 1];
  double u_ip2 = u[im + 2], u_ip3 = u[im + 3];
  double b21 = u_ip1 - 2. * u_ip2 + u_ip3, b22 = 3. * u_ip1 - 4. * u_ip2 + u_ip3;
  double b11 = u_i - 2. * u_ip1 + u_ip2, b12 = u_i - u_ip2;
  double b01 = u_im1 - 2. * u_i + u_ip1, b02 = u_im1 - 4. * u_i + 3. * u_ip1;
  double b2 = C1312 * b21 * b21 + 0.25 * b22 * b22;
  double b1 = C1312 * b11 * b11 + 0.25 * b12 * b12;
  double b0 = C1312 * b01 * b01 + 0.25 * b02 * b02;
  double e2 = b2 + 1e-40 * 1.0, e1 = b1 + 1e-40 * 1.0, e0 = b0 + 1e-40 * 1.0;
  double o2 = 1. / (e2 * e2), o1 = 6. / (e1 * e1), o0 = 3. / (e0 * e0);
  double oos = 1. / (o0 + o1 + o2);
  double w2 = o2 * oos, w1 = o1 * oos, w0 = o0 * oos;
  double q2 = (11. * oo6) * u_ip1 + (-7. * oo6) * u_ip2 + (2. * oo6) * u_ip3;
  double q1 = (2. * oo6) * u_i + (5. * oo6) * u_ip1 + (-oo6) * u_ip2;
  double q0 = (-oo6) * u_im1 + (5. * oo6) * u_i + (2. * oo6) * u_ip1;
  return w0 * q0 + w1 * q1 + w2 * q2;
}

/* rec1d_p_WENOZ_uniform (rec1d.c:1627-1679,1732-1754): WENO5 with the
   WENO-Z weights optw_k (1 + tau5 / (b_k + eps)), tau5 = |b0 - b2| */
static double wenoz_p(const double *u, int im)
{
  const double oo6 = 1 / 6.;
  double u_im2 = u[im - 2], u_im1 = u[im - 1], u_i = u[im];
  double u_ip1 = u[im + 1], u_ip2 = u[im + 2];
  double b01 = u_im2 - 2. * u_im1 + u_i, b02 = u_im2 - 4. * u_im1 + 3. * u_i;
  double b11 = u_im1 - 2. * u_i + u_ip1, b12 = u_im1 - u_ip1;
  double b21 = u_i - 2. * u_ip1 + u_ip2, b22 = 3. * u_i - 4. * u_ip1 + u_ip2;
  double b0 = C1312 * b01 * b01 + 0.25 * b02 * b02;
  double b1 = C1312 * b11 * b11 + 0.25 * b12 * b12;
  double b2 = C1312 * b21 * b21 + 0.25 * b22 * b22;
  double e0 = b0 + 1e-40 * 1.0, e1 = b1 + 1e-40 * 1.0, e2 = b2 + 1e-40 * 1.0;
  double tau5 = fabs(b0 - b2);
  double o0 = 1. * (1. + tau5 / e0), o1 = 6. * (1. + tau5 / e1), o2 = 3. * (1. + tau5 / e2);
  double oos = 1. / (o0 + o1 + o2);
  double w0 = o0 * oos, w1 = o1 * oos, w2 = o2 * oos;
  double q0 = (2. * oo6) * u_im2 + (-7. * oo6) * u_im1 + (11. * oo6) * u_i;
  double q1 = (-oo6) * u_im1 + (5. * oo6) * u_i + (2. * oo6) * u_ip1;
  double q2 = (2. * oo6) * u_i + (5. * oo6) * u_ip1 + (-oo6) * u_ip2;
  return w0 * q0 + w1 * q1 + w2 * q2;
}

/* rec1d_m_WENOZ_uniform (rec1d.c:1681-1730,1756-1780) */
static double wenoz_m(const double *u, int im)
{
  const double oo6 = 1 / 6.;
  double u_im1 = u[im - 1], u_i = u[im], u_ip1 = u[im + 1];
  double u_ip2 = u[im + 2], u_ip3 = u[im + 3];
  double b21 = u_ip1 - 2. * u_ip2 + u_ip3, b22 = 3. * u_ip1 - 4. * u_ip2 + u_ip3;
  double b11 = u_i - 2. * u_ip1 + u_ip2, b12 = u_i - u_ip2;
  double b01 = u_im1 - 2. * u_i + u_ip1, b02 = u_im1 - 4. * u_i + 3. * u_ip1;
  double b2 = C1312 * b21 * b21 + 0.25 * b22 * b22;
  double b1 = C1312 * b11 * b11 + 0.25 * b12 * b12;
  double b0 = C1312 * b01 * b01 + 0.25 * b02 * b02;
  double e2 = b2 + 1e-40 * 1.0, e1 = b1 + 1e-40 * 1.0, e0 = b0 + 1e-40 * 1.0;
  double tau5 = fabs(b0 - b2);
  double o2 = 1. * (1. + tau5 / e2), o1 = 6. * (1. + tau5 / e1), o0 = 3. * (1. + tau5 / e0);
  double oos = 1. / (o0 + o1 + o2);
  double w2 = o2 * oos, w1 = o1 * oos, w0 = o0 * oos;
  double q2 = (11. * oo6) * u_ip1 + (-7. * oo6) * u_ip2 + (2. * oo6) * u_ip3;
  double q1 = (2. * oo6) * u_i + (5. * oo6) * u_ip1 + (-oo6) * u_ip2;
  double q0 = (-oo6) * u_im1 + (5. * oo6) * u_i + (2. * oo6) * u_ip1;
  return w0 * q0 + w1 * q1 + w2 * q2;
}

/* left state at midpoint im (0..n-2) of a pencil of n values */
static double rec_p(int mode, int n, const double *u, int im, double r3)
{
  if (mode == NMO_REC_1) return u[im];
  if (mode == NMO_REC_WENOM5_2 && im >= 2 && im <= n - 3) return weno5_p(u, im);
  if (mode == NMO_REC_WENOMZ_2 && im >= 2 && im <= n - 3) return wenoz_p(u, im);
  /* rec1d_p_WENOm3_2 */
  if (im >= 1 && im <= n - 2) return weno3_p(u, im, 1., r3, -0.5, 1.5, 0.5, 0.5);
  if (n < 3) return u[im];
  return 0.5 * u[0] + 0.5 * u[1];            /* im == 0 */
}

/* right state at midpoint im */
static double rec_m(int mode, int n, const double *u, int im, double r3)
{
  if (mode == NMO_REC_1) return u[im + 1];
  if (mode == NMO_REC_WENOM5_2 && im >= 1 && im <= n - 4) return weno5_m(u, im);
  if (mode == NMO_REC_WENOMZ_2 && im >= 1 && im <= n - 4) return wenoz_m(u, im);
  /* rec1d_m_WENOm3_2 */
  if (im >= 0 && im <= n - 3) return weno3_m(u, im, r3, 1., 0.5, 0.5, 1.5, -0.5);
  if (n < 3) return u[im + 1];
  return 0.5 * u[n - 2] + 0.5 * u[n - 1];    /* im == n-2 */
}

/* det(dXb/dx) at node ijk (coordinates_init_node) */
static double det_dXbdx(const nmo_mesh *m, int e, int ijk)
{
  int np = m->n * m->n * m->n, a, b;
  const double *bb = m->bbox + 6 * e;
  double d0 = 2. / (bb[1] - bb[0]), d1 = 2. / (bb[3] - bb[2]);
  double d2 = 2. / (bb[5] - bb[4]);
  double det = d0 * d1 * d2, M[3][3];
  if (!m->curvi[e]) return det;
  for (a = 0; a < 3; a++)
    for (b = 0; b < 3; b++) M[a][b] = m->dXdx[((size_t)e * 9 + a * 3 + b) * np + ijk];
  return det * (M[0][0] * M[1][1] * M[2][2] - M[0][2] * M[1][1] * M[2][0] +
                M[0][1] * M[1][2] * M[2][0] + M[0][2] * M[1][0] * M[2][1] -
                M[0][0] * M[1][2] * M[2][1] - M[0][1] * M[1][0] * M[2][2]);
}

/* RHS of one fin.-vol. element (scalarwave1_vol_rhs_u / _surf_rhs_u with
   use_fv: fv_divf, then the surface terms).  tmp holds 8*np doubles. */
/* coordinates_midpoint_data = yes on a curvilinear element: sqrtgdiag_d,
   det(dXb/dx) and the unit normal of direction d at the midpoint right of
   node ijk (coordinates.c:337-420, utilities.c:48-80,90-103) */
static void midpoint_factors(const nmo_mesh *m, int e, int d, int ijk, double *sgm,
                             double *oojm, double nrm[3])
{
  int np = m->n * m->n * m->n, a, b, l;
  const double *bb = m->bbox + 6 * e;
  double d0 = 2. / (bb[1] - bb[0]), d1 = 2. / (bb[3] - bb[2]), d2 = 2. / (bb[5] - bb[4]);
  double dXbdX[3] = {d0, d1, d2}, M[3][3], g = 0., smag;
  for (a = 0; a < 3; a++)
    for (b = 0; b < 3; b++) M[a][b] = m->dXdxm[(((size_t)e * 3 + d) * 9 + a * 3 + b) * np + ijk];
  for (l = 0; l < 3; l++) g += M[d][l] * M[d][l];
  *sgm = dXbdX[d] * sqrt(g);
  *oojm = d0 * d1 * d2 * (M[0][0] * M[1][1] * M[2][2] - M[0][2] * M[1][1] * M[2][0] +
                          M[0][1] * M[1][2] * M[2][0] + M[0][2] * M[1][0] * M[2][1] -
                          M[0][0] * M[1][2] * M[2][1] - M[0][1] * M[1][0] * M[2][2]);
  smag = 1. * sqrt(M[d][0] * M[d][0] + M[d][1] * M[d][1] + M[d][2] * M[d][2]);
  if (smag == 0.0) smag = 1.;
  for (l = 0; l < 3; l++) nrm[l] = M[d][l] / smag;
}

static void rhs_elem_fv(const nmo_mesh *m, const nmo_pts *P, double t,
                        const double *w, double *r, int e, double *tmp)
{
  int n = m->n, np = n * n * n, i, j, k, f, l, dir, a, b, i0;
  const double *we = w + (size_t)e * NF * np;
  double *re = r + (size_t)e * NF * np;
  const double *bb = m->bbox + 6 * e;
  double *divf = tmp, *ooJ = tmp + 4 * np, *sg = tmp + 5 * np;
  double Xb[64], Xbm[64], dXb[64], distXb[6];
  double fnumR[4] = {0., 0., 0., 0.}, fnumL[4] = {0., 0., 0., 0.};
  const int addsurf = (m->fv_extrap == 1);     /* dnfn_extrap1 */
  const double r3 = m->fv_w3ratio;

  /* points, midpoints and the n distances dXb (set_nm_nodemidpoint_distsXb_dir) */
  nmo_uniform(n, Xb);
  for (i = 0; i < n - 1; i++) Xbm[i] = 0.5 * (Xb[i] + Xb[i + 1]);
  for (f = 0; f < 6; f++) {
    int d = f / 2, right = f % 2, id = (n - 2) * right;
    double Xbf = (2. * bb[f] - (bb[2 * d + 1] + bb[2 * d])) / (bb[2 * d + 1] - bb[2 * d]);
    distXb[f] = fabs(Xbm[id] - Xbf);
  }
  for (i = 0; i < np; i++) {
    ooJ[i] = det_dXbdx(m, e, i);
    for (dir = 0; dir < 3; dir++) sg[dir * np + i] = sqrtgdiag(m, e, dir, i);
  }
  for (i = 0; i < 4 * np; i++) divf[i] = 0.;

  for (dir = 0; dir < 3; dir++) {
    const int st = (dir == 0) ? 1 : (dir == 1) ? n : n * n;
    const double *sgd = sg + dir * np;
    dXb[0] = distXb[2 * dir];
    dXb[n - 1] = distXb[2 * dir + 1];
    for (i = 1; i < n - 1; i++) dXb[i] = Xbm[i] - Xbm[i - 1];
    for (b = 0; b < n; b++)
      for (a = 0; a < n; a++) {
        const int base = face_node(n, 2 * dir, a, b);   /* i0 = 0 of this pencil */
        double qc[NF][64], df[4][64];
        for (i0 = 0; i0 < n; i0++)
          for (l = 0; l < NF; l++) qc[l][i0] = we[l * np + base + i0 * st];
        for (i0 = 0; i0 < n; i0++) {
          const int ccc = base + i0 * st;
          const int g0 = (i0 > 0), lN = (i0 < n - 1);
          const int cccL = base + (g0 ? i0 - 1 : i0) * st;
          const int cccR = base + (lN ? i0 : i0 - 1) * st;
          const double wc = dXb[i0];
          const int mid = m->dXdxm && m->curvi[e];
          double JR, JL, sgR = sgd[cccR], ojR = ooJ[cccR], sgL = sgd[cccL], ojL = ooJ[cccL];
          if (mid) {   /* the midpoint arrays replace the grid ones (fv.c:126-137) */
            double nn_[3];
            if (lN) midpoint_factors(m, e, dir, cccR, &sgR, &ojR, nn_);
            if (g0) midpoint_factors(m, e, dir, cccL, &sgL, &ojL, nn_);
          }
          if (g0 && lN) {
            JR = sgR / (ojR * wc);
            JL = sgL / (ojL * wc);
          } else if (!g0 && lN) {
            JR = sgR / (ojR * wc);
            JL = sgd[ccc] / (ooJ[ccc] * wc);
          } else if (g0 && !lN) {
            JR = sgd[ccc] / (ooJ[ccc] * wc);
            JL = sgL / (ojL * wc);
          } else {
            JR = JL = sgd[ccc] / (ooJ[ccc] * wc);
          }
          if (!addsurf) { JR = lN * JR; JL = g0 * JL; }
          if (g0) {
            for (l = 0; l < 4; l++) fnumL[l] = -fnumR[l];
          } else if (addsurf) {
            double fi[5], fn[5];
            face_fnum(m, P, e, 2 * dir, ccc, a + n * b, t, w, fi, fn);
            for (l = 0; l < 4; l++) fnumL[l] = fn[l];
          }
          if (lN) {
            double ui[5], ua[5], fi[5], fa[5], fn[5], norm[3];
            if (mid) {   /* DGINFO_MIDPTNORM: normal at the midpoint */
              double s_, o_;
              midpoint_factors(m, e, dir, ccc, &s_, &o_, norm);
            } else {
              node_normal(m, e, 2 * dir + 1, ccc, norm);
            }
            for (l = 0; l < NF; l++) {
              ui[l] = rec_p(m->fv_rec, n, qc[l], i0, r3);
              ua[l] = rec_m(m->fv_rec, n, qc[l], i0, r3);
            }
            flux1d(fi, norm, ui);
            flux1d(fa, norm, ua);
            if (m->numflux == 1) upwind(ui, ua, norm, fn);
            else llf(ui, ua, fi, fa, fn);
            for (l = 0; l < 4; l++) fnumR[l] = fn[l];
          } else if (addsurf) {
            double fi[5], fn[5];
            face_fnum(m, P, e, 2 * dir + 1, ccc, a + n * b, t, w, fi, fn);
            for (l = 0; l < 4; l++) fnumR[l] = fn[l];
          }
          for (l = 0; l < 4; l++) {
            double fR = fnumR[l] - 0., fL = fnumL[l] - 0.;
            df[l][i0] = JR * fR + JL * fL;
          }
        }
        if (addsurf && n > 2) {    /* FV_DNFN_EXTRAP1, s1 = 0, s2 = DBL_MAX */
          const double w0 = 1. / 0.75, w1 = 1. - w0;
          for (l = 0; l < 4; l++) {
            df[l][0] = w0 * df[l][0] + w1 * df[l][1];
            df[l][n - 1] = w0 * df[l][n - 1] + w1 * df[l][n - 2];
          }
        }
        for (i0 = 0; i0 < n; i0++) {
          const int ccc = base + i0 * st;
          for (l = 0; l < 4; l++) divf[l * np + ccc] += df[l][i0] * ooJ[ccc];
        }
      }
  }

  /* volume RHS */
  for (k = 0; k < n; k++)
    for (j = 0; j < n; j++)
      for (i = 0; i < n; i++) {
        int ijk = i + n * (j + n * k);
        int onface = (i == 0 || i == n - 1 || j == 0 || j == n - 1 ||
                      k == 0 || k == n - 1);
        double interior = !onface;
        re[4 * np + ijk] = we[ijk];
        for (l = 0; l < 4; l++) re[l * np + ijk] = -divf[l * np + ijk] * interior;
      }

  /* surface terms on fin.-vol. faces: only when fv_divf did not add them */
  if (!addsurf)
    for (f = 0; f < 6; f++) {
      int d = f / 2;
      double oow = 1. / (0. + distXb[f] * 1.);
      for (b = 0; b < n; b++)
        for (a = 0; a < n; a++) {
          int ijk = face_node(n, f, a, b);
          double fi[5], fn[5], gd_ow;
          face_fnum(m, P, e, f, ijk, a + n * b, t, w, fi, fn);
          gd_ow = sg[d * np + ijk] * oow;
          for (l = 0; l < 4; l++) {
            double F = (fn[l] - fi[l] * 0.) * 1.0;
            divf[l * np + ijk] += F * gd_ow;
          }
        }
    }

  /* vladdto_onfaces(r, -1, divf) */
  for (k = 0; k < n; k++)
    for (j = 0; j < n; j++)
      for (i = 0; i < n; i++)
        if (i == 0 || i == n - 1 || j == 0 || j == n - 1 || k == 0 || k == n - 1) {
          int ijk = i + n * (j + n * k);
          for (l = 0; l < 4; l++) re[l * np + ijk] += -1. * divf[l * np + ijk];
        }
}

/* ------------------------------------------------------------------ */
/* trouble indicators                                                  */
/* ------------------------------------------------------------------ */
static double legendre_p(int l, double x)       /* basis_LegendreP */
{
  double Pk = 0., P0 = 1.0, P1 = x;
  int k;
  if (l == 0) return P0;
  if (l == 1) return P1;
  for (k = 2; k <= l; k++) {
    Pk = (x * (2 * k - 1) * P1 - (k - 1) * P0) / k;
    P0 = P1;
    P1 = Pk;
  }
  return Pk;
}

/* Persson's indicator of one field on LGL points, all n^3 coefficients
   (evolve_Persson_array_indicator with the analysis matrices of
   LGL_AT_ST_matrices) */
double nmo_persson(int n, const double *u, double u_scale)
{
  double x[64], w[64], A[64 * 64];
  int np = n * n * n, N = n - 1, i, j, k, l, d;
  double *c = (double *)malloc(sizeof(double) * 2 * np), *t = c + np;
  double c2_sum = 0., c2_hi = 0., se;
  nmo_lgl(n, x, w);
  for (i = 0; i < n; i++) {
    double ooci = 0.5 * (2 * i + 1), oosci;
    if (i == N && N != 0) ooci = 0.5 * i;
    oosci = sqrt(ooci);
    for (j = 0; j < n; j++) A[i * n + j] = w[j] * (legendre_p(i, x[j]) * oosci);
  }
  memcpy(t, u, sizeof(double) * np);
  for (d = 0; d < 3; d++) {
    const int st = (d == 0) ? 1 : (d == 1) ? n : n * n;
    for (k = 0; k < np; k++) {
      const int ii = (d == 0) ? k % n : (d == 1) ? (k / n) % n : k / (n * n);
      const double *line = t + k - ii * st;
      double sum = 0.0;
      for (l = 0; l < n; l++) sum += A[ii * n + l] * line[l * st];
      c[k] = sum;
    }
    memcpy(t, c, sizeof(double) * np);
  }
  if (u_scale >= 0.) c[0] = u_scale * 2. * sqrt(2.);
  for (k = 0; k < n; k++)
    for (j = 0; j < n; j++)
      for (i = 0; i < n; i++) {
        double co = c[i + n * (j + n * k)];
        c2_sum += co * co;
      }
  for (k = 0; k < n; k++)
    for (j = 0; j < n; j++)
      for (i = 0; i < n; i++)
        if ((i == n - 1 && n > 1) || (j == n - 1 && n > 1) || (k == n - 1 && n > 1)) {
          double co = c[i + n * (j + n * k)];
          c2_hi += co * co;
        }
  se = log10(c2_hi / (c2_sum + 2.2250738585072014e-308) + 1e-50);
  free(c);
  return se;
}

/* neighbour element across face f of element e, -1 on outer faces */
static int64_t face_neighbour(const nmo_mesh *m, int e, int f)
{
  int n = m->n, np = n * n * n;
  int64_t nb = m->nbnode[((size_t)e * 6 + f) * n * n];
  if (nb >= 0) return nb / np;
  if (nb == -2) return m->mixface[((size_t)e * 6 + f) * 3];
  return -1;
}

/* Trouble flags of all elements for state u against u_p: relaxed discrete
   maximum principle over the element and its face neighbours
   (evolve_RDMP_trouble) on every element, Persson's indicator above
   persson_max on DG elements.  Flags: DG troubled 1, DG fine 0, FV troubled
   0, FV fine -1.  pers[E][5] gets the indicators (0 on FV elements). */
int nmo_trouble(const nmo_mesh *m, const double *u, const double *u_p, double deltafac,
                double delta0, double epsilon, double persson_max, double uscale,
                int32_t *flags, double *pers)
{
  int n = m->n, np = n * n * n, e;
  double *mm = (double *)malloc(sizeof(double) * (size_t)m->nelem * NF * 2);
  if (!mm) return 2;
  for (e = 0; e < m->nelem; e++) {
    int l, q;
    for (l = 0; l < NF; l++) {
      const double *v = u_p + ((size_t)e * NF + l) * np;
      double lo = v[0], hi = v[0];
      for (q = 1; q < np; q++) {
        if (v[q] < lo) lo = v[q];
        if (v[q] > hi) hi = v[q];
      }
      mm[((size_t)e * NF + l) * 2] = lo;
      mm[((size_t)e * NF + l) * 2 + 1] = hi;
    }
  }
#pragma omp parallel for schedule(static)
  for (e = 0; e < m->nelem; e++) {
    int l, q, f, bad = 0;
    int efv = m->fv && m->fv[e];
    for (l = 0; l < NF; l++) {
      double lo = mm[((size_t)e * NF + l) * 2], hi = mm[((size_t)e * NF + l) * 2 + 1];
      double delta, lower, upper;
      const double *v = u + ((size_t)e * NF + l) * np;
      for (f = 0; f < 6; f++) {
        int64_t e2 = face_neighbour(m, e, f);
        if (e2 < 0) continue;
        if (mm[((size_t)e2 * NF + l) * 2] < lo) lo = mm[((size_t)e2 * NF + l) * 2];
        if (mm[((size_t)e2 * NF + l) * 2 + 1] > hi) hi = mm[((size_t)e2 * NF + l) * 2 + 1];
      }
      delta = deltafac * fmax(delta0, epsilon * (hi - lo));
      lower = lo - delta;
      upper = hi + delta;
      for (q = 0; q < np; q++)
        if (v[q] < lower || v[q] > upper) bad = 1;
      if (!efv) {
        double se = nmo_persson(n, v, uscale);
        if (pers) pers[(size_t)e * NF + l] = se;
        if (se > persson_max) bad = 1;
      } else if (pers) {
        pers[(size_t)e * NF + l] = 0.;
      }
    }
    flags[e] = efv ? (bad ? 0 : -1) : (bad ? 1 : 0);
  }
  free(mm);
  return 0;
}

static void basis(int n, double *D, double *wq)
{
  double x[64];
  nmo_lgl(n, x, wq);
  nmo_diffmat(n, x, D);
}

/* r = RHS(w, t) on all elements */
int nmo_rhs(const nmo_mesh *m, double t, const double *w, double *r)
{
  int n = m->n, np = n * n * n, i, j;
  double D[64 * 64], wq[64];
  nmo_pts P;
  if (n < 2 || n > 64) return 1;
  basis(n, D, wq);
  nmo_lgl(n, P.xl, wq);
  nmo_uniform(n, P.xu);
  for (i = 0; i < n; i++) {          /* Lagrange_winterp */
    double denom = 1.;
    for (j = 0; j < n; j++) if (j != i) denom *= (P.xl[i] - P.xl[j]);
    P.wl[i] = 1. / denom;
  }
#pragma omp parallel
  {
    double *tmp = (double *)malloc(sizeof(double) * 18 * np);
    int e;
#pragma omp for schedule(static)
    for (e = 0; e < m->nelem; e++) {
      if (m->fv && m->fv[e]) rhs_elem_fv(m, &P, t, w, r, e, tmp);
      else rhs_elem(m, &P, D, wq, t, w, r, e, tmp);
    }
    free(tmp);
  }
  return 0;
}

/* one classic RK4 step in place (evolve_RK4_mesh); work holds 3 states */
int nmo_rk4_step(const nmo_mesh *m, double t, double dt, double *u,
                 double *work)
{
  size_t N = (size_t)m->nelem * NF * m->n * m->n * m->n, i;
  double *u_p = work, *w = work + N, *r = work + 2 * N;
  const double c[4] = {dt / 6., dt / 3., dt / 3., dt / 6.};
  const double a[3] = {dt / 2., dt / 2., dt};
  const double ts[4] = {t, t + 0.5 * dt, t + 0.5 * dt, t + dt};
  int s;
  memcpy(u_p, u, N * sizeof(double));
  memcpy(w, u, N * sizeof(double));
  for (s = 0; s < 4; s++) {
    if (nmo_rhs(m, ts[s], w, r)) return 1;
#pragma omp parallel for schedule(static)
    for (i = 0; i < N; i++) {
      u[i] += c[s] * r[i];
      if (s < 3) w[i] = 1. * u_p[i] + a[s] * r[i];
    }
  }
  return 0;
}

/* One Euler (method 1) or sspRK3 (method 2) step (evolve_Euler_mesh,
   evolve_sspRK3_mesh, src/main/evolve/RungeKutta.c:84-200), the vector
   operations in the reference's order. */
static int nmo_other_step(const nmo_mesh *m, int method, double t, double dt, double *u,
                          double *work)
{
  size_t N = (size_t)m->nelem * NF * m->n * m->n * m->n, i;
  double *u_p = work, *w = work + N, *r = work + 2 * N;
  memcpy(u_p, u, N * sizeof(double));
  memcpy(w, u, N * sizeof(double));
  if (nmo_rhs(m, t, w, r)) return 1;                       /* r = RHS(w, t) */
  if (method == 1) {
    for (i = 0; i < N; i++) u[i] += dt * r[i];             /* u += r dt */
    return 0;
  }
  for (i = 0; i < N; i++) {
    u[i] += dt / 6. * r[i];                                /* u += r dt/6 */
    w[i] = 1. * u_p[i] + dt * r[i];                        /* w = u_p + r dt */
  }
  if (nmo_rhs(m, t + dt, w, r)) return 1;                  /* r = RHS(w, t+dt) */
  for (i = 0; i < N; i++) {
    u[i] += dt / 6. * r[i];                                /* u += r dt/6 */
    w[i] += dt * r[i];                                     /* w += r dt */
    w[i] = 0.75 * u_p[i] + 0.25 * w[i];                    /* w = 0.75 u_p + 0.25 w */
  }
  if (nmo_rhs(m, t + 0.5 * dt, w, r)) return 1;            /* r = RHS(w, t+dt/2) */
  for (i = 0; i < N; i++) u[i] += dt * 2. / 3. * r[i];     /* u += r dt*2/3 */
  return 0;
}

/* nsteps steps of method 0 (RK4), 1 (Euler) or 2 (sspRK3), times
   accumulated as in evolve_mesh */
int nmo_evolve(const nmo_mesh *m, int method, double t, double dt, int nsteps, double *u)
{
  size_t N = (size_t)m->nelem * NF * m->n * m->n * m->n;
  double *work = (double *)malloc(3 * N * sizeof(double));
  long double Te = t, te = 0.;
  int s, rc = 0;
  if (!work) return 2;
  for (s = 0; s < nsteps && !rc; s++) {
    double ts = (double)(Te + te);
    rc = method == 0 ? nmo_rk4_step(m, ts, dt, u, work) : nmo_other_step(m, method, ts, dt, u, work);
    te += dt;
  }
  free(work);
  return rc;
}

/* u of one 1D direction d of an element array: out = M in along d */
static void mm_dir(int n, const double *M, int d, const double *in, double *out)
{
  int np = n * n * n, st = d == 0 ? 1 : d == 1 ? n : n * n, q, j;
  for (q = 0; q < np; q++) {
    int i = d == 0 ? q % n : d == 1 ? (q / n) % n : q / (n * n);
    const double *line = in + q - i * st;
    double s = 0.;
    for (j = 0; j < n; j++) s += M[i * n + j] * line[j * st];
    out[q] = s;
  }
}

/* Exponential filter of every field of every element after a step
   (evolve_filter_evosys_mesh -> expfilter_var, src/main/basis/filter.c:
   15-96, src/main/evolve/evolve.c:656-700): u -> u / (1/J) (jpow = 1),
   coefficients c = A^3 u, c_ijk *= f_i f_j f_k with f_k = exp(-alp
   (k/(n-1-dn))^s), u = S^3 c, u -> u (1/J); A, S the normalised-Legendre
   analysis and synthesis matrices of the element's points (LGL: A_ij =
   w_j S_ji; equally spaced: A = S^-1, Legendre.c:277-310,723-729). */
/* The MRS limiter of every element (limdata_MRS and limiter_MRS,
   src/main/limiter/limiter.c:61-204, with var_nodeaverage,
   src/main/basis/basis.c:462-510): node averages and extrema of all
   elements first, then per element theta = min(1, min over fields of the
   ratios against the face neighbours' extrema widened by alpha h^1.5) and
   u <- ubar + theta (u - ubar).  limited (may be NULL): 1 where theta < 1. */
static double mrs_theta(double M, double wbar, double wM)
{
  double den = wM - wbar, y;
  if (den == 0.) return 1.;
  y = (M - wbar) / den;
  if (y < 0.) return 0.;
  return y / 1.1 < 1. ? y / 1.1 : 1.;
}

int nmo_limiter_mrs(const nmo_mesh *m, double *u, double alpha, int32_t *limited)
{
  int n = m->n, np = n * n * n, nn = n * n, e, l, i, j, k, f, N = n - 1;
  double wl[64], wu[64], x[64];
  double *lim = (double *)malloc(sizeof(double) * (size_t)m->nelem * NF * 3);
  int *nbs = (int *)malloc(sizeof(int) * 6 * 4 * nn);
  if (!lim || !nbs) return 2;
  nmo_lgl(n, x, wl);
  for (i = 0; i <= N; i++) wu[i] = (i == 0 || i == N) ? 1. / N : 2. / N;
  for (e = 0; e < m->nelem; e++) {
    const double *w = (m->fv && m->fv[e]) ? wu : wl;
    for (l = 0; l < NF; l++) {
      const double *v = u + ((size_t)e * NF + l) * np;
      double I = 0., lo = v[0], hi = v[0];
      for (k = 0; k < n; k++) {
        double t = 0.;
        for (j = 0; j < n; j++) {
          double s = 0.;
          for (i = 0; i < n; i++) s += w[i] * v[i + n * (j + n * k)];
          t += w[j] * s;
        }
        I += w[k] * t;
      }
      for (i = 0; i < np; i++) {
        if (v[i] < lo) lo = v[i];
        if (v[i] > hi) hi = v[i];
      }
      lim[((size_t)e * NF + l) * 3] = I * 0.125;
      lim[((size_t)e * NF + l) * 3 + 1] = lo;
      lim[((size_t)e * NF + l) * 3 + 2] = hi;
    }
  }
  for (e = 0; e < m->nelem; e++) {
    const double *bb = m->bbox + (size_t)e * 6;
    double h = bb[1] - bb[0], ah, thM = DBL_MAX, thm = DBL_MAX, th;
    int nnb = 0, q, c;
    if (bb[3] - bb[2] > h) h = bb[3] - bb[2];
    if (bb[5] - bb[4] > h) h = bb[5] - bb[4];
    ah = alpha * pow(h, 1.5);
    /* face neighbours: the element across a conforming face, every source
       element of a non-conforming one */
    for (f = 0; f < 6; f++) {
      int64_t nb = m->nbnode[((size_t)e * 6 + f) * nn];
      if (nb >= 0) nbs[nnb++] = (int)(nb / np);
      else if (nb == -2) nbs[nnb++] = m->mixface[((size_t)e * 6 + f) * 3];
      else if (nb == -3) {
        int first = nnb;
        for (q = 0; q < nn; q++) {
          size_t qq = ((size_t)e * 6 + f) * nn + q;
          for (c = m->hang_off[qq]; c < m->hang_off[qq + 1]; c++) {
            int e2 = m->hang_src[2 * c], seen = 0, z;
            for (z = first; z < nnb; z++) seen |= nbs[z] == e2;
            if (!seen) nbs[nnb++] = e2;
          }
        }
      }
    }
    for (l = 0; l < NF; l++) {
      const double *L = lim + ((size_t)e * NF + l) * 3;
      double wbar = L[0], wmi = L[1], wMi = L[2], Mi = -DBL_MAX, mi = DBL_MAX, a, b;
      for (q = 0; q < nnb; q++) {
        const double *B = lim + ((size_t)nbs[q] * NF + l) * 3;
        if (B[1] < mi) mi = B[1];
        if (B[2] > Mi) Mi = B[2];
      }
      mi = wbar - ah < mi ? wbar - ah : mi;
      Mi = wbar + ah > Mi ? wbar + ah : Mi;
      a = mrs_theta(Mi, wbar, wMi);
      b = mrs_theta(mi, wbar, wmi);
      if (a < thM) thM = a;
      if (b < thm) thm = b;
    }
    th = thm < thM ? thm : thM;
    if (th > 1.) th = 1.;
    if (limited) limited[e] = th < 1.;
    if (th < 1.)
      for (l = 0; l < NF; l++) {
        double qbar = lim[((size_t)e * NF + l) * 3], *v = u + ((size_t)e * NF + l) * np;
        for (i = 0; i < np; i++) v[i] = qbar + th * (v[i] - qbar);
      }
  }
  free(lim);
  free(nbs);
  return 0;
}

/* S_ij = P_j(x_i) / sqrt(c_j), 1/c_j = (2j+1)/2 (j/2 for j = N), and the
   analysis matrix A of the LGL points (typ 0: A_ij = w_j S_ji) or of the
   equally spaced points (typ 1: A = S^-1 by Gauss-Jordan elimination with
   partial pivoting) (LGL_AT_ST_matrices, Legendre_AT_ST_matrices,
   src/main/basis/Legendre.c:277-310,723-729) */
static void legendre_as(int n, int typ, double *S, double *A)
{
  int nn = n * n, i, j, q;
  double x[64], w[64];
  if (typ == 0) nmo_lgl(n, x, w);
  else nmo_uniform(n, x);
  for (i = 0; i < n; i++)
    for (j = 0; j < n; j++) {
      double ooc = 0.5 * (2 * j + 1);
      if (j == n - 1 && n - 1 != 0) ooc = 0.5 * j;
      S[i * n + j] = legendre_p(j, x[i]) * sqrt(ooc);
    }
  if (typ == 0) {
    for (i = 0; i < n; i++)
      for (j = 0; j < n; j++) A[i * n + j] = w[j] * S[j * n + i];
  } else {
    double M[4096], I[4096];
    int col, r;
    for (q = 0; q < nn; q++) { M[q] = S[q]; I[q] = 0.; }
    for (i = 0; i < n; i++) I[i * n + i] = 1.;
    for (col = 0; col < n; col++) {
      int piv = col;
      double dd;
      for (r = col + 1; r < n; r++)
        if (fabs(M[r * n + col]) > fabs(M[piv * n + col])) piv = r;
      for (q = 0; q < n; q++) {
        double t1 = M[col * n + q], t2 = I[col * n + q];
        M[col * n + q] = M[piv * n + q]; M[piv * n + q] = t1;
        I[col * n + q] = I[piv * n + q]; I[piv * n + q] = t2;
      }
      dd = M[col * n + col];
      for (q = 0; q < n; q++) { M[col * n + q] /= dd; I[col * n + q] /= dd; }
      for (r = 0; r < n; r++)
        if (r != col) {
          double fac = M[r * n + col];
          for (q = 0; q < n; q++) {
            M[r * n + q] -= fac * M[col * n + q];
            I[r * n + q] -= fac * I[col * n + q];
          }
        }
    }
    for (q = 0; q < nn; q++) A[q] = I[q];
  }
}

int nmo_filter(const nmo_mesh *m, double *u, double alp, double s, int dn, int jpow,
               int filter_fv)
{
  int n = m->n, np = n * n * n, e, l, i, j, k, q, typ;
  double S[2][4096], A[2][4096], f[64], Nf = n - 1 - dn;
  double *a = (double *)malloc(sizeof(double) * np), *b = (double *)malloc(sizeof(double) * np);
  double *ooJ = (double *)malloc(sizeof(double) * np);
  if (!a || !b || !ooJ) return 2;
  if (Nf <= 0.) Nf = 1.;
  for (k = 0; k < n; k++) f[k] = exp(-alp * pow(k / Nf, s));
  for (typ = 0; typ < 2; typ++) legendre_as(n, typ, S[typ], A[typ]);
  for (e = 0; e < m->nelem; e++) {
    int efv = m->fv && m->fv[e];
    if (efv && !filter_fv) continue;
    for (q = 0; q < np; q++) ooJ[q] = det_dXbdx(m, e, q);
    for (l = 0; l < NF; l++) {
      double *v = u + ((size_t)e * NF + l) * np;
      for (q = 0; q < np; q++) a[q] = jpow ? v[q] / ooJ[q] : v[q];
      mm_dir(n, A[efv], 0, a, b);
      mm_dir(n, A[efv], 1, b, a);
      mm_dir(n, A[efv], 2, a, b);
      for (k = 0; k < n; k++)
        for (j = 0; j < n; j++)
          for (i = 0; i < n; i++) b[i + n * (j + n * k)] *= f[i] * f[j] * f[k];
      mm_dir(n, S[efv], 0, b, a);
      mm_dir(n, S[efv], 1, a, b);
      mm_dir(n, S[efv], 2, b, a);
      for (q = 0; q < np; q++) v[q] = jpow ? a[q] * ooJ[q] : a[q];
    }
  }
  free(a); free(b); free(ooJ);
  return 0;
}

/* The face neighbours of face f of element e (nfnb / fnb): the element
   across a conforming face, every distinct source element of a
   non-conforming one, none on an outer face; returns their number */
static int face_neighbours(const nmo_mesh *m, int e, int f, int *nbs)
{
  int n = m->n, nn = n * n, np = nn * n, cnt = 0, q, c, z;
  int64_t nb = m->nbnode[((size_t)e * 6 + f) * nn];
  if (nb >= 0) nbs[cnt++] = (int)(nb / np);
  else if (nb == -2) nbs[cnt++] = m->mixface[((size_t)e * 6 + f) * 3];
  else if (nb == -3)
    for (q = 0; q < nn; q++) {
      size_t qq = ((size_t)e * 6 + f) * nn + q;
      for (c = m->hang_off[qq]; c < m->hang_off[qq + 1]; c++) {
        int e2 = m->hang_src[2 * c], seen = 0;
        for (z = 0; z < cnt; z++) seen |= nbs[z] == e2;
        if (!seen) nbs[cnt++] = e2;
      }
    }
  return cnt;
}

static double minmod3(double a, double b, double c)
{
  if (a * b >= 0 && b * c >= 0) {
    double m3 = fabs(a);
    if (fabs(b) < m3) m3 = fabs(b);
    if (fabs(c) < m3) m3 = fabs(c);
    return (a > 0. ? 1. : -1.) * m3;
  }
  return 0.;
}

static double minmod3b(double a, double b, double c, double bound)
{
  return fabs(a) <= bound ? a : minmod3(a, b, c);
}

/* dequal with the reference's absolute tolerance 1e-10
   (src/main/main/nmesh_main.h:32-34) */
static int dequal10(double a, double b) { return !(a < b - 1e-10 || b < a - 1e-10); }

/* The minmodB limiter of every element (limdata_c000_100_010_001 and
   limiter_minmodB, src/main/limiter/limiter.c:201-380): the coefficients
   c000, c100, c010, c001 of every element's normalised-Legendre expansion
   (analysis along x, then y, then z: basis_array_analysis3,
   src/main/basis/basis.c:183-188) first; then per element and field the
   face averages w0[f] (mean of the neighbours' c000 across face f, 0 on an
   outer face), the bound alpha h (times the mean of |w0[f]| if
   scale_bound), and the slopes limited by minmod3B against beta/sqrt3 times
   the jumps of the averages; where a slope changes by more than 1e-10 the
   field becomes c000 + the three limited linear modes (synthesis along x,
   y, z).  limited (may be NULL): 1 where any field was limited. */
int nmo_limiter_minmodb(const nmo_mesh *m, double *u, double alpha, double beta,
                        int scale_bound, int32_t *limited)
{
  int n = m->n, np = n * n * n, nn = n * n, e, l, i, j, k, f, typ;
  double S[2][4096], A[2][4096];
  const double bos3 = beta / sqrt(3.);
  double *lim = (double *)malloc(sizeof(double) * (size_t)m->nelem * NF * 4);
  double *t0 = (double *)malloc(sizeof(double) * 2 * nn), *t1 = t0 + nn;
  int *nbs = (int *)malloc(sizeof(int) * 4 * nn);
  if (!lim || !t0 || !nbs) return 2;
  if (n < 2) return 3;
  for (typ = 0; typ < 2; typ++) legendre_as(n, typ, S[typ], A[typ]);
  for (e = 0; e < m->nelem; e++) {
    const double *Ae = A[(m->fv && m->fv[e]) ? 1 : 0];
    const double *A0 = Ae, *A1 = Ae + n;   /* rows 0 and 1 */
    for (l = 0; l < NF; l++) {
      const double *v = u + ((size_t)e * NF + l) * np;
      double *L = lim + ((size_t)e * NF + l) * 4, c000 = 0., c100 = 0., c010 = 0., c001 = 0.;
      for (k = 0; k < n; k++)
        for (j = 0; j < n; j++) {
          double a0 = 0., a1 = 0.;
          for (i = 0; i < n; i++) {
            a0 += A0[i] * v[i + n * (j + n * k)];
            a1 += A1[i] * v[i + n * (j + n * k)];
          }
          t0[j + n * k] = a0;
          t1[j + n * k] = a1;
        }
      for (k = 0; k < n; k++) {
        double s00 = 0., s10 = 0., s01 = 0.;
        for (j = 0; j < n; j++) {
          s00 += A0[j] * t0[j + n * k];
          s10 += A0[j] * t1[j + n * k];
          s01 += A1[j] * t0[j + n * k];
        }
        c000 += A0[k] * s00;
        c100 += A0[k] * s10;
        c010 += A0[k] * s01;
        c001 += A1[k] * s00;
      }
      L[0] = c000; L[1] = c100; L[2] = c010; L[3] = c001;
    }
  }
  for (e = 0; e < m->nelem; e++) {
    const double *bb = m->bbox + (size_t)e * 6, *Se = S[(m->fv && m->fv[e]) ? 1 : 0];
    double h = bb[1] - bb[0], Mt_h, w0[6][NF], w0L1[NF];
    int nlim = 0;
    if (bb[3] - bb[2] > h) h = bb[3] - bb[2];
    if (bb[5] - bb[4] > h) h = bb[5] - bb[4];
    Mt_h = alpha * h;
    for (l = 0; l < NF; l++) w0L1[l] = 0.;
    for (f = 0; f < 6; f++) {
      int cnt = face_neighbours(m, e, f, nbs), z;
      for (l = 0; l < NF; l++) {
        double av = 0.;
        for (z = 0; z < cnt; z++) av += lim[((size_t)nbs[z] * NF + l) * 4];
        if (cnt > 0) av = av / cnt;
        w0[f][l] = av;
        w0L1[l] += fabs(av) * 0.166666666666667;
      }
    }
    for (l = 0; l < NF; l++) {
      const double *L = lim + ((size_t)e * NF + l) * 4;
      double w0c = L[0], bound = scale_bound ? Mt_h * w0L1[l] : Mt_h;
      double wl100 = minmod3b(L[1], bos3 * (w0c - w0[0][l]), bos3 * (w0[1][l] - w0c), bound);
      double wl010 = minmod3b(L[2], bos3 * (w0c - w0[2][l]), bos3 * (w0[3][l] - w0c), bound);
      double wl001 = minmod3b(L[3], bos3 * (w0c - w0[4][l]), bos3 * (w0[5][l] - w0c), bound);
      if (!dequal10(wl100, L[1]) || !dequal10(wl010, L[2]) || !dequal10(wl001, L[3])) {
        double *v = u + ((size_t)e * NF + l) * np;
        for (k = 0; k < n; k++)
          for (j = 0; j < n; j++)
            for (i = 0; i < n; i++) {
              /* S^3 of the four non-zero coefficients, x, then y, then z */
              double tx0 = Se[i * n] * w0c + Se[i * n + 1] * wl100;
              double tx1 = Se[i * n] * wl010, tx2 = Se[i * n] * wl001;
              double ty0 = Se[j * n] * tx0 + Se[j * n + 1] * tx1, ty1 = Se[j * n] * tx2;
              v[i + n * (j + n * k)] = Se[k * n] * ty0 + Se[k * n + 1] * ty1;
            }
        nlim++;
      }
    }
    if (limited) limited[e] = nlim > 0;
  }
  free(lim);
  free(t0);
  free(nbs);
  return 0;
}

/* nsteps RK4 steps; the time of each step is accumulated in long double as
   in evolve_mesh (src/main/main/main.c:610-626) */
int nmo_rk4(const nmo_mesh *m, double t, double dt, int nsteps, double *u)
{
  size_t N = (size_t)m->nelem * NF * m->n * m->n * m->n;
  double *work = (double *)malloc(3 * N * sizeof(double));
  long double Te = t, te = 0.;
  int s, rc = 0;
  if (!work) return 2;
  for (s = 0; s < nsteps && !rc; s++) {
    double ts = (double)(Te + te);
    rc = nmo_rk4_step(m, ts, dt, u, work);
    te += dt;
  }
  free(work);
  return rc;
}

/* ------------------------------------------------------------------ */
/* GRHD conservative-to-primitive recovery (config 3's physics)        */
/* ------------------------------------------------------------------ */
/* Newton-Raphson with bracketing and bisection fallback in [x1, x2]
   (newton1d_brak, src/utility/numerics/newton1d_brak.c:20-121); returns the
   number of iterations (>= 0) or a negative error code, the root in *x0. */
int nmo_newton1d_brak(double *x0, void (*fdf)(double, void *, double *, double *),
                      double x1, double x2, void *par, int maxits, double xacc)
{
  int j, bisect;
  double f, fh, fl, df, xh, xl, xrt, dx, dxold, tmp;
  if (!isfinite(x1) || !isfinite(x2)) return -2 * maxits - 2;
  if ((x1 <= *x0 && *x0 <= x2) || (x2 <= *x0 && *x0 <= x1)) xrt = *x0;
  else xrt = 0.5 * (x1 + x2);
  fdf(x1, par, &fl, &df);
  fdf(x2, par, &fh, &df);
  j = 0;
  if (fl <= 0.0 && fh >= 0.0) j = 1;
  if (fl >= 0.0 && fh <= 0.0) j = 1;
  if (!j) return -2 * maxits - 3;
  if (fl == 0.0) { *x0 = x1; return 0; }
  if (fh == 0.0) { *x0 = x2; return 0; }
  if (fl < 0.0) { xl = x1; xh = x2; }
  else { xh = x1; xl = x2; }
  dxold = fabs(x2 - x1);
  dx = dxold;
  for (j = 1; j <= maxits; j++) {
    fdf(xrt, par, &f, &df);
    if (!isfinite(f)) return -j;
    if (f == 0.0) { *x0 = xrt; return j; }
    if (f < 0.0) xl = xrt;
    else xh = xrt;
    if (!isfinite(df)) bisect = 1;
    else bisect = (fabs(2.0 * f) > fabs(dxold * df));
    if (bisect == 0) {
      dxold = dx;
      dx = f / df;
      tmp = xrt;
      xrt -= dx;
      if (((xrt - xh) * (xrt - xl) > 0.0) || (tmp == xrt)) {
        bisect = 1; xrt = tmp; dx = dxold;
      }
    }
    if (bisect) {
      dxold = dx;
      dx = 0.5 * (xh - xl);
      xrt = xl + dx;
      if (xl == xrt) { *x0 = xrt; return j; }
    }
    if (fabs(dx) < xacc) { *x0 = xrt; return j; }
  }
  *x0 = xrt;
  return j;
}

/* Ideal-gas GRHD on a conformally flat 3-metric gamma_ij = psi^4 delta_ij
   (restated; the reference has no GRHD, so this is parity unpinned):
   conserved (D, S_i, tau) densitized by sqrt(gamma) = psi^6,
   D = psi^6 rho W, S_i = psi^6 rho h W^2 v_i, tau = psi^6 (rho h W^2 - p) - D,
   v_i = psi^4 v^i, W = 1/sqrt(1 - v_i v^i), h = 1 + eps + p/rho,
   p = (gamma - 1) rho eps.  Primitives (rho, v^1, v^2, v^3, p). */
typedef struct nmo_grhd {
  double gamma, rho_atm, p_atm, tol;
  int maxits;
} nmo_grhd;

typedef struct nmo_c2p_par {
  double D, tau, S2, gm1, gam;
} nmo_c2p_par;

/* f(p) = (gamma-1) rho(p) eps(p) - p and the approximation
   f'(p) = v^2 c_s^2 - 1 */
static void c2p_fdf(double p, void *vp, double *f, double *df)
{
  const nmo_c2p_par *q = (const nmo_c2p_par *)vp;
  double E = q->tau + q->D + p;
  double v2 = q->S2 / (E * E);
  double W = 1. / sqrt(1. - v2);
  double rho = q->D / W;
  double eps = (q->tau + q->D * (1. - W) + p * (1. - W * W)) / (q->D * W);
  double cs2 = q->gam * q->gm1 * eps / (1. + q->gam * eps);
  *f = q->gm1 * rho * eps - p;
  *df = v2 * cs2 - 1.;
}

void nmo_grhd_prim2con(const nmo_grhd *g, int64_t npts, const double *psi, const double *prim,
                       double *cons)
{
  int64_t i;
  for (i = 0; i < npts; i++) {
    double ps = psi ? psi[i] : 1.;
    double ps4 = ps * ps * ps * ps, ps6 = ps4 * ps * ps;
    double rho = prim[i], vx = prim[npts + i], vy = prim[2 * npts + i];
    double vz = prim[3 * npts + i], p = prim[4 * npts + i];
    double v2 = ps4 * (vx * vx + vy * vy + vz * vz);
    double W = 1. / sqrt(1. - v2);
    double eps = p / ((g->gamma - 1.) * rho);
    double h = 1. + eps + p / rho;
    double rhW2 = rho * h * W * W;
    cons[i] = ps6 * rho * W;
    cons[npts + i] = ps6 * rhW2 * ps4 * vx;
    cons[2 * npts + i] = ps6 * rhW2 * ps4 * vy;
    cons[3 * npts + i] = ps6 * rhW2 * ps4 * vz;
    cons[4 * npts + i] = ps6 * (rhW2 - p) - cons[i];
  }
}

/* con2prim with pressure as the unknown (newton1d_brak on f above; the
   previous prim[4] is the starting guess).  Points that are below the
   atmosphere density or where the root finder fails are set to the
   atmosphere (rho_atm, v = 0, p_atm) and their conserved variables are
   reset to match.  status[i] = iterations (>= 0) or < 0 (atmosphere). */
void nmo_grhd_con2prim(const nmo_grhd *g, int64_t npts, const double *psi, double *cons,
                       double *prim, int32_t *status)
{
  int64_t i;
  for (i = 0; i < npts; i++) {
    double ps = psi ? psi[i] : 1.;
    double ps4 = ps * ps * ps * ps, ps6 = ps4 * ps * ps;
    double D = cons[i] / ps6, Sx = cons[npts + i] / ps6, Sy = cons[2 * npts + i] / ps6;
    double Sz = cons[3 * npts + i] / ps6, tau = cons[4 * npts + i] / ps6;
    double S2 = (Sx * Sx + Sy * Sy + Sz * Sz) / ps4;
    nmo_c2p_par q;
    double plo, phi, p, f, df, xacc;
    int rc = -1, k;
    q.D = D; q.tau = tau; q.S2 = S2; q.gm1 = g->gamma - 1.; q.gam = g->gamma;
    if (D >= g->rho_atm && isfinite(D) && isfinite(tau) && isfinite(S2)) {
      double S = sqrt(S2);
      plo = S - tau - D;
      plo = plo > 0. ? plo * (1. + 1e-14) : 0.;
      phi = q.gm1 * (tau + D);
      if (phi < plo) phi = 2. * plo;
      if (phi <= 0.) phi = 1e-300;
      for (k = 0; k < 200; k++) {      /* widen upwards until f(phi) < 0 */
        c2p_fdf(phi, &q, &f, &df);
        if (f < 0.) break;
        phi *= 2.;
      }
      p = prim[4 * npts + i];
      xacc = g->tol * phi;
      rc = nmo_newton1d_brak(&p, c2p_fdf, plo, phi, &q, g->maxits, xacc);
      if (rc >= 0) {
        double E = tau + D + p, W, rho;
        double v2 = S2 / (E * E);
        W = 1. / sqrt(1. - v2);
        rho = D / W;
        if (!(rho >= g->rho_atm) || !(p > 0.) || !isfinite(W)) rc = -1;
        else {
          double fac = 1. / (E * ps4);          /* v^i = S^i / (E psi^4) */
          prim[i] = rho;
          prim[npts + i] = Sx * fac;
          prim[2 * npts + i] = Sy * fac;
          prim[3 * npts + i] = Sz * fac;
          prim[4 * npts + i] = p;
        }
      }
    }
    if (rc < 0) {                            /* atmosphere, conserved reset */
      double eps_atm = g->p_atm / ((g->gamma - 1.) * g->rho_atm);
      double h = 1. + eps_atm + g->p_atm / g->rho_atm;
      prim[i] = g->rho_atm;
      prim[npts + i] = prim[2 * npts + i] = prim[3 * npts + i] = 0.;
      prim[4 * npts + i] = g->p_atm;
      cons[i] = ps6 * g->rho_atm;
      cons[npts + i] = cons[2 * npts + i] = cons[3 * npts + i] = 0.;
      cons[4 * npts + i] = ps6 * (g->rho_atm * h - g->p_atm) - cons[i];
    }
    status[i] = rc;
  }
}

/* Valencia fluxes, characteristic speeds and Cowling sources on a static
   conformally flat background ds^2 = -alpha^2 dt^2 + psi^4 dx^2 (zero
   shift), from primitives (rho, v^i, p):
     F^d(D) = alpha v^d D, F^d(S_j) = alpha v^d S_j + alpha psi^6 p delta^d_j,
     F^d(tau) = alpha v^d tau + alpha psi^6 p v^d  (densitized D, S_j, tau);
     S(S_j) = psi^6 [2 alpha (d_j psi / psi)(rho h W^2 v^2 + 3 p) - E d_j alpha],
     S(tau) = -psi^6 rho h W^2 v^j d_j alpha,  E = rho h W^2 - p;
   speeds along d: lambda_pm = alpha/(1 - v^2 c_s^2) [v^d (1 - c_s^2) pm
     c_s sqrt((1 - v^2)(psi^-4 (1 - v^2 c_s^2) - v^d v^d (1 - c_s^2)))].
   (restated; the reference has no GRHD) */
void nmo_grhd_fluxes(const nmo_grhd *g, int64_t npts, int d, const double *alpha,
                     const double *psi, const double *prim, double *flux, double *lam)
{
  int64_t i;
  for (i = 0; i < npts; i++) {
    double al = alpha ? alpha[i] : 1., ps = psi ? psi[i] : 1.;
    double ps4 = ps * ps * ps * ps, ps6 = ps4 * ps * ps;
    double rho = prim[i], v[3] = {prim[npts + i], prim[2 * npts + i], prim[3 * npts + i]};
    double p = prim[4 * npts + i];
    double v2 = ps4 * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    double W = 1. / sqrt(1. - v2);
    double eps = p / ((g->gamma - 1.) * rho);
    double h = 1. + eps + p / rho;
    double rhW2 = rho * h * W * W;
    double D = ps6 * rho * W, tau = ps6 * (rhW2 - p) - D, avd = al * v[d];
    double cs2 = g->gamma * p / (rho * h);
    double disc = (1. - v2) * (1. / ps4 * (1. - v2 * cs2) - v[d] * v[d] * (1. - cs2));
    double fac = al / (1. - v2 * cs2);
    int j;
    flux[i] = avd * D;
    for (j = 0; j < 3; j++) {
      double Sj = ps6 * rhW2 * ps4 * v[j];
      flux[(1 + j) * npts + i] = avd * Sj + (j == d ? al * ps6 * p : 0.);
    }
    flux[4 * npts + i] = avd * tau + al * ps6 * p * v[d];
    if (disc < 0.) disc = 0.;
    lam[i] = fac * (v[d] * (1. - cs2) - sqrt(cs2) * sqrt(disc));
    lam[npts + i] = fac * (v[d] * (1. - cs2) + sqrt(cs2) * sqrt(disc));
  }
}

void nmo_grhd_sources(const nmo_grhd *g, int64_t npts, const double *alpha, const double *psi,
                      const double *dalpha, const double *dpsi, const double *prim, double *src)
{
  int64_t i;
  for (i = 0; i < npts; i++) {
    double al = alpha[i], ps = psi[i];
    double ps4 = ps * ps * ps * ps, ps6 = ps4 * ps * ps;
    double rho = prim[i], v[3] = {prim[npts + i], prim[2 * npts + i], prim[3 * npts + i]};
    double p = prim[4 * npts + i];
    double v2 = ps4 * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    double W = 1. / sqrt(1. - v2);
    double eps = p / ((g->gamma - 1.) * rho);
    double h = 1. + eps + p / rho;
    double rhW2 = rho * h * W * W;
    double E = rhW2 - p, vda = 0.;
    int j;
    src[i] = 0.;
    for (j = 0; j < 3; j++) {
      double da = dalpha[j * npts + i], dp = dpsi[j * npts + i];
      src[(1 + j) * npts + i] = ps6 * (2. * al * (dp / ps) * (rhW2 * v2 + 3. * p) - E * da);
      vda += v[j] * da;
    }
    src[4 * npts + i] = -ps6 * rhW2 * vda;
  }
}

/* the midpoint reconstructions for other translation units of the oracle */
double nmo_rec_p(int mode, int n, const double *u, int im, double r3)
{
  return rec_p(mode, n, u, im, r3);
}

double nmo_rec_m(int mode, int n, const double *u, int im, double r3)
{
  return rec_m(mode, n, u, im, r3);
}
