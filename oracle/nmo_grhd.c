/* nmo_grhd.c -- ORACLE (test infrastructure only; never part of the product
 * path): a plain-C restatement of the GRHD evolution in the Cowling
 * approximation that the GPU path runs (nmesh_gb300/csrc/grhd_evolve.cu).
 *
 * The reference has no GRHD (its physics modules live in external
 * repositories), so the physics and the finite-volume form here are parity
 * unpinned.  What is the reference's is restated from it: the DG strong-form
 * divergence with the chain rule (src/main/coordinates/derivs.c:102-181,
 * 756-815), the LLF numerical flux (src/main/dg/numflux1d.c:85-112: F* =
 * (F_l + F_r - a (U_r - U_l))/2 with a the largest characteristic speed on
 * either side), the lift (f* - f_in) sqrtgdiag / w_end (src/main/dg/
 * dg.c:30-151), the WENOm5_2 / WENOm3_2 midpoint reconstructions
 * (src/main/dg/rec1d.c:880-1030,1186-1368, via oracle/nmo.c), the root
 * finder newton1d_brak (src/utility/numerics/newton1d_brak.c:20-121, via
 * nmo_grhd_con2prim), RK4 (src/main/evolve/RungeKutta.c:19-82), and the
 * DG <-> finite-volume transfer of the reference's PARENT_2n_P_UNIFORM
 * switch (src/main/evolve/trouble.c:162-183, src/main/basis/gridpoints.c:
 * 158-200: P = Lagrange interpolation from the n LGL points to nf equally
 * spaced points, back by the pseudo-inverse R = (P^T P)^-1 P^T), here with
 * nf = 2n (the reference's mode) or any other nf >= n.
 *
 * System (densitized conserved U = psi^6 (D, S_j, tau), primitives
 * (rho, v^i, p), ideal gas), on the static isotropic Schwarzschild
 * background of mass M: psi = 1 + M/(2r), alpha = (1 - M/(2r))/(1 + M/(2r)).
 *   dU/dt = -d_i F^i + S (Cowling sources of nmo_grhd_sources)
 *   F^i n_i = alpha v_n U + alpha psi^6 p (0, n_j, v_n),  v_n = v^i n_i
 *
 * DG elements (n LGL points): -div F = -sum_i sum_a dX^a/dx^i (2/dX^a)
 * D_a F^i (strong form) + S; on every face node with a neighbour
 * r -= g (F* - F_in.n), g = |grad X^d| (2/dX^d) / w_end, n the outward unit
 * normal; outer faces copy the interior state (no face term).
 *
 * Finite-volume elements (nf equally spaced points, the element's faces
 * among them): per direction the midpoint fluxes from WENO-reconstructed
 * primitives (first order where a reconstructed state is unphysical),
 * the LLF flux with the map's unit normal and J |grad Xb^a| at the
 * midpoint, and at the face points the LLF flux with the neighbour's trace;
 * div = det(dXb/dx) sum_a (G_{t+1/2} - G_{t-1/2}) / dXb (half cells of
 * width h/2 at the faces).
 *
 * Traces across a DG / finite-volume interface are primitives: from a
 * finite-volume neighbour piecewise linear in each in-plane direction, from
 * a DG neighbour by Lagrange interpolation of its face plane; U = prim2con.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define NF 5
#define MAXN 32

typedef struct nmo_grhd {
  double gamma, rho_atm, p_atm, tol;
  int maxits;
} nmo_grhd;

void nmo_lgl(int npoints, double *x, double *w);
void nmo_uniform(int npoints, double *x);
void nmo_diffmat(int n, const double *x, double *D);
double nmo_rec_p(int mode, int n, const double *u, int im, double r3);
double nmo_rec_m(int mode, int n, const double *u, int im, double r3);
int nmo_mesh_map(int type, const double prm[4], int p, const double X[3], double x[3],
                 double J[3][3]);
void nmo_grhd_prim2con(const nmo_grhd *g, int64_t npts, const double *psi, const double *prim,
                       double *cons);
void nmo_grhd_con2prim(const nmo_grhd *g, int64_t npts, const double *psi, double *cons,
                       double *prim, int32_t *status);

typedef struct nmo_grmesh {
  int nelem, n, nf;
  int mesh_type;
  double prm[4];            /* mesh parameters of nmo_mesh_generate */
  const int32_t *pat;       /* [E] */
  const double *bbox;       /* [E][6] */
  const double *xyz;        /* [E][3][n^3] LGL nodes */
  const double *dXdx;       /* [E][9][n^3] */
  const int32_t *nb;        /* [E][6] neighbour element, -1 outer */
  const int32_t *code;      /* [E][6] neighbour face | orientation << 3 */
  const int32_t *fv;        /* [E] 1: finite-volume element */
  nmo_grhd g;
  double mass;
  int rec;                  /* midpoint reconstruction (oracle/nmo.c modes) */
} nmo_grmesh;

/* ---------------------------------------------------------------------- */
/* pointwise physics                                                       */
/* ---------------------------------------------------------------------- */
/* background: alpha, psi, d_i alpha, d_i psi */
void nmo_gr_background(double mass, const double x[3], double bg[8])
{
  const double r2 = x[0] * x[0] + x[1] * x[1] + x[2] * x[2];
  const double r = sqrt(r2);
  const double a = 0.5 * mass / r;
  const double ps = 1. + a;
  const double c1 = 2. * a / (r2 * (ps * ps)), c2 = -a / r2;
  int i;
  bg[0] = (1. - a) / (1. + a);
  bg[1] = ps;
  for (i = 0; i < 3; i++) {
    bg[2 + i] = c1 * x[i];
    bg[5 + i] = c2 * x[i];
  }
}

/* flux along the unit normal n of the state U with primitives P */
static void flux_n(const double *U, const double *P, const double n[3], double al, double ps,
                   double F[NF])
{
  const double ps2 = ps * ps, ps6 = ps2 * ps2 * ps2;
  const double vn = P[1] * n[0] + P[2] * n[1] + P[3] * n[2];
  const double avn = al * vn, ap = al * ps6 * P[4];
  F[0] = avn * U[0];
  F[1] = avn * U[1] + ap * n[0];
  F[2] = avn * U[2] + ap * n[1];
  F[3] = avn * U[3] + ap * n[2];
  F[4] = avn * U[4] + ap * vn;
}

/* largest |characteristic speed| along the unit normal n */
static double speed_n(const nmo_grhd *g, const double *P, const double n[3], double al, double ps)
{
  const double ps2 = ps * ps, ps4 = ps2 * ps2;
  const double rho = P[0], p = P[4];
  const double vn = P[1] * n[0] + P[2] * n[1] + P[3] * n[2];
  const double v2 = ps4 * (P[1] * P[1] + P[2] * P[2] + P[3] * P[3]);
  const double eps = p / ((g->gamma - 1.) * rho);
  const double h = 1. + eps + p / rho;
  const double cs2 = g->gamma * p / (rho * h);
  double disc = (1. - v2) * (1. / ps4 * (1. - v2 * cs2) - vn * vn * (1. - cs2));
  const double fac = al / (1. - v2 * cs2);
  double lm, lp;
  if (disc < 0.) disc = 0.;
  lm = fac * (vn * (1. - cs2) - sqrt(cs2) * sqrt(disc));
  lp = fac * (vn * (1. - cs2) + sqrt(cs2) * sqrt(disc));
  return fmax(fabs(lm), fabs(lp));
}

static void sources(const nmo_grhd *g, const double *P, const double bg[8], double S[NF])
{
  const double al = bg[0], ps = bg[1];
  const double ps2 = ps * ps, ps4 = ps2 * ps2, ps6 = ps4 * ps2;
  const double rho = P[0], p = P[4];
  const double v2 = ps4 * (P[1] * P[1] + P[2] * P[2] + P[3] * P[3]);
  const double W2 = 1. / (1. - v2);
  const double eps = p / ((g->gamma - 1.) * rho);
  const double h = 1. + eps + p / rho;
  const double rhW2 = rho * h * W2;
  const double E = rhW2 - p;
  double vda = 0.;
  int j;
  S[0] = 0.;
  for (j = 0; j < 3; j++) {
    S[1 + j] = ps6 * (2. * al * (bg[5 + j] / ps) * (rhW2 * v2 + 3. * p) - E * bg[2 + j]);
    vda += P[1 + j] * bg[2 + j];
  }
  S[4] = -ps6 * rhW2 * vda;
}

/* U of primitives P at conformal factor psi */
static void p2c(const nmo_grhd *g, double ps, const double P[NF], double U[NF])
{
  nmo_grhd_prim2con(g, 1, &ps, P, U);
}

/* physical primitive state (else the reconstruction falls back) */
static int physical(const double P[NF], double ps)
{
  const double ps2 = ps * ps, ps4 = ps2 * ps2;
  const double v2 = ps4 * (P[1] * P[1] + P[2] * P[2] + P[3] * P[3]);
  return P[0] > 0. && P[4] > 0. && v2 < 1. && isfinite(P[0] + P[1] + P[2] + P[3] + P[4]);
}

/* LLF flux along n between the interior (Ui, Pi) and exterior (Uo, Po) */
static void llf(const nmo_grhd *g, const double *Ui, const double *Pi, const double *Uo,
                const double *Po, const double n[3], double al, double ps, double Fs[NF],
                double Fi[NF])
{
  double Fo[NF], a;
  int f;
  flux_n(Ui, Pi, n, al, ps, Fi);
  flux_n(Uo, Po, n, al, ps, Fo);
  a = fmax(speed_n(g, Pi, n, al, ps), speed_n(g, Po, n, al, ps));
  for (f = 0; f < NF; f++) Fs[f] = 0.5 * (Fi[f] + Fo[f] - a * (Uo[f] - Ui[f]));
}

/* ---------------------------------------------------------------------- */
/* points, faces, traces                                                   */
/* ---------------------------------------------------------------------- */
static int face_ijk(int n, int f, int a, int b)
{
  const int d = f / 2, q = (f % 2) * (n - 1);
  if (d == 0) return q + n * (a + n * b);
  if (d == 1) return a + n * (q + n * b);
  return a + n * (b + n * q);
}

/* index and in-plane position across a face with orientation o (bit 0:
   swap, bit 1: reverse a, bit 2: reverse b) */
static void orient_ab(int n, int o, int a, int b, int *a2, int *b2)
{
  int aa = (o & 1) ? b : a, bb = (o & 1) ? a : b;
  if (o & 2) aa = n - 1 - aa;
  if (o & 4) bb = n - 1 - bb;
  *a2 = aa;
  *b2 = bb;
}

static void orient_pos(int o, double s, double t, double *s2, double *t2)
{
  double ss = (o & 1) ? t : s, tt = (o & 1) ? s : t;
  if (o & 2) ss = -ss;
  if (o & 4) tt = -tt;
  *s2 = ss;
  *t2 = tt;
}

/* piecewise-linear weights of equally spaced points xu at x: interval k */
static int pw_linear(int n, const double *xu, double x, double *w0, double *w1)
{
  int k = (int)floor((x + 1.) * 0.5 * (n - 1));
  if (k < 0) k = 0;
  if (k > n - 2) k = n - 2;
  *w1 = (x - xu[k]) / (xu[k + 1] - xu[k]);
  *w0 = 1. - *w1;
  return k;
}

/* Lagrange basis of the points xl at x */
static void lagrange(int n, const double *xl, double x, double *l)
{
  int i, j;
  for (i = 0; i < n; i++) {
    double v = 1.;
    for (j = 0; j < n; j++)
      if (j != i) v *= (x - xl[j]) / (xl[i] - xl[j]);
    l[i] = v;
  }
}

typedef struct grpts {
  double xl[MAXN], wl[MAXN], D[MAXN * MAXN], xu[2 * MAXN];
} grpts;

static void grpts_init(const nmo_grmesh *m, grpts *P)
{
  nmo_lgl(m->n, P->xl, P->wl);
  nmo_diffmat(m->n, P->xl, P->D);
  nmo_uniform(m->nf, P->xu);
}

/* map geometry at patch coordinates of element e at Xb: x, dXb/dx */
static void geo_at(const nmo_grmesh *m, int e, const double Xb[3], double x[3], double Mb[3][3])
{
  const double *bb = m->bbox + 6 * (size_t)e;
  double X[3], J[3][3];
  int d, c;
  for (d = 0; d < 3; d++)
    X[d] = 0.5 * ((bb[2 * d + 1] - bb[2 * d]) * Xb[d] + (bb[2 * d + 1] + bb[2 * d]));
  nmo_mesh_map(m->mesh_type, m->prm, m->pat[e], X, x, J);
  for (d = 0; d < 3; d++)
    for (c = 0; c < 3; c++) Mb[d][c] = (2. / (bb[2 * d + 1] - bb[2 * d])) * J[d][c];
}

static double det3(double M[3][3])
{
  return M[0][0] * (M[1][1] * M[2][2] - M[1][2] * M[2][1]) -
         M[0][1] * (M[1][0] * M[2][2] - M[1][2] * M[2][0]) +
         M[0][2] * (M[1][0] * M[2][1] - M[1][1] * M[2][0]);
}

/* exterior primitives at in-plane node (a, b) of face f of element e from
   the neighbour of the other point type (traces across a DG / FV face) */
static void cross_trace(const nmo_grmesh *m, const grpts *P, int e, int f, int a, int b,
                        const double *prim_dg, const double *prim_fv, double Po[NF])
{
  const int e2 = m->nb[6 * e + f], f2 = m->code[6 * e + f] & 7, o = (m->code[6 * e + f] >> 3) & 7;
  const double *xs = m->fv[e] ? P->xu : P->xl;
  double s, t, s2, t2;
  int q;
  orient_pos(o, xs[a], xs[b], &s2, &t2);
  s = s2;
  t = t2;
  if (m->fv[e2]) {
    /* finite-volume neighbour: piecewise linear in each direction */
    const int nf = m->nf, npf = nf * nf * nf;
    double wa0, wa1, wb0, wb1;
    const int ka = pw_linear(nf, P->xu, s, &wa0, &wa1);
    const int kb = pw_linear(nf, P->xu, t, &wb0, &wb1);
    for (q = 0; q < NF; q++) {
      const double *u = prim_fv + ((size_t)e2 * NF + q) * npf;
      const double v0 = wa0 * u[face_ijk(nf, f2, ka, kb)] + wa1 * u[face_ijk(nf, f2, ka + 1, kb)];
      const double v1 =
          wa0 * u[face_ijk(nf, f2, ka, kb + 1)] + wa1 * u[face_ijk(nf, f2, ka + 1, kb + 1)];
      Po[q] = wb0 * v0 + wb1 * v1;
    }
  } else {
    const int n = m->n, np = n * n * n;
    double la[MAXN], lb[MAXN];
    int i, j;
    lagrange(n, P->xl, s, la);
    lagrange(n, P->xl, t, lb);
    for (q = 0; q < NF; q++) {
      const double *u = prim_dg + ((size_t)e2 * NF + q) * np;
      double v = 0.;
      for (j = 0; j < n; j++) {
        double vj = 0.;
        for (i = 0; i < n; i++) vj += la[i] * u[face_ijk(n, f2, i, j)];
        v += lb[j] * vj;
      }
      Po[q] = v;
    }
  }
}

/* exterior (U, P) of face node (a, b) of face f of element e; 0: outer face */
static int exterior(const nmo_grmesh *m, const grpts *P, int e, int f, int a, int b, double ps,
                    const double *w_dg, const double *w_fv, const double *prim_dg,
                    const double *prim_fv, double Uo[NF], double Po[NF])
{
  const int e2 = m->nb[6 * e + f];
  int q;
  if (e2 < 0) return 0;
  if (m->fv[e2] == m->fv[e]) {
    const int nn = m->fv[e] ? m->nf : m->n, npts = nn * nn * nn;
    const int f2 = m->code[6 * e + f] & 7, o = (m->code[6 * e + f] >> 3) & 7;
    const double *W = m->fv[e] ? w_fv : w_dg, *PP = m->fv[e] ? prim_fv : prim_dg;
    int a2, b2, idx;
    orient_ab(nn, o, a, b, &a2, &b2);
    idx = face_ijk(nn, f2, a2, b2);
    for (q = 0; q < NF; q++) {
      Uo[q] = W[((size_t)e2 * NF + q) * npts + idx];
      Po[q] = PP[((size_t)e2 * NF + q) * npts + idx];
    }
    return 1;
  }
  cross_trace(m, P, e, f, a, b, prim_dg, prim_fv, Po);
  p2c(&m->g, ps, Po, Uo);
  return 1;
}

/* ---------------------------------------------------------------------- */
/* right-hand sides                                                        */
/* ---------------------------------------------------------------------- */
static void rhs_dg(const nmo_grmesh *m, const grpts *P, int e, const double *w_dg,
                   const double *w_fv, const double *prim_dg, const double *prim_fv,
                   double *r, double *F)
{
  const int n = m->n, np = n * n * n;
  const double *bb = m->bbox + 6 * (size_t)e;
  const double *U = w_dg + (size_t)e * NF * np, *PP = prim_dg + (size_t)e * NF * np;
  const double *M = m->dXdx + (size_t)e * 9 * np, *xyz = m->xyz + (size_t)e * 3 * np;
  double s[3];
  int q, i, a, f, d;
  for (d = 0; d < 3; d++) s[d] = 2. / (bb[2 * d + 1] - bb[2 * d]);
  /* F[i][f][q]: flux along e_i */
  for (q = 0; q < np; q++) {
    double Uq[NF], Pq[NF], bg[8], x[3], nrm[3], Fq[NF];
    for (f = 0; f < NF; f++) {
      Uq[f] = U[f * np + q];
      Pq[f] = PP[f * np + q];
    }
    for (d = 0; d < 3; d++) x[d] = xyz[d * np + q];
    nmo_gr_background(m->mass, x, bg);
    for (i = 0; i < 3; i++) {
      nrm[0] = nrm[1] = nrm[2] = 0.;
      nrm[i] = 1.;
      flux_n(Uq, Pq, nrm, bg[0], bg[1], Fq);
      for (f = 0; f < NF; f++) F[(i * NF + f) * np + q] = Fq[f];
    }
    sources(&m->g, Pq, bg, Fq);
    for (f = 0; f < NF; f++) r[f * np + q] = Fq[f];
  }
  /* volume: r = S - sum_i sum_a M[a][i] s_a (D_a F^i) */
  for (f = 0; f < NF; f++)
    for (q = 0; q < np; q++) {
      const int ijk[3] = {q % n, (q / n) % n, q / (n * n)};
      const int str[3] = {1, n, n * n};
      double div = 0.;
      for (i = 0; i < 3; i++) {
        const double *Fi = F + (i * NF + f) * np;
        for (a = 0; a < 3; a++) {
          const int base = q - ijk[a] * str[a];
          double ds = 0.;
          int k;
          for (k = 0; k < n; k++) ds += P->D[ijk[a] * n + k] * Fi[base + k * str[a]];
          div += M[(a * 3 + i) * np + q] * (s[a] * ds);
        }
      }
      r[f * np + q] -= div;
    }
  /* faces */
  for (f = 0; f < 6; f++) {
    const int dd = f / 2;
    const double sgn = (f % 2) ? 1. : -1.;
    int aa, bb2;
    for (bb2 = 0; bb2 < n; bb2++)
      for (aa = 0; aa < n; aa++) {
        const int q2 = face_ijk(n, f, aa, bb2);
        double Ui[NF], Pi[NF], Uo[NF], Po[NF], Fs[NF], Fi[NF], bg[8], x[3], nrm[3], nm, g;
        for (d = 0; d < 3; d++) x[d] = xyz[d * np + q2];
        nmo_gr_background(m->mass, x, bg);
        if (!exterior(m, P, e, f, aa, bb2, bg[1], w_dg, w_fv, prim_dg, prim_fv, Uo, Po))
          continue;
        for (q = 0; q < NF; q++) {
          Ui[q] = U[q * np + q2];
          Pi[q] = PP[q * np + q2];
        }
        nm = sqrt(M[(dd * 3 + 0) * np + q2] * M[(dd * 3 + 0) * np + q2] +
                  M[(dd * 3 + 1) * np + q2] * M[(dd * 3 + 1) * np + q2] +
                  M[(dd * 3 + 2) * np + q2] * M[(dd * 3 + 2) * np + q2]);
        for (d = 0; d < 3; d++) nrm[d] = sgn * M[(dd * 3 + d) * np + q2] / nm;
        g = nm * s[dd] / P->wl[0];
        llf(&m->g, Ui, Pi, Uo, Po, nrm, bg[0], bg[1], Fs, Fi);
        for (q = 0; q < NF; q++) r[q * np + q2] -= g * (Fs[q] - Fi[q]);
      }
  }
}

static void rhs_fv(const nmo_grmesh *m, const grpts *P, int e, const double *w_dg,
                   const double *w_fv, const double *prim_dg, const double *prim_fv,
                   double *r)
{
  const int nf = m->nf, npf = nf * nf * nf;
  const double h = 2. / (nf - 1);
  const double *U = w_fv + (size_t)e * NF * npf, *PP = prim_fv + (size_t)e * NF * npf;
  int q, a, f;
  /* sources and det(dXb/dx) at the points */
  double *detp = (double *)malloc(sizeof(double) * npf);
  for (q = 0; q < npf; q++) {
    const double Xb[3] = {P->xu[q % nf], P->xu[(q / nf) % nf], P->xu[q / (nf * nf)]};
    double x[3], Mb[3][3], bg[8], Pq[NF], S[NF];
    geo_at(m, e, Xb, x, Mb);
    nmo_gr_background(m->mass, x, bg);
    detp[q] = det3(Mb);
    for (f = 0; f < NF; f++) Pq[f] = PP[f * npf + q];
    sources(&m->g, Pq, bg, S);
    for (f = 0; f < NF; f++) r[f * npf + q] = S[f];
  }
  for (a = 0; a < 3; a++) {
    const int str[3] = {1, nf, nf * nf};
    const int o1 = a == 0 ? 1 : 0, o2 = a == 2 ? 1 : 2;
    int i1, i2;
    for (i2 = 0; i2 < nf; i2++)
      for (i1 = 0; i1 < nf; i1++) {
        double G[2 * MAXN][NF], Gf[2][NF], pen[NF][2 * MAXN];
        int base = i1 * str[o1] + i2 * str[o2], t, side;
        for (f = 0; f < NF; f++)
          for (t = 0; t < nf; t++) pen[f][t] = PP[f * npf + base + t * str[a]];
        /* midpoint fluxes G_t (t = 0..nf-2), J |grad Xb^a| F*.n */
        for (t = 0; t < nf - 1; t++) {
          double Xb[3], x[3], Mb[3][3], bg[8], PL[NF], PR[NF], UL[NF], UR[NF], Fs[NF], Fi[NF];
          double nrm[3], nm, jg;
          int ok;
          Xb[o1] = P->xu[i1];
          Xb[o2] = P->xu[i2];
          Xb[a] = 0.5 * (P->xu[t] + P->xu[t + 1]);
          geo_at(m, e, Xb, x, Mb);
          nmo_gr_background(m->mass, x, bg);
          nm = sqrt(Mb[a][0] * Mb[a][0] + Mb[a][1] * Mb[a][1] + Mb[a][2] * Mb[a][2]);
          for (f = 0; f < 3; f++) nrm[f] = Mb[a][f] / nm;
          jg = nm / det3(Mb);
          for (f = 0; f < NF; f++) {
            PL[f] = nmo_rec_p(m->rec, nf, pen[f], t, 2.);
            PR[f] = nmo_rec_m(m->rec, nf, pen[f], t, 2.);
          }
          ok = physical(PL, bg[1]);
          if (!ok)
            for (f = 0; f < NF; f++) PL[f] = pen[f][t];
          ok = physical(PR, bg[1]);
          if (!ok)
            for (f = 0; f < NF; f++) PR[f] = pen[f][t + 1];
          p2c(&m->g, bg[1], PL, UL);
          p2c(&m->g, bg[1], PR, UR);
          llf(&m->g, UL, PL, UR, PR, nrm, bg[0], bg[1], Fs, Fi);
          for (f = 0; f < NF; f++) G[t][f] = jg * Fs[f];
        }
        /* face points: outward flux with the neighbour's trace (the
           physical flux on outer faces) */
        for (side = 0; side < 2; side++) {
          const int t0 = side ? nf - 1 : 0, fc = 2 * a + side;
          const int qq = base + t0 * str[a];
          const double Xb[3] = {P->xu[qq % nf], P->xu[(qq / nf) % nf], P->xu[qq / (nf * nf)]};
          const int fa = i1, fb = i2;  /* in-plane (a, b) of face fc */
          double x[3], Mb[3][3], bg[8], Ui[NF], Pi[NF], Uo[NF], Po[NF], Fs[NF], Fi[NF];
          double nrm[3], nm, jg;
          geo_at(m, e, Xb, x, Mb);
          nmo_gr_background(m->mass, x, bg);
          nm = sqrt(Mb[a][0] * Mb[a][0] + Mb[a][1] * Mb[a][1] + Mb[a][2] * Mb[a][2]);
          for (f = 0; f < 3; f++) nrm[f] = (side ? 1. : -1.) * Mb[a][f] / nm;
          jg = nm / det3(Mb);
          for (f = 0; f < NF; f++) {
            Ui[f] = U[f * npf + qq];
            Pi[f] = PP[f * npf + qq];
          }
          if (exterior(m, P, e, fc, fa, fb, bg[1], w_dg, w_fv, prim_dg, prim_fv, Uo, Po))
            llf(&m->g, Ui, Pi, Uo, Po, nrm, bg[0], bg[1], Fs, Fi);
          else
            flux_n(Ui, Pi, nrm, bg[0], bg[1], Fs);
          for (f = 0; f < NF; f++) Gf[side][f] = jg * Fs[f];
        }
        for (t = 0; t < nf; t++) {
          const int qq = base + t * str[a];
          for (f = 0; f < NF; f++) {
            double dv;
            if (t == 0) dv = (G[0][f] + Gf[0][f]) / (0.5 * h);
            else if (t == nf - 1) dv = (Gf[1][f] - G[nf - 2][f]) / (0.5 * h);
            else dv = (G[t][f] - G[t - 1][f]) / h;
            r[f * npf + qq] -= detp[qq] * dv;
          }
        }
      }
  }
  free(detp);
}

/* psi at the points of element e (LGL nodes or equally spaced points) */
static double psi_at(const nmo_grmesh *m, const grpts *P, int e, int q, int fvpts)
{
  double x[3], bg[8];
  if (fvpts) {
    const int nf = m->nf;
    const double Xb[3] = {P->xu[q % nf], P->xu[(q / nf) % nf], P->xu[q / (nf * nf)]};
    double Mb[3][3];
    geo_at(m, e, Xb, x, Mb);
  } else {
    const int np = m->n * m->n * m->n;
    int d;
    for (d = 0; d < 3; d++) x[d] = m->xyz[((size_t)e * 3 + d) * np + q];
  }
  nmo_gr_background(m->mass, x, bg);
  return bg[1];
}

/* con2prim of the stage input on every point in use (atmosphere fixes
   written back into w); returns the number of atmosphere points and the
   total number of root-finder iterations */
int64_t nmo_gr_con2prim(const nmo_grmesh *m, double *w_dg, double *w_fv, double *prim_dg,
                        double *prim_fv, int64_t *iters)
{
  grpts P;
  const int np = m->n * m->n * m->n, npf = m->nf * m->nf * m->nf;
  int64_t natm = 0, it = 0;
  int e;
  grpts_init(m, &P);
#pragma omp parallel for schedule(dynamic) reduction(+ : natm, it)
  for (e = 0; e < m->nelem; e++) {
    const int isfv = m->fv[e] != 0, npts = isfv ? npf : np;
    double *W = isfv ? w_fv + (size_t)e * NF * npf : w_dg + (size_t)e * NF * np;
    double *PP = isfv ? prim_fv + (size_t)e * NF * npf : prim_dg + (size_t)e * NF * np;
    int q, f;
    for (q = 0; q < npts; q++) {
      double ps = psi_at(m, &P, e, q, isfv), U[NF], Pq[NF];
      int32_t st;
      for (f = 0; f < NF; f++) {
        U[f] = W[f * npts + q];
        Pq[f] = PP[f * npts + q];
      }
      nmo_grhd_con2prim(&m->g, 1, &ps, U, Pq, &st);
      for (f = 0; f < NF; f++) {
        W[f * npts + q] = U[f];
        PP[f * npts + q] = Pq[f];
      }
      if (st < 0) natm++;
      else it += st;
    }
  }
  if (iters) *iters = it;
  return natm;
}

/* r = RHS(w) on every element (after nmo_gr_con2prim of w) */
int nmo_gr_rhs(const nmo_grmesh *m, const double *w_dg, const double *w_fv,
               const double *prim_dg, const double *prim_fv, double *r_dg, double *r_fv)
{
  grpts P;
  const int np = m->n * m->n * m->n, npf = m->nf * m->nf * m->nf;
  int e;
  if (m->n > MAXN || m->nf > 2 * MAXN || m->nf < 3) return 1;
  grpts_init(m, &P);
#pragma omp parallel
  {
    double *F = (double *)malloc(sizeof(double) * 3 * NF * np);
#pragma omp for schedule(dynamic)
    for (e = 0; e < m->nelem; e++) {
      if (m->fv[e])
        rhs_fv(m, &P, e, w_dg, w_fv, prim_dg, prim_fv, r_fv + (size_t)e * NF * npf);
      else
        rhs_dg(m, &P, e, w_dg, w_fv, prim_dg, prim_fv, r_dg + (size_t)e * NF * np, F);
    }
    free(F);
  }
  return 0;
}

/* nsteps classic RK4 steps of (u_dg, u_fv) from t (the system is
   autonomous); prim_* are the root finder's starting guesses, updated */
int nmo_gr_rk4(const nmo_grmesh *m, double dt, int nsteps, double *u_dg, double *u_fv,
               double *prim_dg, double *prim_fv)
{
  const size_t ld = (size_t)m->nelem * NF * m->n * m->n * m->n;
  const size_t lf = (size_t)m->nelem * NF * m->nf * m->nf * m->nf;
  const double c[4] = {dt / 6., dt / 3., dt / 3., dt / 6.}, aw[3] = {dt / 2., dt / 2., dt};
  double *up_d = (double *)malloc(sizeof(double) * ld), *w_d = (double *)malloc(sizeof(double) * ld);
  double *r_d = (double *)calloc(ld, sizeof(double));
  double *up_f = (double *)malloc(sizeof(double) * lf), *w_f = (double *)malloc(sizeof(double) * lf);
  double *r_f = (double *)calloc(lf, sizeof(double));
  int s, k, rc = 0;
  size_t i;
  if (!up_d || !w_d || !r_d || !up_f || !w_f || !r_f) rc = 2;
  for (k = 0; k < nsteps && !rc; k++) {
    nmo_gr_con2prim(m, u_dg, u_fv, prim_dg, prim_fv, NULL);
    memcpy(up_d, u_dg, sizeof(double) * ld);
    memcpy(w_d, u_dg, sizeof(double) * ld);
    memcpy(up_f, u_fv, sizeof(double) * lf);
    memcpy(w_f, u_fv, sizeof(double) * lf);
    for (s = 0; s < 4 && !rc; s++) {
      if (s > 0) nmo_gr_con2prim(m, w_d, w_f, prim_dg, prim_fv, NULL);
      rc = nmo_gr_rhs(m, w_d, w_f, prim_dg, prim_fv, r_d, r_f);
      for (i = 0; i < ld; i++) {
        u_dg[i] = u_dg[i] + c[s] * r_d[i];
        if (s < 3) w_d[i] = up_d[i] + aw[s] * r_d[i];
      }
      for (i = 0; i < lf; i++) {
        u_fv[i] = u_fv[i] + c[s] * r_f[i];
        if (s < 3) w_f[i] = up_f[i] + aw[s] * r_f[i];
      }
    }
  }
  free(up_d); free(w_d); free(r_d); free(up_f); free(w_f); free(r_f);
  return rc;
}

/* ---------------------------------------------------------------------- */
/* DG <-> finite-volume transfer                                           */
/* ---------------------------------------------------------------------- */
/* P[q][m] = l_m(xu_q) (nf x n) and R = (P^T P)^-1 P^T (n x nf), built in
   long double */
void nmo_gr_transfer(int n, int nf, double *Pm, double *Rm)
{
  double xl[MAXN], wl[MAXN], xu[2 * MAXN];
  long double PtP[MAXN][2 * MAXN], Pl[2 * MAXN][MAXN];
  int q, i, j, k;
  nmo_lgl(n, xl, wl);
  nmo_uniform(nf, xu);
  for (q = 0; q < nf; q++)
    for (i = 0; i < n; i++) {
      long double v = 1.L;
      for (j = 0; j < n; j++)
        if (j != i) v *= ((long double)xu[q] - xl[j]) / ((long double)xl[i] - xl[j]);
      Pl[q][i] = v;
      Pm[q * n + i] = (double)v;
    }
  /* [P^T P | P^T], Gauss-Jordan with partial pivoting */
  for (i = 0; i < n; i++) {
    for (j = 0; j < n; j++) {
      long double s = 0.L;
      for (q = 0; q < nf; q++) s += Pl[q][i] * Pl[q][j];
      PtP[i][j] = s;
    }
    for (q = 0; q < nf; q++) PtP[i][n + q] = Pl[q][i];
  }
  for (k = 0; k < n; k++) {
    int piv = k;
    long double d;
    for (i = k + 1; i < n; i++)
      if (fabsl(PtP[i][k]) > fabsl(PtP[piv][k])) piv = i;
    if (piv != k)
      for (j = 0; j < n + nf; j++) {
        long double t = PtP[k][j];
        PtP[k][j] = PtP[piv][j];
        PtP[piv][j] = t;
      }
    d = PtP[k][k];
    for (j = 0; j < n + nf; j++) PtP[k][j] /= d;
    for (i = 0; i < n; i++)
      if (i != k) {
        long double fct = PtP[i][k];
        for (j = 0; j < n + nf; j++) PtP[i][j] -= fct * PtP[k][j];
      }
  }
  for (i = 0; i < n; i++)
    for (q = 0; q < nf; q++) Rm[i * nf + q] = (double)PtP[i][n + q];
}

/* out = (A x A x A) in for one field: A is (no x ni), in ni^3, out no^3 */
void nmo_gr_apply3(int ni, int no, const double *A, const double *in, double *out)
{
  double *t1 = (double *)malloc(sizeof(double) * no * ni * ni);
  double *t2 = (double *)malloc(sizeof(double) * no * no * ni);
  int i, j, k, m;
  for (k = 0; k < ni; k++)
    for (j = 0; j < ni; j++)
      for (i = 0; i < no; i++) {
        double s = 0.;
        for (m = 0; m < ni; m++) s += A[i * ni + m] * in[m + ni * (j + ni * k)];
        t1[i + no * (j + ni * k)] = s;
      }
  for (k = 0; k < ni; k++)
    for (j = 0; j < no; j++)
      for (i = 0; i < no; i++) {
        double s = 0.;
        for (m = 0; m < ni; m++) s += A[j * ni + m] * t1[i + no * (m + ni * k)];
        t2[i + no * (j + no * k)] = s;
      }
  for (k = 0; k < no; k++)
    for (j = 0; j < no; j++)
      for (i = 0; i < no; i++) {
        double s = 0.;
        for (m = 0; m < ni; m++) s += A[k * ni + m] * t2[i + no * (j + no * m)];
        out[i + no * (j + no * k)] = s;
      }
  free(t1);
  free(t2);
}

/* coordinates [3][npts] of the points of element e (equally spaced with
   fvpts, else the LGL nodes) */
void nmo_gr_points(const nmo_grmesh *m, int e, int fvpts, double *xyz)
{
  grpts P;
  int q, d;
  grpts_init(m, &P);
  if (!fvpts) {
    const int np = m->n * m->n * m->n;
    memcpy(xyz, m->xyz + (size_t)e * 3 * np, sizeof(double) * 3 * np);
    return;
  }
  for (q = 0; q < m->nf * m->nf * m->nf; q++) {
    const int nf = m->nf, npf = nf * nf * nf;
    const double Xb[3] = {P.xu[q % nf], P.xu[(q / nf) % nf], P.xu[q / (nf * nf)]};
    double x[3], Mb[3][3];
    geo_at(m, e, Xb, x, Mb);
    for (d = 0; d < 3; d++) xyz[d * npf + q] = x[d];
  }
}
