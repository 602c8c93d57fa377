/* nmo_mesh.c -- ORACLE (test infrastructure only; never part of the product
 * path): the oracle's own mesh generator and face matcher, so that the
 * oracle can run a workload without any of the product's code.
 *
 * It restates the reference's setup-time geometry in the reference's
 * operation order (so that, compiled with -ffp-contract=off, coordinates
 * and dX/dx equal the reference's bit for bit):
 *   box patch              src/main/coordinates/setup_Boxes.c:6-25
 *   7 CubedSpheres         src/main/amr/mesh.c:536-540 ->
 *                          src/main/coordinates/setup_CubedSpheres.c:193-218
 *                          (sphere_around_full_box_at_xc), :653-681
 *                          (add_N_CubedSphere_pats, set_AB_min_max_from_Din)
 *   element bboxes         src/main/amr/connections.c:1175-1205
 *                          (amr_set_elm0_bbox: successive halving)
 *   X of Xb                src/main/coordinates/get_coords.c:384-394
 *   cubed-sphere map       src/main/coordinates/coordtrans_CubedSphere.c:
 *                          37-118 (xyz_of_lamAB_CubSph), 257-509
 *                          (dlamAB_dxyz_CubSph), types outerCubedSphere and
 *                          CubedShell with constant sigma
 *   node coordinates       src/main/coordinates/coordinates.c:133-224
 * Shell meshes (6 CubedShell patches between two spheres) use the same map
 * with both surfaces curved; the reference builds such patches but has no
 * mesh type of six of them alone (parity of that layout is unpinned).
 *
 * Face matching: two element faces are neighbours when their corner
 * centroids coincide (modulo a period per axis for a periodic box); the
 * in-plane node correspondence is the dihedral orientation under which the
 * four corners coincide (the reference copies coincident neighbour points,
 * src/main/amr/surface.c:799-900).  Conforming meshes only.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

void nmo_lgl(int npoints, double *x, double *w);
void nmo_uniform(int npoints, double *x);

/* patch kinds */
enum { OP_BOX = 0, OP_OUTER = 1, OP_SHELL = 2 };

typedef struct opatch {
  int kind, dom;
  double bbox[6];
  double xc[3];
  double s0, s1;   /* inner distance (flat) or radius, outer radius */
} opatch;

/* mesh types of nmo_mesh_generate */
enum { NMO_MESH_BOX = 1, NMO_MESH_SHELL6 = 6, NMO_MESH_CUBEDSPHERES7 = 7 };

/* A, B range of cubed-sphere domain dom from the inner distances
   (set_AB_min_max_from_Din) */
static void ab_minmax(int dom, const double Din[6], double ab[4])
{
  static const int nbr[6][4] = {{3, 2, 5, 4}, {2, 3, 4, 5}, {1, 0, 5, 4},
                                {0, 1, 4, 5}, {3, 2, 1, 0}, {2, 3, 0, 1}};
  ab[0] = -Din[nbr[dom][0]] / Din[dom];
  ab[1] = Din[nbr[dom][1]] / Din[dom];
  ab[2] = -Din[nbr[dom][2]] / Din[dom];
  ab[3] = Din[nbr[dom][3]] / Din[dom];
}

static int make_patches(int type, const double prm[4], opatch *P)
{
  int np = 0, d, dom;
  if (type == NMO_MESH_BOX) {
    /* prm: xc (3), half edge */
    memset(&P[0], 0, sizeof(opatch));
    for (d = 0; d < 3; d++) {
      P[0].bbox[2 * d] = prm[d] - prm[3];
      P[0].bbox[2 * d + 1] = prm[d] + prm[3];
    }
    return 1;
  }
  if (type == NMO_MESH_CUBEDSPHERES7) {
    /* prm: dc, r0fac (outer radius r0fac dc), centre at 0 */
    double dc = prm[0], r0 = prm[1] * dc, Din[6];
    memset(&P[0], 0, sizeof(opatch));
    for (d = 0; d < 3; d++) {
      P[0].bbox[2 * d] = 0.0 - dc;
      P[0].bbox[2 * d + 1] = 0.0 + dc;
    }
    np = 1;
    for (d = 0; d < 6; d++) Din[d] = dc;
    for (dom = 0; dom < 6; dom++) {
      double ab[4];
      opatch *c = &P[np++];
      memset(c, 0, sizeof(opatch));
      ab_minmax(dom, Din, ab);
      c->kind = OP_OUTER;
      c->dom = dom;
      c->bbox[0] = 0.; c->bbox[1] = 1.;
      c->bbox[2] = ab[0]; c->bbox[3] = ab[1]; c->bbox[4] = ab[2]; c->bbox[5] = ab[3];
      c->s0 = Din[dom];
      c->s1 = r0;
    }
    return np;
  }
  if (type == NMO_MESH_SHELL6) {
    /* prm: inner radius, outer radius, centre at 0 */
    double Din[6];
    for (d = 0; d < 6; d++) Din[d] = prm[0];
    for (dom = 0; dom < 6; dom++) {
      double ab[4];
      opatch *c = &P[np++];
      memset(c, 0, sizeof(opatch));
      ab_minmax(dom, Din, ab);
      c->kind = OP_SHELL;
      c->dom = dom;
      c->bbox[0] = 0.; c->bbox[1] = 1.;
      c->bbox[2] = ab[0]; c->bbox[3] = ab[1]; c->bbox[4] = ab[2]; c->bbox[5] = ab[3];
      c->s0 = prm[0];
      c->s1 = prm[1];
    }
    return np;
  }
  return -1;
}

/* x and dX/dx of a cubed-sphere patch with constant sigma (the outer
   surface curved; with OP_SHELL also the inner one), in the reference's
   operation order for each direction dir = dom / 2: the radial Cartesian
   index is dir, A runs along ia and B along ib */
static void cs_map(const opatch *P, const double X[3], double x[3], double J[3][3])
{
  const double lam = X[0], A = X[1], B = X[2];
  const int dir = P->dom / 2;
  const int ia = dir == 0 ? 1 : (dir == 1 ? 0 : 1);
  const int ib = dir == 0 ? 2 : (dir == 1 ? 2 : 0);
  const double pm = 2 * (P->dom % 2) - 1;
  const double sq = sqrt(1.0 + A * A + B * B);
  double a0, a1, dA0 = 0.0, dB0 = 0.0, dA1, dB1, da0[3], da1[3];
  double r[3], r2[3], rc2, m[3], m0[3], m1[3], rR, rR2;
  int c;
  /* constant sigma: d sigma / dA = d sigma / dB = 0 */
  dA1 = 0.0 / P->s1;
  dB1 = 0.0 / P->s1;
  a1 = pm * P->s1 / sq;
  if (P->kind == OP_SHELL) {
    dA0 = 0.0 / P->s0;
    dB0 = 0.0 / P->s0;
    a0 = pm * P->s0 / sq;
    for (c = 0; c < 3; c++) da0[c] = a0;   /* marked non-zero */
  } else {
    a0 = pm * P->s0;
    for (c = 0; c < 3; c++) da0[c] = 0.0;
  }
  for (c = 0; c < 3; c++) da1[c] = a1;     /* marked non-zero */
  rR = (a1 - a0) * lam + a0;
  x[dir] = P->xc[dir] + rR;
  x[ia] = P->xc[ia] + A * rR;
  x[ib] = P->xc[ib] + B * rR;
  for (c = 0; c < 3; c++) r[c] = (c == dir) ? rR : x[c] - P->xc[c];
  for (c = 0; c < 3; c++) r2[c] = r[c] * r[c];
  rc2 = r2[0] + r2[1] + r2[2];
  rR2 = r2[dir];
  for (c = 0; c < 3; c++) {
    if (c == dir) {
      m[c] = (1.0 / rR - rR / rc2);
      m0[c] = -dA0 * (r[ia] / rR2) - dB0 * (r[ib] / rR2);
      m1[c] = -dA1 * (r[ia] / rR2) - dB1 * (r[ib] / rR2);
    } else {
      m[c] = (-r[c] / rc2);
      m0[c] = (c == ia) ? dA0 / rR : dB0 / rR;
      m1[c] = (c == ia) ? dA1 / rR : dB1 / rR;
    }
  }
  for (c = 0; c < 3; c++) {
    da0[c] *= (m[c] + m0[c]);
    da1[c] *= (m[c] + m1[c]);
  }
  for (c = 0; c < 3; c++) {
    if (c == dir)
      J[0][c] = (1.0 - da0[c] - (da1[c] - da0[c]) * lam) / (a1 - a0);
    else
      J[0][c] = (-da0[c] - (da1[c] - da0[c]) * lam) / (a1 - a0);
  }
  for (c = 0; c < 3; c++) {
    J[1][c] = 0.0;
    J[2][c] = 0.0;
  }
  J[1][dir] = -r[ia] / rR2;
  J[1][ia] = 1.0 / rR;
  J[2][dir] = -r[ib] / rR2;
  J[2][ib] = J[1][ia];
}

/* x and dX/dx at patch coordinates X of patch p of a generated mesh */
int nmo_mesh_map(int type, const double prm[4], int p, const double X[3], double x[3],
                 double J[3][3])
{
  opatch P[8];
  int npat = make_patches(type, prm, P), d, c;
  if (npat < 0 || p < 0 || p >= npat) return 1;
  if (P[p].kind != OP_BOX) {
    cs_map(&P[p], X, x, J);
  } else {
    for (d = 0; d < 3; d++) {
      x[d] = X[d];
      for (c = 0; c < 3; c++) J[d][c] = (d == c) ? 1. : 0.;
    }
  }
  return 0;
}

/* elements of one patch at uniform level L: count per patch */
int64_t nmo_mesh_count(int type, int luni)
{
  const int np = type == NMO_MESH_BOX ? 1 : (type == NMO_MESH_SHELL6 ? 6 : 7);
  if (luni < 0 || luni > 10 || (type != NMO_MESH_BOX && type != NMO_MESH_SHELL6 &&
                                type != NMO_MESH_CUBEDSPHERES7))
    return -1;
  return (int64_t)np << (3 * luni);
}

/* Generate a uniform mesh of n points per direction (LGL, or equally spaced
   with uniform != 0) at level luni: per element its patch, bbox (patch
   coordinates), a curvilinear flag, x [3][np] and dX/dx [9][np] (identity
   on Cartesian elements); elements patch by patch, Morton order inside. */
int nmo_mesh_generate(int type, int n, int luni, int ndiv, const double prm[4], int uniform,
                      int32_t *pat, double *bbox, int32_t *curvi, double *xyz, double *dXdx)
{
  opatch P[8];
  double px[64], pw[64];
  const int npts = n * n * n;
  const int64_t per = ndiv > 0 ? (int64_t)ndiv * ndiv * ndiv : (int64_t)1 << (3 * luni);
  int npat, p;
  int64_t e = 0, mc;
  if (n < 2 || n > 64 || nmo_mesh_count(type, luni) < 0 || ndiv < 0) return 1;
  npat = make_patches(type, prm, P);
  if (npat < 0) return 1;
  if (uniform) nmo_uniform(n, px);
  else nmo_lgl(n, px, pw);
  for (p = 0; p < npat; p++)
    for (mc = 0; mc < per; mc++, e++) {
      double *bb = bbox + e * 6, LX[3];
      int ix[3] = {0, 0, 0}, bit, d, ll, i, j, k;
      if (ndiv > 0) {
        /* ndiv equal parts per direction, i fastest */
        const double *pb = P[p].bbox;
        ix[0] = (int)(mc % ndiv);
        ix[1] = (int)((mc / ndiv) % ndiv);
        ix[2] = (int)(mc / ((int64_t)ndiv * ndiv));
        for (d = 0; d < 3; d++) {
          bb[2 * d] = pb[2 * d] + (pb[2 * d + 1] - pb[2 * d]) * (double)ix[d] / ndiv;
          bb[2 * d + 1] = ix[d] + 1 == ndiv
                              ? pb[2 * d + 1]
                              : pb[2 * d] + (pb[2 * d + 1] - pb[2 * d]) * (double)(ix[d] + 1) / ndiv;
        }
      } else {
        for (bit = 0; bit < luni; bit++)
          for (d = 0; d < 3; d++) ix[d] |= (int)((mc >> (3 * bit + d)) & 1) << bit;
        /* amr_set_elm0_bbox */
        for (d = 0; d < 6; d++) bb[d] = P[p].bbox[d];
        for (d = 0; d < 3; d++) LX[d] = bb[2 * d + 1] - bb[2 * d];
        for (ll = 1; ll <= luni; ll++)
          for (d = 0; d < 3; d++) {
            LX[d] /= 2.;
            if ((ix[d] >> (luni - ll)) & 1) bb[2 * d] = bb[2 * d + 1] - LX[d];
            else bb[2 * d + 1] = bb[2 * d] + LX[d];
          }
      }
      pat[e] = p;
      curvi[e] = P[p].kind != OP_BOX;
      for (k = 0; k < n; k++)
        for (j = 0; j < n; j++)
          for (i = 0; i < n; i++) {
            const int ijk = i + n * (j + n * k);
            double Xb[3], X[3], x[3], J[3][3];
            int a, c;
            Xb[0] = px[i]; Xb[1] = px[j]; Xb[2] = px[k];
            for (d = 0; d < 3; d++)
              X[d] = 0.5 * ((bb[2 * d + 1] - bb[2 * d]) * Xb[d] + (bb[2 * d + 1] + bb[2 * d]));
            if (P[p].kind != OP_BOX) {
              cs_map(&P[p], X, x, J);
            } else {
              for (d = 0; d < 3; d++) {
                x[d] = X[d];
                for (c = 0; c < 3; c++) J[d][c] = (d == c) ? 1. : 0.;
              }
            }
            for (d = 0; d < 3; d++) xyz[(e * 3 + d) * npts + ijk] = x[d];
            for (a = 0; a < 3; a++)
              for (c = 0; c < 3; c++) dXdx[(e * 9 + a * 3 + c) * npts + ijk] = J[a][c];
          }
    }
  return 0;
}

/* ---------------------------------------------------------------------- */
/* face matching                                                           */
/* ---------------------------------------------------------------------- */
typedef struct fkey {
  int64_t k[3];
  int64_t ef;  /* e * 6 + f */
} fkey;

static int fkey_cmp(const void *pa, const void *pb)
{
  const fkey *a = (const fkey *)pa, *b = (const fkey *)pb;
  int d;
  for (d = 0; d < 3; d++)
    if (a->k[d] != b->k[d]) return a->k[d] < b->k[d] ? -1 : 1;
  return a->ef < b->ef ? -1 : (a->ef > b->ef);
}

/* volume index of in-plane node (a, b) of face f (Ind_n_norm order) */
static int face_ijk(int n, int f, int a, int b)
{
  const int d = f / 2, q = (f % 2) * (n - 1);
  if (d == 0) return q + n * (a + n * b);
  if (d == 1) return a + n * (q + n * b);
  return a + n * (b + n * q);
}

static double wrapc(double v, double period)
{
  double q;
  if (!(period > 0)) return v;
  q = fmod(v, period);
  if (q < 0) q += period;
  if (fabs(q - period) < 1e-7) q = 0.;
  return q;
}

static void corner(const double *xyz, int64_t e, int n, int f, int a, int b, double c[3])
{
  const int npts = n * n * n, ijk = face_ijk(n, f, a, b);
  int d;
  for (d = 0; d < 3; d++) c[d] = xyz[(e * 3 + d) * npts + ijk];
}

static int same_point(const double p[3], const double q[3], const double *period, double tol)
{
  int d;
  for (d = 0; d < 3; d++) {
    double dd = p[d] - q[d];
    if (period && period[d] > 0) dd -= period[d] * floor(dd / period[d] + 0.5);
    if (fabs(dd) > tol) return 0;
  }
  return 1;
}

/* nbnode[E][6][n*n]: global index e'*np + ijk' of the coincident node across
   each face node, -1 on outer faces; nb[E][6] / code[E][6] (may be NULL):
   the neighbour element (-1 outer) and its face | orientation << 3, node
   (a, b) lying at the neighbour's (a', b') = (s ? b : a, s ? a : b),
   reversed per axis by bits 1 and 2 (s = bit 0).  period may be NULL.  Returns 0, or 1
   when a face is matched more than once or its corners do not coincide. */
int nmo_match_faces(int64_t E, int n, const double *xyz, const double *period, int64_t *nbnode,
                    int32_t *nb, int32_t *code)
{
  const int npts = n * n * n, nn = n * n;
  const double h = 1e-6, tol = 1e-9;
  fkey *keys = (fkey *)malloc(sizeof(fkey) * (size_t)E * 6);
  int64_t q, i;
  int rc = 0;
  if (!keys) return 2;
  for (q = 0; q < E * 6 * nn; q++) nbnode[q] = -1;
  if (nb)
    for (q = 0; q < E * 6; q++) nb[q] = -1;
  if (code)
    for (q = 0; q < E * 6; q++) code[q] = 0;
  for (q = 0; q < E * 6; q++) {
    const int64_t e = q / 6;
    const int f = (int)(q % 6);
    double c[4][3], cen[3];
    int d, s;
    corner(xyz, e, n, f, 0, 0, c[0]);
    corner(xyz, e, n, f, n - 1, 0, c[1]);
    corner(xyz, e, n, f, 0, n - 1, c[2]);
    corner(xyz, e, n, f, n - 1, n - 1, c[3]);
    for (d = 0; d < 3; d++) {
      cen[d] = 0.;
      for (s = 0; s < 4; s++) cen[d] += c[s][d];
      cen[d] = wrapc(0.25 * cen[d], period ? period[d] : 0.);
      keys[q].k[d] = (int64_t)llround(cen[d] / h);
    }
    keys[q].ef = q;
  }
  qsort(keys, (size_t)E * 6, sizeof(fkey), fkey_cmp);
  for (i = 0; i < E * 6; i++) {
    int64_t j = i + 1, pair[2];
    int side;
    if (j < E * 6 && memcmp(keys[i].k, keys[j].k, sizeof(keys[i].k)) == 0) {
      if (j + 1 < E * 6 && memcmp(keys[j].k, keys[j + 1].k, sizeof(keys[j].k)) == 0) {
        rc = 1;  /* three faces at one place: not conforming */
        break;
      }
      pair[0] = keys[i].ef;
      pair[1] = keys[j].ef;
      for (side = 0; side < 2; side++) {
        const int64_t e = pair[side] / 6, e2 = pair[1 - side] / 6;
        const int f = (int)(pair[side] % 6), f2 = (int)(pair[1 - side] % 6);
        int o, found = -1, a, b;
        for (o = 0; o < 8 && found < 0; o++) {
          int ok = 1, s;
          for (s = 0; s < 4 && ok; s++) {
            const int ca = (s & 1) ? n - 1 : 0, cb = (s & 2) ? n - 1 : 0;
            int aa = (o & 1) ? cb : ca, bb = (o & 1) ? ca : cb;
            double p1[3], p2[3];
            if (o & 2) aa = n - 1 - aa;
            if (o & 4) bb = n - 1 - bb;
            corner(xyz, e, n, f, ca, cb, p1);
            corner(xyz, e2, n, f2, aa, bb, p2);
            ok = same_point(p1, p2, period, tol);
          }
          if (ok) found = o;
        }
        if (found < 0) {
          rc = 1;
          break;
        }
        if (nb) nb[e * 6 + f] = (int32_t)e2;
        if (code) code[e * 6 + f] = f2 | (found << 3);
        for (b = 0; b < n; b++)
          for (a = 0; a < n; a++) {
            int aa = (found & 1) ? b : a, bb = (found & 1) ? a : b;
            if (found & 2) aa = n - 1 - aa;
            if (found & 4) bb = n - 1 - bb;
            nbnode[(e * 6 + f) * nn + a + n * b] = e2 * npts + face_ijk(n, f2, aa, bb);
          }
      }
      if (rc) break;
      i = j;
    }
  }
  free(keys);
  return rc;
}
