// mesh.cpp -- host-side mesh packer.
//
// Produces the static element/face description that the device context
// uploads: element geometry and metric (a restatement of the reference's
// setup-time coordinate code), and a face table (neighbour element,
// neighbour face, dihedral orientation of the in-plane node order) found by
// matching face-node coordinates.  Runs once per mesh; compiled with
// -ffp-contract=off so that the geometry is bitwise the same on x86-64 and
// aarch64 hosts.
//
// Reference code restated here (paths within nmeshsource/nmesh):
//   LGL nodes/weights     src/main/basis/Legendre.c:59-98,149-213
//   D matrix              src/main/basis/Lagrange.c:15-27,126-147
//   box patch             src/main/coordinates/setup_Boxes.c:6-25
//   7 CubedSpheres        src/main/amr/mesh.c:536-540 ->
//                         src/main/coordinates/setup_CubedSpheres.c:193-218,
//                         653-681,829-880,935-944
//   uniform refinement    src/main/amr/connections.c:1175-1205 (bbox halving)
//   X of Xb               src/main/coordinates/get_coords.c:384-394
//   cubed-sphere map and  src/main/coordinates/coordtrans_CubedSphere.c:37-118,
//   its derivatives         257-509 (outerCubedSphere, constant sigma)
//   node coordinates      src/main/coordinates/coordinates.c:133-224
#include "mesh.h"
#include "../../include/nmg.h"

#include <algorithm>
#include <array>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <new>
#include <unordered_map>

namespace {
thread_local std::string g_mesh_err;

int fail(int code, const std::string &msg) {
  g_mesh_err = msg;
  return code;
}

void legendre_P_dP_Q_dQ(int l, double x, double *P, double *dP, double *Q,
                        double *dQ) {
  double P0 = 1., P1 = x, dP0 = 0., dP1 = 1., Pk = 0., dPk = 0.;
  if (l == 0) { *P = 1.; *dP = 0.; return; }
  if (l == 1) { *P = x; *dP = 1.; return; }
  for (int k = 2; k <= l + 1; k++) {
    Pk = (P1 * x * (2 * k - 1) - P0 * (k - 1)) / k;
    dPk = P1 * (2 * k - 1) + dP0;
    if (k >= l + 1) break;
    P0 = P1; P1 = Pk; dP0 = dP1; dP1 = dPk;
  }
  *P = P1; *dP = dP1; *Q = Pk - P0; *dQ = dPk - dP0;
}

// one patch of the mesh
using nmg::Patch;

// x and dX/dx of an outerCubedSphere patch with constant sigma1 = s1
// (xyz_of_lamAB_CubSph / dlamAB_dxyz_CubSph), same operation order
void cubsph_x_dXdx(const Patch &P, const double X[3], double x[3],
                   double dXdx[3][3]) {
  double lam = X[0], A = X[1], B = X[2];
  int dir = P.dom / 2;
  double pm = 2 * (P.dom % 2) - 1;
  double xc = P.xc[0], yc = P.xc[1], zc = P.xc[2];
  double sqrt_1_A2_B2 = sqrt(1.0 + A * A + B * B);
  double a0 = pm * P.s0;
  double sigma1 = P.s1;
  double dsig1[2] = {0., 0.};
  double dsigma_dA_osigma1 = dsig1[0] / sigma1;
  double dsigma_dB_osigma1 = dsig1[1] / sigma1;
  double a1 = pm * sigma1 / sqrt_1_A2_B2;
  double da0_dx = 0.0, da0_dy = 0.0, da0_dz = 0.0;
  double da1_dx = a1, da1_dy = a1, da1_dz = a1;
  double dsigma_dA_osigma0 = 0.0, dsigma_dB_osigma0 = 0.0;
  if (P.shell) {
    // CubedShell: the inner surface is the sphere of radius s0 too
    double dsig0[2] = {0., 0.};
    dsigma_dA_osigma0 = dsig0[0] / P.s0;
    dsigma_dB_osigma0 = dsig0[1] / P.s0;
    a0 = pm * P.s0 / sqrt_1_A2_B2;
    da0_dx = a0; da0_dy = a0; da0_dz = a0;
  }
  double rx, ry, rz, rx2, ry2, rz2, rc2, mx, my, mz, mx0, my0, mz0, mx1, my1,
      mz1;
  double *dlamdx = &dXdx[0][0], *dlamdy = &dXdx[0][1], *dlamdz = &dXdx[0][2];
  double *dAdx = &dXdx[1][0], *dAdy = &dXdx[1][1], *dAdz = &dXdx[1][2];
  double *dBdx = &dXdx[2][0], *dBdy = &dXdx[2][1], *dBdz = &dXdx[2][2];
  if (dir == 0) {
    rx = (a1 - a0) * lam + a0;
    x[0] = xc + rx; x[1] = yc + A * rx; x[2] = zc + B * rx;
    ry = x[1] - yc; rz = x[2] - zc;
    rx2 = rx * rx; ry2 = ry * ry; rz2 = rz * rz;
    rc2 = rx2 + ry2 + rz2;
    mx = (1.0 / rx - rx / rc2); my = (-ry / rc2); mz = (-rz / rc2);
    mx0 = -dsigma_dA_osigma0 * (ry / rx2) - dsigma_dB_osigma0 * (rz / rx2);
    my0 = dsigma_dA_osigma0 / rx;
    mz0 = dsigma_dB_osigma0 / rx;
    mx1 = -dsigma_dA_osigma1 * (ry / rx2) - dsigma_dB_osigma1 * (rz / rx2);
    my1 = dsigma_dA_osigma1 / rx;
    mz1 = dsigma_dB_osigma1 / rx;
    da0_dx *= (mx + mx0); da0_dy *= (my + my0); da0_dz *= (mz + mz0);
    da1_dx *= (mx + mx1); da1_dy *= (my + my1); da1_dz *= (mz + mz1);
    *dlamdx = (1.0 - da0_dx - (da1_dx - da0_dx) * lam) / (a1 - a0);
    *dlamdy = (-da0_dy - (da1_dy - da0_dy) * lam) / (a1 - a0);
    *dlamdz = (-da0_dz - (da1_dz - da0_dz) * lam) / (a1 - a0);
    *dAdx = -ry / rx2; *dAdy = 1.0 / rx; *dAdz = 0.0;
    *dBdx = -rz / rx2; *dBdy = 0.0; *dBdz = *dAdy;
  } else if (dir == 1) {
    ry = (a1 - a0) * lam + a0;
    x[1] = yc + ry; x[0] = xc + A * ry; x[2] = zc + B * ry;
    rx = x[0] - xc; rz = x[2] - zc;
    rx2 = rx * rx; ry2 = ry * ry; rz2 = rz * rz;
    rc2 = rx2 + ry2 + rz2;
    mx = (-rx / rc2); my = (1.0 / ry - ry / rc2); mz = (-rz / rc2);
    mx0 = dsigma_dA_osigma0 / ry;
    my0 = -dsigma_dA_osigma0 * (rx / ry2) - dsigma_dB_osigma0 * (rz / ry2);
    mz0 = dsigma_dB_osigma0 / ry;
    mx1 = dsigma_dA_osigma1 / ry;
    my1 = -dsigma_dA_osigma1 * (rx / ry2) - dsigma_dB_osigma1 * (rz / ry2);
    mz1 = dsigma_dB_osigma1 / ry;
    da0_dx *= (mx + mx0); da0_dy *= (my + my0); da0_dz *= (mz + mz0);
    da1_dx *= (mx + mx1); da1_dy *= (my + my1); da1_dz *= (mz + mz1);
    *dlamdx = (-da0_dx - (da1_dx - da0_dx) * lam) / (a1 - a0);
    *dlamdy = (1.0 - da0_dy - (da1_dy - da0_dy) * lam) / (a1 - a0);
    *dlamdz = (-da0_dz - (da1_dz - da0_dz) * lam) / (a1 - a0);
    *dAdx = 1.0 / ry; *dAdy = -rx / ry2; *dAdz = 0.0;
    *dBdx = 0.0; *dBdy = -rz / ry2; *dBdz = *dAdx;
  } else {
    rz = (a1 - a0) * lam + a0;
    x[2] = zc + rz; x[1] = yc + A * rz; x[0] = xc + B * rz;
    rx = x[0] - xc; ry = x[1] - yc;
    rx2 = rx * rx; ry2 = ry * ry; rz2 = rz * rz;
    rc2 = rx2 + ry2 + rz2;
    mx = (-rx / rc2); my = (-ry / rc2); mz = (1.0 / rz - rz / rc2);
    mx0 = dsigma_dB_osigma0 / rz;
    my0 = dsigma_dA_osigma0 / rz;
    mz0 = -dsigma_dA_osigma0 * (ry / rz2) - dsigma_dB_osigma0 * (rx / rz2);
    mx1 = dsigma_dB_osigma1 / rz;
    my1 = dsigma_dA_osigma1 / rz;
    mz1 = -dsigma_dA_osigma1 * (ry / rz2) - dsigma_dB_osigma1 * (rx / rz2);
    da0_dx *= (mx + mx0); da0_dy *= (my + my0); da0_dz *= (mz + mz0);
    da1_dx *= (mx + mx1); da1_dy *= (my + my1); da1_dz *= (mz + mz1);
    *dlamdx = (-da0_dx - (da1_dx - da0_dx) * lam) / (a1 - a0);
    *dlamdy = (-da0_dy - (da1_dy - da0_dy) * lam) / (a1 - a0);
    *dlamdz = (1.0 - da0_dz - (da1_dz - da0_dz) * lam) / (a1 - a0);
    *dAdx = 0.0; *dAdy = 1.0 / rz; *dAdz = -ry / rz2;
    *dBdx = *dAdy; *dBdy = 0.0; *dBdz = -rx / rz2;
  }
}

// A, B ranges of cubed-sphere domain dom from the inner distances Din
// (set_AB_min_max_from_Din)
void ab_range(int dom, const double Din[6], double r[4]) {
  static const int ia[6][4] = {{3, 2, 5, 4}, {2, 3, 4, 5}, {1, 0, 5, 4},
                               {0, 1, 4, 5}, {3, 2, 1, 0}, {2, 3, 0, 1}};
  r[0] = -Din[ia[dom][0]] / Din[dom];
  r[1] = Din[ia[dom][1]] / Din[dom];
  r[2] = -Din[ia[dom][2]] / Din[dom];
  r[3] = Din[ia[dom][3]] / Din[dom];
}

// one element of a generated mesh: patch, level, integer position
struct Leaf {
  int p, L;
  int ix[3];
};

// element bbox at level L and integer location (ix,iy,iz) by successive
// halving of the patch bbox (amr_set_elm0_bbox)
void elem_bbox(const double pb[6], int L, const int ixyz[3], double bb[6]) {
  double LX[3];
  for (int f = 0; f < 6; f++) bb[f] = pb[f];
  for (int d = 0; d < 3; d++) LX[d] = bb[2 * d + 1] - bb[2 * d];
  for (int ll = 1; ll <= L; ll++) {
    for (int d = 0; d < 3; d++) {
      int bit = (ixyz[d] >> (L - ll)) & 1;
      LX[d] /= 2.;
      if (bit) bb[2 * d] = bb[2 * d + 1] - LX[d];
      else bb[2 * d + 1] = bb[2 * d] + LX[d];
    }
  }
}

// Cartesian position of the patch coordinates X (set_xyz)
void patch_x(const Patch &P, const double X[3], double x[3]) {
  if (P.cubed) {
    double J[3][3];
    cubsph_x_dXdx(P, X, x, J);
  } else {
    for (int d = 0; d < 3; d++) x[d] = X[d];
  }
}

// the elements of patch p at uniform level L, in Morton (Z) order
void uniform_leaves(int p, int L, std::vector<Leaf> &out) {
  const int64_t per = (int64_t)1 << (3 * L);
  for (int64_t mc = 0; mc < per; mc++) {
    Leaf lf{p, L, {0, 0, 0}};
    for (int bit = 0; bit < L; bit++)
      for (int d = 0; d < 3; d++) lf.ix[d] |= (int)((mc >> (3 * bit + d)) & 1) << bit;
    out.push_back(lf);
  }
}

// Nested-sphere refinement (hrefine_sphere_loadbalance and
// hrefine_once_within_sphere, src/main/amr/refine.c:1025-1100): pass i
// refines every element whose centre -- the patch map of its bbox centre
// (set_nodecenter_xyz, src/main/coordinates/utilities.c:1308-1327) -- lies
// within r_i = radius 2^(levels-1-i) of x = 0 (Cart_distance_x0_x1); a
// refined element is replaced by its eight children (child digit: bit d set
// for the upper half in direction d).
void refine_spheres(const std::vector<Patch> &pats, int levels, double radius,
                    std::vector<Leaf> &leaves) {
  double r = radius * std::pow(2., levels - 1);
  for (int i = 0; i < levels; i++, r *= 0.5) {
    std::vector<Leaf> next;
    next.reserve(leaves.size());
    for (const Leaf &lf : leaves) {
      double bb[6], X[3], x[3];
      elem_bbox(pats[lf.p].bbox, lf.L, lf.ix, bb);
      for (int d = 0; d < 3; d++) X[d] = 0.5 * (bb[2 * d + 1] + bb[2 * d]);
      patch_x(pats[lf.p], X, x);
      double dist2 = 0.;
      for (int d = 0; d < 3; d++) {
        const double tmp = 0. - x[d];
        dist2 += tmp * tmp;
      }
      if (std::sqrt(dist2) <= r) {
        for (int dig = 0; dig < 8; dig++) {
          Leaf c{lf.p, lf.L + 1, {0, 0, 0}};
          for (int d = 0; d < 3; d++) c.ix[d] = 2 * lf.ix[d] + ((dig >> d) & 1);
          next.push_back(c);
        }
      } else {
        next.push_back(lf);
      }
    }
    leaves.swap(next);
  }
}

// fill geometry for the given elements (patch, level, position); elements
// of patches in fvmask get equally spaced points
void fill_geometry(nmg_mesh &m, const std::vector<Patch> &pats, const std::vector<Leaf> &leaves,
                   int32_t fvmask) {
  const int n = m.n, np = n * n * n;
  m.nelem = (int64_t)leaves.size();
  m.patches = pats;
  m.pat.resize(m.nelem);
  m.bbox.resize(m.nelem * 6);
  m.curvi.resize(m.nelem);
  m.xyz.resize(m.nelem * 3 * np);
  m.dXdx.resize(m.nelem * 9 * np);
  m.fv.assign(m.nelem, 0);
  m.names.assign(m.nelem, std::string());
  m.level.assign(m.nelem, 0);
  m.ixyz.assign(m.nelem * 3, 0);
  for (int64_t e = 0; e < m.nelem; e++) {
    const int p = leaves[e].p, Lp = leaves[e].L;
    const int *ixyz = leaves[e].ix;
    if (m.ndiv > 0) {
      // ndiv equal parts per direction
      const double *pb = pats[p].bbox;
      double *bb = &m.bbox[e * 6];
      for (int d = 0; d < 3; d++) {
        bb[2 * d] = pb[2 * d] + (pb[2 * d + 1] - pb[2 * d]) * (double)ixyz[d] / m.ndiv;
        bb[2 * d + 1] = ixyz[d] + 1 == m.ndiv
                            ? pb[2 * d + 1]
                            : pb[2 * d] + (pb[2 * d + 1] - pb[2 * d]) * (double)(ixyz[d] + 1) / m.ndiv;
      }
    } else {
      elem_bbox(pats[p].bbox, Lp, ixyz, &m.bbox[e * 6]);
    }
    // elmname: patch, then one octree child digit per level, bit d set
    // for the upper half in direction d (connections.c:819-866,1186-1200)
    std::string nm = std::to_string(p) + "_";
    for (int ll = 1; ll <= Lp; ll++) {
      int dig = 0;
      for (int d = 0; d < 3; d++) dig |= ((ixyz[d] >> (Lp - ll)) & 1) << d;
      nm += (char)('0' + dig);
    }
    if (m.ndiv > 0)
      nm = std::to_string(p) + "_" + std::to_string(ixyz[0]) + "_" + std::to_string(ixyz[1]) +
           "_" + std::to_string(ixyz[2]);
    m.names[e] = nm;
    m.level[e] = Lp;
    for (int d = 0; d < 3; d++) m.ixyz[e * 3 + d] = ixyz[d];
    m.pat[e] = (int32_t)p;
    m.curvi[e] = pats[p].cubed ? 1 : 0;
    const bool isfv = (fvmask >> p) & 1;
    if (isfv) m.fv[e] = 1;
    nmg::element_geometry(m, e, isfv, &m.xyz[e * 3 * np], &m.dXdx[e * 9 * np]);
  }
}

// Level and integer position of each element of a mesh given element by
// element, from its bbox within its patch's extent (the union of the
// patch's element bboxes): the halvings must agree in the three directions
// and land on integer positions, else the mesh keeps no levels (and is
// matched as conforming only).
void derive_levels(nmg_mesh &m) {
  const int64_t E = m.nelem;
  std::unordered_map<int, std::array<double, 6>> ext;
  for (int64_t e = 0; e < E; e++) {
    const double *bb = &m.bbox[e * 6];
    auto it = ext.find(m.pat[e]);
    if (it == ext.end()) {
      std::array<double, 6> a;
      for (int q = 0; q < 6; q++) a[q] = bb[q];
      ext[m.pat[e]] = a;
    } else {
      for (int d = 0; d < 3; d++) {
        it->second[2 * d] = std::min(it->second[2 * d], bb[2 * d]);
        it->second[2 * d + 1] = std::max(it->second[2 * d + 1], bb[2 * d + 1]);
      }
    }
  }
  std::vector<int32_t> level(E), ixyz(E * 3);
  for (int64_t e = 0; e < E; e++) {
    const double *bb = &m.bbox[e * 6];
    const std::array<double, 6> &a = ext[m.pat[e]];
    int L = -1;
    for (int d = 0; d < 3; d++) {
      const double h = bb[2 * d + 1] - bb[2 * d], ratio = (a[2 * d + 1] - a[2 * d]) / h;
      const int Ld = (int)std::lround(std::log2(ratio));
      const double q = (bb[2 * d] - a[2 * d]) / h;
      if (Ld < 0 || Ld > 20 || std::fabs(ratio - std::ldexp(1., Ld)) > 1e-6 * ratio ||
          std::fabs(q - std::round(q)) > 1e-6 || (L >= 0 && Ld != L))
        return;
      L = Ld;
      ixyz[e * 3 + d] = (int32_t)std::lround(q);
    }
    level[e] = L;
  }
  m.level.swap(level);
  m.ixyz.swap(ixyz);
}

// quantised coordinates for the spatial hash of face centres
struct Key {
  int64_t q[3];
  bool operator==(const Key &o) const {
    return q[0] == o.q[0] && q[1] == o.q[1] && q[2] == o.q[2];
  }
};
struct KeyHash {
  size_t operator()(const Key &k) const {
    uint64_t h = 1469598103934665603ULL;
    for (int d = 0; d < 3; d++) {
      h ^= (uint64_t)k.q[d] + 0x9e3779b97f4a7c15ULL + (h << 6) + (h >> 2);
    }
    return (size_t)h;
  }
};

double wrap1(double v, double period) {
  if (period <= 0) return v;
  double r = std::fmod(v, period);
  if (r < 0) r += period;
  if (std::fabs(r - period) < 1e-9 * period) r = 0.;
  return r;
}

}  // namespace

namespace nmg {

// D[i*n+j] = l_j'(x_i) of the Lagrange polynomials through x (Lagrange_DT,
// src/main/basis/Lagrange.c:126-147, with the weights of Lagrange.c:15-27)
static void lagrange_D(int n, const double *x, double *D) {
  std::vector<double> wi(n);
  for (int i = 0; i < n; i++) {
    double denom = 1.;
    for (int m2 = 0; m2 < n; m2++)
      if (m2 != i) denom *= (x[i] - x[m2]);
    wi[i] = 1. / denom;
  }
  for (int i = 0; i < n; i++) {
    double Dii = 0;
    for (int j = 0; j < n; j++)
      if (i != j) {
        double Dij = (wi[j] / wi[i]) / (x[i] - x[j]);
        Dii -= Dij;
        D[i * n + j] = Dij;
      }
    D[i * n + i] = Dii;
  }
}

void lgl_basis(int n, double *x, double *w, double *D) {
  const double PI = 3.14159265358979323846264338327950;
  int N = n - 1;
  double P, dP, Q, dQ, y, dy;
  if (N == 0) {
    x[0] = 0.; w[0] = 2.;
  } else {
    x[0] = -1.; x[N] = 1.;
    w[0] = 2.0 / (N * (N + 1.0)); w[N] = w[0];
    for (int j = 1; j <= N / 2; j++) {
      if (j == N / 2.0) {
        y = 0.;
      } else {
        y = -cos(PI * (j + 0.25) / N - 3 / (8 * N * PI * (j + 0.25)));
        for (int i = 0; i < 100; i++) {
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
  lagrange_D(n, x, D);
}

void uniform_basis(int n, double *x, double *w, double *D) {
  const int N = n - 1;
  if (N == 0) {
    x[0] = 0.; w[0] = 2.;
  } else {
    x[0] = -1.; x[N] = 1.;
    const double h = 2. / N;
    for (int j = 1; j <= N / 2; j++) {
      const double y = (j == N / 2.0) ? 0. : -1. + j * h;
      x[N - j] = -y;
      x[j] = +y;
    }
    w[N] = w[0] = 1. / N;
    for (int j = 1; j < N; j++) w[j] = 2. / N;
  }
  lagrange_D(n, x, D);
}

bool element_geometry(const nmg_mesh &m, int64_t e, bool uniform, double *xyz, double *dXdx) {
  const int n = m.n, np = n * n * n;
  const double *bb = &m.bbox[e * 6];
  const double *px = uniform ? m.xu.data() : m.x.data();
  const Patch *pat = nullptr;
  if (!m.patches.empty()) pat = &m.patches[m.pat[e]];
  else if (m.curvi[e]) return false;  // map of a described curvilinear element unknown
  for (int k = 0; k < n; k++)
    for (int j = 0; j < n; j++)
      for (int i = 0; i < n; i++) {
        const int ijk = i + n * (j + n * k);
        double Xb[3] = {px[i], px[j], px[k]}, X[3], x[3], J[3][3];
        for (int d = 0; d < 3; d++)
          X[d] = 0.5 * ((bb[2 * d + 1] - bb[2 * d]) * Xb[d] + (bb[2 * d + 1] + bb[2 * d]));
        if (pat && pat->cubed) {
          cubsph_x_dXdx(*pat, X, x, J);
        } else {
          for (int d = 0; d < 3; d++) {
            x[d] = X[d];
            for (int c = 0; c < 3; c++) J[d][c] = (d == c) ? 1. : 0.;
          }
        }
        for (int d = 0; d < 3; d++) xyz[d * np + ijk] = x[d];
        for (int a = 0; a < 3; a++)
          for (int c = 0; c < 3; c++) dXdx[(a * 3 + c) * np + ijk] = J[a][c];
      }
  return true;
}

// midpoint positions set_nodemidpoint_XbYbZb (src/main/coordinates/
// get_coords.c:1703-1740) and the map as at the grid points
// (coordinates.c:283-375)
bool element_midpoint_dXdx(const nmg_mesh &m, int64_t e, double *dXdxm) {
  const int n = m.n, np = n * n * n;
  const double *bb = &m.bbox[e * 6];
  const double *px = m.xu.data();
  const Patch *pat = nullptr;
  if (!m.patches.empty()) pat = &m.patches[m.pat[e]];
  else if (m.curvi[e]) return false;
  for (int q = 0; q < 3 * 9 * np; q++) dXdxm[q] = 0.;
  for (int d = 0; d < 3; d++)
    for (int k = 0; k < n; k++)
      for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++) {
          const int id[3] = {i, j, k};
          if (id[d] >= n - 1) continue;
          const int ijk = i + n * (j + n * k);
          double Xb[3] = {px[i], px[j], px[k]}, X[3], x[3], J[3][3];
          Xb[d] = 0.5 * (px[id[d]] + px[id[d] + 1]);
          for (int c = 0; c < 3; c++)
            X[c] = 0.5 * ((bb[2 * c + 1] - bb[2 * c]) * Xb[c] + (bb[2 * c + 1] + bb[2 * c]));
          if (pat && pat->cubed) {
            cubsph_x_dXdx(*pat, X, x, J);
          } else {
            for (int a = 0; a < 3; a++)
              for (int c = 0; c < 3; c++) J[a][c] = (a == c) ? 1. : 0.;
          }
          for (int a = 0; a < 3; a++)
            for (int c = 0; c < 3; c++) dXdxm[((d * 9) + a * 3 + c) * np + ijk] = J[a][c];
        }
  return true;
}

std::string pack_faces(nmg_mesh &m, const int64_t *nbnode, const double period[3]) {
  const int n = m.n, np = n * n * n, nn = n * n;
  const int64_t E = m.nelem;
  m.nb.assign(E * 6, -1);
  m.code.assign(E * 6, 0);
  double per[3] = {0, 0, 0};
  if (period)
    for (int d = 0; d < 3; d++) per[d] = period[d];
  // characteristic length for the tolerance
  double lmax = 0;
  for (int64_t i = 0; i < E * 3 * np; i++) lmax = std::max(lmax, std::fabs(m.xyz[i]));
  const double tol = 1e-9 * std::max(1.0, lmax);
  const double cell = 1e3 * tol;

  auto pos = [&](int64_t e, int ijk, double q[3]) {
    for (int d = 0; d < 3; d++) q[d] = wrap1(m.xyz[(e * 3 + d) * np + ijk], per[d]);
  };
  auto dist2 = [&](const double *a, const double *b) {
    double s = 0;
    for (int d = 0; d < 3; d++) {
      double v = std::fabs(a[d] - b[d]);
      if (per[d] > 0) v = std::min(v, per[d] - v);
      s += v * v;
    }
    return s;
  };
  // face centre = average of the 4 corner nodes (an element face never
  // straddles a period, so average first and wrap the centre)
  auto centre = [&](int64_t e, int f, double c[3]) {
    int corner[4][2] = {{0, 0}, {n - 1, 0}, {0, n - 1}, {n - 1, n - 1}};
    for (int d = 0; d < 3; d++) {
      double s = 0;
      for (int t = 0; t < 4; t++)
        s += m.xyz[(e * 3 + d) * np + face_node(n, f, corner[t][0], corner[t][1])];
      c[d] = wrap1(0.25 * s, per[d]);
    }
  };

  if (nbnode) {
    // explicit node table: derive neighbour element, face and orientation
    for (int64_t e = 0; e < E; e++)
      for (int f = 0; f < 6; f++) {
        const int64_t *t = nbnode + (e * 6 + f) * nn;
        if (t[0] < 0) {
          for (int q = 1; q < nn; q++)
            if (t[q] >= 0) return "face with partial neighbour table";
          continue;
        }
        int64_t e2 = t[0] / np;
        int f2 = -1;
        for (int g = 0; g < 6 && f2 < 0; g++) {
          int ok = 1;
          for (int q = 0; q < nn && ok; q++) {
            int idx = (int)(t[q] - e2 * np);
            int ii = idx % n, jj = (idx / n) % n, kk = idx / nn;
            int c[3] = {ii, jj, kk};
            if (t[q] / np != e2 || c[g >> 1] != (g & 1) * (n - 1)) ok = 0;
          }
          if (ok) f2 = g;
        }
        if (f2 < 0) return "neighbour nodes do not lie on one face";
        int found = -1;
        for (int o = 0; o < 8 && found < 0; o++) {
          int ok = 1;
          for (int b = 0; b < n && ok; b++)
            for (int a = 0; a < n && ok; a++) {
              int a2, b2;
              orient_map(n, o, a, b, &a2, &b2);
              if (t[a + n * b] != e2 * np + face_node(n, f2, a2, b2)) ok = 0;
            }
          if (ok) found = o;
        }
        if (found < 0) return "face node map is not a dihedral permutation";
        m.nb[e * 6 + f] = (int32_t)e2;
        m.code[e * 6 + f] = f2 | (found << 3);
      }
    return "";
  }

  // spatial hash of face centres
  std::unordered_map<Key, std::vector<int64_t>, KeyHash> h;
  h.reserve((size_t)E * 6);
  auto kcell = [&](const double c[3], const int off[3]) {
    Key k;
    for (int d = 0; d < 3; d++) k.q[d] = (int64_t)std::floor(c[d] / cell) + off[d];
    return k;
  };
  std::vector<double> cen(E * 6 * 3);
  for (int64_t e = 0; e < E; e++)
    for (int f = 0; f < 6; f++) {
      double *c = &cen[(e * 6 + f) * 3];
      centre(e, f, c);
      int z[3] = {0, 0, 0};
      h[kcell(c, z)].push_back(e * 6 + f);
    }
  for (int64_t e = 0; e < E; e++)
    for (int f = 0; f < 6; f++) {
      const double *c = &cen[(e * 6 + f) * 3];
      int64_t match = -1;
      int nmatch = 0;
      for (int dz = -1; dz <= 1; dz++)
        for (int dy = -1; dy <= 1; dy++)
          for (int dx = -1; dx <= 1; dx++) {
            int off[3] = {dx, dy, dz};
            Key k = kcell(c, off);
            if (per[0] > 0 || per[1] > 0 || per[2] > 0) {
              // cells wrap around with the period
              for (int d = 0; d < 3; d++)
                if (per[d] > 0) {
                  int64_t ncell = (int64_t)std::floor(per[d] / cell) + 1;
                  k.q[d] = ((k.q[d] % ncell) + ncell) % ncell;
                }
            }
            auto it = h.find(k);
            if (it == h.end()) continue;
            for (int64_t g : it->second) {
              if (g == e * 6 + f) continue;  // (a periodic element may be its own neighbour)
              if (dist2(c, &cen[g * 3]) < tol * tol) {
                if (g != match) nmatch++;
                if (nmatch > 1)
                  return "faces " + std::to_string(match) + " and " + std::to_string(g) +
                         " both match face " + std::to_string(f) + " of element " +
                         std::to_string(e) + " (non-conforming mesh)";
                match = g;
              }
            }
          }
      if (nmatch == 0) continue;  // outer face
      if (nmatch > 1)
        return "more than one face matches face " + std::to_string(f) + " of element " +
               std::to_string(e) + " (non-conforming mesh)";
      int64_t e2 = match / 6;
      int f2 = (int)(match % 6);
      // orientation: every face node must coincide with the oriented image;
      // between a DG and a finite-volume element (different points) only
      // the corners do
      const bool mixed = !m.fv.empty() && (m.fv[e] != 0) != (m.fv[e2] != 0);
      int found = -1;
      for (int o = 0; o < 8 && found < 0; o++) {
        int ok = 1;
        for (int b = 0; b < n && ok; b++)
          for (int a = 0; a < n && ok; a++) {
            if (mixed && !((a == 0 || a == n - 1) && (b == 0 || b == n - 1))) continue;
            int a2, b2;
            orient_map(n, o, a, b, &a2, &b2);
            double p1[3], p2[3];
            pos(e, face_node(n, f, a, b), p1);
            pos(e2, face_node(n, f2, a2, b2), p2);
            if (dist2(p1, p2) > tol * tol) ok = 0;
          }
        if (ok) found = o;
      }
      if (found < 0) return "face nodes of neighbours do not coincide (non-conforming)";
      m.nb[e * 6 + f] = (int32_t)e2;
      m.code[e * 6 + f] = f2 | (found << 3) | (mixed ? NMG_CODE_MIXED : 0);
    }
  if (m.level.empty()) return "";

  // Non-conforming faces (elements of different levels: patch-wise,
  // amr_hrefine_p, or nested spheres): a face without a conforming
  // neighbour that lies on its parent's face is matched against the coarser
  // elements' faces by the parent face's corners, which the elements at
  // those corners carry (the siblings, or their descendants where the
  // siblings are refined further).  The neighbour relation set_ajsurf_vl
  // (src/main/amr/surface.c:799-1360) works with: each face node takes the
  // average of the neighbour faces that contain it, each interpolated at the
  // node's position (basis_interp2d_toIpoints).  Only jumps of one level
  // are built: a coarse face must meet exactly four finer faces.
  struct LKey {
    int64_t v[2];
    bool operator==(const LKey &o) const { return v[0] == o.v[0] && v[1] == o.v[1]; }
  };
  struct LKeyHash {
    size_t operator()(const LKey &k) const {
      return (size_t)(k.v[0] * 0x9e3779b97f4a7c15ULL ^ (k.v[1] + 0x632be59bd9b4e019ULL));
    }
  };
  auto lkey = [](int p, int L, const int q[3]) {
    return LKey{{((int64_t)p << 8) | L, ((int64_t)q[0] << 42) | ((int64_t)q[1] << 21) | q[2]}};
  };
  std::unordered_map<LKey, int64_t, LKeyHash> where;
  int levmax = 0;
  for (int64_t e = 0; e < E; e++) {
    where[lkey(m.pat[e], m.level[e], &m.ixyz[e * 3])] = e;
    levmax = std::max(levmax, (int)m.level[e]);
  }
  // corners (and their centre) of face f of e's ancestor `up` levels up;
  // false if the patch is not tiled there
  auto ancestor_face = [&](int64_t e, int f, int up, double corner[4][3], double pc[3]) {
    const int d = f >> 1, s = f & 1, d1 = d == 0 ? 1 : 0, d2 = d == 2 ? 1 : 2;
    for (int dd = 0; dd < 3; dd++) pc[dd] = 0.;
    for (int t = 0; t < 4; t++) {
      int bits[3], q[3];
      bits[d] = s;
      bits[d1] = t & 1;
      bits[d2] = t >> 1;
      int lv = m.level[e] - up;
      for (int dd = 0; dd < 3; dd++) q[dd] = m.ixyz[e * 3 + dd] >> up;
      auto it = where.find(lkey(m.pat[e], lv, q));
      while (it == where.end() && lv < levmax) {
        for (int dd = 0; dd < 3; dd++) q[dd] = 2 * q[dd] + bits[dd];
        it = where.find(lkey(m.pat[e], ++lv, q));
      }
      if (it == where.end()) return false;
      const int node = face_node(n, f, (t & 1) * (n - 1), (t >> 1) * (n - 1));
      pos(it->second, node, corner[t]);
      for (int dd = 0; dd < 3; dd++) pc[dd] += m.xyz[(it->second * 3 + dd) * np + node];
    }
    for (int dd = 0; dd < 3; dd++) pc[dd] = wrap1(0.25 * pc[dd], per[dd]);
    return true;
  };
  // an outer face of an element of level Lc whose centre is pc
  auto find_outer = [&](const double pc[3], int Lc) {
    for (int dz = -1; dz <= 1; dz++)
      for (int dy = -1; dy <= 1; dy++)
        for (int dx = -1; dx <= 1; dx++) {
          int off[3] = {dx, dy, dz};
          auto it = h.find(kcell(pc, off));
          if (it == h.end()) continue;
          for (int64_t g : it->second)
            if (m.nb[g] < 0 && m.level[g / 6] == Lc && dist2(pc, &cen[g * 3]) < tol * tol)
              return g;
        }
    return (int64_t)-1;
  };
  struct HPair { int64_t fe; int ff; int64_t ce; int cf; int A, B, o; };
  std::vector<HPair> pairs;
  for (int64_t e = 0; e < E; e++)
    for (int f = 0; f < 6; f++) {
      const int L = m.level[e];
      if (m.nb[e * 6 + f] >= 0 || L < 1) continue;
      const int d = f >> 1, s = f & 1, d1 = d == 0 ? 1 : 0, d2 = d == 2 ? 1 : 2;
      const int *q = &m.ixyz[e * 3];
      if ((q[d] & 1) != s) continue;  // not on the parent's face f
      double corner[4][3], pc[3];
      if (!ancestor_face(e, f, 1, corner, pc)) return "element levels do not tile the patch";
      const int64_t match = find_outer(pc, L - 1);
      if (match < 0) {
        // no coarser neighbour one level up: a face two or more levels up
        // that meets an element is a level jump this mesh does not build
        for (int up = 2; up <= L && ((q[d] >> (up - 1)) & 1) == s; up++) {
          if (!ancestor_face(e, f, up, corner, pc)) return "element levels do not tile the patch";
          if (find_outer(pc, L - up) >= 0)
            return "element " + std::to_string(e) + " face " + std::to_string(f) +
                   ": a level jump of more than one across a face is not supported";
        }
        continue;  // outer face
      }
      const int64_t e2 = match / 6;
      const int f2 = (int)(match % 6);
      int found = -1;
      for (int o = 0; o < 8 && found < 0; o++) {
        int ok = 1;
        for (int t = 0; t < 4 && ok; t++) {
          int a2, b2;
          orient_map(n, o, (t & 1) * (n - 1), (t >> 1) * (n - 1), &a2, &b2);
          double p2[3];
          pos(e2, face_node(n, f2, a2, b2), p2);
          if (dist2(corner[t], p2) > tol * tol) ok = 0;
        }
        if (ok) found = o;
      }
      if (found < 0) return "non-conforming face corners do not coincide";
      pairs.push_back({e, f, e2, f2, q[d1] & 1, q[d2] & 1, found});
    }
  if (pairs.empty()) return "";

  const double tq = 1e-10;  // a node on the line between two fine faces belongs to both
  const std::vector<double> &x = m.x;
  auto add_face = [&](int64_t e, int f) {
    m.hface.push_back((int32_t)e);
    m.hface.push_back(f);
  };
  auto add_src = [&](int64_t e, int f, double u, double v) {
    m.hsrc.push_back((int32_t)e);
    m.hsrc.push_back(f);
    m.hpos.push_back(u);
    m.hpos.push_back(v);
  };
  m.hoff.assign(1, 0);
  // fine faces: one contribution per node, the coarse face at the node's
  // position in the parent face mapped by the orientation
  for (const HPair &P : pairs) {
    add_face(P.fe, P.ff);
    const int sw = P.o & 1, fa = (P.o >> 1) & 1, fb = (P.o >> 2) & 1;
    for (int b = 0; b < n; b++)
      for (int a = 0; a < n; a++) {
        const double pa = (x[a] + (2 * P.A - 1)) * 0.5, pb = (x[b] + (2 * P.B - 1)) * 0.5;
        double u = sw ? pb : pa, v = sw ? pa : pb;
        if (fa) u = -u;
        if (fb) v = -v;
        add_src(P.ce, P.cf, u, v);
        m.hoff.push_back((int32_t)(m.hsrc.size() / 2));
      }
    m.nb[P.fe * 6 + P.ff] = (int32_t)P.ce;
    m.code[P.fe * 6 + P.ff] = P.cf | (P.o << 3) | NMG_CODE_HANG;
  }
  // coarse faces: each node averages the fine faces that contain it
  std::vector<size_t> order(pairs.size());
  for (size_t i = 0; i < order.size(); i++) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](size_t i, size_t j) {
    if (pairs[i].ce != pairs[j].ce) return pairs[i].ce < pairs[j].ce;
    if (pairs[i].cf != pairs[j].cf) return pairs[i].cf < pairs[j].cf;
    return pairs[i].A + 2 * pairs[i].B < pairs[j].A + 2 * pairs[j].B;
  });
  for (size_t i = 0; i < order.size(); i += 4) {
    const HPair &P0 = pairs[order[i]];
    if (i + 3 >= order.size() || pairs[order[i + 3]].ce != P0.ce || pairs[order[i + 3]].cf != P0.cf)
      return "coarse face of element " + std::to_string(P0.ce) +
             " does not have four finer neighbours";
    add_face(P0.ce, P0.cf);
    const int sw = P0.o & 1, fa = (P0.o >> 1) & 1, fb = (P0.o >> 2) & 1;
    for (int b2 = 0; b2 < n; b2++)
      for (int a2 = 0; a2 < n; a2++) {
        const double u = fa ? -x[a2] : x[a2], v = fb ? -x[b2] : x[b2];
        const double pa = sw ? v : u, pb = sw ? u : v;
        for (int t = 0; t < 4; t++) {
          const HPair &P = pairs[order[i + t]];
          const bool ina = P.A ? pa >= -tq : pa <= tq, inb = P.B ? pb >= -tq : pb <= tq;
          if (ina && inb) add_src(P.fe, P.ff, 2 * pa - (2 * P.A - 1), 2 * pb - (2 * P.B - 1));
        }
        m.hoff.push_back((int32_t)(m.hsrc.size() / 2));
      }
    m.nb[P0.ce * 6 + P0.cf] = (int32_t)P0.fe;
    m.code[P0.ce * 6 + P0.cf] = P0.ff | NMG_CODE_HANG;
  }
  return "";
}

}  // namespace nmg

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

const char *nmg_mesh_last_error(void) { return g_mesh_err.c_str(); }

int nmg_basis(int32_t n, double *x, double *w, double *D) {
  if (n < 2 || n > 32 || !x || !w || !D) return fail(NMG_EINVAL, "nmg_basis: bad argument");
  nmg::lgl_basis(n, x, w, D);
  return NMG_OK;
}

int nmg_mesh_build(const nmg_mesh_params *p, nmg_mesh **out) {
  if (!p || !out) return fail(NMG_EINVAL, "nmg_mesh_build: null argument");
  *out = nullptr;
  if (p->n < 2 || p->n > 16) return fail(NMG_EUNSUP, "nmg_mesh_build: n must be in [2,16]");
  if (p->luni < 0 || p->luni > 8) return fail(NMG_EINVAL, "nmg_mesh_build: luni must be in [0,8]");
  if (p->sphere_levels < 0 || p->sphere_levels > 8 || !(p->sphere_radius >= 0.))
    return fail(NMG_EINVAL, "nmg_mesh_build: sphere_levels must be in [0,8], sphere_radius >= 0");
  nmg_mesh *m = new (std::nothrow) nmg_mesh;
  if (!m) return fail(NMG_ENOMEM, "nmg_mesh_build: out of memory");
  try {
    m->n = p->n;
    m->x.resize(p->n); m->w.resize(p->n); m->D.resize(p->n * p->n);
    nmg::lgl_basis(p->n, m->x.data(), m->w.data(), m->D.data());
    {
      std::vector<double> wu(p->n), Du((size_t)p->n * p->n);
      m->xu.resize(p->n);
      nmg::uniform_basis(p->n, m->xu.data(), wu.data(), Du.data());
    }
    std::vector<Patch> pats;
    double period[3] = {0, 0, 0};
    if (p->mesh_type == NMG_MESH_BOX) {
      if (!(p->box_dout > 0)) { delete m; return fail(NMG_EINVAL, "box_dout must be > 0"); }
      Patch b;
      for (int d = 0; d < 3; d++) {
        b.bbox[2 * d] = p->xc[d] - p->box_dout;
        b.bbox[2 * d + 1] = p->xc[d] + p->box_dout;
        if (p->periodic) period[d] = 2 * p->box_dout;
      }
      pats.push_back(b);
    } else if (p->mesh_type == NMG_MESH_CUBEDSPHERES7) {
      if (!(p->cs_dc > 0) || !(p->cs_r0fac > sqrt(3.))) {
        delete m;
        return fail(NMG_EINVAL, "cubed spheres need cs_dc > 0 and cs_r0fac > sqrt(3)");
      }
      if (p->periodic) { delete m; return fail(NMG_EINVAL, "periodic only for the box"); }
      double dc = p->cs_dc, r0 = p->cs_r0fac * dc;
      Patch b;
      for (int d = 0; d < 3; d++) {
        b.bbox[2 * d] = p->xc[d] - dc;
        b.bbox[2 * d + 1] = p->xc[d] + dc;
      }
      pats.push_back(b);
      double Din[6], r[4];
      for (int f = 0; f < 6; f++) Din[f] = dc;
      for (int dom = 0; dom < 6; dom++) {
        Patch c;
        ab_range(dom, Din, r);
        double bb[6] = {0., 1., r[0], r[1], r[2], r[3]};
        std::memcpy(c.bbox, bb, sizeof(bb));
        c.cubed = true;
        c.dom = dom;
        for (int d = 0; d < 3; d++) c.xc[d] = p->xc[d];
        c.s0 = Din[dom];
        c.s1 = r0;
        pats.push_back(c);
      }
    } else if (p->mesh_type == NMG_MESH_CUBEDSHELL6) {
      if (!(p->shell_rin > 0) || !(p->shell_rout > p->shell_rin)) {
        delete m;
        return fail(NMG_EINVAL, "cubed shells need 0 < shell_rin < shell_rout");
      }
      if (p->periodic) { delete m; return fail(NMG_EINVAL, "periodic only for the box"); }
      double Din[6], r[4];
      for (int f = 0; f < 6; f++) Din[f] = p->shell_rin;
      for (int dom = 0; dom < 6; dom++) {
        Patch c;
        ab_range(dom, Din, r);
        double bb[6] = {0., 1., r[0], r[1], r[2], r[3]};
        std::memcpy(c.bbox, bb, sizeof(bb));
        c.cubed = true;
        c.shell = true;
        c.dom = dom;
        for (int d = 0; d < 3; d++) c.xc[d] = p->xc[d];
        c.s0 = p->shell_rin;
        c.s1 = p->shell_rout;
        pats.push_back(c);
      }
    } else {
      delete m;
      return fail(NMG_EUNSUP, "nmg_mesh_build: unknown mesh_type");
    }
    if (p->ndiv < 0 || p->ndiv > 256 ||
        (p->ndiv > 0 && (p->hrefine || p->sphere_levels > 0))) {
      delete m;
      return fail(NMG_EINVAL, "nmg_mesh_build: ndiv must be in [0,256], without refinement");
    }
    m->ndiv = p->ndiv;
    std::vector<Leaf> leaves;
    auto wanted = [&](size_t q) { return p->patch_mask == 0 || ((p->patch_mask >> q) & 1); };
    if (p->ndiv > 0) {
      for (size_t q = 0; q < pats.size(); q++)
        if (wanted(q))
          for (int k = 0; k < p->ndiv; k++)
            for (int j = 0; j < p->ndiv; j++)
              for (int i = 0; i < p->ndiv; i++) leaves.push_back(Leaf{(int)q, 0, {i, j, k}});
    } else {
      for (size_t q = 0; q < pats.size(); q++)
        if (wanted(q)) uniform_leaves((int)q, p->luni + (((p->hrefine >> q) & 1) ? 1 : 0), leaves);
    }
    if (leaves.empty()) {
      delete m;
      return fail(NMG_EINVAL, "nmg_mesh_build: patch_mask selects no patch");
    }
    if (p->sphere_levels > 0) refine_spheres(pats, p->sphere_levels, p->sphere_radius, leaves);
    fill_geometry(*m, pats, leaves, p->fv);
    bool anyfv = false;
    for (int64_t e = 0; e < m->nelem; e++) anyfv = anyfv || m->fv[e];
    if (!anyfv) m->fv.clear();
    if (m->ndiv > 0) m->level.clear();  // not an octree: conforming faces only
    std::string err = nmg::pack_faces(*m, nullptr, period);
    if (!err.empty()) { delete m; return fail(NMG_EMESH, err); }
  } catch (const std::bad_alloc &) {
    delete m;
    return fail(NMG_ENOMEM, "nmg_mesh_build: out of memory");
  }
  *out = m;
  return NMG_OK;
}

int nmg_mesh_from_desc(const nmg_mesh_desc *d, nmg_mesh **out) {
  if (!d || !out || !d->bbox || !d->curvi || !d->xyz) return fail(NMG_EINVAL, "nmg_mesh_from_desc: null argument");
  *out = nullptr;
  if (d->n < 2 || d->n > 16 || d->nelem <= 0) return fail(NMG_EUNSUP, "nmg_mesh_from_desc: bad n or nelem");
  const int n = d->n, np = n * n * n;
  const int64_t E = d->nelem;
  for (int64_t e = 0; e < E; e++)
    if (d->curvi[e] && !d->dXdx) return fail(NMG_EINVAL, "curvilinear element without dXdx");
  nmg_mesh *m = new (std::nothrow) nmg_mesh;
  if (!m) return fail(NMG_ENOMEM, "out of memory");
  try {
    m->n = n;
    m->nelem = E;
    m->x.resize(n); m->w.resize(n); m->D.resize(n * n);
    nmg::lgl_basis(n, m->x.data(), m->w.data(), m->D.data());
    {
      std::vector<double> wu(n), Du((size_t)n * n);
      m->xu.resize(n);
      nmg::uniform_basis(n, m->xu.data(), wu.data(), Du.data());
    }
    int64_t nfv = 0;
    if (d->fv)
      for (int64_t e = 0; e < E; e++) nfv += d->fv[e] ? 1 : 0;
    if (nfv > 0) {
      m->fv.assign(E, 0);
      for (int64_t e = 0; e < E; e++) m->fv[e] = d->fv[e] ? 1 : 0;
    }
    m->pat.assign(E, 0);
    if (d->pat) std::memcpy(m->pat.data(), d->pat, E * sizeof(int32_t));
    m->bbox.assign(d->bbox, d->bbox + E * 6);
    m->curvi.assign(d->curvi, d->curvi + E);
    m->xyz.assign(d->xyz, d->xyz + E * 3 * np);
    m->dXdx.assign(E * 9 * np, 0.);
    for (int64_t e = 0; e < E; e++) {
      double *M9 = &m->dXdx[e * 9 * np];
      if (m->curvi[e]) {
        std::memcpy(M9, d->dXdx + e * 9 * np, 9 * np * sizeof(double));
      } else {
        for (int a = 0; a < 3; a++)
          for (int i = 0; i < np; i++) M9[(a * 3 + a) * np + i] = 1.;
      }
      for (int q = 0; q < 3; q++)
        if (!(m->bbox[e * 6 + 2 * q + 1] > m->bbox[e * 6 + 2 * q])) {
          delete m;
          return fail(NMG_EINVAL, "element bbox must have positive extent");
        }
    }
    if (!d->nbnode) derive_levels(*m);  // non-conforming faces are found from the levels
    std::string err = nmg::pack_faces(*m, d->nbnode, d->period);
    if (!err.empty()) { delete m; return fail(NMG_EMESH, err); }
  } catch (const std::bad_alloc &) {
    delete m;
    return fail(NMG_ENOMEM, "out of memory");
  }
  *out = m;
  return NMG_OK;
}

int64_t nmg_mesh_nelem(const nmg_mesh *m) { return m ? m->nelem : -1; }
int32_t nmg_mesh_n(const nmg_mesh *m) { return m ? m->n : -1; }

int nmg_mesh_get_elements(const nmg_mesh *m, int32_t *pat, double *bbox) {
  if (!m) return fail(NMG_EINVAL, "null mesh");
  if (pat) std::memcpy(pat, m->pat.data(), m->nelem * sizeof(int32_t));
  if (bbox) std::memcpy(bbox, m->bbox.data(), m->nelem * 6 * sizeof(double));
  return NMG_OK;
}

int nmg_mesh_get_coords(const nmg_mesh *m, double *xyz) {
  if (!m || !xyz) return fail(NMG_EINVAL, "null argument");
  std::memcpy(xyz, m->xyz.data(), m->xyz.size() * sizeof(double));
  return NMG_OK;
}

int nmg_mesh_get_dXdx(const nmg_mesh *m, double *dXdx) {
  if (!m || !dXdx) return fail(NMG_EINVAL, "null argument");
  std::memcpy(dXdx, m->dXdx.data(), m->dXdx.size() * sizeof(double));
  return NMG_OK;
}

int nmg_mesh_get_faces(const nmg_mesh *m, int32_t *nb, int32_t *code) {
  if (!m) return fail(NMG_EINVAL, "null mesh");
  if (nb) std::memcpy(nb, m->nb.data(), m->nb.size() * sizeof(int32_t));
  if (code) std::memcpy(code, m->code.data(), m->code.size() * sizeof(int32_t));
  return NMG_OK;
}

int nmg_mesh_get_fv(const nmg_mesh *m, int32_t *fv) {
  if (!m || !fv) return fail(NMG_EINVAL, "null argument");
  for (int64_t e = 0; e < m->nelem; e++) fv[e] = m->fv.empty() ? 0 : m->fv[e];
  return NMG_OK;
}

int nmg_mesh_get_hanging(const nmg_mesh *m, int64_t *nface, int64_t *ncontrib, int32_t *hface,
                         int32_t *hoff, int32_t *hsrc, double *hpos) {
  if (!m || !nface || !ncontrib) return fail(NMG_EINVAL, "nmg_mesh_get_hanging: null argument");
  *nface = (int64_t)m->hface.size() / 2;
  *ncontrib = (int64_t)m->hsrc.size() / 2;
  if (hface) std::copy(m->hface.begin(), m->hface.end(), hface);
  if (hoff) std::copy(m->hoff.begin(), m->hoff.end(), hoff);
  if (hsrc) std::copy(m->hsrc.begin(), m->hsrc.end(), hsrc);
  if (hpos) std::copy(m->hpos.begin(), m->hpos.end(), hpos);
  return NMG_OK;
}

// dt = auto (update_elm_eid_dt -> adapt_node_dt_and_mesh_dt,
// src/main/amr/storage.c:1305-1365, src/main/coordinates/utilities.c:
// 972-1124,1225-1300): per element hmin = the smallest distance between a
// corner point and its axis neighbours (starting from the bbox diagonal /
// sqrt(3)), dt = dtfac hmin, or uniform_dtfac hmin when that pair lies along
// a direction of equally spaced points; the mesh dt is the minimum.
int nmg_mesh_auto_dt(const nmg_mesh *m, double dtfac, double uniform_dtfac, double *dt) {
  if (!m || !dt) return fail(NMG_EINVAL, "nmg_mesh_auto_dt: null argument");
  const int n = m->n, np = n * n * n;
  double mdt = DBL_MAX * 0.1;
  auto dist = [](const double a[3], const double b[3]) {
    double d2 = 0.;
    for (int d = 0; d < 3; d++) {
      const double dx = b[d] - a[d];
      d2 += dx * dx;
    }
    return sqrt(d2);
  };
  for (int64_t e = 0; e < m->nelem; e++) {
    const double *X = &m->xyz[(size_t)e * 3 * np];
    auto pt = [&](int i, int j, int k, double p[3]) {
      const int ijk = i + n * (j + n * k);
      for (int d = 0; d < 3; d++) p[d] = X[d * np + ijk];
    };
    // space diagonal of the bbox through the patch map (the corner points
    // of an element without a known map)
    const double *bb = &m->bbox[e * 6];
    double c0[3], c1[3];
    const Patch *pat = m->patches.empty() ? nullptr : &m->patches[m->pat[e]];
    if (pat) {
      const double X0[3] = {bb[0], bb[2], bb[4]}, X1[3] = {bb[1], bb[3], bb[5]};
      double J[3][3];
      if (pat->cubed) {
        cubsph_x_dXdx(*pat, X0, c0, J);
        cubsph_x_dXdx(*pat, X1, c1, J);
      } else {
        for (int d = 0; d < 3; d++) { c0[d] = X0[d]; c1[d] = X1[d]; }
      }
    } else {
      pt(0, 0, 0, c0);
      pt(n - 1, n - 1, n - 1, c1);
    }
    double hmin = dist(c0, c1) / sqrt(3.);
    int best0 = -1, best1 = -1;
    for (int c = 0; c < 8; c++) {
      const int i = (c & 1) * (n - 1), j = ((c >> 1) & 1) * (n - 1), k = ((c >> 2) & 1) * (n - 1);
      double p0[3];
      pt(i, j, k, p0);
      for (int kk = -1; kk <= 1; kk++)
        for (int jj = -1; jj <= 1; jj++)
          for (int ii = -1; ii <= 1; ii++) {
            const int in = i + ii, jn = j + jj, kn = k + kk;
            if (in < 0 || in >= n || jn < 0 || jn >= n || kn < 0 || kn >= n) continue;
            if (in == i && jn == j && kn == k) continue;
            if ((in != i) + (jn != j) + (kn != k) != 1) continue;
            double p1[3];
            pt(in, jn, kn, p1);
            const double dd = dist(p0, p1);
            if (dd < hmin) {
              hmin = dd;
              best0 = i + n * (j + n * k);
              best1 = in + n * (jn + n * kn);
            }
          }
    }
    const bool uni = !m->fv.empty() && m->fv[e] && best0 >= 0 && best1 >= 0;
    const double dtm = (uni ? uniform_dtfac : dtfac) * hmin;
    if (dtm < mdt) mdt = dtm;
  }
  *dt = mdt;
  return NMG_OK;
}

int nmg_mesh_get_midpoint_dXdx(const nmg_mesh *m, double *dXdxm) {
  if (!m || !dXdxm) return fail(NMG_EINVAL, "nmg_mesh_get_midpoint_dXdx: null argument");
  const size_t per = (size_t)27 * m->n * m->n * m->n;
  for (int64_t e = 0; e < m->nelem; e++)
    if (!nmg::element_midpoint_dXdx(*m, e, dXdxm + e * per))
      return fail(NMG_EUNSUP, "nmg_mesh_get_midpoint_dXdx: element map unknown");
  return NMG_OK;
}

int nmg_uniform_points(int32_t n, double *x) {
  if (n < 1 || n > 64 || !x) return fail(NMG_EINVAL, "nmg_uniform_points: bad argument");
  std::vector<double> w(n), D((size_t)n * n);
  nmg::uniform_basis(n, x, w.data(), D.data());
  return NMG_OK;
}

void nmg_mesh_free(nmg_mesh *m) { delete m; }

int nmg_mesh_concat(const nmg_mesh *const *ms, int32_t count, nmg_mesh **out) {
  if (!ms || count <= 0 || !out) return fail(NMG_EINVAL, "nmg_mesh_concat: bad argument");
  *out = nullptr;
  const int n = ms[0] ? ms[0]->n : 0;
  for (int i = 0; i < count; i++)
    if (!ms[i] || ms[i]->n != n)
      return fail(NMG_EINVAL, "nmg_mesh_concat: meshes must exist and share n");
  for (int i = 0; i < count; i++)
    if (!ms[i]->fv.empty())
      return fail(NMG_EUNSUP, "nmg_mesh_concat: finite-volume meshes are not concatenated");
  nmg_mesh *m = new (std::nothrow) nmg_mesh;
  if (!m) return fail(NMG_ENOMEM, "nmg_mesh_concat: out of memory");
  try {
    m->n = n;
    m->x = ms[0]->x;
    m->w = ms[0]->w;
    m->D = ms[0]->D;
    m->xu = ms[0]->xu;
    int64_t off = 0;
    m->hoff.assign(1, 0);
    for (int i = 0; i < count; i++) {
      const nmg_mesh &a = *ms[i];
      for (int64_t e = 0; e < a.nelem; e++) m->pat.push_back(a.pat[e]);
      m->bbox.insert(m->bbox.end(), a.bbox.begin(), a.bbox.end());
      m->curvi.insert(m->curvi.end(), a.curvi.begin(), a.curvi.end());
      m->xyz.insert(m->xyz.end(), a.xyz.begin(), a.xyz.end());
      m->dXdx.insert(m->dXdx.end(), a.dXdx.begin(), a.dXdx.end());
      for (size_t q = 0; q < a.nb.size(); q++)
        m->nb.push_back(a.nb[q] < 0 ? -1 : (int32_t)(a.nb[q] + off));
      m->code.insert(m->code.end(), a.code.begin(), a.code.end());
      // non-conforming faces keep their interpolation lists, renumbered
      for (size_t q = 0; q < a.hface.size(); q += 2) {
        m->hface.push_back((int32_t)(a.hface[q] + off));
        m->hface.push_back(a.hface[q + 1]);
      }
      const int32_t c0 = m->hoff.back();
      for (size_t q = 1; q < a.hoff.size(); q++) m->hoff.push_back(c0 + a.hoff[q]);
      for (size_t q = 0; q < a.hsrc.size(); q += 2) {
        m->hsrc.push_back((int32_t)(a.hsrc[q] + off));
        m->hsrc.push_back(a.hsrc[q + 1]);
      }
      m->hpos.insert(m->hpos.end(), a.hpos.begin(), a.hpos.end());
      off += a.nelem;
    }
    m->nelem = off;
    if (m->hface.empty()) m->hoff.clear();
  } catch (const std::bad_alloc &) {
    delete m;
    return fail(NMG_ENOMEM, "nmg_mesh_concat: out of memory");
  }
  *out = m;
  return NMG_OK;
}

}  // extern "C"
