// grhd_evolve.cu -- GRHD evolution in the Cowling approximation on a cubed
// shell: DG elements (LGL points) with LLF faces, finite-volume elements on
// nf equally spaced points (WENO-reconstructed primitives, LLF midpoint
// fluxes), con2prim with atmosphere every stage, the DG <-> finite-volume
// switch with the reference's data transfer (PARENT_2n_P_UNIFORM,
// src/main/evolve/trouble.c:162-183, src/main/basis/gridpoints.c:158-200),
// RK4 stages with the update fused into each kernel, graph-captured steps.
//
// The reference has no GRHD (its physics lives in external repositories),
// so the physics and the finite-volume form are parity unpinned; they are
// restated step by step in the oracle (oracle/nmo_grhd.c), which the tests
// hold this file to.  From the reference come the DG strong form with the
// chain rule (src/main/coordinates/derivs.c:102-181,756-815), the LLF flux
// (src/main/dg/numflux1d.c:85-112), the lift (src/main/dg/dg.c:30-151), the
// WENO reconstructions (src/main/dg/rec1d.c, weno.cuh), the root finder
// newton1d_brak (grhd.cuh) and RK4 (src/main/evolve/RungeKutta.c:19-82).
//
// Device layout: DG states [E][5][n^3] for every element (rows of
// finite-volume elements unused), finite-volume states [slot][5][nf^3] for
// the elements in finite-volume mode (slots in ascending element order),
// per DG node the background (alpha, psi, d alpha, d psi) [E][8][n^3], per
// finite-volume slot the geometry of its points and midpoints
// [slot][kGeo][nf^3] computed on the device from the shell map, and per
// DG / finite-volume face a trace slot of primitives [5][max(n,nf)^2].
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/nmg.h"
#include "mesh.h"
#include "tc_device.cuh"

namespace {

#include "grhd.cuh"
// the finite-volume midpoint reconstructions with one division per
// reconstruction (the nonlinear weights normalised together)
#define NMG_FV_FAST
#include "weno.cuh"
#undef NMG_FV_FAST

constexpr int NF = 5;
constexpr int kMaxN = 10;   // DG points per direction
constexpr int kMaxNF = 16;  // finite-volume points per direction
// per finite-volume point: det(dXb/dx), background (8), per direction the
// unit normal and J |grad Xb^a| (4 x 3), per direction at the midpoint right
// of the point: unit normal, J |grad Xb^a|, alpha, psi (6 x 3)
constexpr int kGeo = 39;
constexpr int kNT = 256;
constexpr int kNTF = 512;  // finite-volume kernel: one CTA per SM, 16 warps

struct ShellMap {
  int dom[6];
  double s0[6], s1[6], xc[3];
};

// x and dXb/dx-free dX/dx of the CubedShell map (constant radii s0 < s1),
// the operation order of the reference's xyz_of_lamAB_CubSph /
// dlamAB_dxyz_CubSph (src/main/coordinates/coordtrans_CubedSphere.c:37-118,
// 257-509) for dom / 2 = dir
__device__ void shell_map(const ShellMap &S, int p, const double X[3], double x[3],
                          double J[3][3]) {
  const double lam = X[0], A = X[1], B = X[2];
  const int dom = S.dom[p], dir = dom / 2;
  const int ia = dir == 1 ? 0 : 1, ib = dir == 2 ? 0 : 2;
  const double pm = 2 * (dom % 2) - 1;
  const double sq = sqrt(1.0 + A * A + B * B);
  const double a0 = pm * S.s0[p] / sq, a1 = pm * S.s1[p] / sq;
  const double rR = (a1 - a0) * lam + a0;
  x[dir] = S.xc[dir] + rR;
  x[ia] = S.xc[ia] + A * rR;
  x[ib] = S.xc[ib] + B * rR;
  double r[3];
  for (int c = 0; c < 3; c++) r[c] = (c == dir) ? rR : x[c] - S.xc[c];
  const double rc2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
  const double rR2 = r[dir] * r[dir];
  for (int c = 0; c < 3; c++) {
    const double m = (c == dir) ? (1.0 / rR - rR / rc2) : (-r[c] / rc2);
    const double da0 = a0 * m, da1 = a1 * m;
    J[0][c] = ((c == dir ? 1.0 : 0.0) - da0 - (da1 - da0) * lam) / (a1 - a0);
    J[1][c] = 0.;
    J[2][c] = 0.;
  }
  J[1][dir] = -r[ia] / rR2;
  J[1][ia] = 1.0 / rR;
  J[2][dir] = -r[ib] / rR2;
  J[2][ib] = J[1][ia];
}

__host__ __device__ inline void background(double mass, const double x[3], double bg[8]) {
  const double r2 = x[0] * x[0] + x[1] * x[1] + x[2] * x[2];
  const double r = sqrt(r2);
  const double a = 0.5 * mass / r;
  const double ps = 1. + a;
  const double c1 = 2. * a / (r2 * (ps * ps)), c2 = -a / r2;
  bg[0] = (1. - a) / (1. + a);
  bg[1] = ps;
  for (int i = 0; i < 3; i++) {
    bg[2 + i] = c1 * x[i];
    bg[5 + i] = c2 * x[i];
  }
}

__device__ __forceinline__ void flux_n(const double *U, const double *P, const double n[3],
                                       double al, double ps, double F[NF]) {
  const double ps2 = ps * ps, ps6 = ps2 * ps2 * ps2;
  const double vn = P[1] * n[0] + P[2] * n[1] + P[3] * n[2];
  const double avn = al * vn, ap = al * ps6 * P[4];
  F[0] = avn * U[0];
  F[1] = avn * U[1] + ap * n[0];
  F[2] = avn * U[2] + ap * n[1];
  F[3] = avn * U[3] + ap * n[2];
  F[4] = avn * U[4] + ap * vn;
}

__device__ __forceinline__ double speed_n(const nmg_grhd_params &g, const double *P,
                                          const double n[3], double al, double ps) {
  const double ps2 = ps * ps, ps4 = ps2 * ps2;
  const double rho = P[0], p = P[4];
  const double vn = P[1] * n[0] + P[2] * n[1] + P[3] * n[2];
  const double v2 = ps4 * (P[1] * P[1] + P[2] * P[2] + P[3] * P[3]);
  const double eps = p / ((g.gamma - 1.) * rho);
  const double h = 1. + eps + p / rho;
  const double cs2 = g.gamma * p / (rho * h);
  double disc = (1. - v2) * (1. / ps4 * (1. - v2 * cs2) - vn * vn * (1. - cs2));
  const double fac = al / (1. - v2 * cs2);
  if (disc < 0.) disc = 0.;
  const double lm = fac * (vn * (1. - cs2) - sqrt(cs2) * sqrt(disc));
  const double lp = fac * (vn * (1. - cs2) + sqrt(cs2) * sqrt(disc));
  return fmax(fabs(lm), fabs(lp));
}

__device__ __forceinline__ void sources(const nmg_grhd_params &g, const double *P,
                                        const double *bg, int bstride, double S[NF]) {
  const double al = bg[0], ps = bg[bstride];
  const double ps2 = ps * ps, ps4 = ps2 * ps2, ps6 = ps4 * ps2;
  const double rho = P[0], p = P[4];
  const double v2 = ps4 * (P[1] * P[1] + P[2] * P[2] + P[3] * P[3]);
  const double W2 = 1. / (1. - v2);
  const double eps = p / ((g.gamma - 1.) * rho);
  const double h = 1. + eps + p / rho;
  const double rhW2 = rho * h * W2;
  const double E = rhW2 - p;
  double vda = 0.;
  S[0] = 0.;
  for (int j = 0; j < 3; j++) {
    const double da = bg[(2 + j) * bstride], dp = bg[(5 + j) * bstride];
    S[1 + j] = ps6 * (2. * al * (dp / ps) * (rhW2 * v2 + 3. * p) - E * da);
    vda += P[1 + j] * da;
  }
  S[4] = -ps6 * rhW2 * vda;
}

__device__ __forceinline__ bool physical(const double P[NF], double ps) {
  const double ps2 = ps * ps, ps4 = ps2 * ps2;
  const double v2 = ps4 * (P[1] * P[1] + P[2] * P[2] + P[3] * P[3]);
  return P[0] > 0. && P[4] > 0. && v2 < 1. && isfinite(P[0] + P[1] + P[2] + P[3] + P[4]);
}

// conserved state U, flux F along the unit normal n and the largest
// |characteristic speed| of the primitives P (as p2c_point, flux_n and
// speed_n compute them, sharing 1/rho, W and c_s)
__device__ __forceinline__ double side_state(const nmg_grhd_params &g, const double *P,
                                             const double n[3], double al, double ps4,
                                             double ps6, double ips4, double U[NF],
                                             double F[NF]) {
  const double rho = P[0], p = P[4];
  const double v2 = ps4 * (P[1] * P[1] + P[2] * P[2] + P[3] * P[3]);
  const double pr = p / rho;
  const double eps = pr / (g.gamma - 1.);
  const double h = 1. + eps + pr;
  const double W2 = 1. / (1. - v2), W = sqrt(W2);
  const double rhW2 = rho * h * W2;
  U[0] = ps6 * rho * W;
  U[1] = ps6 * rhW2 * ps4 * P[1];
  U[2] = ps6 * rhW2 * ps4 * P[2];
  U[3] = ps6 * rhW2 * ps4 * P[3];
  U[4] = ps6 * (rhW2 - p) - U[0];
  const double vn = P[1] * n[0] + P[2] * n[1] + P[3] * n[2];
  const double avn = al * vn, ap = al * ps6 * p;
  F[0] = avn * U[0];
  F[1] = avn * U[1] + ap * n[0];
  F[2] = avn * U[2] + ap * n[1];
  F[3] = avn * U[3] + ap * n[2];
  F[4] = avn * U[4] + ap * vn;
  const double cs2 = g.gamma * pr / h;
  double disc = (1. - v2) * (ips4 * (1. - v2 * cs2) - vn * vn * (1. - cs2));
  if (disc < 0.) disc = 0.;
  const double fac = al / (1. - v2 * cs2);
  const double lm = fac * (vn * (1. - cs2) - sqrt(cs2) * sqrt(disc));
  const double lp = fac * (vn * (1. - cs2) + sqrt(cs2) * sqrt(disc));
  return fmax(fabs(lm), fabs(lp));
}

__device__ __forceinline__ void llf(const nmg_grhd_params &g, const double *Ui, const double *Pi,
                                    const double *Uo, const double *Po, const double n[3],
                                    double al, double ps, double Fs[NF], double Fi[NF]) {
  double Fo[NF];
  flux_n(Ui, Pi, n, al, ps, Fi);
  flux_n(Uo, Po, n, al, ps, Fo);
  const double a = fmax(speed_n(g, Pi, n, al, ps), speed_n(g, Po, n, al, ps));
  for (int f = 0; f < NF; f++) Fs[f] = 0.5 * (Fi[f] + Fo[f] - a * (Uo[f] - Ui[f]));
}

__host__ __device__ __forceinline__ int face_ijk(int n, int f, int a, int b) {
  const int d = f >> 1, q = (f & 1) * (n - 1);
  return d == 0 ? q + n * (a + n * b) : d == 1 ? a + n * (q + n * b) : a + n * (b + n * q);
}

__device__ __forceinline__ void orient_ab(int n, int o, int a, int b, int *a2, int *b2) {
  int aa = (o & 1) ? b : a, bb = (o & 1) ? a : b;
  if (o & 2) aa = n - 1 - aa;
  if (o & 4) bb = n - 1 - bb;
  *a2 = aa;
  *b2 = bb;
}

__device__ __forceinline__ double det3(const double M[3][3]) {
  return M[0][0] * (M[1][1] * M[2][2] - M[1][2] * M[2][1]) -
         M[0][1] * (M[1][0] * M[2][2] - M[1][2] * M[2][0]) +
         M[0][2] * (M[1][0] * M[2][1] - M[1][1] * M[2][0]);
}

// parameters of every stage kernel
struct GrP {
  int n, np, nn, nf, npf, nnf, tpts;
  int ndg, nfv;
  nmg_grhd_params g;
  double mass;
  int rec;
  const int *dglist;     // [ndg] DG elements
  const int *slotelem;   // [nfv] element of each finite-volume slot
  const int *fvslot;     // [E] slot, -1: DG
  const int *nb, *code;  // [E][6]
  const int *tslot;      // [E][6] trace slot of a DG / FV face, -1: none
  const int *tface;      // [ntr][2] element, face of each trace slot
  int ntr;
  const double *dXdx;    // [E][9][np]
  const double *bgd;     // [E][8][np]
  const double *bbox;    // [E][6]
  const double *basis;   // D [n*n], wl [n], xl [n], xu [nf], barycentric weights [n]
  const double *geo;     // [slot][kGeo][npf]
  double *trace;         // [ntr][5][tpts]
  // stage buffers
  const double *win_d, *win_f, *u0_d, *u0_f;
  double *acc_d, *acc_f, *wout_d, *wout_f;
  const double *prim_d, *prim_f;
  double *rbuf;          // [slot][5][npf] finite-volume r
  int mode;              // 0: r into acc; 1..4: RK4 stage s
  double cacc, cw;
  int pencils;           // finite-volume pencils per chunk
};

__device__ __forceinline__ void epilogue(const GrP &P, double r, size_t idx, const double *u0,
                                         double *acc, double *wout) {
  if (P.mode == 0) {
    acc[idx] = r;
  } else if (P.mode == 1) {
    const double u = u0[idx];
    acc[idx] = u + P.cacc * r;
    wout[idx] = u + P.cw * r;
  } else if (P.mode <= 3) {
    acc[idx] += P.cacc * r;
    wout[idx] = u0[idx] + P.cw * r;
  } else {
    acc[idx] += P.cacc * r;
  }
}

// con2prim of the stage input on every point in use, atmosphere fixes
// written back; stats[0] += iterations, stats[1] += atmosphere points
__global__ void c2p_kernel(GrP P, double *w_d, double *w_f, double *prim_d, double *prim_f,
                           unsigned long long *stats) {
  const int64_t nd = (int64_t)P.ndg * P.np, tot = nd + (int64_t)P.nfv * P.npf;
  unsigned long long it = 0, atm = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < tot;
       i += (int64_t)gridDim.x * blockDim.x) {
    double *W, *PP, ps;
    int64_t npts, q;
    if (i < nd) {
      const int e = P.dglist[i / P.np];
      q = i % P.np;
      npts = P.np;
      W = w_d + (size_t)e * NF * P.np;
      PP = prim_d + (size_t)e * NF * P.np;
      ps = P.bgd[((size_t)e * 8 + 1) * P.np + q];
    } else {
      const int64_t j = i - nd;
      const int s = (int)(j / P.npf);
      q = j % P.npf;
      npts = P.npf;
      W = w_f + (size_t)s * NF * P.npf;
      PP = prim_f + (size_t)s * NF * P.npf;
      ps = P.geo[((size_t)s * kGeo + 2) * P.npf + q];
    }
    double U[NF], Pq[NF];
    for (int f = 0; f < NF; f++) {
      U[f] = W[f * npts + q];
      Pq[f] = PP[f * npts + q];
    }
    const int rc = c2p_point(P.g, ps, U, Pq);
    for (int f = 0; f < NF; f++) {
      W[f * npts + q] = U[f];
      PP[f * npts + q] = Pq[f];
    }
    if (rc < 0) atm++;
    else it += rc;
  }
  // one atomic per warp
  for (int o = 16; o > 0; o >>= 1) {
    it += __shfl_down_sync(0xffffffffu, it, o);
    atm += __shfl_down_sync(0xffffffffu, atm, o);
  }
  if ((threadIdx.x & 31) == 0 && (it || atm)) {
    atomicAdd(stats, it);
    atomicAdd(stats + 1, atm);
  }
}

// primitives across every DG / finite-volume face at this face's points:
// piecewise linear in each in-plane direction from a finite-volume
// neighbour, Lagrange interpolation of a DG neighbour's face plane
__global__ void trace_kernel(GrP P, const double *prim_d, const double *prim_f) {
  const int64_t tot = (int64_t)P.ntr * P.tpts;
  const double *D = P.basis;
  const double *xl = D + P.n * P.n + P.n, *xu = xl + P.n;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < tot;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int t = (int)(i / P.tpts), ab = (int)(i % P.tpts);
    const int e = P.tface[2 * t], f = P.tface[2 * t + 1];
    const bool fv = P.fvslot[e] >= 0;
    const int mine = fv ? P.nf : P.n;
    const int a = ab % mine, b = ab / mine;
    if (b >= mine) continue;
    const int e2 = P.nb[6 * e + f], f2 = P.code[6 * e + f] & 7, o = (P.code[6 * e + f] >> 3) & 7;
    const double *xs = fv ? xu : xl;
    double s = (o & 1) ? xs[b] : xs[a], u = (o & 1) ? xs[a] : xs[b];
    if (o & 2) s = -s;
    if (o & 4) u = -u;
    double *out = P.trace + (size_t)t * NF * P.tpts;
    if (fv) {
      // DG neighbour: Lagrange basis of the LGL points at (s, u), in the
      // barycentric form (weights bw = 1 / prod_{j != k} (x_k - x_j))
      const double *bw = xu + P.nf;
      double la[kMaxN], lb[kMaxN];
      for (int k = 0; k < P.n; k++) {
        double va = bw[k], vb = bw[k];
        for (int j = 0; j < P.n; j++)
          if (j != k) {
            va *= s - xl[j];
            vb *= u - xl[j];
          }
        la[k] = va;
        lb[k] = vb;
      }
      for (int q = 0; q < NF; q++) {
        const double *src = prim_d + ((size_t)e2 * NF + q) * P.np;
        double v = 0.;
        for (int j = 0; j < P.n; j++) {
          double vj = 0.;
          for (int k = 0; k < P.n; k++) vj += la[k] * src[face_ijk(P.n, f2, k, j)];
          v += lb[j] * vj;
        }
        out[q * P.tpts + a + mine * b] = v;
      }
    } else {
      // finite-volume neighbour: piecewise linear
      const int nf = P.nf;
      int ka = (int)floor((s + 1.) * 0.5 * (nf - 1)), kb = (int)floor((u + 1.) * 0.5 * (nf - 1));
      ka = min(max(ka, 0), nf - 2);
      kb = min(max(kb, 0), nf - 2);
      const double wa1 = (s - xu[ka]) / (xu[ka + 1] - xu[ka]), wa0 = 1. - wa1;
      const double wb1 = (u - xu[kb]) / (xu[kb + 1] - xu[kb]), wb0 = 1. - wb1;
      const int s2 = P.fvslot[e2];
      for (int q = 0; q < NF; q++) {
        const double *src = prim_f + ((size_t)s2 * NF + q) * P.npf;
        const double v0 = wa0 * src[face_ijk(nf, f2, ka, kb)] + wa1 * src[face_ijk(nf, f2, ka + 1, kb)];
        const double v1 =
            wa0 * src[face_ijk(nf, f2, ka, kb + 1)] + wa1 * src[face_ijk(nf, f2, ka + 1, kb + 1)];
        out[q * P.tpts + a + mine * b] = wb0 * v0 + wb1 * v1;
      }
    }
  }
}

// exterior state of face node (a, b) of face f of element e; false: outer
// face.  Same-type neighbours are read at the coincident point, the others
// from the trace slot (primitives; U from prim2con at psi ps).
__device__ bool exterior(const GrP &P, int e, int f, int a, int b, double ps, double Uo[NF],
                         double Po[NF]) {
  const int e2 = P.nb[6 * e + f];
  if (e2 < 0) return false;
  const bool fv = P.fvslot[e] >= 0, fv2 = P.fvslot[e2] >= 0;
  if (fv == fv2) {
    const int nn = fv ? P.nf : P.n, npts = fv ? P.npf : P.np;
    const int f2 = P.code[6 * e + f] & 7, o = (P.code[6 * e + f] >> 3) & 7;
    int a2, b2;
    orient_ab(nn, o, a, b, &a2, &b2);
    const int idx = face_ijk(nn, f2, a2, b2);
    const size_t row = fv ? (size_t)P.fvslot[e2] : (size_t)e2;
    const double *W = fv ? P.win_f : P.win_d, *PP = fv ? P.prim_f : P.prim_d;
    for (int q = 0; q < NF; q++) {
      Uo[q] = W[(row * NF + q) * npts + idx];
      Po[q] = PP[(row * NF + q) * npts + idx];
    }
    return true;
  }
  const int t = P.tslot[6 * e + f];
  const int mine = fv ? P.nf : P.n;
  const double *tr = P.trace + (size_t)t * NF * P.tpts;
  for (int q = 0; q < NF; q++) Po[q] = tr[q * P.tpts + a + mine * b];
  p2c_point(P.g, ps, Po, Uo);
  return true;
}

// DG faces (LLF with the fluid's characteristic speeds, lifted with
// |grad X^d| (2/dX^d) / w_end), one direction at a time (its two faces are
// disjoint), then the stage update of the element's r (shared by the DG
// kernels)
__device__ __forceinline__ void dg_faces_epilogue(const GrP &P, int e, const double *sP,
                                                  double *sR, const double *Ug,
                                                  const double *M, const double *bg,
                                                  const double *s, double w_end) {
  const int n = P.n, np = P.np, nn = P.nn;
  // faces, one direction at a time (its two faces are disjoint)
  for (int d = 0; d < 3; d++) {
    for (int task = threadIdx.x; task < 2 * nn; task += blockDim.x) {
      const int side = task / nn, ab = task - side * nn, a = ab % n, b = ab / n;
      const int f = 2 * d + side, q2 = face_ijk(n, f, a, b);
      const double al = bg[q2], ps = bg[np + q2];
      double Ui[NF], Pi[NF], Uo[NF], Po[NF], Fs[NF], Fi[NF], nr[3];
      if (!exterior(P, e, f, a, b, ps, Uo, Po)) continue;
      for (int q = 0; q < NF; q++) {
        Ui[q] = Ug[q * np + q2];
        Pi[q] = sP[q * np + q2];
      }
      const double m0 = M[(d * 3 + 0) * np + q2], m1 = M[(d * 3 + 1) * np + q2],
                   m2 = M[(d * 3 + 2) * np + q2];
      const double nm = sqrt(m0 * m0 + m1 * m1 + m2 * m2);
      const double sg = side ? 1. : -1.;
      nr[0] = sg * m0 / nm;
      nr[1] = sg * m1 / nm;
      nr[2] = sg * m2 / nm;
      const double g = nm * s[d] / w_end;
      llf(P.g, Ui, Pi, Uo, Po, nr, al, ps, Fs, Fi);
      for (int q = 0; q < NF; q++) sR[q * np + q2] -= g * (Fs[q] - Fi[q]);
    }
    __syncthreads();
  }
  for (int i = threadIdx.x; i < NF * np; i += blockDim.x)
    epilogue(P, sR[i], (size_t)e * NF * np + i, P.u0_d, P.acc_d, P.wout_d);
}

// DG elements: one CTA per element
__global__ void __launch_bounds__(kNT) dg_kernel(GrP P) {
  extern __shared__ double sm[];
  const int n = P.n, np = P.np, nn = P.nn;
  double *sF = sm, *sP = sF + 15 * np, *sR = sP + NF * np, *sD = sR + NF * np;
  const int e = P.dglist[blockIdx.x];
  const double *Pg = P.prim_d + (size_t)e * NF * np, *Ug = P.win_d + (size_t)e * NF * np;
  const double *M = P.dXdx + (size_t)e * 9 * np, *bg = P.bgd + (size_t)e * 8 * np;
  const double *bb = P.bbox + 6 * (size_t)e;
  const double s[3] = {2. / (bb[1] - bb[0]), 2. / (bb[3] - bb[2]), 2. / (bb[5] - bb[4])};
  const double w_end = P.basis[n * n];
  for (int i = threadIdx.x; i < NF * np; i += blockDim.x) sP[i] = Pg[i];
  for (int i = threadIdx.x; i < n * n; i += blockDim.x) sD[i] = P.basis[i];
  __syncthreads();
  for (int q = threadIdx.x; q < np; q += blockDim.x) {
    double Uq[NF], Pq[NF], Fq[NF], nr[3];
    for (int f = 0; f < NF; f++) {
      Uq[f] = Ug[f * np + q];
      Pq[f] = sP[f * np + q];
    }
    const double al = bg[q], ps = bg[np + q];
    for (int i = 0; i < 3; i++) {
      nr[0] = nr[1] = nr[2] = 0.;
      nr[i] = 1.;
      flux_n(Uq, Pq, nr, al, ps, Fq);
      for (int f = 0; f < NF; f++) sF[(i * NF + f) * np + q] = Fq[f];
    }
    sources(P.g, Pq, bg + q, np, Fq);
    for (int f = 0; f < NF; f++) sR[f * np + q] = Fq[f];
  }
  __syncthreads();
  // strong-form divergence with the chain rule
  for (int task = threadIdx.x; task < NF * np; task += blockDim.x) {
    const int f = task / np, q = task - f * np;
    const int ijk[3] = {q % n, (q / n) % n, q / nn};
    const int str[3] = {1, n, nn};
    double div = 0.;
    for (int i = 0; i < 3; i++) {
      const double *Fi = sF + (i * NF + f) * np;
      for (int a = 0; a < 3; a++) {
        const int base = q - ijk[a] * str[a];
        const double *Dr = sD + ijk[a] * n;
        double ds = 0.;
        for (int k = 0; k < n; k++) ds += Dr[k] * Fi[base + k * str[a]];
        div += M[(a * 3 + i) * np + q] * (s[a] * ds);
      }
    }
    sR[f * np + q] -= div;
  }
  __syncthreads();
  dg_faces_epilogue(P, e, sP, sR, Ug, M, bg, s, w_end);
}

// DG elements with the divergence's line derivatives on the tensor cores
// (n = 7, 8, 9; the exact integer digit products of stage_tc.cu): the fluxes
// F^i along x^i are formed one i at a time for the five fields, split into
// digits, and D applied along every direction a by 16-line MMA tiles (the
// line left over at odd n in FP64); the chain rule M[a][i] (2/dX^a) D_a F^i,
// the sources, the faces and the update are dg_kernel's FP64 code.
constexpr int kNTD = 160;  // five warps: the 5 fields x 3 tiles of a pass at n = 7
template <int N>
constexpr size_t dg_tc_smem() {
  return sizeof(double) * 3 * NF * N * N * N + sizeof(uint4) * NF * N * N * N;
}

template <int N>
__global__ void __launch_bounds__(kNTD, 3) dg_tc_kernel(GrP P) {
  using S = nmgk::TcShape<N>;
  constexpr int np = S::NP, nn = S::NN, TILES = S::TILES, NWARP = kNTD / 32;
  extern __shared__ __align__(16) unsigned char gsm[];
  // the digits first: ldmatrix rows and uint4 stores want 16-byte addresses,
  // and 15 np doubles are not a multiple of 16 bytes at odd np
  uint4 *sDig = reinterpret_cast<uint4 *>(gsm);                 // [5][np] digits of sF
  double *sP = reinterpret_cast<double *>(sDig + NF * np);      // [5][np] primitives
  double *sR = sP + NF * np;                                    // [5][np] r
  double *sF = sR + NF * np;                                    // [5][np] fluxes along x^i
  __shared__ int sEmax[3][NF];
  const int e = P.dglist[blockIdx.x];
  const double *Pg = P.prim_d + (size_t)e * NF * np, *Ug = P.win_d + (size_t)e * NF * np;
  const double *M = P.dXdx + (size_t)e * 9 * np, *bg = P.bgd + (size_t)e * 8 * np;
  const double *bb = P.bbox + 6 * (size_t)e;
  const double s[3] = {2. / (bb[1] - bb[0]), 2. / (bb[3] - bb[2]), 2. / (bb[5] - bb[4])};
  const double w_end = P.basis[N * N];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, g = lane >> 2, tq = lane & 3;
  if (tid < 3 * NF) sEmax[tid / NF][tid % NF] = 0;
  for (int i = tid; i < NF * np; i += kNTD) sP[i] = Pg[i];
  __syncthreads();
  for (int q = tid; q < np; q += kNTD) {
    double Pq[NF], Fq[NF];
    for (int f = 0; f < NF; f++) Pq[f] = sP[f * np + q];
    sources(P.g, Pq, bg + q, np, Fq);
    for (int f = 0; f < NF; f++) sR[f * np + q] = Fq[f];
  }
  const uint32_t digbase = (uint32_t)__cvta_generic_to_shared(sDig);
  const int fd0 = nmgk::cTcRowExp[N - 7][tq], fd1 = nmgk::cTcRowExp[N - 7][min(tq + 4, 8)];
  const int fd8 = nmgk::cTcRowExp[N - 7][8];
  const uint4 *gB = &nmgk::gTcB[N - 7][0][0][0];
  const double *gD = nmgk::gTcD[N - 7];
#pragma unroll 1
  for (int i = 0; i < 3; i++) {
    {
      // the fluxes along x^i and each field's largest exponent
      int em[NF] = {0, 0, 0, 0, 0};
      for (int q = tid; q < np; q += kNTD) {
        double Uq[NF], Pq[NF], Fq[NF], nr[3] = {0., 0., 0.};
        nr[i] = 1.;
        for (int f = 0; f < NF; f++) {
          Uq[f] = Ug[f * np + q];
          Pq[f] = sP[f * np + q];
        }
        flux_n(Uq, Pq, nr, bg[q], bg[np + q], Fq);
        for (int f = 0; f < NF; f++) {
          sF[f * np + q] = Fq[f];
          em[f] = max(em[f], (int)((unsigned long long)__double_as_longlong(Fq[f]) >> 52) & 0x7FF);
        }
      }
#pragma unroll
      for (int f = 0; f < NF; f++) {
        const unsigned m = __reduce_max_sync(0xffffffffu, (unsigned)em[f]);
        if (lane == 0) atomicMax(&sEmax[i][f], (int)m);
      }
    }
    __syncthreads();
    for (int q = tid; q < NF * np; q += kNTD) sDig[q] = nmgk::tc_digits(sF[q], sEmax[i][q / np]);
    __syncthreads();
#pragma unroll 1
    for (int a = 0; a < 3; a++) {
      const double sa = s[a];
      const double *Mai = M + (a * 3 + i) * np;
#pragma unroll 1
      for (int task = warp; task < NF * TILES; task += NWARP) {
        const int f = task / TILES, tile = task - f * TILES;
        const int Lr = min(tile * 16 + (lane & 15), nn - 1), chunk = lane >> 4;
        const int ps = a == 0 ? 1 : (a == 1 ? N : nn);
        const int nb = a == 0 ? N * Lr : (a == 1 ? (Lr % N) + nn * (Lr / N) : Lr);
        // owned output slots as in stage_tc.cu's kernel, and M[a][i] (2/dX^a) there
        int nodeS[5];
        bool okS[5];
        double mS[5];
#pragma unroll
        for (int sl = 0; sl < 5; sl++) {
          const int L = tile * 16 + g + (sl < 4 ? (sl >> 1) * 8 : tq * 8);
          const int io = sl < 4 ? tq + (sl & 1) * 4 : N - 1;
          okS[sl] = L < nn && io < N && (sl < 4 ? true : (N == 9 && tq < 2));
          nodeS[sl] = okS[sl] ? nmgk::tc_node<N>(a, L, io) : 0;
          mS[sl] = okS[sl] ? Mai[nodeS[sl]] * sa : 0.;
        }
        double dv[5];
        nmgk::tc_derivs<N>(gB, digbase + (uint32_t)(f * np + nb) * 16u, (uint32_t)ps * 16u,
                           chunk, lane, tq, sEmax[i][f], fd0, fd1, fd8, dv);
#pragma unroll
        for (int sl = 0; sl < 5; sl++)
          if (okS[sl]) sR[f * np + nodeS[sl]] -= mS[sl] * dv[sl];
      }
      if (S::LAST) {
        // the line left over (l0 = l1 = n - 1) in FP64
        for (int t = tid; t < NF * N; t += kNTD) {
          const int f = t / N, io = t - f * N, L = nn - 1;
          double d = 0.;
          for (int p = 0; p < N; p++)
            d = fma(__ldg(gD + io * N + p), sF[f * np + nmgk::tc_node<N>(a, L, p)], d);
          const int node = nmgk::tc_node<N>(a, L, io);
          sR[f * np + node] -= Mai[node] * sa * d;
        }
      }
      __syncthreads();
    }
  }
  dg_faces_epilogue(P, e, sP, sR, Ug, M, bg, s, w_end);
}

// finite-volume elements: one CTA per slot.  Per direction and chunk of
// pencils: (1) per cell and field both face values of the cell's
// reconstruction (the cell's smoothness indicators serve its two faces),
// (2) per midpoint the LLF flux of the two states meeting there, per face
// point the outward flux, (3) per point the flux difference.
__global__ void __launch_bounds__(kNTF, 1) fv_kernel(GrP P) {
  extern __shared__ double sm[];
  const int nf = P.nf, npf = P.npf, nnf = P.nnf;
  const int slot = blockIdx.x, e = P.slotelem[slot];
  const int per = nf + 1;  // nf - 1 midpoints + 2 face points per pencil
  double *sP = sm, *sG = sP + NF * npf;  // sG: [pencils][nf + 1][5]
  double *sQ = sG + (size_t)P.pencils * per * NF;  // [2: left, right face][5][pencils][nf]
  const int qst = P.pencils * nf;                   // stride of one (face, field) plane
  const double *Pg = P.prim_f + (size_t)slot * NF * npf, *Ug = P.win_f + (size_t)slot * NF * npf;
  const double *G = P.geo + (size_t)slot * kGeo * npf;
  double *R = P.rbuf + (size_t)slot * NF * npf;
  const double ih = (nf - 1) / 2., ih2 = 2. * ih;  // 1/h, 1/(h/2): h = 2/(nf-1)
  for (int i = threadIdx.x; i < NF * npf; i += blockDim.x) sP[i] = Pg[i];
  __syncthreads();
  for (int q = threadIdx.x; q < npf; q += blockDim.x) {
    double Pq[NF], S[NF];
    for (int f = 0; f < NF; f++) Pq[f] = sP[f * npf + q];
    sources(P.g, Pq, G + npf + q, npf, S);
    for (int f = 0; f < NF; f++) R[f * npf + q] = S[f];
  }
  for (int a = 0; a < 3; a++) {
    const int str[3] = {1, nf, nnf};
    const int o1 = a == 0 ? 1 : 0, o2 = a == 2 ? 1 : 2;
    for (int c0 = 0; c0 < nnf; c0 += P.pencils) {
      const int cp = min(P.pencils, nnf - c0);
      __syncthreads();
      for (int task = threadIdx.x; task < cp * nf * NF; task += blockDim.x) {
        const int c = task % nf, kf = task / nf, k = kf % cp, f = kf / cp, pen = c0 + k;
        const int base = (pen % nf) * str[o1] + (pen / nf) * str[o2];
        const double *u = sP + f * npf + base;
        double v[5];
        for (int j = 0; j < 5; j++) {
          const int ii = c - 2 + j;
          v[j] = (ii >= 0 && ii < nf) ? u[ii * str[a]] : 0.;
        }
        double lft, rgt;
        rec_cell(P.rec, nf, v, c, 2., &lft, &rgt);
        sQ[f * qst + k * nf + c] = lft;
        sQ[(NF + f) * qst + k * nf + c] = rgt;
      }
      __syncthreads();
      for (int task = threadIdx.x; task < cp * per; task += blockDim.x) {
        const int k = task / per, t = task - k * per, pen = c0 + k;
        const int i1 = pen % nf, i2 = pen / nf;
        const int base = i1 * str[o1] + i2 * str[o2];
        double Fs[NF], Fi[NF];
        if (t < nf - 1) {
          // midpoint t (between points t and t+1)
          const int qm = base + t * str[a];
          const double *gm = G + (21 + 6 * a) * npf + qm;
          const double nr[3] = {gm[0], gm[npf], gm[2 * npf]};
          const double jg = gm[3 * npf], al = gm[4 * npf], ps = gm[5 * npf];
          double PL[NF], PR[NF], UL[NF], UR[NF];
          for (int f = 0; f < NF; f++) {
            PL[f] = sQ[(NF + f) * qst + k * nf + t];  // right face of cell t
            PR[f] = sQ[f * qst + k * nf + t + 1];     // left face of cell t+1
          }
          if (!physical(PL, ps))
            for (int f = 0; f < NF; f++) PL[f] = sP[f * npf + qm];
          if (!physical(PR, ps))
            for (int f = 0; f < NF; f++) PR[f] = sP[f * npf + qm + str[a]];
          // both sides' conserved state, flux and largest speed from one
          // evaluation of their primitives (fewer divisions than p2c_point
          // followed by llf; the same quantities)
          const double ps2 = ps * ps, ps4 = ps2 * ps2, ps6 = ps4 * ps2, ips4 = 1. / ps4;
          double FL[NF], FR[NF];
          const double aL = side_state(P.g, PL, nr, al, ps4, ps6, ips4, UL, FL);
          const double aR = side_state(P.g, PR, nr, al, ps4, ps6, ips4, UR, FR);
          const double am = fmax(aL, aR);
          for (int f = 0; f < NF; f++)
            sG[(k * per + t) * NF + f] = jg * (0.5 * (FL[f] + FR[f] - am * (UR[f] - UL[f])));
        } else {
          // face point of side t - (nf - 1): outward flux
          const int side = t - (nf - 1), t0 = side ? nf - 1 : 0, fc = 2 * a + side;
          const int qq = base + t0 * str[a];
          const double sg = side ? 1. : -1.;
          const double *gq = G + (9 + 4 * a) * npf + qq;
          const double nr[3] = {sg * gq[0], sg * gq[npf], sg * gq[2 * npf]};
          const double jg = gq[3 * npf];
          const double al = G[npf + qq], ps = G[2 * npf + qq];
          double Ui[NF], Pi[NF], Uo[NF], Po[NF];
          for (int f = 0; f < NF; f++) {
            Ui[f] = Ug[f * npf + qq];
            Pi[f] = sP[f * npf + qq];
          }
          if (exterior(P, e, fc, i1, i2, ps, Uo, Po))
            llf(P.g, Ui, Pi, Uo, Po, nr, al, ps, Fs, Fi);
          else
            flux_n(Ui, Pi, nr, al, ps, Fs);
          for (int f = 0; f < NF; f++) sG[(k * per + t) * NF + f] = jg * Fs[f];
        }
      }
      __syncthreads();
      for (int task = threadIdx.x; task < cp * nf; task += blockDim.x) {
        const int k = task / nf, t = task - k * nf, pen = c0 + k;
        const int i1 = pen % nf, i2 = pen / nf;
        const int qq = i1 * str[o1] + i2 * str[o2] + t * str[a];
        const double *g0 = sG + k * per * NF;
        // det / h (det / (h/2) at the pencil ends) times the flux difference
        const double dh = G[qq] * ((t == 0 || t == nf - 1) ? ih2 : ih);
        for (int f = 0; f < NF; f++) {
          double df;
          if (t == 0) df = g0[f] + g0[(nf - 1) * NF + f];
          else if (t == nf - 1) df = g0[nf * NF + f] - g0[(nf - 2) * NF + f];
          else df = g0[t * NF + f] - g0[(t - 1) * NF + f];
          R[f * npf + qq] -= dh * df;
        }
      }
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < NF * npf; i += blockDim.x)
    epilogue(P, R[i], (size_t)slot * NF * npf + i, P.u0_f, P.acc_f, P.wout_f);
}

// geometry of the finite-volume slots (points and midpoints) from the map
__global__ void fvgeo_kernel(GrP P, ShellMap S, const int *pat, double *geo) {
  const int nf = P.nf, npf = P.npf;
  const double *xu = P.basis + P.n * P.n + 2 * P.n;
  const int64_t tot = (int64_t)P.nfv * npf;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < tot;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int slot = (int)(i / npf), q = (int)(i % npf), e = P.slotelem[slot];
    const int id[3] = {q % nf, (q / nf) % nf, q / (nf * nf)};
    const double *bb = P.bbox + 6 * (size_t)e;
    double *G = geo + (size_t)slot * kGeo * npf + q;
    auto eval = [&](const double Xb[3], double x[3], double Mb[3][3]) {
      double X[3], J[3][3];
      for (int d = 0; d < 3; d++)
        X[d] = 0.5 * ((bb[2 * d + 1] - bb[2 * d]) * Xb[d] + (bb[2 * d + 1] + bb[2 * d]));
      shell_map(S, pat[e], X, x, J);
      for (int d = 0; d < 3; d++)
        for (int c = 0; c < 3; c++) Mb[d][c] = (2. / (bb[2 * d + 1] - bb[2 * d])) * J[d][c];
    };
    double Xb[3] = {xu[id[0]], xu[id[1]], xu[id[2]]}, x[3], Mb[3][3], bgv[8];
    eval(Xb, x, Mb);
    const double det = det3(Mb);
    background(P.mass, x, bgv);
    G[0] = det;
    for (int k = 0; k < 8; k++) G[(1 + k) * npf] = bgv[k];
    for (int a = 0; a < 3; a++) {
      const double nm = sqrt(Mb[a][0] * Mb[a][0] + Mb[a][1] * Mb[a][1] + Mb[a][2] * Mb[a][2]);
      for (int c = 0; c < 3; c++) G[(9 + 4 * a + c) * npf] = Mb[a][c] / nm;
      G[(12 + 4 * a) * npf] = nm / det;
    }
    for (int a = 0; a < 3; a++) {
      double *Gm = G + (21 + 6 * a) * npf;
      if (id[a] >= nf - 1) {
        for (int k = 0; k < 6; k++) Gm[k * npf] = 0.;
        continue;
      }
      double Xm[3] = {Xb[0], Xb[1], Xb[2]}, xm[3], Mm[3][3], bm[8];
      Xm[a] = 0.5 * (xu[id[a]] + xu[id[a] + 1]);
      eval(Xm, xm, Mm);
      background(P.mass, xm, bm);
      const double nm = sqrt(Mm[a][0] * Mm[a][0] + Mm[a][1] * Mm[a][1] + Mm[a][2] * Mm[a][2]);
      for (int c = 0; c < 3; c++) Gm[c * npf] = Mm[a][c] / nm;
      Gm[3 * npf] = nm / det3(Mm);
      Gm[4 * npf] = bm[0];
      Gm[5 * npf] = bm[1];
    }
  }
}

// out = (A x A x A) in for every field of the listed elements, A (no x ni);
// src/dst rows given per element (in row isrc[k], out row idst[k])
__global__ void convert_kernel(const double *A, int ni, int no, const int *isrc,
                               const int *idst, const double *src, double *dst) {
  extern __shared__ double sm[];
  const int ni3 = ni * ni * ni, no3 = no * no * no;
  double *sIn = sm, *t1 = sIn + ni3, *t2 = t1 + no * ni * ni, *sA = t2 + no * no * ni;
  const int k = blockIdx.x;
  for (int i = threadIdx.x; i < no * ni; i += blockDim.x) sA[i] = A[i];
  for (int f = 0; f < NF; f++) {
    const double *in = src + ((size_t)isrc[k] * NF + f) * ni3;
    double *out = dst + ((size_t)idst[k] * NF + f) * no3;
    __syncthreads();
    for (int i = threadIdx.x; i < ni3; i += blockDim.x) sIn[i] = in[i];
    __syncthreads();
    for (int t = threadIdx.x; t < no * ni * ni; t += blockDim.x) {
      const int i = t % no, jk = t / no;
      double s = 0.;
      for (int m = 0; m < ni; m++) s += sA[i * ni + m] * sIn[m + ni * jk];
      t1[t] = s;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < no * no * ni; t += blockDim.x) {
      const int i = t % no, j = (t / no) % no, kk = t / (no * no);
      double s = 0.;
      for (int m = 0; m < ni; m++) s += sA[j * ni + m] * t1[i + no * (m + ni * kk)];
      t2[t] = s;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < no3; t += blockDim.x) {
      const int i = t % no, j = (t / no) % no, kk = t / (no * no);
      double s = 0.;
      for (int m = 0; m < ni; m++) s += sA[kk * ni + m] * t2[i + no * (j + no * m)];
      out[t] = s;
    }
  }
}

// copy rows (element states of 5 fields) between slot layouts
__global__ void copy_rows_kernel(int64_t rowlen, const int *isrc, const int *idst,
                                 const double *src, double *dst) {
  const int k = blockIdx.y;
  const double *in = src + (size_t)isrc[k] * rowlen;
  double *out = dst + (size_t)idst[k] * rowlen;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < rowlen;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = in[i];
}

// Persson's modal indicator of D (field 0) per element (the reference's
// evolve_Persson_array_indicator, src/main/evolve/trouble.c:505-564): the
// LGL nodal values (a finite-volume element's projected back by R x R x R)
// analysed into normalised Legendre coefficients c by A x A x A, then
// log10(sum of c^2 over the modes of highest degree in some direction /
// sum of all c^2).  One CTA per element.
__global__ void persson_kernel(GrP P, const double *u_d, const double *u_f, const double *A,
                               const double *R, double *ind) {
  extern __shared__ double sm[];
  const int n = P.n, np = P.np, nf = P.nf;
  const int e = blockIdx.x, slot = P.fvslot[e];
  double *sU = sm, *t1 = sU + max(np, P.npf), *t2 = t1 + max(n * nf * nf, np);
  double *sC = t2 + max(n * n * nf, np), *red = sC + np;
  // nodal values of D on the LGL points
  if (slot < 0) {
    for (int q = threadIdx.x; q < np; q += blockDim.x) sU[q] = u_d[(size_t)e * NF * np + q];
  } else {
    const int npf = P.npf;
    for (int q = threadIdx.x; q < npf; q += blockDim.x) sU[q] = u_f[(size_t)slot * NF * npf + q];
    __syncthreads();
    for (int t = threadIdx.x; t < n * nf * nf; t += blockDim.x) {
      const int i = t % n, jk = t / n;
      double s = 0.;
      for (int m = 0; m < nf; m++) s += R[i * nf + m] * sU[m + nf * jk];
      t1[t] = s;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < n * n * nf; t += blockDim.x) {
      const int i = t % n, j = (t / n) % n, k = t / (n * n);
      double s = 0.;
      for (int m = 0; m < nf; m++) s += R[j * nf + m] * t1[i + n * (m + nf * k)];
      t2[t] = s;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < np; t += blockDim.x) {
      const int i = t % n, j = (t / n) % n, k = t / (n * n);
      double s = 0.;
      for (int m = 0; m < nf; m++) s += R[k * nf + m] * t2[i + n * (j + n * m)];
      sC[t] = s;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < np; t += blockDim.x) sU[t] = sC[t];
  }
  __syncthreads();
  // modal analysis, one direction at a time (as nmo_persson)
  for (int d = 0; d < 3; d++) {
    const int st = d == 0 ? 1 : (d == 1 ? n : n * n);
    for (int k = threadIdx.x; k < np; k += blockDim.x) {
      const int ii = d == 0 ? k % n : (d == 1 ? (k / n) % n : k / (n * n));
      const double *line = sU + k - ii * st;
      double sum = 0.;
      for (int l = 0; l < n; l++) sum += A[ii * n + l] * line[l * st];
      sC[k] = sum;
    }
    __syncthreads();
    for (int k = threadIdx.x; k < np; k += blockDim.x) sU[k] = sC[k];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double all = 0., hi = 0.;
    for (int k = 0; k < n; k++)
      for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++) {
          const double co = sU[i + n * (j + n * k)];
          all += co * co;
          if (i == n - 1 || j == n - 1 || k == n - 1) hi += co * co;
        }
    ind[e] = log10(hi / (all + 2.2250738585072014e-308) + 1e-50);
  }
  (void)red;
}

__global__ void p2c_kernel(nmg_grhd_params g, int64_t nrows, int npts, const double *psi_rows,
                           int psi_stride, const int *psi_row_of, const double *prim,
                           double *cons) {
  const int64_t tot = nrows * npts;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < tot;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = i / npts, q = i % npts;
    const int pr = psi_row_of ? psi_row_of[r] : (int)r;
    const double ps = psi_rows[(size_t)pr * psi_stride + q];
    double P[NF], U[NF];
    for (int f = 0; f < NF; f++) P[f] = prim[(r * NF + f) * npts + q];
    p2c_point(g, ps, P, U);
    for (int f = 0; f < NF; f++) cons[(r * NF + f) * npts + q] = U[f];
  }
}


}  // namespace

// ---------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------
struct nmg_grhd_ctx {
  std::string err;
  int device = -1;
  cudaStream_t stream = nullptr;
  nmg_grhd_evolve_params prm{};
  int n = 0, np = 0, nn = 0, nf = 0, npf = 0, nnf = 0, tpts = 0;
  int64_t E = 0;
  ShellMap shell{};
  std::vector<int32_t> h_nb, h_code, h_fv, h_slot;
  std::vector<double> h_bbox;
  // device mesh
  int *d_nb = nullptr, *d_code = nullptr, *d_pat = nullptr;
  double *d_dXdx = nullptr, *d_bgd = nullptr, *d_bbox = nullptr, *d_basis = nullptr;
  double *d_Pm = nullptr, *d_Rm = nullptr, *d_A = nullptr, *d_ind = nullptr;
  // DG states and guesses
  double *d_ud[4] = {nullptr, nullptr, nullptr, nullptr};
  double *d_pd = nullptr;
  // finite-volume slots
  int nfv = 0, cap = 0;
  double *d_uf[4] = {nullptr, nullptr, nullptr, nullptr};
  double *d_pf = nullptr, *d_rbuf = nullptr, *d_geo = nullptr;
  int *d_slotelem = nullptr, *d_fvslot = nullptr, *d_dglist = nullptr;
  int ndg = 0;
  // DG / finite-volume faces
  int ntr = 0;
  int *d_tslot = nullptr, *d_tface = nullptr;
  double *d_trace = nullptr;
  int cur = 0;
  unsigned long long *d_stats = nullptr;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  double graph_dt = 0.;
  int64_t launches = 0, graph_launches = 0;
  size_t smem_dg = 0, smem_fv = 0;
  int pencils = 0;
  bool dg_tc = false;  // DG divergence on the tensor cores (n = 7, 8, 9)
};

namespace {

int gset(nmg_grhd_ctx *c, int code, const std::string &msg) {
  if (c) c->err = msg;
  return code;
}

#define GCK(call)                                                                        \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess)                                                               \
      return gset(c, NMG_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_));     \
  } while (0)

template <class T>
int dalloc(nmg_grhd_ctx *c, T **p, size_t count) {
  if (*p) cudaFree(*p);
  *p = nullptr;
  if (count == 0) return NMG_OK;
  if (cudaMalloc((void **)p, count * sizeof(T)) != cudaSuccess) {
    cudaGetLastError();
    return gset(c, NMG_ENOMEM, "nmg_grhd: device allocation failed");
  }
  return NMG_OK;
}

template <class T>
int upload(nmg_grhd_ctx *c, T **p, const std::vector<T> &v) {
  int rc = dalloc(c, p, v.size());
  if (rc || v.empty()) return rc;
  GCK(cudaMemcpyAsync(*p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, c->stream));
  return NMG_OK;
}

void drop_graphs(nmg_grhd_ctx *c) {
  for (auto &g : c->graph)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
}

// LGL -> equally spaced interpolation P (nf x n) and its pseudo-inverse
// R = (P^T P)^-1 P^T (n x nf), in long double (gridpoints.c:158-200 with
// Inverse_InterpMatT_pseudo)
void transfer_matrices(int n, int nf, const std::vector<double> &xl, const std::vector<double> &xu,
                       std::vector<double> &Pm, std::vector<double> &Rm) {
  std::vector<long double> Pl((size_t)nf * n), A((size_t)n * (n + nf));
  Pm.assign((size_t)nf * n, 0.);
  Rm.assign((size_t)n * nf, 0.);
  for (int q = 0; q < nf; q++)
    for (int i = 0; i < n; i++) {
      long double v = 1.L;
      for (int j = 0; j < n; j++)
        if (j != i) v *= ((long double)xu[q] - xl[j]) / ((long double)xl[i] - xl[j]);
      Pl[(size_t)q * n + i] = v;
      Pm[(size_t)q * n + i] = (double)v;
    }
  const int w = n + nf;
  for (int i = 0; i < n; i++) {
    for (int j = 0; j < n; j++) {
      long double s = 0.L;
      for (int q = 0; q < nf; q++) s += Pl[(size_t)q * n + i] * Pl[(size_t)q * n + j];
      A[(size_t)i * w + j] = s;
    }
    for (int q = 0; q < nf; q++) A[(size_t)i * w + n + q] = Pl[(size_t)q * n + i];
  }
  for (int k = 0; k < n; k++) {
    int piv = k;
    for (int i = k + 1; i < n; i++)
      if (fabsl(A[(size_t)i * w + k]) > fabsl(A[(size_t)piv * w + k])) piv = i;
    if (piv != k)
      for (int j = 0; j < w; j++) std::swap(A[(size_t)k * w + j], A[(size_t)piv * w + j]);
    const long double d = A[(size_t)k * w + k];
    for (int j = 0; j < w; j++) A[(size_t)k * w + j] /= d;
    for (int i = 0; i < n; i++)
      if (i != k) {
        const long double f = A[(size_t)i * w + k];
        for (int j = 0; j < w; j++) A[(size_t)i * w + j] -= f * A[(size_t)k * w + j];
      }
  }
  for (int i = 0; i < n; i++)
    for (int q = 0; q < nf; q++) Rm[(size_t)i * nf + q] = (double)A[(size_t)i * w + n + q];
}

// normalised Legendre analysis of n LGL points: A[i][j] = w_j P_i(x_j)
// sqrt(c_i), c_i = (2i+1)/2 and n/2-1/2 ... (N/2 for the top mode), as the
// reference's LGL_AT_ST_matrices (src/main/basis/Legendre.c:277-310)
std::vector<double> analysis_matrix(const std::vector<double> &x, const std::vector<double> &w) {
  const int n = (int)x.size(), N = n - 1;
  std::vector<double> A((size_t)n * n);
  for (int i = 0; i < n; i++) {
    double ooci = 0.5 * (2 * i + 1);
    if (i == N && N != 0) ooci = 0.5 * i;
    const double oosci = std::sqrt(ooci);
    for (int j = 0; j < n; j++) {
      double Pk = 0., P0 = 1.0, P1 = x[j], Pi;
      if (i == 0) Pi = P0;
      else if (i == 1) Pi = P1;
      else {
        for (int k = 2; k <= i; k++) {
          Pk = (x[j] * (2 * k - 1) * P1 - (k - 1) * P0) / k;
          P0 = P1;
          P1 = Pk;
        }
        Pi = Pk;
      }
      A[(size_t)i * n + j] = w[j] * (Pi * oosci);
    }
  }
  return A;
}

GrP base_params(nmg_grhd_ctx *c) {
  GrP P;
  std::memset(&P, 0, sizeof(P));
  P.n = c->n; P.np = c->np; P.nn = c->nn;
  P.nf = c->nf; P.npf = c->npf; P.nnf = c->nnf; P.tpts = c->tpts;
  P.ndg = c->ndg; P.nfv = c->nfv;
  P.g = c->prm.eos;
  P.mass = c->prm.mass;
  P.rec = c->prm.rec;
  P.dglist = c->d_dglist; P.slotelem = c->d_slotelem; P.fvslot = c->d_fvslot;
  P.nb = c->d_nb; P.code = c->d_code; P.tslot = c->d_tslot; P.tface = c->d_tface;
  P.ntr = c->ntr;
  P.dXdx = c->d_dXdx; P.bgd = c->d_bgd; P.bbox = c->d_bbox; P.basis = c->d_basis;
  P.geo = c->d_geo; P.trace = c->d_trace; P.rbuf = c->d_rbuf;
  P.pencils = c->pencils;
  return P;
}

int grid_for(int64_t work) {
  return (int)std::max<int64_t>(1, std::min<int64_t>((work + kNT - 1) / kNT, 152 * 16));
}

// one stage: con2prim of the input (in place), traces, DG and FV kernels;
// with ev (8 events), each kernel class is bracketed by a pair of events
int enqueue_stage(nmg_grhd_ctx *c, GrP P, double *win_d, double *win_f,
                  cudaEvent_t *ev = nullptr) {
  P.win_d = win_d;
  P.win_f = win_f;
  P.prim_d = c->d_pd;
  P.prim_f = c->d_pf;
  auto mark = [&](int k) {
    if (ev) cudaEventRecord(ev[k], c->stream);
  };
  const int64_t work = (int64_t)c->ndg * c->np + (int64_t)c->nfv * c->npf;
  mark(0);
  if (work > 0) {
    c2p_kernel<<<grid_for(work), kNT, 0, c->stream>>>(P, win_d, win_f, c->d_pd, c->d_pf,
                                                      c->d_stats);
    GCK(cudaGetLastError());
    c->launches++;
  }
  mark(1);
  mark(2);
  if (c->ntr > 0) {
    trace_kernel<<<grid_for((int64_t)c->ntr * c->tpts), kNT, 0, c->stream>>>(P, c->d_pd, c->d_pf);
    GCK(cudaGetLastError());
    c->launches++;
  }
  mark(3);
  mark(4);
  if (c->ndg > 0) {
    if (!c->dg_tc)
      dg_kernel<<<c->ndg, kNT, c->smem_dg, c->stream>>>(P);
    else if (c->n == 7)
      dg_tc_kernel<7><<<c->ndg, kNTD, dg_tc_smem<7>(), c->stream>>>(P);
    else if (c->n == 8)
      dg_tc_kernel<8><<<c->ndg, kNTD, dg_tc_smem<8>(), c->stream>>>(P);
    else
      dg_tc_kernel<9><<<c->ndg, kNTD, dg_tc_smem<9>(), c->stream>>>(P);
    GCK(cudaGetLastError());
    c->launches++;
  }
  mark(5);
  mark(6);
  if (c->nfv > 0) {
    fv_kernel<<<c->nfv, kNTF, c->smem_fv, c->stream>>>(P);
    GCK(cudaGetLastError());
    c->launches++;
  }
  mark(7);
  return NMG_OK;
}

// one RK4 step of the state in buffer cur (the result goes to 1 - cur);
// with ms, the step runs stage by stage and ms[k] accumulates the time of
// kernel class k (con2prim, traces, DG, finite volume)
int enqueue_step(nmg_grhd_ctx *c, int cur, double dt, double *ms = nullptr) {
  cudaEvent_t ev[8];
  if (ms)
    for (int k = 0; k < 8; k++) GCK(cudaEventCreate(&ev[k]));
  double *Ud = c->d_ud[cur], *Ad = c->d_ud[1 - cur], *WAd = c->d_ud[2], *WBd = c->d_ud[3];
  double *Uf = c->d_uf[cur], *Af = c->d_uf[1 - cur], *WAf = c->d_uf[2], *WBf = c->d_uf[3];
  const double cacc[4] = {dt / 6., dt / 3., dt / 3., dt / 6.};
  const double cw[4] = {dt / 2., dt / 2., dt, 0.};
  double *wind[4] = {Ud, WAd, WBd, WAd}, *winf[4] = {Uf, WAf, WBf, WAf};
  double *woutd[4] = {WAd, WBd, WAd, nullptr}, *woutf[4] = {WAf, WBf, WAf, nullptr};
  for (int s = 0; s < 4; s++) {
    GrP P = base_params(c);
    P.u0_d = Ud; P.u0_f = Uf;
    P.acc_d = Ad; P.acc_f = Af;
    P.wout_d = woutd[s]; P.wout_f = woutf[s];
    P.mode = s + 1;
    P.cacc = cacc[s];
    P.cw = cw[s];
    int rc = enqueue_stage(c, P, wind[s], winf[s], ms ? ev : nullptr);
    if (rc) return rc;
    if (ms) {
      GCK(cudaEventSynchronize(ev[7]));
      for (int k = 0; k < 4; k++) {
        float t = 0.f;
        GCK(cudaEventElapsedTime(&t, ev[2 * k], ev[2 * k + 1]));
        ms[k] += t;
      }
    }
  }
  if (ms)
    for (int k = 0; k < 8; k++) cudaEventDestroy(ev[k]);
  return NMG_OK;
}

// the element types: slots, lists, traces (host tables to the device)
int upload_types(nmg_grhd_ctx *c) {
  const int64_t E = c->E;
  std::vector<int> dgl, slotelem, fvslot(E, -1), tslot(E * 6, -1), tface;
  for (int64_t e = 0; e < E; e++) {
    if (c->h_fv[e]) {
      fvslot[e] = (int)slotelem.size();
      slotelem.push_back((int)e);
    } else {
      dgl.push_back((int)e);
    }
  }
  for (int64_t e = 0; e < E; e++)
    for (int f = 0; f < 6; f++) {
      const int e2 = c->h_nb[e * 6 + f];
      if (e2 >= 0 && (c->h_fv[e] != 0) != (c->h_fv[e2] != 0)) {
        tslot[e * 6 + f] = (int)(tface.size() / 2);
        tface.push_back((int)e);
        tface.push_back(f);
      }
    }
  c->ndg = (int)dgl.size();
  c->nfv = (int)slotelem.size();
  c->ntr = (int)(tface.size() / 2);
  c->h_slot = fvslot;
  int rc;
  if ((rc = upload(c, &c->d_dglist, dgl)) || (rc = upload(c, &c->d_slotelem, slotelem)) ||
      (rc = upload(c, &c->d_fvslot, fvslot)) || (rc = upload(c, &c->d_tslot, tslot)) ||
      (rc = upload(c, &c->d_tface, tface)))
    return rc;
  return dalloc(c, &c->d_trace, (size_t)c->ntr * NF * c->tpts);
}

}  // namespace

extern "C" {

int nmg_grhd_create(const nmg_mesh *m, const nmg_grhd_evolve_params *p, nmg_grhd_ctx **out) {
  if (!m || !p || !out) return NMG_EINVAL;
  *out = nullptr;
  nmg_grhd_ctx *c = new (std::nothrow) nmg_grhd_ctx;
  if (!c) return NMG_ENOMEM;
  *out = c;
  c->prm = *p;
  const nmg_grhd_params &g = p->eos;
  if (!(g.gamma > 1.) || !(g.rho_atm > 0.) || !(g.p_atm > 0.) || !(g.tol > 0.) || g.maxits <= 0 ||
      g.maxits > 100000 || !(p->mass >= 0.))
    return gset(c, NMG_EINVAL, "nmg_grhd_create: bad physical parameters");
  if (p->rec < NMG_FV_REC_1 || p->rec > NMG_FV_REC_WENOMZ_2)
    return gset(c, NMG_EINVAL, "nmg_grhd_create: unknown reconstruction");
  if (m->patches.size() != 6)
    return gset(c, NMG_EUNSUP, "nmg_grhd_create: the mesh must be NMG_MESH_CUBEDSHELL6");
  for (int q = 0; q < 6; q++) {
    const nmg::Patch &P = m->patches[q];
    if (!P.cubed || !P.shell) return gset(c, NMG_EUNSUP, "nmg_grhd_create: not a cubed shell");
    c->shell.dom[q] = P.dom;
    c->shell.s0[q] = P.s0;
    c->shell.s1[q] = P.s1;
  }
  for (int d = 0; d < 3; d++) c->shell.xc[d] = m->patches[0].xc[d];
  if (!m->fv.empty()) return gset(c, NMG_EUNSUP, "nmg_grhd_create: DG mesh expected");
  c->n = m->n;
  c->nf = p->nf > 0 ? p->nf : 2 * m->n;
  if (c->n < 3 || c->n > kMaxN)
    return gset(c, NMG_EUNSUP, "nmg_grhd_create: n must be in [3,10]");
  if (c->nf < 4 || c->nf > kMaxNF)
    return gset(c, NMG_EUNSUP, "nmg_grhd_create: nf must be in [4,16]");
  c->np = c->n * c->n * c->n;
  c->nn = c->n * c->n;
  c->npf = c->nf * c->nf * c->nf;
  c->nnf = c->nf * c->nf;
  c->tpts = std::max(c->nn, c->nnf);
  c->E = m->nelem;
  cudaError_t ce = cudaGetDevice(&c->device);
  if (ce != cudaSuccess) return gset(c, NMG_ECUDA, cudaGetErrorString(ce));
  GCK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  // shared memory of the kernels
  c->smem_dg = sizeof(double) * ((size_t)25 * c->np + c->nn);
  int optin = 0;
  GCK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device));
  // per pencil: the fluxes of its nf + 1 flux points and both face values
  // of its nf cells
  const size_t per_pencil = sizeof(double) * ((size_t)(c->nf + 1) * NF + (size_t)c->nf * 2 * NF);
  const size_t sp = sizeof(double) * (size_t)NF * c->npf;
  if (sp + per_pencil > (size_t)optin || c->smem_dg > (size_t)optin)
    return gset(c, NMG_EUNSUP, "nmg_grhd_create: element too large for shared memory");
  c->pencils = (int)std::min<size_t>((size_t)c->nnf, ((size_t)optin - sp) / per_pencil);
  c->smem_fv = sp + per_pencil * c->pencils;
  GCK(cudaFuncSetAttribute(dg_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)c->smem_dg));
  GCK(cudaFuncSetAttribute(fv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)c->smem_fv));
  // the tensor-core DG kernel at n = 7, 8, 9 (NMG_GRHD_DG=fp64 keeps the FP64 one)
  {
    const char *ev = std::getenv("NMG_GRHD_DG");
    c->dg_tc = c->n >= 7 && c->n <= 9 && !(ev && std::strcmp(ev, "fp64") == 0);
  }
  if (c->dg_tc) {
    GCK(nmgk::tc_upload_tables(c->n, m->D.data(), false));
    if (c->n == 7)
      GCK(cudaFuncSetAttribute(dg_tc_kernel<7>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)dg_tc_smem<7>()));
    else if (c->n == 8)
      GCK(cudaFuncSetAttribute(dg_tc_kernel<8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)dg_tc_smem<8>()));
    else
      GCK(cudaFuncSetAttribute(dg_tc_kernel<9>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)dg_tc_smem<9>()));
  }
  // mesh tables
  const int64_t E = c->E;
  c->h_nb.assign(m->nb.begin(), m->nb.end());
  c->h_code.resize(E * 6);
  for (int64_t i = 0; i < E * 6; i++) c->h_code[i] = m->code[i] & 63;
  c->h_bbox = m->bbox;
  c->h_fv.assign(E, 0);
  std::vector<double> bgd((size_t)E * 8 * c->np);
  for (int64_t e = 0; e < E; e++)
    for (int q = 0; q < c->np; q++) {
      double x[3], b[8];
      for (int d = 0; d < 3; d++) x[d] = m->xyz[((size_t)e * 3 + d) * c->np + q];
      background(p->mass, x, b);
      for (int k = 0; k < 8; k++) bgd[((size_t)e * 8 + k) * c->np + q] = b[k];
    }
  std::vector<double> basis;
  basis.insert(basis.end(), m->D.begin(), m->D.end());
  basis.insert(basis.end(), m->w.begin(), m->w.end());
  basis.insert(basis.end(), m->x.begin(), m->x.end());
  std::vector<double> xu(c->nf);
  {
    std::vector<double> wu(c->nf), Du((size_t)c->nf * c->nf);
    nmg::uniform_basis(c->nf, xu.data(), wu.data(), Du.data());
  }
  basis.insert(basis.end(), xu.begin(), xu.end());
  for (int k = 0; k < c->n; k++) {  // barycentric weights of the LGL points
    double den = 1.;
    for (int j = 0; j < c->n; j++)
      if (j != k) den *= m->x[k] - m->x[j];
    basis.push_back(1. / den);
  }
  std::vector<double> Pm, Rm;
  transfer_matrices(c->n, c->nf, m->x, xu, Pm, Rm);
  int rc;
  if ((rc = upload(c, &c->d_nb, c->h_nb)) || (rc = upload(c, &c->d_code, c->h_code)) ||
      (rc = upload(c, &c->d_pat, m->pat)) || (rc = upload(c, &c->d_dXdx, m->dXdx)) ||
      (rc = upload(c, &c->d_bgd, bgd)) || (rc = upload(c, &c->d_bbox, m->bbox)) ||
      (rc = upload(c, &c->d_basis, basis)) || (rc = upload(c, &c->d_Pm, Pm)) ||
      (rc = upload(c, &c->d_Rm, Rm)) || (rc = upload(c, &c->d_A, analysis_matrix(m->x, m->w))) ||
      (rc = dalloc(c, &c->d_ind, (size_t)m->nelem)))
    return rc;
  const size_t ld = (size_t)E * NF * c->np;
  for (int b = 0; b < 4; b++)
    if ((rc = dalloc(c, &c->d_ud[b], ld))) return rc;
  if ((rc = dalloc(c, &c->d_pd, ld)) || (rc = dalloc(c, &c->d_stats, 2))) return rc;
  GCK(cudaMemsetAsync(c->d_ud[0], 0, ld * sizeof(double), c->stream));
  GCK(cudaMemsetAsync(c->d_pd, 0, ld * sizeof(double), c->stream));
  GCK(cudaMemsetAsync(c->d_stats, 0, 2 * sizeof(unsigned long long), c->stream));
  if ((rc = upload_types(c))) return rc;
  GCK(cudaStreamSynchronize(c->stream));
  return NMG_OK;
}

void nmg_grhd_destroy(nmg_grhd_ctx *c) {
  if (!c) return;
  drop_graphs(c);
  if (c->stream) cudaStreamSynchronize(c->stream);
  void *ptrs[] = {c->d_nb, c->d_code, c->d_pat, c->d_dXdx, c->d_bgd, c->d_bbox, c->d_basis,
                  c->d_Pm, c->d_Rm, c->d_A, c->d_ind, c->d_ud[0], c->d_ud[1], c->d_ud[2], c->d_ud[3], c->d_pd,
                  c->d_uf[0], c->d_uf[1], c->d_uf[2], c->d_uf[3], c->d_pf, c->d_rbuf, c->d_geo,
                  c->d_slotelem, c->d_fvslot, c->d_dglist, c->d_tslot, c->d_tface, c->d_trace,
                  c->d_stats};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

const char *nmg_grhd_last_error(const nmg_grhd_ctx *c) { return c ? c->err.c_str() : "null context"; }

int64_t nmg_grhd_fv_count(const nmg_grhd_ctx *c) { return c ? c->nfv : -1; }

int nmg_grhd_sizes(const nmg_grhd_ctx *c, int32_t *n, int32_t *nf, int64_t *nelem) {
  if (!c) return NMG_EINVAL;
  if (n) *n = c->n;
  if (nf) *nf = c->nf;
  if (nelem) *nelem = c->E;
  return NMG_OK;
}

int nmg_grhd_set_fv_elements(nmg_grhd_ctx *c, const int32_t *fv) {
  if (!c || !fv) return gset(c, NMG_EINVAL, "nmg_grhd_set_fv_elements: null argument");
  const int64_t E = c->E;
  std::vector<int32_t> nfv(E);
  for (int64_t e = 0; e < E; e++) nfv[e] = fv[e] ? 1 : 0;
  if (nfv == c->h_fv) return NMG_OK;
  // new slots: ascending elements
  std::vector<int> old_slot = c->h_slot, new_slot(E, -1);
  int count = 0;
  for (int64_t e = 0; e < E; e++)
    if (nfv[e]) new_slot[e] = count++;
  std::vector<int> keep_src, keep_dst, tofv_e, tofv_s, todg_s, todg_e;
  for (int64_t e = 0; e < E; e++) {
    if (nfv[e] && c->h_fv[e]) {
      keep_src.push_back(old_slot[e]);
      keep_dst.push_back(new_slot[e]);
    } else if (nfv[e]) {
      tofv_e.push_back((int)e);
      tofv_s.push_back(new_slot[e]);
    } else if (c->h_fv[e]) {
      todg_s.push_back(old_slot[e]);
      todg_e.push_back((int)e);
    }
  }
  const size_t lf = (size_t)count * NF * c->npf;
  double *nu = nullptr, *np_ = nullptr;
  int rc;
  if ((rc = dalloc(c, &nu, lf)) || (rc = dalloc(c, &np_, lf))) return rc;
  int *d_lists = nullptr;
  std::vector<int> all;
  auto put = [&](const std::vector<int> &v) {
    const size_t off = all.size();
    all.insert(all.end(), v.begin(), v.end());
    return off;
  };
  const size_t o_ks = put(keep_src), o_kd = put(keep_dst), o_fe = put(tofv_e), o_fs = put(tofv_s),
               o_ds = put(todg_s), o_de = put(todg_e);
  if ((rc = upload(c, &d_lists, all))) return rc;
  double *U = c->d_ud[c->cur], *Uf = c->d_uf[c->cur];
  if (!keep_src.empty()) {
    dim3 grid(8, (unsigned)keep_src.size());
    copy_rows_kernel<<<grid, kNT, 0, c->stream>>>((int64_t)NF * c->npf, d_lists + o_ks,
                                                  d_lists + o_kd, Uf, nu);
    copy_rows_kernel<<<grid, kNT, 0, c->stream>>>((int64_t)NF * c->npf, d_lists + o_ks,
                                                  d_lists + o_kd, c->d_pf, np_);
    GCK(cudaGetLastError());
  }
  const size_t sm_to = sizeof(double) * ((size_t)c->np + (size_t)c->nf * c->nn +
                                         (size_t)c->nf * c->nf * c->n + (size_t)c->nf * c->n);
  const size_t sm_back = sizeof(double) * ((size_t)c->npf + (size_t)c->n * c->nnf +
                                           (size_t)c->n * c->n * c->nf + (size_t)c->nf * c->n);
  GCK(cudaFuncSetAttribute(convert_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)std::max(sm_to, sm_back)));
  if (!tofv_e.empty()) {
    convert_kernel<<<(unsigned)tofv_e.size(), kNT, sm_to, c->stream>>>(
        c->d_Pm, c->n, c->nf, d_lists + o_fe, d_lists + o_fs, U, nu);
    convert_kernel<<<(unsigned)tofv_e.size(), kNT, sm_to, c->stream>>>(
        c->d_Pm, c->n, c->nf, d_lists + o_fe, d_lists + o_fs, c->d_pd, np_);
    GCK(cudaGetLastError());
  }
  if (!todg_s.empty()) {
    convert_kernel<<<(unsigned)todg_s.size(), kNT, sm_back, c->stream>>>(
        c->d_Rm, c->nf, c->n, d_lists + o_ds, d_lists + o_de, Uf, U);
    convert_kernel<<<(unsigned)todg_s.size(), kNT, sm_back, c->stream>>>(
        c->d_Rm, c->nf, c->n, d_lists + o_ds, d_lists + o_de, c->d_pf, c->d_pd);
    GCK(cudaGetLastError());
  }
  GCK(cudaStreamSynchronize(c->stream));
  cudaFree(d_lists);
  // swap in the new slot arrays
  for (int b = 0; b < 4; b++) {
    if (c->d_uf[b]) cudaFree(c->d_uf[b]);
    c->d_uf[b] = nullptr;
  }
  if (c->d_pf) cudaFree(c->d_pf);
  c->d_uf[c->cur] = nu;
  c->d_pf = np_;
  for (int b = 0; b < 4; b++)
    if (b != c->cur && (rc = dalloc(c, &c->d_uf[b], lf))) return rc;
  if ((rc = dalloc(c, &c->d_rbuf, lf)) || (rc = dalloc(c, &c->d_geo, (size_t)count * kGeo * c->npf)))
    return rc;
  c->h_fv = nfv;
  if ((rc = upload_types(c))) return rc;
  if (c->nfv > 0) {
    GrP P = base_params(c);
    fvgeo_kernel<<<grid_for((int64_t)c->nfv * c->npf), kNT, 0, c->stream>>>(P, c->shell, c->d_pat,
                                                                          c->d_geo);
    GCK(cudaGetLastError());
  }
  GCK(cudaStreamSynchronize(c->stream));
  drop_graphs(c);
  return NMG_OK;
}

int nmg_grhd_trouble_indicators(nmg_grhd_ctx *c, double *ind) {
  if (!c || !ind) return gset(c, NMG_EINVAL, "nmg_grhd_trouble_indicators: null argument");
  const int n = c->n, nf = c->nf, np = c->np;
  const size_t smem = sizeof(double) * ((size_t)std::max(np, c->npf) +
                                        std::max(n * nf * nf, np) + std::max(n * n * nf, np) + np);
  GCK(cudaFuncSetAttribute(persson_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  GrP P = base_params(c);
  persson_kernel<<<(unsigned)c->E, kNT, smem, c->stream>>>(P, c->d_ud[c->cur], c->d_uf[c->cur],
                                                          c->d_A, c->d_Rm, c->d_ind);
  GCK(cudaGetLastError());
  GCK(cudaMemcpyAsync(ind, c->d_ind, sizeof(double) * c->E, cudaMemcpyDeviceToHost, c->stream));
  GCK(cudaStreamSynchronize(c->stream));
  return NMG_OK;
}

int nmg_grhd_update_troubled(nmg_grhd_ctx *c, double persson_max, double back_margin,
                             int32_t *switched) {
  if (!c || !(back_margin >= 0.))
    return gset(c, NMG_EINVAL, "nmg_grhd_update_troubled: bad argument");
  std::vector<double> ind(c->E);
  int rc = nmg_grhd_trouble_indicators(c, ind.data());
  if (rc) return rc;
  std::vector<int32_t> fv = c->h_fv;
  int to_fv = 0, to_dg = 0;
  for (int64_t e = 0; e < c->E; e++) {
    if (!fv[e] && ind[e] > persson_max) {
      fv[e] = 1;
      to_fv++;
    } else if (fv[e] && ind[e] < persson_max - back_margin) {
      fv[e] = 0;
      to_dg++;
    }
  }
  if (switched) {
    switched[0] = to_fv;
    switched[1] = to_dg;
  }
  return (to_fv || to_dg) ? nmg_grhd_set_fv_elements(c, fv.data()) : NMG_OK;
}

int nmg_grhd_get_fv_elements(nmg_grhd_ctx *c, int32_t *fv) {
  if (!c || !fv) return gset(c, NMG_EINVAL, "nmg_grhd_get_fv_elements: null argument");
  std::memcpy(fv, c->h_fv.data(), sizeof(int32_t) * c->E);
  return NMG_OK;
}

// host layouts: DG [E][5][n^3] (rows of finite-volume elements ignored or
// zero), finite volume [nfv][5][nf^3] in ascending element order
int nmg_grhd_set_prim(nmg_grhd_ctx *c, const double *prim_dg, const double *prim_fv) {
  if (!c || !prim_dg || (c->nfv > 0 && !prim_fv))
    return gset(c, NMG_EINVAL, "nmg_grhd_set_prim: null argument");
  const size_t ld = (size_t)c->E * NF * c->np, lf = (size_t)c->nfv * NF * c->npf;
  GCK(cudaMemcpyAsync(c->d_pd, prim_dg, ld * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  p2c_kernel<<<grid_for((int64_t)c->E * c->np), kNT, 0, c->stream>>>(
      c->prm.eos, c->E, c->np, c->d_bgd + c->np, 8 * c->np, nullptr, c->d_pd, c->d_ud[c->cur]);
  GCK(cudaGetLastError());
  if (lf) {
    GCK(cudaMemcpyAsync(c->d_pf, prim_fv, lf * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    p2c_kernel<<<grid_for((int64_t)c->nfv * c->npf), kNT, 0, c->stream>>>(
        c->prm.eos, c->nfv, c->npf, c->d_geo + 2 * c->npf, kGeo * c->npf, nullptr, c->d_pf,
        c->d_uf[c->cur]);
    GCK(cudaGetLastError());
  }
  GCK(cudaStreamSynchronize(c->stream));
  return NMG_OK;
}

int nmg_grhd_set_state(nmg_grhd_ctx *c, const double *u_dg, const double *u_fv,
                       const double *prim_dg, const double *prim_fv) {
  if (!c || !u_dg || (c->nfv > 0 && !u_fv))
    return gset(c, NMG_EINVAL, "nmg_grhd_set_state: null argument");
  const size_t ld = (size_t)c->E * NF * c->np, lf = (size_t)c->nfv * NF * c->npf;
  GCK(cudaMemcpyAsync(c->d_ud[c->cur], u_dg, ld * sizeof(double), cudaMemcpyHostToDevice,
                      c->stream));
  if (prim_dg)
    GCK(cudaMemcpyAsync(c->d_pd, prim_dg, ld * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  if (lf) {
    GCK(cudaMemcpyAsync(c->d_uf[c->cur], u_fv, lf * sizeof(double), cudaMemcpyHostToDevice,
                        c->stream));
    if (prim_fv)
      GCK(cudaMemcpyAsync(c->d_pf, prim_fv, lf * sizeof(double), cudaMemcpyHostToDevice,
                          c->stream));
  }
  GCK(cudaStreamSynchronize(c->stream));
  return NMG_OK;
}

int nmg_grhd_get_state(nmg_grhd_ctx *c, double *u_dg, double *u_fv, double *prim_dg,
                       double *prim_fv) {
  if (!c) return NMG_EINVAL;
  const size_t ld = (size_t)c->E * NF * c->np, lf = (size_t)c->nfv * NF * c->npf;
  if (u_dg)
    GCK(cudaMemcpyAsync(u_dg, c->d_ud[c->cur], ld * sizeof(double), cudaMemcpyDeviceToHost,
                        c->stream));
  if (prim_dg)
    GCK(cudaMemcpyAsync(prim_dg, c->d_pd, ld * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  if (lf && u_fv)
    GCK(cudaMemcpyAsync(u_fv, c->d_uf[c->cur], lf * sizeof(double), cudaMemcpyDeviceToHost,
                        c->stream));
  if (lf && prim_fv)
    GCK(cudaMemcpyAsync(prim_fv, c->d_pf, lf * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  GCK(cudaStreamSynchronize(c->stream));
  return NMG_OK;
}

// r = RHS of the resident state after its con2prim (which, as in the first
// stage of a step, may reset atmosphere points of the state in place)
int nmg_grhd_rhs(nmg_grhd_ctx *c, double *r_dg, double *r_fv) {
  if (!c || !r_dg) return gset(c, NMG_EINVAL, "nmg_grhd_rhs: null argument");
  GrP P = base_params(c);
  P.acc_d = c->d_ud[1 - c->cur];
  P.acc_f = c->d_uf[1 - c->cur];
  P.mode = 0;
  int rc = enqueue_stage(c, P, c->d_ud[c->cur], c->d_uf[c->cur]);
  if (rc) return rc;
  const size_t ld = (size_t)c->E * NF * c->np, lf = (size_t)c->nfv * NF * c->npf;
  GCK(cudaMemcpyAsync(r_dg, c->d_ud[1 - c->cur], ld * sizeof(double), cudaMemcpyDeviceToHost,
                      c->stream));
  if (lf && r_fv)
    GCK(cudaMemcpyAsync(r_fv, c->d_uf[1 - c->cur], lf * sizeof(double), cudaMemcpyDeviceToHost,
                        c->stream));
  GCK(cudaStreamSynchronize(c->stream));
  return NMG_OK;
}

int nmg_grhd_rk4_steps(nmg_grhd_ctx *c, double dt, int32_t nsteps) {
  if (!c || nsteps < 0 || !(dt > 0.)) return gset(c, NMG_EINVAL, "nmg_grhd_rk4_steps: bad argument");
  if (nsteps == 0) return NMG_OK;
  if (dt != c->graph_dt) {
    drop_graphs(c);
    c->graph_dt = dt;
  }
  for (int g = 0; g < 2; g++) {
    if (c->graph[g]) continue;
    cudaGraph_t gr;
    GCK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    const int64_t l0 = c->launches;
    int rc = enqueue_step(c, g, dt);
    cudaGraph_t tmp = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(c->stream, &tmp);
    gr = tmp;
    c->graph_launches = c->launches - l0;
    c->launches = l0;
    if (rc) {
      if (gr) cudaGraphDestroy(gr);
      return rc;
    }
    GCK(e2);
    cudaError_t e3 = cudaGraphInstantiate(&c->graph[g], gr, 0);
    cudaGraphDestroy(gr);
    GCK(e3);
  }
  for (int s = 0; s < nsteps; s++) {
    GCK(cudaGraphLaunch(c->graph[c->cur], c->stream));
    c->launches += c->graph_launches;
    c->cur = 1 - c->cur;
  }
  GCK(cudaStreamSynchronize(c->stream));
  return NMG_OK;
}

int nmg_grhd_profile_step(nmg_grhd_ctx *c, double dt, double *ms) {
  if (!c || !ms || !(dt > 0.)) return gset(c, NMG_EINVAL, "nmg_grhd_profile_step: bad argument");
  for (int k = 0; k < 4; k++) ms[k] = 0.;
  int rc = enqueue_step(c, c->cur, dt, ms);
  if (rc) return rc;
  c->cur = 1 - c->cur;
  GCK(cudaStreamSynchronize(c->stream));
  return NMG_OK;
}

int nmg_grhd_stats(nmg_grhd_ctx *c, int64_t *c2p_iterations, int64_t *atmosphere_points,
                   int64_t *launches) {
  if (!c) return NMG_EINVAL;
  unsigned long long h[2] = {0, 0};
  GCK(cudaMemcpyAsync(h, c->d_stats, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  GCK(cudaStreamSynchronize(c->stream));
  if (c2p_iterations) *c2p_iterations = (int64_t)h[0];
  if (atmosphere_points) *atmosphere_points = (int64_t)h[1];
  if (launches) *launches = c->launches;
  return NMG_OK;
}

int nmg_grhd_reset_stats(nmg_grhd_ctx *c) {
  if (!c) return NMG_EINVAL;
  GCK(cudaMemsetAsync(c->d_stats, 0, 2 * sizeof(unsigned long long), c->stream));
  GCK(cudaStreamSynchronize(c->stream));
  return NMG_OK;
}

void *nmg_grhd_stream(nmg_grhd_ctx *c) { return c ? (void *)c->stream : nullptr; }

}  // extern "C"
