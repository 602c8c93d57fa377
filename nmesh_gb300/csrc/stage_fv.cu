// stage_fv.cu -- fused finite-volume RHS + RK4 stage kernel for elements in
// the reference's finite-volume mode (scalarwave1, FP64).
//
// Reference semantics (paths within nmeshsource/nmesh):
//   fv_divf            src/main/dg/fv.c:115-624 (use_only_right_flux,
//                      coordinates_midpoint_data = no, fv_flux = fnum)
//   midpoint states    src/tests/scalarwave1/scalarwave1.c:761-802
//   WENO3 / WENOm3_2   src/main/dg/rec1d.c:16-27,121-227,880-1030
//   WENO5 / WENOm5_2   src/main/dg/rec1d.c:1186-1368
//   dnfn extrapolation src/main/dg/rec1d.c:542-628 (s1 = 0, s2 = DBL_MAX)
//   face fluxes        src/tests/scalarwave1/scalarwave1.c:139-209,
//                      src/main/dg/numflux1d.c:85-112
//   surface terms      src/main/dg/dg.c:30-151 (fin.-vol. weight 1/|distXb|)
//   stage update       src/main/evolve/RungeKutta.c:19-82
//
// Two variants are built from this file:
//   "fvx" (this translation unit, compiled with -fmad=false): every FP64
//         product and sum is rounded separately in the reference's order,
//         with IEEE division, so on meshes without exact-data outer faces
//         (whose sin/cos come from a different math library) the result
//         equals the reference's bit for bit;
//   "fv"  (stage_fv_fast.cu defines NMG_FV_FAST and includes this file):
//         FMA contraction allowed and the nonlinear weights normalised with
//         one division per reconstruction, w_k = g_k prod_{j!=k} e_j^2 /
//         sum_k g_k prod_{j!=k} e_j^2 (the same weights as g_k/e_k^2 over
//         their sum, in exact arithmetic); within FP64 rounding of "fvx".
//
// Work split inside one CTA (one element): the element's pi, c state is
// staged in shared memory; per direction and chunk of pencils, one thread
// per (cell, field) reconstructs both face values of the cell (its
// smoothness indicators serve both faces; the same expressions as the
// per-midpoint rec_p / rec_m), then one thread per midpoint forms the
// flux of the two states meeting there (stored in shared memory); then one
// thread per node forms the conservative difference with the J sqrtgdiag /
// dXb factors and accumulates div f; the face terms and the RK4 update
// follow.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cstdint>

#include "stage.cuh"

#ifdef NMG_FV_FAST
#define NMG_FVNS fv_fast
#define NMG_FV_NAME "fv"
#else
#define NMG_FVNS fv_exact
#define NMG_FV_NAME "fvx"
#endif

namespace nmgk {
namespace NMG_FVNS {
namespace {

constexpr int kGeo = 13;  // per-node FV geometry of curvilinear elements

#include "weno.cuh"

__device__ __forceinline__ int fnode(int n, int f, int a, int b) {
  const int d = f >> 1, p = (f & 1) * (n - 1);
  return d == 0 ? p + n * (a + n * b) : d == 1 ? a + n * (p + n * b) : a + n * (b + n * p);
}

// pencils per chunk of the per-cell face-value phase ("fvc"): all pencils
// of a direction, or as many as fit under the 227 KB limit per CTA
__host__ __device__ inline int fv_chunk(int n) {
  const int np = n * n * n, nn = n * n;
  const int base = 8 * np + 4 * (n - 1) * nn;  // doubles
  int c = (28900 - base) / (8 * n);
  if (c > nn) c = nn;
  return c < 1 ? 1 : c;
}

// pencil P (in-plane index a + n b of the face-2d plane) -> its i0 = 0 node
__device__ __forceinline__ int pencil_base(int n, int d, int P) {
  return fnode(n, 2 * d, P % n, P / n);
}

// unit normal at node for face 2d+1 (node_normal_at_ijk); the face-2d normal
// is its negation (x / -m == -(x / m) exactly)
__device__ __forceinline__ void normal_at(const StageParams &P, const double *G, int np, int d,
                                          int node, double nr[3]) {
  if (G) {
    nr[0] = __ldg(G + (4 + 3 * d + 0) * np + node);
    nr[1] = __ldg(G + (4 + 3 * d + 1) * np + node);
    nr[2] = __ldg(G + (4 + 3 * d + 2) * np + node);
  } else {
    nr[0] = d == 0 ? 1. : 0.;
    nr[1] = d == 1 ? 1. : 0.;
    nr[2] = d == 2 ? 1. : 0.;
  }
}

// sqrtgdiag_d and 1/J at node
__device__ __forceinline__ double sg_at(const double *G, int np, const double *sc, int d,
                                        int node) {
  return G ? __ldg(G + (1 + d) * np + node) : sc[d];
}
__device__ __forceinline__ double ooj_at(const double *G, int np, double oojc, int node) {
  return G ? __ldg(G + node) : oojc;
}

// LLF flux (amax = 1) of the four fluxed fields for normal nr
__device__ __forceinline__ void llf4(const double *ui, const double *ua, const double nr[3],
                                     double *fn) {
  const double fi0 = -(ui[1] * nr[0] + ui[2] * nr[1] + ui[3] * nr[2]);
  const double fa0 = -(ua[1] * nr[0] + ua[2] * nr[1] + ua[3] * nr[2]);
  fn[0] = 0.5 * (fa0 + fi0 - (ua[0] - ui[0]));
#pragma unroll
  for (int l = 1; l < 4; l++) {
    const double fil = -ui[0] * nr[l - 1], fal = -ua[0] * nr[l - 1];
    fn[l] = 0.5 * (fal + fil - (ua[l] - ui[l]));
  }
}

// upwind flux (scalarwave1_numflux1d_upwind): R diag(lam+) R^-1 u_in +
// R diag(lam-) R^-1 u_adj with the characteristic matrices of the normal,
// evaluated as the matrix products in that order (so that "fvx" stays
// bit-exact), eigenvalues (1, -1, 0, 0)
__device__ void upwind4(const double *ui, const double *ua, const double nr[3], double *fn) {
  const double lam[4] = {1.0, -1.0, 0.0, 0.0};
  const double nx = nr[0], ny = nr[1], nz = nr[2];
  double lp[4][4], ln[4][4], ip[4][4], in_[4][4], sp[4][4], sn[4][4], fi[4], fa[4];
  double R[4][4], Ri[4][4];
  for (int l = 0; l < 4; l++) {
    for (int m = 0; m < 4; m++) lp[l][m] = ln[l][m] = ip[l][m] = in_[l][m] = sp[l][m] = sn[l][m] = 0.;
    fi[l] = fa[l] = 0.;
  }
  for (int l = 0; l < 4; l++) {
    if (lam[l] > 0.) lp[l][l] = lam[l];
    else ln[l][l] = lam[l];
  }
  R[0][0] = 1.0; R[0][1] = 1.0; R[0][2] = 0.0; R[0][3] = 0.0;
  R[1][0] = -nx; R[1][1] = nx; R[2][0] = -ny; R[2][1] = ny; R[3][0] = -nz; R[3][1] = nz;
  Ri[0][0] = 1.0 / 2.0; Ri[0][1] = -nx / 2.0; Ri[0][2] = -ny / 2.0; Ri[0][3] = -nz / 2.0;
  Ri[1][0] = 1.0 / 2.0; Ri[1][1] = nx / 2.0; Ri[1][2] = ny / 2.0; Ri[1][3] = nz / 2.0;
  Ri[2][0] = 0.0; Ri[3][0] = 0.0;
  if (nz != 0) {
    R[1][2] = 0.0; R[1][3] = nz; R[2][2] = nz; R[2][3] = 0.0; R[3][2] = -ny; R[3][3] = -nx;
    Ri[2][1] = -(nx * ny) / nz; Ri[2][2] = (nx * nx + nz * nz) / nz; Ri[2][3] = -ny;
    Ri[3][1] = (ny * ny + nz * nz) / nz; Ri[3][2] = -(nx * ny) / nz; Ri[3][3] = -nx;
  } else if (nx != 0) {
    R[1][2] = -nz; R[1][3] = -ny; R[2][2] = 0.0; R[2][3] = nx; R[3][2] = nx; R[3][3] = 0.0;
    Ri[2][1] = -nz; Ri[2][2] = -(ny * nz) / nx; Ri[2][3] = (nx * nx + ny * ny) / nx;
    Ri[3][1] = -ny; Ri[3][2] = (nx * nx + nz * nz) / nx; Ri[3][3] = -(ny * nz) / nx;
  } else {
    R[1][2] = 0.0; R[1][3] = ny; R[2][2] = -nz; R[2][3] = -nx; R[3][2] = ny; R[3][3] = 0.0;
    Ri[2][1] = -(nx * nz) / ny; Ri[2][2] = -nz; Ri[2][3] = (nx * nx + ny * ny) / ny;
    Ri[3][1] = (ny * ny + nz * nz) / ny; Ri[3][2] = -nx; Ri[3][3] = -(nx * nz) / ny;
  }
  for (int l = 0; l < 4; l++)
    for (int m = 0; m < 4; m++)
      for (int q = 0; q < 4; q++) {
        ip[l][m] += lp[l][q] * Ri[q][m];
        in_[l][m] += ln[l][q] * Ri[q][m];
      }
  for (int l = 0; l < 4; l++)
    for (int m = 0; m < 4; m++)
      for (int q = 0; q < 4; q++) {
        sp[l][m] += R[l][q] * ip[q][m];
        sn[l][m] += R[l][q] * in_[q][m];
      }
  for (int l = 0; l < 4; l++)
    for (int m = 0; m < 4; m++) {
      fi[l] += sp[l][m] * ui[m];
      fa[l] += sn[l][m] * ua[m];
    }
  for (int l = 0; l < 4; l++) fn[l] = fi[l] + fa[l];
}

__device__ __forceinline__ void numflux4(int kind, const double *ui, const double *ua,
                                         const double nr[3], double *fn) {
  if (kind == NMG_NUMFLUX_UPWIND) upwind4(ui, ua, nr, fn);
  else llf4(ui, ua, nr, fn);
}

// LLF flux f* through face f at face node (a, b) of element e with interior
// state ui (scalarwave1_fluxes_pt: neighbour trace, exact plane wave or the
// outgoing-radiation exterior state)
__device__ void face_fnum(const StageParams &P, int e, int f, int a, int b, const double *ui,
                          const double nrp[3], double t, double *fn) {
  const int n = P.n, np = n * n * n, nn = n * n;
  const double sg = (f & 1) ? 1. : -1.;
  double nr[3];
  for (int q = 0; q < 3; q++) nr[q] = sg > 0. ? nrp[q] : -nrp[q];
  double ua[4];
  const int nbe = __ldg(P.nb + e * 6 + f);
  if (nbe >= 0) {
    const int cd = __ldg(P.code + e * 6 + f), f2 = cd & 7, o = cd >> 3;
    if (cd & kCodeMixed) {
      const double *G = P.ghost + (size_t)__ldg(P.bslot + e * 6 + f) * 4 * nn + a + n * b;
      for (int l = 0; l < 4; l++) ua[l] = G[l * nn];
    } else {
      const int sw = o & 1, fa = (o >> 1) & 1, fb = (o >> 2) & 1;
      int aa = sw ? b : a, bb = sw ? a : b;
      aa = fa ? n - 1 - aa : aa;
      bb = fb ? n - 1 - bb : bb;
      const double *W2 = P.win + (size_t)nbe * NF * np + fnode(n, f2, aa, bb);
      for (int l = 0; l < 4; l++) ua[l] = __ldg(W2 + l * np);
    }
  } else {
    const int bs = __ldg(P.bslot + e * 6 + f), ab = a + n * b;
    if (P.bc == NMG_BC_EXACT_PLANEWAVE) {
      const double *X = P.fvbxyz + (size_t)bs * 3 * nn + ab;
      const double arg = P.k0 * X[0] + P.k1 * X[nn] + P.k2 * X[2 * nn] - P.om * t;
      double sn, cn;
      sincos(arg, &sn, &cn);
      ua[0] = -P.om * cn;
      ua[1] = P.k0 * cn;
      ua[2] = P.k1 * cn;
      ua[3] = P.k2 * cn;
    } else {
      const double cnv = ui[1] * nr[0] + ui[2] * nr[1] + ui[3] * nr[2];
      const double wo = ui[0] - cnv;
      const double pie = 0.5 * wo, cne = -0.5 * wo;
      ua[0] = pie;
      for (int l = 0; l < 3; l++) ua[1 + l] = ui[1 + l] + (cne - cnv) * nr[l];
    }
  }
  numflux4(P.numflux, ui, ua, nr, fn);
}

// J sqrtgdiag / dXb factors of node i0 of a pencil (fv.c:384-411)
__device__ __forceinline__ void jgdow(const double *G, const double *Gm, int np,
                                      const double *sc, double oojc, int d, int n, int base,
                                      int st, int i0, double wc, bool addsurf, double &JR,
                                      double &JL) {
  const int g0 = i0 > 0, lN = i0 < n - 1;
  const int ccc = base + i0 * st;
  const int cccL = base + (g0 ? i0 - 1 : i0) * st, cccR = base + (lN ? i0 : i0 - 1) * st;
  // the factors of the midpoints (indices cccR, cccL): from the midpoint
  // data when given, else those of the grid points there
  const double sgR = Gm ? __ldg(Gm + (d * 5 + 0) * np + cccR) : sg_at(G, np, sc, d, cccR);
  const double ojR = Gm ? __ldg(Gm + (d * 5 + 1) * np + cccR) : ooj_at(G, np, oojc, cccR);
  const double sgL = Gm ? __ldg(Gm + (d * 5 + 0) * np + cccL) : sg_at(G, np, sc, d, cccL);
  const double ojL = Gm ? __ldg(Gm + (d * 5 + 1) * np + cccL) : ooj_at(G, np, oojc, cccL);
  if (g0 && lN) {
    JR = sgR / (ojR * wc);
    JL = sgL / (ojL * wc);
  } else if (!g0 && lN) {
    JR = sgR / (ojR * wc);
    JL = sg_at(G, np, sc, d, ccc) / (ooj_at(G, np, oojc, ccc) * wc);
  } else if (g0 && !lN) {
    JR = sg_at(G, np, sc, d, ccc) / (ooj_at(G, np, oojc, ccc) * wc);
    JL = sgL / (ojL * wc);
  } else {
    JR = JL = sg_at(G, np, sc, d, ccc) / (ooj_at(G, np, oojc, ccc) * wc);
  }
  if (!addsurf) {
    JR = (double)lN * JR;
    JL = (double)g0 * JL;
  }
}

template <int NT, bool CELL>
__global__ void __launch_bounds__(NT) fv_kernel(const StageParams P) {
  extern __shared__ double smem[];
  const int n = P.n, np = n * n * n, nn = n * n, nm = n - 1;
  const int e = P.fvlist ? __ldg(P.fvlist + blockIdx.x) : P.ebase + (int)blockIdx.x;
  if (e >= P.nelem) return;
  double *sW = smem;             // [4][np]  pi, cx, cy, cz of w
  double *sD = sW + 4 * np;      // [4][np]  div f accumulators
  double *sF = sD + 4 * np;      // [4][nm][nn] midpoint fluxes of one direction
  __shared__ double sSc[3], sDist[6], sOoJc;
  __shared__ int sCs;
  const double t = stage_time(P);
  const bool addsurf = P.fv_extrap == NMG_FV_EXTRAP_DNFN1;
  const double r3 = P.fv_w3ratio;

  if (threadIdx.x == 0) {
    sCs = __ldg(P.cslot + e);
    for (int d = 0; d < 3; d++) sSc[d] = __ldg(P.scale + e * 3 + d);
    sOoJc = sSc[0] * sSc[1] * sSc[2];
    for (int f = 0; f < 6; f++) sDist[f] = __ldg(P.fvdist + e * 6 + f);
  }
  for (int q = threadIdx.x; q < 4 * np; q += NT) {
    sW[q] = __ldg(P.win + (size_t)e * NF * np + q);
    sD[q] = 0.;
  }
  __syncthreads();
  const double *G = sCs >= 0 ? P.fvgeo + (size_t)sCs * kGeo * np : nullptr;
  // midpoint data of a curvilinear element (affine maps: equal to the grid's)
  const double *Gm = (sCs >= 0 && P.fvmid) ? P.fvmid + (size_t)sCs * 15 * np : nullptr;
  const double oojc = sOoJc;

  double *sQ = sF + 4 * nm * nn;  // CELL: [2 faces][4 fields][n cells][chunk pencils]
  const int pch = CELL ? fv_chunk(n) : 0;

#pragma unroll 1
  for (int d = 0; d < 3; d++) {
    const int st = d == 0 ? 1 : d == 1 ? n : nn;
    if constexpr (!CELL) {
      // midpoint fluxes fnumR of midpoint im (normal at its left node)
      for (int q = threadIdx.x; q < nm * nn; q += NT) {
        const int im = q / nn, Pn = q - im * nn;
        const int base = pencil_base(n, d, Pn);
        double ui[4], ua[4];
#pragma unroll
        for (int l = 0; l < 4; l++) {
          const double *u = sW + l * np + base;
          double v[6];
#pragma unroll
          for (int j = 0; j < 6; j++) {
            const int i = im - 2 + j;
            v[j] = (i >= 0 && i < n) ? u[i * st] : 0.;
          }
          ui[l] = rec_p(P.fv_rec, n, v, im, r3);
          ua[l] = rec_m(P.fv_rec, n, v, im, r3);
        }
        double nr[3], fn[4];
        if (Gm) {
#pragma unroll
          for (int c = 0; c < 3; c++) nr[c] = __ldg(Gm + (d * 5 + 2 + c) * np + base + im * st);
        } else {
          normal_at(P, G, np, d, base + im * st, nr);
        }
        numflux4(P.numflux, ui, ua, nr, fn);
#pragma unroll
        for (int l = 0; l < 4; l++) sF[(l * nm + im) * nn + Pn] = fn[l];
      }
      __syncthreads();
    } else {
#pragma unroll 1
      for (int c0 = 0; c0 < nn; c0 += pch) {
        const int cp = min(pch, nn - c0);
        // both face values of every cell of the chunk's pencils (one set of
        // smoothness indicators per cell and field)
        for (int q = threadIdx.x; q < cp * n * 4; q += NT) {
          const int k = q % cp, lc = q / cp, c = lc % n, l = lc / n;
          const double *u = sW + l * np + pencil_base(n, d, c0 + k);
          double v[5];
#pragma unroll
          for (int j = 0; j < 5; j++) {
            const int i = c - 2 + j;
            v[j] = (i >= 0 && i < n) ? u[i * st] : 0.;
          }
          double lft, rgt;
          rec_cell(P.fv_rec, n, v, c, r3, &lft, &rgt);
          sQ[((0 * 4 + l) * n + c) * pch + k] = lft;
          sQ[((1 * 4 + l) * n + c) * pch + k] = rgt;
        }
        __syncthreads();
        // midpoint fluxes fnumR of midpoint im (normal at its left node): the
        // right face of cell im meets the left face of cell im + 1
        for (int q = threadIdx.x; q < cp * nm; q += NT) {
          const int im = q / cp, k = q - im * cp, Pn = c0 + k;
          const int base = pencil_base(n, d, Pn);
          double ui[4], ua[4];
#pragma unroll
          for (int l = 0; l < 4; l++) {
            ui[l] = sQ[((1 * 4 + l) * n + im) * pch + k];
            ua[l] = sQ[((0 * 4 + l) * n + im + 1) * pch + k];
          }
          double nr[3], fn[4];
          if (Gm) {
#pragma unroll
            for (int c = 0; c < 3; c++) nr[c] = __ldg(Gm + (d * 5 + 2 + c) * np + base + im * st);
          } else {
            normal_at(P, G, np, d, base + im * st, nr);
          }
          numflux4(P.numflux, ui, ua, nr, fn);
#pragma unroll
          for (int l = 0; l < 4; l++) sF[(l * nm + im) * nn + Pn] = fn[l];
        }
        __syncthreads();
      }
    }
    // conservative difference at every node of the direction's pencils
    for (int q = threadIdx.x; q < np; q += NT) {
      const int i0 = q / nn, Pn = q - i0 * nn;
      const int base = pencil_base(n, d, Pn);
      const int node = base + i0 * st;
      const double wc = i0 == 0 ? sDist[2 * d] : i0 == n - 1 ? sDist[2 * d + 1] : __ldg(P.fvdxb + i0);
      double JR, JL;
      jgdow(G, Gm, np, sSc, oojc, d, n, base, st, i0, wc, addsurf, JR, JL);
      double fR[4], fL[4];
      if (i0 < n - 1) {
        for (int l = 0; l < 4; l++) fR[l] = sF[(l * nm + i0) * nn + Pn];
      } else if (addsurf) {
        double ui[4], nr[3];
        for (int l = 0; l < 4; l++) ui[l] = sW[l * np + node];
        normal_at(P, G, np, d, node, nr);
        face_fnum(P, e, 2 * d + 1, Pn % n, Pn / n, ui, nr, t, fR);
      } else {
        for (int l = 0; l < 4; l++) fR[l] = 0.;
      }
      if (i0 > 0) {
        for (int l = 0; l < 4; l++) fL[l] = -sF[(l * nm + i0 - 1) * nn + Pn];
      } else if (addsurf) {
        double ui[4], nr[3];
        for (int l = 0; l < 4; l++) ui[l] = sW[l * np + node];
        normal_at(P, G, np, d, node, nr);
        face_fnum(P, e, 2 * d, Pn % n, Pn / n, ui, nr, t, fL);
      } else {
        for (int l = 0; l < 4; l++) fL[l] = 0.;
      }
      double df[4];
      for (int l = 0; l < 4; l++) df[l] = JR * fR[l] + JL * fL[l];
      if (addsurf && n > 2 && (i0 == 0 || i0 == n - 1)) {
        // dnfn extrapolation: df_face = w0 df_face + w1 df_next
        const int i1 = i0 == 0 ? 1 : n - 2;
        const double wc1 = (i1 == 0 || i1 == n - 1) ? sDist[2 * d + (i1 != 0)] : __ldg(P.fvdxb + i1);
        double JR1, JL1;
        jgdow(G, Gm, np, sSc, oojc, d, n, base, st, i1, wc1, addsurf, JR1, JL1);
        const double w0 = 1. / 0.75, w1 = 1. - w0;
        for (int l = 0; l < 4; l++) {
          const double fR1 = sF[(l * nm + i1) * nn + Pn], fL1 = -sF[(l * nm + i1 - 1) * nn + Pn];
          const double df1 = JR1 * fR1 + JL1 * fL1;
          df[l] = w0 * df[l] + w1 * df1;
        }
      }
      const double oj = ooj_at(G, np, oojc, node);
      for (int l = 0; l < 4; l++) sD[l * np + node] += df[l] * oj;
    }
    __syncthreads();
  }

  // surface terms of fin.-vol. faces when fv_divf did not add them
  if (!addsurf) {
#pragma unroll 1
    for (int d = 0; d < 3; d++) {
      for (int q = threadIdx.x; q < 2 * nn; q += NT) {
        const int s = q / nn, ab = q - s * nn, f = 2 * d + s;
        const int a = ab % n, b = ab / n, node = fnode(n, f, a, b);
        double ui[4], nr[3], fn[4];
        for (int l = 0; l < 4; l++) ui[l] = sW[l * np + node];
        normal_at(P, G, np, d, node, nr);
        face_fnum(P, e, f, a, b, ui, nr, t, fn);
        const double oow = 1. / sDist[f];
        const double gd_ow = sg_at(G, np, sSc, d, node) * oow;
        for (int l = 0; l < 4; l++) sD[l * np + node] += fn[l] * gd_ow;
      }
      __syncthreads();
    }
  }

  // r = -div f (r_phi = pi) and the RK4 stage update
  for (int q = threadIdx.x; q < NF * np; q += NT) {
    const int f = q / np, node = q - f * np;
    const size_t idx = (size_t)e * NF * np + q;
    const double r = f < 4 ? -sD[f * np + node] : sW[node];
    if (P.mode == 0) {
      P.rout[idx] = r;
    } else if (P.mode == 1) {
      const double u = __ldg(P.u0 + idx);
      P.acc[idx] = u + P.cacc * r;
      P.wout[idx] = u + P.cw * r;
    } else if (P.mode == 4) {
      P.acc[idx] = P.acc[idx] + P.cacc * r;
    } else if (P.mode == 5) {
      P.acc[idx] = __ldg(P.u0 + idx) + P.cacc * r;
    } else if (P.mode == 6) {
      P.acc[idx] = P.acc[idx] + P.cacc * r;
      const double w = __ldg(P.win + idx) + P.cw * r;
      P.wout[idx] = 0.75 * __ldg(P.u0 + idx) + 0.25 * w;
    } else {
      P.acc[idx] = P.acc[idx] + P.cacc * r;
      P.wout[idx] = __ldg(P.u0 + idx) + P.cw * r;
    }
  }
}

template <int NT, bool CELL>
cudaError_t launch_fv(const StageParams &P, cudaStream_t st) {
  const size_t smem = fv_smem(P.n) + (CELL ? sizeof(double) * 8 * P.n * fv_chunk(P.n) : 0);
  if (P.nelem == 0)
    return cudaFuncSetAttribute(fv_kernel<NT, CELL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)smem);
  const int grid = P.fvlist ? P.nfvel : (P.ecount > 0 ? P.ecount : P.nelem);
  if (grid == 0) return cudaSuccess;
  fv_kernel<NT, CELL><<<grid, NT, smem, st>>>(P);
  return cudaGetLastError();
}

}  // namespace

int variants(int n, Variant *out, int cap) {
  if (n < 2 || n > kFvMaxN || cap < 3) return 0;
  out[0] = {NMG_FV_NAME, 1, 128, launch_fv<128, false>};
  out[1] = {NMG_FV_NAME, 1, 256, launch_fv<256, false>};
  out[2] = {NMG_FV_NAME, 1, 512, launch_fv<512, false>};
#ifdef NMG_FV_FAST
  // "fvc": the per-cell face-value phase (fewer FP64 instructions, more
  // shared memory and barriers); the autotuner chooses
  if (cap < 6) return 3;
  out[3] = {"fvc", 1, 128, launch_fv<128, true>};
  out[4] = {"fvc", 1, 256, launch_fv<256, true>};
  out[5] = {"fvc", 1, 512, launch_fv<512, true>};
  return 6;
#else
  return 3;
#endif
}

}  // namespace NMG_FVNS

#ifndef NMG_FV_FAST
namespace fv_fast {
int variants(int n, Variant *out, int cap);
}

size_t fv_smem(int n) {
  const size_t np = (size_t)n * n * n, nn = (size_t)n * n;
  return (8 * np + 4 * (n - 1) * nn) * sizeof(double);
}

// the fast variants first, then the exact ones
int fv_variants(int n, Variant *out, int cap) {
  int k = fv_fast::variants(n, out, cap);
  return k + fv_exact::variants(n, out + k, cap - k);
}

namespace {
// One thread per (slot, field, face node): the neighbour's face plane
// interpolated to this face's node, sum_b sum_a v(a,b) B1[a] B2[b] with the
// neighbour's basis (basis_array_interp2d, src/main/basis/interpolate.c:296),
// rounded in that order (this file has no FMA contraction).
__global__ void __launch_bounds__(256) ghost_kernel(int nghost, int n, const int *gtab,
                                                   const unsigned char *isfv, const double *M,
                                                   const double *win, double *ghost) {
  const int nn = n * n, np = nn * n;
  const int64_t total = (int64_t)nghost * 4 * nn;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total;
       q += (int64_t)gridDim.x * blockDim.x) {
    const int g = (int)(q / (4 * nn)), rem = (int)(q - (int64_t)g * 4 * nn);
    const int l = rem / nn, ab = rem - l * nn, a = ab % n, b = ab / n;
    const int e2 = __ldg(gtab + 4 * g + 2), cd = __ldg(gtab + 4 * g + 3);
    const int f2 = cd & 7, o = (cd >> 3) & 7;
    const int sw = o & 1, fa = (o >> 1) & 1, fb = (o >> 2) & 1;
    int aa = sw ? b : a, bb = sw ? a : b;
    aa = fa ? n - 1 - aa : aa;
    bb = fb ? n - 1 - bb : bb;
    // basis of the neighbour's points at this face's point positions
    const double *Mk = M + (isfv[e2] ? 1 : 0) * nn;
    const double *v = win + ((size_t)e2 * NF + l) * np;
    double sum = 0.;
    for (int k = 0; k < n; k++) {
      const double B2 = __ldg(Mk + bb * n + k);
      for (int j = 0; j < n; j++)
        sum += __ldg(v + fv_exact::fnode(n, f2, j, k)) * __ldg(Mk + aa * n + j) * B2;
    }
    ghost[(size_t)g * 4 * nn + l * nn + ab] = sum;
  }
}
}  // namespace

namespace {
// One thread per (slot, field, face node) of a non-conforming face: each
// contribution is the source face's plane interpolated at the node,
// sum_b sum_a v(a,b) B1[a] B2[b] (basis_interp2d_toIpoints), and the node
// takes their average (set_ajsurf_vl, src/main/amr/surface.c:1320-1337),
// rounded in that order (this file has no FMA contraction).
__global__ void __launch_bounds__(256) hang_kernel(int nhang, int n, const int *hoff,
                                                  const int *hsrc, const double *hw,
                                                  const double *win, double *ghost) {
  const int nn = n * n, np = nn * n;
  const int64_t total = (int64_t)nhang * 4 * nn;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total;
       q += (int64_t)gridDim.x * blockDim.x) {
    const int h = (int)(q / (4 * nn)), rem = (int)(q - (int64_t)h * 4 * nn);
    const int l = rem / nn, ab = rem - l * nn;
    const int c0 = __ldg(hoff + (size_t)h * nn + ab), c1 = __ldg(hoff + (size_t)h * nn + ab + 1);
    double acc = 0.;
    for (int c = c0; c < c1; c++) {
      const int e2 = __ldg(hsrc + 2 * c), f2 = __ldg(hsrc + 2 * c + 1);
      const double *B1 = hw + (size_t)c * 2 * n, *B2 = B1 + n;
      const double *v = win + ((size_t)e2 * NF + l) * np;
      double sum = 0.;
      for (int k = 0; k < n; k++) {
        const double b2 = __ldg(B2 + k);
        for (int j = 0; j < n; j++)
          sum += __ldg(v + fv_exact::fnode(n, f2, j, k)) * __ldg(B1 + j) * b2;
      }
      acc += sum;
    }
    if (c1 - c0 > 1) acc /= (c1 - c0);
    ghost[(size_t)h * 4 * nn + l * nn + ab] = acc;
  }
}

// Transpose of the non-conforming traces for the adjoint: the neighbour part
// of a face lift (g d pi + gn . d c, gn d pi + g d c) on slot h's face, with
// d the trace, becomes, per field, the adjoint tb = (g rbar_pi + gn . rbar_c,
// gn rbar_pi + g rbar_c) at the owner's face node; every trace value is a
// weighted sum of source-face values, so each source-face node of each
// non-conforming face gathers sum w tb over the (slot, node) pairs that read
// it (toff/tsrc/tw: that list, built on the host from the forward one).
// The sums land in the slot of the source face, where the transposed stage
// kernel adds them to the face's interior-side terms.
__global__ void __launch_bounds__(256) hang_adj_kernel(int nhang, int n, const int *toff,
                                                      const int *tsrc, const double *tw,
                                                      const int *hface, const int *cslot,
                                                      const double *fac, const double *gcart,
                                                      const double *rbar, double *out) {
  const int nn = n * n, np = nn * n;
  const int64_t total = (int64_t)nhang * 4 * nn;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total;
       q += (int64_t)gridDim.x * blockDim.x) {
    const int h2 = (int)(q / (4 * nn)), rem = (int)(q - (int64_t)h2 * 4 * nn);
    const int l = rem / nn, jk = rem - l * nn;
    const int i0 = __ldg(toff + (size_t)h2 * nn + jk), i1 = __ldg(toff + (size_t)h2 * nn + jk + 1);
    double acc = 0.;
    for (int i = i0; i < i1; i++) {
      const int src = __ldg(tsrc + i), h = src / nn, t = src - h * nn;
      const int e = __ldg(hface + 2 * h), f = __ldg(hface + 2 * h + 1), d = f >> 1;
      const int node = fv_exact::fnode(n, f, t % n, t / n);
      const double *R = rbar + (size_t)e * NF * np + node;
      const double rp = __ldg(R), r0 = __ldg(R + np), r1 = __ldg(R + 2 * np), r2 = __ldg(R + 3 * np);
      double gn0, gn1, gn2, g;
      const int cs = __ldg(cslot + e);
      if (cs < 0) {
        g = __ldg(gcart + e * 3 + d);
        const double sg = (f & 1) ? g : -g;
        gn0 = d == 0 ? sg : 0.;
        gn1 = d == 1 ? sg : 0.;
        gn2 = d == 2 ? sg : 0.;
      } else {
        const double *F4 = fac + (((size_t)cs * 6 + f) * nn + t) * 4;
        gn0 = __ldg(F4); gn1 = __ldg(F4 + 1); gn2 = __ldg(F4 + 2); g = __ldg(F4 + 3);
      }
      double tb;
      if (l == 0) tb = g * rp + (gn0 * r0 + gn1 * r1 + gn2 * r2);
      else if (l == 1) tb = gn0 * rp + g * r0;
      else if (l == 2) tb = gn1 * rp + g * r1;
      else tb = gn2 * rp + g * r2;
      acc += __ldg(tw + i) * tb;
    }
    out[(size_t)h2 * 4 * nn + l * nn + jk] = acc;
  }
}
}  // namespace

cudaError_t hang_adj_launch(int nhang, int n, const int *toff, const int *tsrc, const double *tw,
                            const int *hface, const int *cslot, const double *fac,
                            const double *gcart, const double *rbar, double *out,
                            cudaStream_t st) {
  if (nhang <= 0) return cudaSuccess;
  const int64_t total = (int64_t)nhang * 4 * n * n;
  const int grid = (int)std::min<int64_t>((total + 255) / 256, 152 * 16);
  hang_adj_kernel<<<grid, 256, 0, st>>>(nhang, n, toff, tsrc, tw, hface, cslot, fac, gcart, rbar,
                                        out);
  return cudaGetLastError();
}

cudaError_t hang_launch(int nhang, int n, const int *hoff, const int *hsrc, const double *hw,
                        const double *win, double *ghost, cudaStream_t st) {
  if (nhang <= 0) return cudaSuccess;
  const int64_t total = (int64_t)nhang * 4 * n * n;
  const int grid = (int)std::min<int64_t>((total + 255) / 256, 152 * 16);
  hang_kernel<<<grid, 256, 0, st>>>(nhang, n, hoff, hsrc, hw, win, ghost);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// element switches and trouble indicators
// ---------------------------------------------------------------------------
namespace {
// out = M along direction d of in (one field of one element, n^3 values)
__device__ void apply_dir(int n, const double *M, int d, const double *in, double *out) {
  const int np = n * n * n, st = d == 0 ? 1 : d == 1 ? n : n * n;
  for (int q = threadIdx.x; q < np; q += blockDim.x) {
    const int i = d == 0 ? q % n : d == 1 ? (q / n) % n : q / (n * n);
    const double *line = in + q - i * st;
    double s = 0.;
    for (int j = 0; j < n; j++) s += M[i * n + j] * line[j * st];
    out[q] = s;
  }
  __syncthreads();
}

// u of the listed elements <- (M x M x M) u, all five fields, in place
__global__ void __launch_bounds__(256) convert_kernel(int n, const int *list, const double *M,
                                                     double *u) {
  extern __shared__ double sm[];
  const int np = n * n * n;
  double *a = sm, *b = sm + np, *sM = sm + 2 * np;
  for (int q = threadIdx.x; q < n * n; q += blockDim.x) sM[q] = M[q];
  const int e = __ldg(list + blockIdx.x);
  for (int l = 0; l < NF; l++) {
    double *v = u + ((size_t)e * NF + l) * np;
    __syncthreads();
    for (int q = threadIdx.x; q < np; q += blockDim.x) a[q] = v[q];
    __syncthreads();
    apply_dir(n, sM, 0, a, b);
    apply_dir(n, sM, 1, b, a);
    apply_dir(n, sM, 2, a, b);
    for (int q = threadIdx.x; q < np; q += blockDim.x) v[q] = b[q];
  }
}

// Exponential filter of every field of every element (expfilter_var,
// src/main/basis/filter.c:15-96): u -> u J^p, (F x F x F) u with
// F = S diag(exp(-alp (k/N)^s)) A in the element's point type, u -> u J^-p
// (1/J = det(dXb/dx) per node: oojdg on curvilinear DG elements, the FV
// geometry on FV ones, constant on Cartesian ones).
__global__ void __launch_bounds__(256) filter_kernel(int n, double *u, const unsigned char *isfv,
                                                    const double *F, const int *cslot,
                                                    const double *oojdg, const double *fvgeo,
                                                    const double *scale, int jpow,
                                                    int filter_fv, int allfv) {
  extern __shared__ double sm[];
  const int np = n * n * n, nn = n * n;
  double *a = sm, *b = sm + np, *sM = sm + 2 * np, *sJ = sm + 2 * np + nn;
  const int e = blockIdx.x;
  const bool efv = allfv || (isfv && isfv[e]);
  if (efv && !filter_fv) return;
  for (int q = threadIdx.x; q < nn; q += blockDim.x) sM[q] = F[(efv ? nn : 0) + q];
  const int cs = __ldg(cslot + e);
  const double ojc = __ldg(scale + 3 * e) * __ldg(scale + 3 * e + 1) * __ldg(scale + 3 * e + 2);
  for (int q = threadIdx.x; q < np && jpow; q += blockDim.x)
    sJ[q] = cs < 0 ? ojc : efv ? __ldg(fvgeo + (size_t)cs * 13 * np + q)
                               : __ldg(oojdg + (size_t)cs * np + q);
  for (int l = 0; l < NF; l++) {
    double *v = u + ((size_t)e * NF + l) * np;
    __syncthreads();
    for (int q = threadIdx.x; q < np; q += blockDim.x) a[q] = jpow ? v[q] / sJ[q] : v[q];
    __syncthreads();
    apply_dir(n, sM, 0, a, b);
    apply_dir(n, sM, 1, b, a);
    apply_dir(n, sM, 2, a, b);
    for (int q = threadIdx.x; q < np; q += blockDim.x) v[q] = jpow ? b[q] * sJ[q] : b[q];
  }
}

// min and max of each field over each element (limdata_MRS)
__global__ void __launch_bounds__(256) minmax_kernel(int n, int nelem, const double *u,
                                                    double *mm) {
  __shared__ double smin[256], smax[256];
  const int np = n * n * n;
  const int e = blockIdx.x;
  if (e >= nelem) return;
  for (int l = 0; l < NF; l++) {
    const double *v = u + ((size_t)e * NF + l) * np;
    double lo = v[threadIdx.x < np ? threadIdx.x : 0], hi = lo;
    for (int q = threadIdx.x; q < np; q += blockDim.x) {
      lo = fmin(lo, v[q]);
      hi = fmax(hi, v[q]);
    }
    smin[threadIdx.x] = lo;
    smax[threadIdx.x] = hi;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
      if (threadIdx.x < w) {
        smin[threadIdx.x] = fmin(smin[threadIdx.x], smin[threadIdx.x + w]);
        smax[threadIdx.x] = fmax(smax[threadIdx.x], smax[threadIdx.x + w]);
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      mm[((size_t)e * NF + l) * 2] = smin[0];
      mm[((size_t)e * NF + l) * 2 + 1] = smax[0];
    }
    __syncthreads();
  }
}

// Trouble flag of each element: the relaxed discrete maximum principle
// (evolve_RDMP_trouble, src/main/evolve/trouble.c:438-503: u must stay
// within [min - delta, max + delta] of u_p over the element and its face
// neighbours, delta = deltafac max(delta0, epsilon (max - min))) and, on DG
// elements, Persson's modal indicator (evolve_Persson_array_indicator,
// trouble.c:505-564) above persson_max.  Flag: DG troubled 1, DG fine 0,
// finite-volume troubled 0, finite-volume fine -1.
__global__ void __launch_bounds__(256) trouble_kernel(int n, int nelem, const double *u,
                                                     const double *mm, const int *nb,
                                                     const unsigned char *isfv, const double *A,
                                                     double deltafac, double delta0,
                                                     double epsilon, double persson_max,
                                                     double uscale, int *flag, double *pers) {
  extern __shared__ double sm[];
  const int np = n * n * n, nn = n * n;
  double *a = sm, *b = sm + np, *sA = sm + 2 * np;
  __shared__ double red[2][256];
  __shared__ int bad;
  const int e = blockIdx.x;
  if (e >= nelem) return;
  for (int q = threadIdx.x; q < nn; q += blockDim.x) sA[q] = A[q];
  if (threadIdx.x == 0) bad = 0;
  const bool efv = isfv && isfv[e];
  __syncthreads();
  for (int l = 0; l < NF; l++) {
    double lo = mm[((size_t)e * NF + l) * 2], hi = mm[((size_t)e * NF + l) * 2 + 1];
    for (int f = 0; f < 6; f++) {
      const int e2 = __ldg(nb + e * 6 + f);
      if (e2 < 0) continue;
      const double lo2 = mm[((size_t)e2 * NF + l) * 2], hi2 = mm[((size_t)e2 * NF + l) * 2 + 1];
      if (lo2 < lo) lo = lo2;
      if (hi2 > hi) hi = hi2;
    }
    const double delta = deltafac * fmax(delta0, epsilon * (hi - lo));
    const double lower = lo - delta, upper = hi + delta;
    const double *v = u + ((size_t)e * NF + l) * np;
    for (int q = threadIdx.x; q < np; q += blockDim.x)
      if (v[q] < lower || v[q] > upper) bad = 1;
    if (!efv) {  // Persson's indicator of this field
      __syncthreads();
      for (int q = threadIdx.x; q < np; q += blockDim.x) a[q] = v[q];
      __syncthreads();
      apply_dir(n, sA, 0, a, b);
      apply_dir(n, sA, 1, b, a);
      apply_dir(n, sA, 2, a, b);
      if (threadIdx.x == 0 && uscale >= 0.) b[0] = uscale * 2. * sqrt(2.);
      __syncthreads();
      double s2 = 0., sh = 0.;
      for (int q = threadIdx.x; q < np; q += blockDim.x) {
        const int i = q % n, j = (q / n) % n, k = q / nn;
        const double co = b[q];
        s2 += co * co;
        if ((i == n - 1 && n > 1) || (j == n - 1 && n > 1) || (k == n - 1 && n > 1)) sh += co * co;
      }
      red[0][threadIdx.x] = s2;
      red[1][threadIdx.x] = sh;
      __syncthreads();
      for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
          red[0][threadIdx.x] += red[0][threadIdx.x + w];
          red[1][threadIdx.x] += red[1][threadIdx.x + w];
        }
        __syncthreads();
      }
      if (threadIdx.x == 0) {
        const double se = log10(red[1][0] / (red[0][0] + 2.2250738585072014e-308) + 1e-50);
        if (pers) pers[(size_t)e * NF + l] = se;
        if (se > persson_max) bad = 1;
      }
    } else if (threadIdx.x == 0 && pers) {
      pers[(size_t)e * NF + l] = 0.;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) flag[e] = efv ? (bad ? 0 : -1) : (bad ? 1 : 0);
}
}  // namespace

// MRS limiter (limdata_MRS / limiter_MRS, src/main/limiter/limiter.c:61-204):
// per element and field the node average (the LGL or uniform quadrature
// along x, then y, then z, times 1/8: var_nodeaverage, src/main/basis/
// basis.c:462-510), the minimum and the maximum.
__global__ void __launch_bounds__(256) limdata_kernel(int n, const double *u,
                                                     const unsigned char *isfv, int allfv,
                                                     const double *wl, const double *wu,
                                                     double *lim) {
  __shared__ double s1[256], red[2][256];
  const int np = n * n * n, nn = n * n, e = blockIdx.x;
  const bool efv = allfv || (isfv && isfv[e]);
  const double *w = efv ? wu : wl;
  for (int l = 0; l < NF; l++) {
    const double *v = u + ((size_t)e * NF + l) * np;
    for (int q = threadIdx.x; q < nn; q += blockDim.x) {  // q = j + n k
      double s = 0.;
      for (int i = 0; i < n; i++) s += __ldg(w + i) * v[i + n * q];
      s1[q] = s;
    }
    double lo = v[0], hi = v[0];
    for (int q = threadIdx.x; q < np; q += blockDim.x) {
      lo = fmin(lo, v[q]);
      hi = fmax(hi, v[q]);
    }
    red[0][threadIdx.x] = lo;
    red[1][threadIdx.x] = hi;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
      if (threadIdx.x < h) {
        red[0][threadIdx.x] = fmin(red[0][threadIdx.x], red[0][threadIdx.x + h]);
        red[1][threadIdx.x] = fmax(red[1][threadIdx.x], red[1][threadIdx.x + h]);
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      double I = 0.;
      for (int k = 0; k < n; k++) {
        double t = 0.;
        for (int j = 0; j < n; j++) t += __ldg(w + j) * s1[j + n * k];
        I += __ldg(w + k) * t;
      }
      double *L = lim + ((size_t)e * NF + l) * 3;
      L[0] = I * 0.125;
      L[1] = red[0][0];
      L[2] = red[1][0];
    }
    __syncthreads();
  }
}

__device__ __forceinline__ double mrs_theta(double M, double wbar, double wM) {
  const double den = wM - wbar;
  if (den == 0.) return 1.;
  const double y = (M - wbar) / den;
  if (y < 0.) return 0.;
  return fmin(y / 1.1, 1.);
}

// u <- ubar + theta (u - ubar) with theta = min(1, min over fields of the
// MRS ratios against the neighbours' extrema widened by alpha h^1.5)
__global__ void __launch_bounds__(256) limiter_kernel(int n, double *u, const double *lim,
                                                     const int *nboff, const int *nbl,
                                                     const double *alpha_h, int *limited) {
  __shared__ double sth;
  const int np = n * n * n, e = blockIdx.x;
  if (threadIdx.x == 0) {
    double thM = DBL_MAX, thm = DBL_MAX;
    const double ah = __ldg(alpha_h + e);
    for (int l = 0; l < NF; l++) {
      const double *L = lim + ((size_t)e * NF + l) * 3;
      const double wbar = L[0], wmi = L[1], wMi = L[2];
      double Mi = -DBL_MAX, mi = DBL_MAX;
      for (int k = __ldg(nboff + 6 * e); k < __ldg(nboff + 6 * e + 6); k++) {
        const double *N = lim + ((size_t)__ldg(nbl + k) * NF + l) * 3;
        if (N[1] < mi) mi = N[1];
        if (N[2] > Mi) Mi = N[2];
      }
      mi = fmin(wbar - ah, mi);
      Mi = fmax(wbar + ah, Mi);
      const double a = mrs_theta(Mi, wbar, wMi), b = mrs_theta(mi, wbar, wmi);
      if (a < thM) thM = a;
      if (b < thm) thm = b;
    }
    sth = fmin(1., fmin(thm, thM));
    limited[e] = sth < 1. ? 1 : 0;
  }
  __syncthreads();
  const double th = sth;
  if (th >= 1.) return;
  for (int q = threadIdx.x; q < NF * np; q += blockDim.x) {
    const int l = q / np;
    const double qbar = lim[((size_t)e * NF + l) * 3];
    double *v = u + (size_t)e * NF * np + q;
    *v = qbar + th * (*v - qbar);
  }
}

// minmodB limiter (limdata_c000_100_010_001 / limiter_minmodB, src/main/
// limiter/limiter.c:201-380).  Products and sums are rounded one by one
// (no contraction into FMAs) in the oracle's order, so that the limiter's
// decisions and outputs are reproducible from the same input bit for bit.
//
// Data: the coefficients c000, c100, c010, c001 of every element's
// normalised-Legendre expansion, analysis along x, then y, then z
// (basis_array_analysis3, src/main/basis/basis.c:183-188).  ana = [typ][2][n]
// rows 0 and 1 of the analysis matrix, typ 0 LGL and 1 equally spaced.
__global__ void __launch_bounds__(256) mmb_limdata_kernel(int n, const double *u,
                                                         const unsigned char *isfv, int allfv,
                                                         const double *ana, double *lim) {
  __shared__ double t0[256], t1[256], s3[3][16];
  const int np = n * n * n, nn = n * n, e = blockIdx.x;
  const bool efv = allfv || (isfv && isfv[e]);
  const double *A0 = ana + (efv ? 2 * n : 0), *A1 = A0 + n;
  for (int l = 0; l < NF; l++) {
    const double *v = u + ((size_t)e * NF + l) * np;
    for (int q = threadIdx.x; q < nn; q += blockDim.x) {  // q = j + n k
      double a0 = 0., a1 = 0.;
      for (int i = 0; i < n; i++) {
        const double x = v[i + n * q];
        a0 = __dadd_rn(a0, __dmul_rn(__ldg(A0 + i), x));
        a1 = __dadd_rn(a1, __dmul_rn(__ldg(A1 + i), x));
      }
      t0[q] = a0;
      t1[q] = a1;
    }
    __syncthreads();
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
      double s00 = 0., s10 = 0., s01 = 0.;
      for (int j = 0; j < n; j++) {
        s00 = __dadd_rn(s00, __dmul_rn(__ldg(A0 + j), t0[j + n * k]));
        s10 = __dadd_rn(s10, __dmul_rn(__ldg(A0 + j), t1[j + n * k]));
        s01 = __dadd_rn(s01, __dmul_rn(__ldg(A1 + j), t0[j + n * k]));
      }
      s3[0][k] = s00;
      s3[1][k] = s10;
      s3[2][k] = s01;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double c000 = 0., c100 = 0., c010 = 0., c001 = 0.;
      for (int k = 0; k < n; k++) {
        c000 = __dadd_rn(c000, __dmul_rn(__ldg(A0 + k), s3[0][k]));
        c100 = __dadd_rn(c100, __dmul_rn(__ldg(A0 + k), s3[1][k]));
        c010 = __dadd_rn(c010, __dmul_rn(__ldg(A0 + k), s3[2][k]));
        c001 = __dadd_rn(c001, __dmul_rn(__ldg(A1 + k), s3[0][k]));
      }
      double *L = lim + ((size_t)e * NF + l) * 4;
      L[0] = c000;
      L[1] = c100;
      L[2] = c010;
      L[3] = c001;
    }
    __syncthreads();
  }
}

__device__ __forceinline__ double mmb_minmod3(double a, double b, double c) {
  if (__dmul_rn(a, b) >= 0. && __dmul_rn(b, c) >= 0.)
    return (a > 0. ? 1. : -1.) * fmin(fabs(a), fmin(fabs(b), fabs(c)));
  return 0.;
}

__device__ __forceinline__ double mmb_minmod3b(double a, double b, double c, double bound) {
  return fabs(a) <= bound ? a : mmb_minmod3(a, b, c);
}

// dequal: equal within the absolute tolerance 1e-10
// (src/main/main/nmesh_main.h:32-34)
__device__ __forceinline__ bool mmb_dequal(double a, double b) {
  return !(a < __dadd_rn(b, -1e-10) || b < __dadd_rn(a, -1e-10));
}

// per element and field: face averages w0[f] (mean of the neighbours' c000
// across face f, foff = [E*6+1] CSR over nbl; 0 on outer faces), bound
// mt_h (= alpha h) times the mean |w0[f]| if scale_bound, slopes limited by
// minmod3B against bos3 (= beta/sqrt3) times the jumps of the averages;
// where a slope moves by more than 1e-10 the field becomes c000 plus the
// three limited linear modes (synthesis along x, y, z; syn = [typ][2][n]
// columns 0 and 1 of the synthesis matrix).  limited[e]: any field limited.
__global__ void __launch_bounds__(256) mmb_limiter_kernel(
    int n, double *u, const unsigned char *isfv, int allfv, const double *syn, const double *lim,
    const int *foff, const int *nbl, const double *mt_h, double bos3, int scale_bound,
    int *limited) {
  __shared__ double coef[NF][4];
  __shared__ int flag[NF];
  const int np = n * n * n, e = blockIdx.x;
  const int l = threadIdx.x;
  if (l < NF) {
    double w0[6], w0L1 = 0.;
    for (int f = 0; f < 6; f++) {
      const int b = __ldg(foff + 6 * e + f), z = __ldg(foff + 6 * e + f + 1);
      double av = 0.;
      for (int k = b; k < z; k++)
        av = __dadd_rn(av, lim[((size_t)__ldg(nbl + k) * NF + l) * 4]);
      if (z > b) av = __ddiv_rn(av, (double)(z - b));
      w0[f] = av;
      w0L1 = __dadd_rn(w0L1, __dmul_rn(fabs(av), 0.166666666666667));
    }
    const double *L = lim + ((size_t)e * NF + l) * 4;
    const double w0c = L[0];
    const double mh = __ldg(mt_h + e);
    const double bound = scale_bound ? __dmul_rn(mh, w0L1) : mh;
    double wl[3];
    bool lim_any = false;
    for (int d = 0; d < 3; d++) {
      const double lo = __dmul_rn(bos3, __dadd_rn(w0c, -w0[2 * d]));
      const double hi = __dmul_rn(bos3, __dadd_rn(w0[2 * d + 1], -w0c));
      wl[d] = mmb_minmod3b(L[1 + d], lo, hi, bound);
      lim_any |= !mmb_dequal(wl[d], L[1 + d]);
    }
    coef[l][0] = w0c;
    coef[l][1] = wl[0];
    coef[l][2] = wl[1];
    coef[l][3] = wl[2];
    flag[l] = lim_any ? 1 : 0;
  }
  __syncthreads();
  int any = 0;
  for (int k = 0; k < NF; k++) any |= flag[k];
  if (threadIdx.x == 0) limited[e] = any;
  if (!any) return;
  const bool efv = allfv || (isfv && isfv[e]);
  const double *S0 = syn + (efv ? 2 * n : 0), *S1 = S0 + n;
  for (int q = threadIdx.x; q < NF * np; q += blockDim.x) {
    const int f = q / np, p = q - f * np;
    if (!flag[f]) continue;
    const int i = p % n, j = (p / n) % n, k = p / (n * n);
    const double c0 = coef[f][0], cx = coef[f][1], cy = coef[f][2], cz = coef[f][3];
    const double tx0 = __dadd_rn(__dmul_rn(__ldg(S0 + i), c0), __dmul_rn(__ldg(S1 + i), cx));
    const double tx1 = __dmul_rn(__ldg(S0 + i), cy), tx2 = __dmul_rn(__ldg(S0 + i), cz);
    const double ty0 = __dadd_rn(__dmul_rn(__ldg(S0 + j), tx0), __dmul_rn(__ldg(S1 + j), tx1));
    const double ty1 = __dmul_rn(__ldg(S0 + j), tx2);
    u[(size_t)e * NF * np + q] =
        __dadd_rn(__dmul_rn(__ldg(S0 + k), ty0), __dmul_rn(__ldg(S1 + k), ty1));
  }
}

cudaError_t mmb_limiter_launch(int n, int nelem, double *u, const unsigned char *isfv, int allfv,
                               const double *ana, const double *syn, double *lim,
                               const int *foff, const int *nbl, const double *mt_h, double bos3,
                               int scale_bound, int *limited, cudaStream_t st) {
  if (nelem <= 0) return cudaSuccess;
  if (n < 2 || n > 16) return cudaErrorInvalidValue;
  mmb_limdata_kernel<<<nelem, 256, 0, st>>>(n, u, isfv, allfv, ana, lim);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  mmb_limiter_kernel<<<nelem, 256, 0, st>>>(n, u, isfv, allfv, syn, lim, foff, nbl, mt_h, bos3,
                                            scale_bound, limited);
  return cudaGetLastError();
}

size_t filter_smem(int n) { return sizeof(double) * (3 * (size_t)n * n * n + (size_t)n * n); }

cudaError_t filter_prepare(int n) {
  return cudaFuncSetAttribute(filter_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)filter_smem(n));
}

cudaError_t limiter_launch(int n, int nelem, double *u, const unsigned char *isfv, int allfv,
                           const double *wl, const double *wu, double *lim, const int *nboff,
                           const int *nbl, const double *alpha_h, int *limited, cudaStream_t st) {
  if (nelem <= 0) return cudaSuccess;
  limdata_kernel<<<nelem, 256, 0, st>>>(n, u, isfv, allfv, wl, wu, lim);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  limiter_kernel<<<nelem, 256, 0, st>>>(n, u, lim, nboff, nbl, alpha_h, limited);
  return cudaGetLastError();
}

cudaError_t filter_launch(int n, int nelem, double *u, const unsigned char *isfv, const double *F,
                          const int *cslot, const double *oojdg, const double *fvgeo,
                          const double *scale, int jpow, int filter_fv, int allfv,
                          cudaStream_t st) {
  if (nelem <= 0) return cudaSuccess;
  filter_kernel<<<nelem, 256, filter_smem(n), st>>>(n, u, isfv, F, cslot, oojdg, fvgeo, scale,
                                                    jpow, filter_fv, allfv);
  return cudaGetLastError();
}

cudaError_t convert_launch(int n, const int *list, int count, const double *M, double *u,
                           cudaStream_t st) {
  if (count <= 0) return cudaSuccess;
  const size_t smem = sizeof(double) * (2 * (size_t)n * n * n + (size_t)n * n);
  cudaError_t e = cudaFuncSetAttribute(convert_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  convert_kernel<<<count, 256, smem, st>>>(n, list, M, u);
  return cudaGetLastError();
}

cudaError_t trouble_launch(int n, int nelem, const double *u, const double *u_p, double *mm,
                           const int *nb, const unsigned char *isfv, const double *A,
                           double deltafac, double delta0, double epsilon, double persson_max,
                           double uscale, int *flag, double *pers, cudaStream_t st) {
  minmax_kernel<<<nelem, 256, 0, st>>>(n, nelem, u_p, mm);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const size_t smem = sizeof(double) * (2 * (size_t)n * n * n + (size_t)n * n);
  e = cudaFuncSetAttribute(trouble_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  trouble_kernel<<<nelem, 256, smem, st>>>(n, nelem, u, mm, nb, isfv, A, deltafac, delta0,
                                           epsilon, persson_max, uscale, flag, pers);
  return cudaGetLastError();
}

cudaError_t ghost_launch(int nghost, int n, const int *gtab, const unsigned char *isfv,
                         const double *M, const double *win, double *ghost, cudaStream_t st) {
  if (nghost <= 0) return cudaSuccess;
  const int64_t total = (int64_t)nghost * 4 * n * n;
  const int grid = (int)std::min<int64_t>((total + 255) / 256, 152 * 16);
  ghost_kernel<<<grid, 256, 0, st>>>(nghost, n, gtab, isfv, M, win, ghost);
  return cudaGetLastError();
}
#endif

}  // namespace nmgk
