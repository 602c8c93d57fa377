// stage.cuh -- parameters and shared device code of the fused DG RHS + RK4
// stage kernels (scalarwave1, FP64).
//
// Reference semantics (paths within nmeshsource/nmesh):
//   volume terms  src/tests/scalarwave1/scalarwave1.c:62-134,242-284 with
//                 src/main/coordinates/derivs.c:154-181,756-815
//   face terms    src/tests/scalarwave1/scalarwave1.c:139-209,287-321 with
//                 src/main/dg/dg.c:30-151 and src/main/dg/numflux1d.c:85-112
//   stage update  src/main/evolve/RungeKutta.c:19-82
//
// r_pi = div c, r_c = grad pi (the flux of the first-order wave is
// f_pi^i = -c_i, f_{c_j}^i = -pi delta^i_j, scalarwave1.c:39-48) plus, on
// face nodes, the LLF lift (f* - f_in) sqrtgdiag / w_end with the wave
// speed 1: r_pi += g (dpi + dc.n), r_c += g (dc + dpi n), where d = exterior
// minus interior and g = sqrtgdiag / (2 w_end).  r_phi = pi.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>

#include "../../include/nmg.h"

#define NF 5
#define NMAX 12

namespace nmgk {

struct StageParams {
  int nelem;
  int ebase, ecount;    // element range of this launch (ecount 0: all nelem)
  const int *elist;     // if set: the launch's elements are elist[ebase .. ebase+ecount)
  const double *win;    // w read by the RHS (neighbour traces too)
  const double *u0;     // u at the start of the step
  double *acc;          // u accumulator
  double *wout;         // next stage's w
  double *rout;         // RHS output (mode 0)
  int mode;             // 0: r only; 1..4: RK4 stage (1: acc = u0 + cacc r,
                        // w = u0 + cw r; 2, 3: acc += cacc r, w = u0 + cw r;
                        // 4: acc += cacc r); 5: acc = u0 + cacc r (Euler);
                        // 6: acc += cacc r, w = 0.75 u0 + 0.25 (win + cw r)
                        // (sspRK3 stage 2)
  double t;             // time of this RHS evaluation
  double cacc, cw;      // stage coefficients: acc += cacc*r, wout = u0 + cw*r
  const double *tdev;   // if non-null: step time read from tdev[*stepdev]
  const int *stepdev;
  double tofs_dt;       // stage time = step time + tofs_dt
  // mesh
  const int *nb;        // [E][6] neighbour element, -1 on outer faces
  const int *code;      // [E][6] neighbour face | orientation << 3
  const int *cslot;     // [E] curvilinear slot or -1 (Cartesian)
  const int *bslot;     // [E][6] outer-face slot or -1
  const int *cmask;     // [C] 9-bit mask of nonzero metric entries (a*3+i)
  const double *scale;  // [E][3] dXb/dx of Cartesian elements
  const double *gcart;  // [E][3] dXb/dx / (2 w_end): lift factor of Cartesian faces
  const double *metric;  // [C][9][np] M[a][i] = dXb^a/dx^i (node-major)
  const double *metricp; // [C][3 a][3 i][n q][n*n line]: pass-major layout
  const double *fac;    // [C][6][nn][4] (g*n0, g*n1, g*n2, g)
  const double *bxyz;   // [B][3][nn] coordinates of outer-face nodes
  const double *bnrm;   // [B][3][nn] outward unit normals there
  int bc;               // NMG_BC_*
  double k0, k1, k2, om;
  const double *D;      // [n][n] D[i*n+j] = l_j'(x_i)
  // finite-volume elements (stage_fv.cu)
  int n;                // points per direction
  int fv_rec;           // NMG_FV_REC_*
  int fv_extrap;        // NMG_FV_EXTRAP_*
  double fv_w3ratio;    // WENOm3 optimal-weight ratio
  const double *fvgeo;  // [C][13][np]: 1/J, sqrtgdiag[3], unit normals n_d[3] (d-major)
  const double *fvdist; // [E][6] distance (element coords) of each face to its nearest midpoint
  const double *fvdxb;  // [n] midpoint spacings dXb[i] = Xbm[i] - Xbm[i-1], 1 <= i <= n-2
  // mixed DG / finite-volume meshes
  const unsigned char *skip;  // [E] 1: finite-volume element (DG kernels write nothing)
  const int *fvlist;    // [nfvel] finite-volume elements (FV kernel grid), or null: all
  int nfvel;
  const double *fvmid;  // [cslot][3][5][np] midpoint sqrtgdiag_d, 1/J, normal_d
                        // (coordinates_midpoint_data = yes), or null
  const double *ghost;  // [G][4][nn] interpolated traces of faces with code & 64;
                        // slot G = bslot[e*6+f]
  int numflux;          // NMG_NUMFLUX_LLF or NMG_NUMFLUX_UPWIND
  const double *fvbxyz; // [B][3][nn] outer-face coordinates on equally spaced points
  const double *fvbnrm; // [B][3][nn] outer-face unit normals there
};

constexpr int kCodeMixed = 64;  // face-table bit: neighbour of the other point type

template <int N>
__device__ __forceinline__ int face_node_d(int f, int a, int b) {
  const int d = f >> 1, p = (f & 1) * (N - 1);
  return d == 0 ? p + N * (a + N * b) : d == 1 ? a + N * (p + N * b) : a + N * (b + N * p);
}

// element of tile slot i (i = ebase + tile * EPB + le): i itself, or the
// i-th entry of the launch's element list (nelem past its end: no element)
__device__ __forceinline__ int elem_at(const StageParams &P, int i) {
  if (!P.elist) return i;
  return i < P.ebase + P.ecount ? __ldg(P.elist + i) : P.nelem;
}

__device__ __forceinline__ double stage_time(const StageParams &P) {
  return P.tdev ? P.tdev[*P.stepdev] + P.tofs_dt : P.t;
}

// copy pi, cx, cy, cz of w for EPB elements into sW[4][EPB][NP]
template <int N, int EPB, int NT>
__device__ __forceinline__ void stage_in(const StageParams &P, double *sW, int e0) {
  constexpr int NP = N * N * N;
  for (int q = threadIdx.x; q < EPB * 4 * NP; q += NT) {
    const int le = q / (4 * NP), rem = q - le * 4 * NP, f = rem / NP, node = rem - f * NP;
    const int e = elem_at(P, e0 + le);
    double v = 0.;
    if (e < P.nelem) v = __ldg(P.win + ((size_t)e * NF + f) * NP + node);
    sW[(f * EPB + le) * NP + node] = v;
  }
}

// Face terms, one direction at a time (faces 2d and 2d+1 are disjoint node
// sets, so no two threads of a pass touch the same node).  Accumulates
// into sR[f][EPB][NP] for f = 0 (r_pi), 1..3 (r_c).
template <int N, int EPB, int NT>
__device__ __forceinline__ void face_terms(const StageParams &P, const double *sW, double *sR,
                                           const int *sCs, const double (*sG)[3], int e0,
                                           double t) {
  constexpr int NP = N * N * N, NN = N * N;
#pragma unroll 1
  for (int d = 0; d < 3; d++) {
    for (int q = threadIdx.x; q < EPB * 2 * NN; q += NT) {
      const int le = q / (2 * NN), rem = q - le * 2 * NN, s = rem / NN, ab = rem - s * NN;
      const int e = elem_at(P, e0 + le);
      if (e >= P.nelem) continue;
      const int a = ab % N, b = ab / N, f = 2 * d + s;
      const int node = face_node_d<N>(f, a, b);
      const double ui0 = sW[(0 * EPB + le) * NP + node];
      const double ui1 = sW[(1 * EPB + le) * NP + node];
      const double ui2 = sW[(2 * EPB + le) * NP + node];
      const double ui3 = sW[(3 * EPB + le) * NP + node];
      double gn0, gn1, gn2, g;
      const int cs = sCs[le];
      if (cs < 0) {
        g = sG[le][d];
        const double sg = (f & 1) ? g : -g;
        gn0 = d == 0 ? sg : 0.;
        gn1 = d == 1 ? sg : 0.;
        gn2 = d == 2 ? sg : 0.;
      } else {
        const double2 *F2 = reinterpret_cast<const double2 *>(P.fac) +
                            (((size_t)cs * 6 + f) * NN + ab) * 2;
        const double2 fa = __ldg(F2), fb = __ldg(F2 + 1);
        gn0 = fa.x; gn1 = fa.y; gn2 = fb.x; g = fb.y;
      }
      double ua0, ua1, ua2, ua3;
      const int nbe = __ldg(P.nb + e * 6 + f);
      if (nbe >= 0) {
        const int cd = __ldg(P.code + e * 6 + f), f2 = cd & 7, o = cd >> 3;
        if (cd & kCodeMixed) {
          const double *G = P.ghost + (size_t)__ldg(P.bslot + e * 6 + f) * 4 * NN + ab;
          ua0 = G[0];
          ua1 = G[NN];
          ua2 = G[2 * NN];
          ua3 = G[3 * NN];
        } else {
          const int sw = o & 1, fa = (o >> 1) & 1, fb = (o >> 2) & 1;
          int aa = sw ? b : a, bb = sw ? a : b;
          aa = fa ? N - 1 - aa : aa;
          bb = fb ? N - 1 - bb : bb;
          const double *W2 = P.win + (size_t)nbe * NF * NP + face_node_d<N>(f2, aa, bb);
          ua0 = __ldg(W2);
          ua1 = __ldg(W2 + NP);
          ua2 = __ldg(W2 + 2 * NP);
          ua3 = __ldg(W2 + 3 * NP);
        }
      } else {
        const int bs = __ldg(P.bslot + e * 6 + f);
        if (P.bc == NMG_BC_EXACT_PLANEWAVE) {
          const double *X = P.bxyz + (size_t)bs * 3 * NN + ab;
          const double arg = P.k0 * X[0] + P.k1 * X[NN] + P.k2 * X[2 * NN] - P.om * t;
          double sn, cn;
          sincos(arg, &sn, &cn);
          ua0 = -P.om * cn;
          ua1 = P.k0 * cn;
          ua2 = P.k1 * cn;
          ua3 = P.k2 * cn;
        } else {
          // outgoing radiation: zero incoming characteristic pi + c.n
          const double *Nr = P.bnrm + (size_t)bs * 3 * NN + ab;
          const double n0 = Nr[0], n1 = Nr[NN], n2 = Nr[2 * NN];
          const double cnv = ui1 * n0 + ui2 * n1 + ui3 * n2;
          const double wo = ui0 - cnv;
          const double dcn = -0.5 * wo - cnv;  // exterior c.n minus interior c.n
          ua0 = 0.5 * wo;
          ua1 = fma(dcn, n0, ui1);
          ua2 = fma(dcn, n1, ui2);
          ua3 = fma(dcn, n2, ui3);
        }
      }
      const double dpi = ua0 - ui0, dcx = ua1 - ui1, dcy = ua2 - ui2, dcz = ua3 - ui3;
      double *r0 = sR + (0 * EPB + le) * NP + node;
      double *r1 = sR + (1 * EPB + le) * NP + node;
      double *r2 = sR + (2 * EPB + le) * NP + node;
      double *r3 = sR + (3 * EPB + le) * NP + node;
      *r0 = fma(dcx, gn0, fma(dcy, gn1, fma(dcz, gn2, fma(g, dpi, *r0))));
      if (P.numflux == NMG_NUMFLUX_UPWIND) {
        // upwind: only the normal part of the c jump is lifted
        const double q = dpi + fma(gn0, dcx, fma(gn1, dcy, gn2 * dcz)) / g;
        *r1 = fma(q, gn0, *r1);
        *r2 = fma(q, gn1, *r2);
        *r3 = fma(q, gn2, *r3);
      } else {
        *r1 = fma(dpi, gn0, fma(g, dcx, *r1));
        *r2 = fma(dpi, gn1, fma(g, dcy, *r2));
        *r3 = fma(dpi, gn2, fma(g, dcz, *r3));
      }
    }
    __syncthreads();
  }
}

// Face data of one face node, split so that the global loads can be issued
// early and the arithmetic done later: the lift factors (g n, g) and either
// the neighbour's interior values, the exact exterior state, or (outgoing
// boundary) the unit normal.
struct FaceData {
  double gn0, gn1, gn2, g;
  double v0, v1, v2, v3;  // neighbour / exterior state, or normal (kind 2)
  int kind;               // 0: neighbour or exact exterior state, 2: outgoing
};

template <int N>
__device__ __forceinline__ void face_fetch(const StageParams &P, int e, int f, int ab, int cs,
                                           double gcart_d, double t, FaceData &F) {
  constexpr int NP = N * N * N, NN = N * N;
  const int d = f >> 1, a = ab % N, b = ab / N;
  if (cs < 0) {
    const double sg = (f & 1) ? gcart_d : -gcart_d;
    F.g = gcart_d;
    F.gn0 = d == 0 ? sg : 0.;
    F.gn1 = d == 1 ? sg : 0.;
    F.gn2 = d == 2 ? sg : 0.;
  } else {
    const double2 *F2 = reinterpret_cast<const double2 *>(P.fac) + (((size_t)cs * 6 + f) * NN + ab) * 2;
    const double2 fa = __ldg(F2), fb = __ldg(F2 + 1);
    F.gn0 = fa.x; F.gn1 = fa.y; F.gn2 = fb.x; F.g = fb.y;
  }
  const int nbe = __ldg(P.nb + e * 6 + f);
  F.kind = 0;
  if (nbe >= 0) {
    const int cd = __ldg(P.code + e * 6 + f), f2 = cd & 7, o = cd >> 3;
    if (cd & kCodeMixed) {
      const double *G = P.ghost + (size_t)__ldg(P.bslot + e * 6 + f) * 4 * NN + ab;
      F.v0 = G[0];
      F.v1 = G[NN];
      F.v2 = G[2 * NN];
      F.v3 = G[3 * NN];
    } else {
      const int sw = o & 1, fa = (o >> 1) & 1, fb = (o >> 2) & 1;
      int aa = sw ? b : a, bb = sw ? a : b;
      aa = fa ? N - 1 - aa : aa;
      bb = fb ? N - 1 - bb : bb;
      const double *W2 = P.win + (size_t)nbe * NF * NP + face_node_d<N>(f2, aa, bb);
      F.v0 = __ldg(W2);
      F.v1 = __ldg(W2 + NP);
      F.v2 = __ldg(W2 + 2 * NP);
      F.v3 = __ldg(W2 + 3 * NP);
    }
  } else {
    const int bs = __ldg(P.bslot + e * 6 + f);
    if (P.bc == NMG_BC_EXACT_PLANEWAVE) {
      const double *X = P.bxyz + (size_t)bs * 3 * NN + ab;
      const double arg = P.k0 * X[0] + P.k1 * X[NN] + P.k2 * X[2 * NN] - P.om * t;
      double sn, cn;
      sincos(arg, &sn, &cn);
      F.v0 = -P.om * cn;
      F.v1 = P.k0 * cn;
      F.v2 = P.k1 * cn;
      F.v3 = P.k2 * cn;
    } else {
      const double *Nr = P.bnrm + (size_t)bs * 3 * NN + ab;
      F.v0 = __ldg(Nr);
      F.v1 = __ldg(Nr + NN);
      F.v2 = __ldg(Nr + 2 * NN);
      F.kind = 2;
    }
  }
}

// LLF (or upwind) lift of one face node given the interior state ui: adds to r[0..3]
__device__ __forceinline__ void face_apply(const FaceData &F, double ui0, double ui1, double ui2,
                                           double ui3, double &r0, double &r1, double &r2,
                                           double &r3, int numflux = NMG_NUMFLUX_LLF) {
  double ua0, ua1, ua2, ua3;
  if (F.kind == 0) {
    ua0 = F.v0; ua1 = F.v1; ua2 = F.v2; ua3 = F.v3;
  } else {
    // outgoing radiation: zero incoming characteristic pi + c.n
    const double n0 = F.v0, n1 = F.v1, n2 = F.v2;
    const double cnv = ui1 * n0 + ui2 * n1 + ui3 * n2;
    const double wo = ui0 - cnv;
    const double dcn = -0.5 * wo - cnv;
    ua0 = 0.5 * wo;
    ua1 = fma(dcn, n0, ui1);
    ua2 = fma(dcn, n1, ui2);
    ua3 = fma(dcn, n2, ui3);
  }
  const double dpi = ua0 - ui0, dcx = ua1 - ui1, dcy = ua2 - ui2, dcz = ua3 - ui3;
  r0 = fma(dcx, F.gn0, fma(dcy, F.gn1, fma(dcz, F.gn2, fma(F.g, dpi, r0))));
  if (numflux == NMG_NUMFLUX_UPWIND) {
    const double q = dpi + fma(F.gn0, dcx, fma(F.gn1, dcy, F.gn2 * dcz)) / F.g;
    r1 = fma(q, F.gn0, r1);
    r2 = fma(q, F.gn1, r2);
    r3 = fma(q, F.gn2, r3);
  } else {
    r1 = fma(dpi, F.gn0, fma(F.g, dcx, r1));
    r2 = fma(dpi, F.gn1, fma(F.g, dcy, r2));
    r3 = fma(dpi, F.gn2, fma(F.g, dcz, r3));
  }
}

// r out (mode 0) or RK4 stage update.  r_pi = sR[0] (+ sR[4] + sR[5] for
// elements whose divergence is split over three partial sums).
template <int N, int EPB, int NT, bool SPLIT>
__device__ __forceinline__ void epilogue(const StageParams &P, const double *sW, const double *sR,
                                         const int *sCs, int e0) {
  constexpr int NP = N * N * N;
  for (int q = threadIdx.x; q < EPB * NF * NP; q += NT) {
    const int le = q / (NF * NP), rem = q - le * NF * NP, f = rem / NP, node = rem - f * NP;
    const int e = elem_at(P, e0 + le);
    if (e >= P.nelem || (P.skip && P.skip[e])) continue;
    const size_t idx = ((size_t)e * NF + f) * NP + node;
    double r;
    if (f < 4) {
      r = sR[(f * EPB + le) * NP + node];
      if (SPLIT && f == 0 && sCs[le] >= 0)
        r += sR[(4 * EPB + le) * NP + node] + sR[(5 * EPB + le) * NP + node];
    } else {
      r = sW[(0 * EPB + le) * NP + node];  // r_phi = pi
    }
    if (P.mode == 0) {
      P.rout[idx] = r;
    } else if (P.mode == 1) {
      const double u = __ldg(P.u0 + idx);
      P.acc[idx] = fma(P.cacc, r, u);
      P.wout[idx] = fma(P.cw, r, u);
    } else if (P.mode == 4) {
      P.acc[idx] = fma(P.cacc, r, P.acc[idx]);
    } else if (P.mode == 5) {
      P.acc[idx] = fma(P.cacc, r, __ldg(P.u0 + idx));
    } else if (P.mode == 6) {
      P.acc[idx] = fma(P.cacc, r, P.acc[idx]);
      P.wout[idx] = fma(0.25, fma(P.cw, r, __ldg(P.win + idx)), 0.75 * __ldg(P.u0 + idx));
    } else {
      P.acc[idx] = fma(P.cacc, r, P.acc[idx]);
      P.wout[idx] = fma(P.cw, r, __ldg(P.u0 + idx));
    }
  }
}

// Transposed face terms and epilogue of the vector-Jacobian stage (shared by
// the FP64 and the tensor-core transposed kernels): sW holds rbar (pi, c) of
// the CTA's elements ([field][EPB][NP]; for one element a pointer into rbar
// in global memory works too), sR the transposed volume terms.
template <int N, int EPB, int NT>
__device__ __forceinline__ void vjp_faces_epilogue(const StageParams &P, const double *sW,
                                                   double *sR, const int *sCs,
                                                   const double (*sG)[3], int e0) {
  constexpr int NP = N * N * N, NN = N * N;
  const int tid = threadIdx.x;
  // ---- transposed face terms, one direction at a time ----
#pragma unroll 1
  for (int d = 0; d < 3; d++) {
    for (int q = tid; q < EPB * 2 * NN; q += NT) {
      const int le = q / (2 * NN), rem = q - le * 2 * NN, s = rem / NN, ab = rem - s * NN;
      const int e = e0 + le;
      if (e >= P.nelem) continue;
      const int a = ab % N, b = ab / N, f = 2 * d + s;
      const int node = face_node_d<N>(f, a, b);
      const double rp = sW[(0 * EPB + le) * NP + node];
      const double rc0 = sW[(1 * EPB + le) * NP + node];
      const double rc1 = sW[(2 * EPB + le) * NP + node];
      const double rc2 = sW[(3 * EPB + le) * NP + node];
      double gn0, gn1, gn2, g;
      const int cs = sCs[le];
      if (cs < 0) {
        g = sG[le][d];
        const double sg = (f & 1) ? g : -g;
        gn0 = d == 0 ? sg : 0.;
        gn1 = d == 1 ? sg : 0.;
        gn2 = d == 2 ? sg : 0.;
      } else {
        const double2 *F2 = reinterpret_cast<const double2 *>(P.fac) +
                            (((size_t)cs * 6 + f) * NN + ab) * 2;
        const double2 fa = __ldg(F2), fb = __ldg(F2 + 1);
        gn0 = fa.x; gn1 = fa.y; gn2 = fb.x; g = fb.y;
      }
      double dp, dc0, dc1, dc2;
      const int nbe = __ldg(P.nb + e * 6 + f);
      if (nbe >= 0 || P.bc == NMG_BC_EXACT_PLANEWAVE) {
        dp = -fma(g, rp, fma(gn0, rc0, fma(gn1, rc1, gn2 * rc2)));
        dc0 = -fma(gn0, rp, g * rc0);
        dc1 = -fma(gn1, rp, g * rc1);
        dc2 = -fma(gn2, rp, g * rc2);
        const int cdh = nbe >= 0 ? __ldg(P.code + e * 6 + f) : 0;
        if (cdh & kCodeMixed) {
          // non-conforming face: the neighbours' part, transposed through
          // the trace interpolation, waits in this face's slot
          const double *T = P.ghost + (size_t)__ldg(P.bslot + e * 6 + f) * 4 * NN + ab;
          dp += T[0];
          dc0 += T[NN];
          dc1 += T[2 * NN];
          dc2 += T[3 * NN];
        } else if (nbe >= 0) {
          const int cd = cdh, f2 = cd & 7, o = cd >> 3;
          const int sw = o & 1, fa = (o >> 1) & 1, fb = (o >> 2) & 1;
          int aa = sw ? b : a, bb = sw ? a : b;
          aa = fa ? N - 1 - aa : aa;
          bb = fb ? N - 1 - bb : bb;
          const double *W2 = P.win + (size_t)nbe * NF * NP + face_node_d<N>(f2, aa, bb);
          const double yp = __ldg(W2), yc0 = __ldg(W2 + NP), yc1 = __ldg(W2 + 2 * NP),
                       yc2 = __ldg(W2 + 3 * NP);
          double hn0, hn1, hn2, h;
          const int cs2 = __ldg(P.cslot + nbe);
          if (cs2 < 0) {
            const int d2 = f2 >> 1;
            h = __ldg(P.gcart + nbe * 3 + d2);
            const double sg = (f2 & 1) ? h : -h;
            hn0 = d2 == 0 ? sg : 0.;
            hn1 = d2 == 1 ? sg : 0.;
            hn2 = d2 == 2 ? sg : 0.;
          } else {
            const double2 *F2 = reinterpret_cast<const double2 *>(P.fac) +
                                (((size_t)cs2 * 6 + f2) * NN + aa + N * bb) * 2;
            const double2 fa2 = __ldg(F2), fb2 = __ldg(F2 + 1);
            hn0 = fa2.x; hn1 = fa2.y; hn2 = fb2.x; h = fb2.y;
          }
          dp += fma(h, yp, fma(hn0, yc0, fma(hn1, yc1, hn2 * yc2)));
          dc0 += fma(hn0, yp, h * yc0);
          dc1 += fma(hn1, yp, h * yc1);
          dc2 += fma(hn2, yp, h * yc2);
        }
      } else {
        // outgoing radiation
        const int bs = __ldg(P.bslot + e * 6 + f);
        const double *Nr = P.bnrm + (size_t)bs * 3 * NN + ab;
        const double n0 = Nr[0], n1 = Nr[NN], n2 = Nr[2 * NN];
        const double gsb = g * fma(n0, rc0, fma(n1, rc1, fma(n2, rc2, rp)));
        dp = -gsb;
        dc0 = -gsb * n0;
        dc1 = -gsb * n1;
        dc2 = -gsb * n2;
      }
      sR[(0 * EPB + le) * NP + node] += dp;
      sR[(1 * EPB + le) * NP + node] += dc0;
      sR[(2 * EPB + le) * NP + node] += dc1;
      sR[(3 * EPB + le) * NP + node] += dc2;
    }
    __syncthreads();
  }

  // ---- epilogue: wbar = (pibar + rbar_phi, cbar, 0) ----
  for (int q = tid; q < EPB * NF * NP; q += NT) {
    const int le = q / (NF * NP), rem = q - le * NF * NP, f = rem / NP, node = rem - f * NP;
    const int e = e0 + le;
    if (e >= P.nelem) continue;
    const size_t idx = ((size_t)e * NF + f) * NP + node;
    double r;
    if (f == 0)
      r = sR[le * NP + node] + __ldg(P.win + ((size_t)e * NF + 4) * NP + node);
    else if (f < 4)
      r = sR[(f * EPB + le) * NP + node];
    else
      r = 0.;
    if (P.mode == 0) {
      P.rout[idx] = r;
    } else if (P.mode == 1) {
      const double u = __ldg(P.u0 + idx);
      P.acc[idx] = fma(P.cacc, r, u);
      P.wout[idx] = fma(P.cw, r, u);
    } else if (P.mode == 4) {
      P.acc[idx] = fma(P.cacc, r, P.acc[idx]);
    } else {
      P.acc[idx] = fma(P.cacc, r, P.acc[idx]);
      P.wout[idx] = fma(P.cw, r, __ldg(P.u0 + idx));
    }
  }
}

// host-side launch entry points of the kernel variants
typedef cudaError_t (*LaunchFn)(const StageParams &, cudaStream_t);
struct Variant {
  const char *name;  // "gather" or "eo"
  int epb, nt;       // elements per CTA, threads per CTA
  LaunchFn launch;   // nelem == 0: set the smem limit only
};
// all compiled variants for n (returns count, fills out[])
int gather_variants(int n, Variant *out, int cap);
int eo_variants(int n, Variant *out, int cap);
// tensor-core variant: derivatives by exact integer digit products (n = 9)
int tc_variants(int n, Variant *out, int cap);
// digits of D and D^T for the tensor-core variants (no-op for other n)
cudaError_t tc_upload(int n, const double *D);
// tensor-core transposed (vector-Jacobian) stage kernel for n = 7, 8, 9
int tcvjp_variants(int n, Variant *out, int cap);
// transposed (vector-Jacobian) stage kernel for n
int vjp_variants(int n, Variant *out, int cap);
// batched persistent kernel over element groups of different n (2..10)
constexpr int kBatchMaxN = 10;
int batch_epb(int n);        // elements per tile for n (0: unsupported n)
size_t batch_smem(int n);    // dynamic shared memory of an n tile
cudaError_t batch_prepare(size_t smem);
cudaError_t batch_launch(const StageParams *d_params, const int *d_gn, const int *d_gblk0,
                         int ngroup, int ntile, int grid, size_t smem, cudaStream_t st);
// even-odd coefficients of D for n into constant memory
cudaError_t eo_upload(int n, const double *D);
// finite-volume stage kernels (all n up to kFvMaxN)
constexpr int kFvMaxN = 13;
size_t fv_smem(int n);
int fv_variants(int n, Variant *out, int cap);
// interpolated traces of the faces between DG and finite-volume elements:
// gtab[g] = (e, f, e2, code), M = [2][n][n] (Lagrange weights of the LGL
// points at the equally spaced positions; piecewise-linear weights of the
// equally spaced points at the LGL positions)
// exponential filter of all elements (set the smem limit once first)
cudaError_t filter_prepare(int n);
cudaError_t filter_launch(int n, int nelem, double *u, const unsigned char *isfv, const double *F,
                          const int *cslot, const double *oojdg, const double *fvgeo,
                          const double *scale, int jpow, int filter_fv, int allfv,
                          cudaStream_t st);
// MRS limiter of every element of u: node averages and extrema (lim,
// [e][field][3]; nboff: CSR over nbl per element face, [E*6+1]), then
// u <- ubar + theta (u - ubar); limited[e] = theta < 1
cudaError_t limiter_launch(int n, int nelem, double *u, const unsigned char *isfv, int allfv,
                           const double *wl, const double *wu, double *lim, const int *nboff,
                           const int *nbl, const double *alpha_h, int *limited, cudaStream_t st);
// minmodB limiter of every element of u (n in [2, 16]): coefficients c000,
// c100, c010, c001 (lim, [e][field][4]), then per field the bounded minmod
// of the linear modes against the face neighbours' averages (foff: CSR over
// nbl per element face, [E*6+1]); limited[e]: some field limited
cudaError_t mmb_limiter_launch(int n, int nelem, double *u, const unsigned char *isfv, int allfv,
                               const double *ana, const double *syn, double *lim,
                               const int *foff, const int *nbl, const double *mt_h, double bos3,
                               int scale_bound, int *limited, cudaStream_t st);
// traces of non-conforming faces: per slot, field and face node the average
// over its contributions of the source face interpolated at the node
cudaError_t hang_launch(int nhang, int n, const int *hoff, const int *hsrc, const double *hw,
                        const double *win, double *ghost, cudaStream_t st);
// adjoint of those traces: per slot, field and face node, the sum over the
// (slot, node) pairs that read that source-face node of weight times the
// lift adjoint of rbar there (toff/tsrc/tw: the transposed list)
cudaError_t hang_adj_launch(int nhang, int n, const int *toff, const int *tsrc, const double *tw,
                            const int *hface, const int *cslot, const double *fac,
                            const double *gcart, const double *rbar, double *out,
                            cudaStream_t st);
cudaError_t ghost_launch(int nghost, int n, const int *gtab, const unsigned char *isfv,
                         const double *M, const double *win, double *ghost, cudaStream_t st);
// u of the listed elements <- (M x M x M) u (all fields), in place
cudaError_t convert_launch(int n, const int *list, int count, const double *M, double *u,
                           cudaStream_t st);
// per-element min/max of u_p, then the trouble flag of every element (RDMP
// on all elements, Persson's indicator with the modal analysis matrix A on
// DG elements); pers[E][5] receives the indicators (may be null)
cudaError_t trouble_launch(int n, int nelem, const double *u, const double *u_p, double *mm,
                           const int *nb, const unsigned char *isfv, const double *A,
                           double deltafac, double delta0, double epsilon, double persson_max,
                           double uscale, int *flag, double *pers, cudaStream_t st);

}  // namespace nmgk
