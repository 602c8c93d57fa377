// stage_eo.cu -- "eo" variant of the fused stage kernel: line-parallel
// directional derivatives with the even-odd split of the LGL
// differentiation matrix.
//
// D of symmetric nodes is centro-antisymmetric (D[n-1-i][n-1-j] = -D[i][j]),
// so with e_j = u_j + u_{n-1-j}, o_j = u_j - u_{n-1-j} one line derivative
// costs ~n^2/2 + 2n FP64 operations instead of n^2 (56 instead of 81 at
// n = 9):  S_i = sum_j A_ij e_j (+ D_ic u_c), T_i = sum_j B_ij o_j,
// (Du)_i = S_i + T_i, (Du)_{n-1-i} = T_i - S_i, with
// A_ij = (D_ij + D_i,n-1-j)/2, B_ij = (D_ij - D_i,n-1-j)/2.
// A thread owns one (line, field) pair of one direction per task; the
// chain-rule factors dXb^a/dx^i are read in a pass-major layout so that
// neighbouring lines are neighbouring addresses, and metric entries that
// vanish identically on an element (cubed-sphere maps have two) are never
// loaded or multiplied.  r_pi is split over three partial sums so that the
// three c-component tasks of one line never write the same address.
#include <algorithm>
#include <cstdio>

#include "stage.cuh"

namespace nmgk {
namespace {

constexpr int MMAX = NMAX / 2;
// [0]: coefficients of D, [1]: of its transpose (also centro-antisymmetric)
__constant__ double cEA[2][NMAX + 1][MMAX][MMAX + 1];  // A_ij, j < m; A_im = D_ic (odd n)
__constant__ double cEB[2][NMAX + 1][MMAX][MMAX];      // B_ij
__constant__ double cEC[2][NMAX + 1][MMAX];            // middle row (odd n): B_cj

template <int N, int TR>
__device__ __forceinline__ void line_deriv(const double *__restrict__ s, int st, double *out) {
  constexpr int M = N / 2;
  constexpr bool ODD = (N & 1) != 0;
  double e[M], o[M];
#pragma unroll
  for (int j = 0; j < M; j++) {
    const double a = s[j * st], b = s[(N - 1 - j) * st];
    e[j] = a + b;
    o[j] = a - b;
  }
  const double uc = ODD ? s[M * st] : 0.;
#pragma unroll
  for (int i = 0; i < M; i++) {
    double S = ODD ? cEA[TR][N][i][M] * uc : cEA[TR][N][i][0] * e[0];
    double T = cEB[TR][N][i][0] * o[0];
#pragma unroll
    for (int j = ODD ? 0 : 1; j < M; j++) S = fma(cEA[TR][N][i][j], e[j], S);
#pragma unroll
    for (int j = 1; j < M; j++) T = fma(cEB[TR][N][i][j], o[j], T);
    out[i] = S + T;
    out[N - 1 - i] = T - S;
  }
  if (ODD) {
    double c = cEC[TR][N][0] * o[0];
#pragma unroll
    for (int j = 1; j < M; j++) c = fma(cEC[TR][N][j], o[j], c);
    out[M] = c;
  }
}

// one CTA's work: elements [blk*EPB, blk*EPB+EPB) of P
template <int N, int EPB, int NT>
__device__ __forceinline__ void eo_body(const StageParams &P, int blk) {
  constexpr int NP = N * N * N, NN = N * N;
  extern __shared__ double smem[];
  double *sW = smem;                 // [4][EPB][NP]: pi, cx, cy, cz of w
  double *sR = smem + 4 * EPB * NP;  // [6][EPB][NP]: r_pi^0, r_c(3), r_pi^1, r_pi^2
  __shared__ int sCs[EPB];
  __shared__ int sMask[EPB];
  __shared__ double sScale[EPB][3];
  __shared__ double sG[EPB][3];
  __shared__ unsigned char sPair[3][4 * EPB];  // per pass: le*4 + field
  __shared__ int sNPair[3];

  const int e0 = P.ebase + blk * EPB;
  const int tid = threadIdx.x;
  for (int q = tid; q < EPB; q += NT) {
    const int e = elem_at(P, e0 + q);
    const int cs = (e < P.nelem) ? P.cslot[e] : -1;
    sCs[q] = cs;
    sMask[q] = (e >= P.nelem) ? 0 : (cs >= 0 ? P.cmask[cs] : (1 | (1 << 4) | (1 << 8)));
    for (int d = 0; d < 3; d++) sScale[q][d] = (e < P.nelem) ? P.scale[e * 3 + d] : 0.;
    for (int d = 0; d < 3; d++) sG[q][d] = (e < P.nelem) ? P.gcart[e * 3 + d] : 0.;
  }
  for (int q = tid; q < 6 * EPB * NP; q += NT) sR[q] = 0.;
  const double t = stage_time(P);
  stage_in<N, EPB, NT>(P, sW, e0);
  __syncthreads();
  if (tid < 3) {
    const int a = tid;
    int np = 0;
    for (int le = 0; le < EPB; le++) {
      const int row = (sMask[le] >> (3 * a)) & 7;
      if (!row) continue;
      sPair[a][np++] = (unsigned char)(le * 4 + 0);
      for (int i = 0; i < 3; i++)
        if (row & (1 << i)) sPair[a][np++] = (unsigned char)(le * 4 + 1 + i);
    }
    sNPair[a] = np;
  }
  __syncthreads();

  // ---- volume terms, one direction per pass ----
#pragma unroll 1
  for (int a = 0; a < 3; a++) {
    const int ntask = sNPair[a] * NN;
    const int st = a == 0 ? 1 : (a == 1 ? N : NN);
    for (int q = tid; q < ntask; q += NT) {
      const int p = q / NN, L = q - p * NN;
      const int pr = sPair[a][p], le = pr >> 2, fld = pr & 3;
      const int l0 = L % N, l1 = L / N;
      const int base = a == 0 ? N * (l0 + N * l1) : (a == 1 ? l0 + NN * l1 : l0 + N * l1);
      double out[N];
      line_deriv<N, 0>(sW + (fld * EPB + le) * NP + base, st, out);
      const int cs = sCs[le];
      const int row = (sMask[le] >> (3 * a)) & 7;
      if (fld == 0) {
        // d_a pi -> r_c[i] for every i with M[a][i] != 0
#pragma unroll
        for (int i = 0; i < 3; i++) {
          if (!(row & (1 << i))) continue;
          double *r = sR + ((1 + i) * EPB + le) * NP + base;
          if (cs < 0) {
            const double s = sScale[le][a];
#pragma unroll
            for (int qq = 0; qq < N; qq++) r[qq * st] = fma(s, out[qq], r[qq * st]);
          } else {
            const double *Mp = P.metricp + (((size_t)cs * 3 + a) * 3 + i) * N * NN + L;
#pragma unroll
            for (int qq = 0; qq < N; qq++)
              r[qq * st] = fma(__ldg(Mp + qq * NN), out[qq], r[qq * st]);
          }
        }
      } else {
        // d_a c_i -> r_pi partial sum of component i
        const int i = fld - 1;
        if (cs < 0) {
          double *r = sR + (0 * EPB + le) * NP + base;
          const double s = sScale[le][a];
#pragma unroll
          for (int qq = 0; qq < N; qq++) r[qq * st] = fma(s, out[qq], r[qq * st]);
        } else {
          const int slot = i == 0 ? 0 : 3 + i;
          double *r = sR + (slot * EPB + le) * NP + base;
          const double *Mp = P.metricp + (((size_t)cs * 3 + a) * 3 + i) * N * NN + L;
#pragma unroll
          for (int qq = 0; qq < N; qq++)
            r[qq * st] = fma(__ldg(Mp + qq * NN), out[qq], r[qq * st]);
        }
      }
    }
    __syncthreads();
  }
  face_terms<N, EPB, NT>(P, sW, sR, sCs, sG, e0, t);
  epilogue<N, EPB, NT, true>(P, sW, sR, sCs, e0);
}

template <int N, int EPB, int NT>
__global__ void __launch_bounds__(NT) eo_kernel(StageParams P) {
  eo_body<N, EPB, NT>(P, blockIdx.x);
}

template <int N, int EPB, int NT>
cudaError_t launch_eo(const StageParams &P, cudaStream_t st) {
  constexpr int NP = N * N * N;
  const size_t shmem = sizeof(double) * 10 * EPB * NP;
  if (P.nelem <= 0)
    return cudaFuncSetAttribute(eo_kernel<N, EPB, NT>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shmem);
  const int ne = P.ecount > 0 ? P.ecount : P.nelem;
  eo_kernel<N, EPB, NT><<<(ne + EPB - 1) / EPB, NT, shmem, st>>>(P);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// "eof": the eo kernel with the face terms folded into the volume passes.
// The a-line through a face node of faces 2a / 2a+1 ends on that face, so
// the pi task of each a-line also applies the LLF lift at its two end nodes
// (neighbour values and lift factors are fetched before the line transform
// so that their latency overlaps the arithmetic).  In pass a that task is
// the only writer of r_c at its nodes; its r_pi face part goes to a
// seventh accumulator.  This removes the three separate face passes.
template <int N, int EPB, int NT>
__device__ __forceinline__ void eof_body(const StageParams &P, int blk) {
  constexpr int NP = N * N * N, NN = N * N;
  extern __shared__ double smem[];
  double *sW = smem;                 // [4][EPB][NP]: pi, cx, cy, cz of w
  double *sR = smem + 4 * EPB * NP;  // [7][EPB][NP]: r_pi^0, r_c(3), r_pi^1, r_pi^2, r_pi^face
  __shared__ int sCs[EPB];
  __shared__ int sMask[EPB];
  __shared__ double sScale[EPB][3];
  __shared__ double sG[EPB][3];
  __shared__ unsigned char sPair[3][4 * EPB];
  __shared__ int sNPair[3];

  const int e0 = P.ebase + blk * EPB;
  const int tid = threadIdx.x;
  for (int q = tid; q < EPB; q += NT) {
    const int e = elem_at(P, e0 + q);
    const int cs = (e < P.nelem) ? P.cslot[e] : -1;
    sCs[q] = cs;
    sMask[q] = (e >= P.nelem) ? -1 : (cs >= 0 ? P.cmask[cs] : (1 | (1 << 4) | (1 << 8)));
    for (int d = 0; d < 3; d++) sScale[q][d] = (e < P.nelem) ? P.scale[e * 3 + d] : 0.;
    for (int d = 0; d < 3; d++) sG[q][d] = (e < P.nelem) ? P.gcart[e * 3 + d] : 0.;
  }
  for (int q = tid; q < 7 * EPB * NP; q += NT) sR[q] = 0.;
  const double t = stage_time(P);
  stage_in<N, EPB, NT>(P, sW, e0);
  __syncthreads();
  if (tid < 3) {
    const int a = tid;
    int np = 0;
    for (int le = 0; le < EPB; le++) {
      if (sMask[le] < 0) continue;  // past the last element
      const int row = (sMask[le] >> (3 * a)) & 7;
      sPair[a][np++] = (unsigned char)(le * 4 + 0);  // always: it carries the faces
      for (int i = 0; i < 3; i++)
        if (row & (1 << i)) sPair[a][np++] = (unsigned char)(le * 4 + 1 + i);
    }
    sNPair[a] = np;
  }
  __syncthreads();

#pragma unroll 1
  for (int a = 0; a < 3; a++) {
    const int ntask = sNPair[a] * NN;
    const int st = a == 0 ? 1 : (a == 1 ? N : NN);
    for (int q = tid; q < ntask; q += NT) {
      const int p = q / NN, L = q - p * NN;
      const int pr = sPair[a][p], le = pr >> 2, fld = pr & 3;
      const int l0 = L % N, l1 = L / N;
      const int base = a == 0 ? N * (l0 + N * l1) : (a == 1 ? l0 + NN * l1 : l0 + N * l1);
      const int cs = sCs[le];
      const int row = (sMask[le] >> (3 * a)) & 7;
      if (fld == 0) {
        FaceData FL, FR;
        face_fetch<N>(P, elem_at(P, e0 + le), 2 * a, L, cs, sG[le][a], t, FL);
        face_fetch<N>(P, elem_at(P, e0 + le), 2 * a + 1, L, cs, sG[le][a], t, FR);
        double out[N];
        line_deriv<N, 0>(sW + (0 * EPB + le) * NP + base, st, out);
#pragma unroll
        for (int i = 0; i < 3; i++) {
          if (!(row & (1 << i))) continue;
          double *r = sR + ((1 + i) * EPB + le) * NP + base;
          if (cs < 0) {
            const double s = sScale[le][a];
#pragma unroll
            for (int qq = 0; qq < N; qq++) r[qq * st] = fma(s, out[qq], r[qq * st]);
          } else {
            const double *Mp = P.metricp + (((size_t)cs * 3 + a) * 3 + i) * N * NN + L;
#pragma unroll
            for (int qq = 0; qq < N; qq++)
              r[qq * st] = fma(__ldg(Mp + qq * NN), out[qq], r[qq * st]);
          }
        }
        // face terms at the two ends of the line
#pragma unroll
        for (int side = 0; side < 2; side++) {
          const int node = base + (side ? (N - 1) * st : 0);
          const double *w = sW + le * NP + node;
          double *r = sR + le * NP + node;
          double r0 = r[6 * EPB * NP], r1 = r[1 * EPB * NP], r2 = r[2 * EPB * NP],
                 r3 = r[3 * EPB * NP];
          face_apply(side ? FR : FL, w[0], w[EPB * NP], w[2 * EPB * NP], w[3 * EPB * NP], r0,
                     r1, r2, r3, P.numflux);
          r[6 * EPB * NP] = r0;
          r[1 * EPB * NP] = r1;
          r[2 * EPB * NP] = r2;
          r[3 * EPB * NP] = r3;
        }
      } else {
        double out[N];
        line_deriv<N, 0>(sW + (fld * EPB + le) * NP + base, st, out);
        const int i = fld - 1;
        if (cs < 0) {
          double *r = sR + (0 * EPB + le) * NP + base;
          const double s = sScale[le][a];
#pragma unroll
          for (int qq = 0; qq < N; qq++) r[qq * st] = fma(s, out[qq], r[qq * st]);
        } else {
          const int slot = i == 0 ? 0 : 3 + i;
          double *r = sR + (slot * EPB + le) * NP + base;
          const double *Mp = P.metricp + (((size_t)cs * 3 + a) * 3 + i) * N * NN + L;
#pragma unroll
          for (int qq = 0; qq < N; qq++)
            r[qq * st] = fma(__ldg(Mp + qq * NN), out[qq], r[qq * st]);
        }
      }
    }
    __syncthreads();
  }

  // epilogue: r_pi = r_pi^0 (+ r_pi^1 + r_pi^2) + r_pi^face, r_phi = pi
  for (int q = tid; q < EPB * NF * NP; q += NT) {
    const int le = q / (NF * NP), rem = q - le * NF * NP, f = rem / NP, node = rem - f * NP;
    const int e = elem_at(P, e0 + le);
    if (e >= P.nelem || (P.skip && P.skip[e])) continue;
    const size_t idx = ((size_t)e * NF + f) * NP + node;
    double r;
    if (f == 0) {
      r = sR[le * NP + node];
      if (sCs[le] >= 0) r += sR[(4 * EPB + le) * NP + node] + sR[(5 * EPB + le) * NP + node];
      r += sR[(6 * EPB + le) * NP + node];
    } else if (f < 4) {
      r = sR[(f * EPB + le) * NP + node];
    } else {
      r = sW[le * NP + node];
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

// MINB: minimum resident CTAs per SM asked of the register allocator
// (1: no register cap)
template <int N, int EPB, int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB) eof_kernel(StageParams P) {
  eof_body<N, EPB, NT>(P, blockIdx.x);
}

template <int N, int EPB, int NT, int MINB>
cudaError_t launch_eof(const StageParams &P, cudaStream_t st) {
  constexpr int NP = N * N * N;
  const size_t shmem = sizeof(double) * 11 * EPB * NP;
  if (P.nelem <= 0)
    return cudaFuncSetAttribute(eof_kernel<N, EPB, NT, MINB>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shmem);
  const int ne = P.ecount > 0 ? P.ecount : P.nelem;
  eof_kernel<N, EPB, NT, MINB><<<(ne + EPB - 1) / EPB, NT, shmem, st>>>(P);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Batched persistent kernel: several element groups, each with its own
// order n and its own StageParams (one group = all problems of one order,
// merged into one mesh), walked by persistent CTAs in one launch.  Tile
// t -> (group g, block t - gblk0[g]); tiles of the highest order come first
// so that the long tiles start early.  Tile shape per n: EPB = bEPB(n),
// 256 threads (the eo:<bEPB>:256 variant, bitwise the same arithmetic).
constexpr int kBatchNT = 256;
constexpr int bEPB(int n) { return (128 / (2 * n * n)) > 1 ? (128 / (2 * n * n)) : 1; }

template <int N>
__device__ __forceinline__ void batch_tile(const StageParams *params, int g, int blk) {
  const StageParams P = params[g];
  eo_body<N, bEPB(N), kBatchNT>(P, blk);
}

__global__ void __launch_bounds__(kBatchNT, 2)
    batch_kernel(const StageParams *params, const int *gn, const int *gblk0, int ngroup,
                 int ntile) {
  for (int b = blockIdx.x; b < ntile; b += gridDim.x) {
    int g = 0;
    while (g + 1 < ngroup && b >= gblk0[g + 1]) g++;
    const int blk = b - gblk0[g];
    __syncthreads();  // the previous tile's epilogue has read its shared memory
    switch (gn[g]) {
      case 2: batch_tile<2>(params, g, blk); break;
      case 3: batch_tile<3>(params, g, blk); break;
      case 4: batch_tile<4>(params, g, blk); break;
      case 5: batch_tile<5>(params, g, blk); break;
      case 6: batch_tile<6>(params, g, blk); break;
      case 7: batch_tile<7>(params, g, blk); break;
      case 8: batch_tile<8>(params, g, blk); break;
      case 9: batch_tile<9>(params, g, blk); break;
      case 10: batch_tile<10>(params, g, blk); break;
      default: break;
    }
  }
}

// ---------------------------------------------------------------------------
// Transposed stage kernel (vector-Jacobian product).  The scalar-wave RHS is
// linear in w, r = L w (+ exterior plane-wave data that does not depend on
// w), so its VJP is wbar = L^T rbar, evaluated here from `win` = rbar:
//   volume  pibar  = sum_a D_a^T (sum_i M[a][i] rbar_c_i),
//           cbar_i = sum_a D_a^T (M[a][i] rbar_pi),   pibar += rbar_phi;
//   faces   for face node x of element e with neighbour node y of e':
//           pibar_x -= g_x rbar_pi(x) + gn_x . rbar_c(x)
//           cbar_x  -= gn_x rbar_pi(x) + g_x rbar_c(x)
//           pibar_x += g_y rbar_pi(y) + gn_y . rbar_c(y)     (y's lift
//           cbar_x  += gn_y rbar_pi(y) + g_y rbar_c(y)        depends on x)
//   outgoing outer faces (r += -g s (1, n), s = pi + c.n):
//           pibar_x -= g sb, cbar_x -= g sb n, sb = rbar_pi + n . rbar_c.
// Every contribution is gathered by the node that receives it, so there
// are no atomics and the result is deterministic.  D^T is centro-
// antisymmetric too, so the even-odd line transform applies unchanged.
template <int N, int EPB, int NT>
__global__ void __launch_bounds__(NT) vjp_kernel(StageParams P) {
  constexpr int NP = N * N * N, NN = N * N;
  extern __shared__ double smem[];
  double *sW = smem;                 // [4][EPB][NP]: rbar pi, c (from win)
  double *sR = smem + 4 * EPB * NP;  // [4][EPB][NP]: wbar pi, c
  __shared__ int sCs[EPB];
  __shared__ int sMask[EPB];
  __shared__ double sScale[EPB][3];
  __shared__ double sG[EPB][3];
  __shared__ unsigned char sPair[3][4 * EPB];
  __shared__ int sNPair[3];

  const int e0 = blockIdx.x * EPB;
  const int tid = threadIdx.x;
  for (int q = tid; q < EPB; q += NT) {
    const int e = e0 + q;
    const int cs = (e < P.nelem) ? P.cslot[e] : -1;
    sCs[q] = cs;
    sMask[q] = (e >= P.nelem) ? 0 : (cs >= 0 ? P.cmask[cs] : (1 | (1 << 4) | (1 << 8)));
    for (int d = 0; d < 3; d++) sScale[q][d] = (e < P.nelem) ? P.scale[e * 3 + d] : 0.;
    for (int d = 0; d < 3; d++) sG[q][d] = (e < P.nelem) ? P.gcart[e * 3 + d] : 0.;
  }
  for (int q = tid; q < 4 * EPB * NP; q += NT) sR[q] = 0.;
  stage_in<N, EPB, NT>(P, sW, e0);
  __syncthreads();
  if (tid < 3) {
    const int a = tid;
    int np = 0;
    for (int le = 0; le < EPB; le++) {
      const int row = (sMask[le] >> (3 * a)) & 7;
      if (!row) continue;
      sPair[a][np++] = (unsigned char)(le * 4 + 0);
      for (int i = 0; i < 3; i++)
        if (row & (1 << i)) sPair[a][np++] = (unsigned char)(le * 4 + 1 + i);
    }
    sNPair[a] = np;
  }
  __syncthreads();

  // ---- transposed volume terms, one direction per pass ----
#pragma unroll 1
  for (int a = 0; a < 3; a++) {
    const int ntask = sNPair[a] * NN;
    const int st = a == 0 ? 1 : (a == 1 ? N : NN);
    for (int q = tid; q < ntask; q += NT) {
      const int p = q / NN, L = q - p * NN;
      const int pr = sPair[a][p], le = pr >> 2, fld = pr & 3;
      const int l0 = L % N, l1 = L / N;
      const int base = a == 0 ? N * (l0 + N * l1) : (a == 1 ? l0 + NN * l1 : l0 + N * l1);
      const int cs = sCs[le];
      const int row = (sMask[le] >> (3 * a)) & 7;
      double y[N], out[N];
      if (fld == 0) {
        // y = sum_i M[a][i] rbar_c_i along the line
#pragma unroll
        for (int qq = 0; qq < N; qq++) y[qq] = 0.;
#pragma unroll
        for (int i = 0; i < 3; i++) {
          if (!(row & (1 << i))) continue;
          const double *rc = sW + ((1 + i) * EPB + le) * NP + base;
          if (cs < 0) {
            const double s = sScale[le][a];
#pragma unroll
            for (int qq = 0; qq < N; qq++) y[qq] = fma(s, rc[qq * st], y[qq]);
          } else {
            const double *Mp = P.metricp + (((size_t)cs * 3 + a) * 3 + i) * N * NN + L;
#pragma unroll
            for (int qq = 0; qq < N; qq++) y[qq] = fma(__ldg(Mp + qq * NN), rc[qq * st], y[qq]);
          }
        }
      } else {
        const int i = fld - 1;
        const double *rp = sW + (0 * EPB + le) * NP + base;
        if (cs < 0) {
          const double s = sScale[le][a];
#pragma unroll
          for (int qq = 0; qq < N; qq++) y[qq] = s * rp[qq * st];
        } else {
          const double *Mp = P.metricp + (((size_t)cs * 3 + a) * 3 + i) * N * NN + L;
#pragma unroll
          for (int qq = 0; qq < N; qq++) y[qq] = __ldg(Mp + qq * NN) * rp[qq * st];
        }
      }
      line_deriv<N, 1>(y, 1, out);
      double *r = sR + (fld * EPB + le) * NP + base;
#pragma unroll
      for (int qq = 0; qq < N; qq++) r[qq * st] += out[qq];
    }
    __syncthreads();
  }

  vjp_faces_epilogue<N, EPB, NT>(P, sW, sR, sCs, sG, e0);
}

template <int N, int EPB, int NT>
cudaError_t launch_vjp(const StageParams &P, cudaStream_t st) {
  constexpr int NP = N * N * N;
  const size_t shmem = sizeof(double) * 8 * EPB * NP;
  if (P.nelem <= 0)
    return cudaFuncSetAttribute(vjp_kernel<N, EPB, NT>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shmem);
  vjp_kernel<N, EPB, NT><<<(P.nelem + EPB - 1) / EPB, NT, shmem, st>>>(P);
  return cudaGetLastError();
}

template <int N>
int add_vjp(Variant *out, int cap) {
  constexpr int NN = N * N;
  constexpr int E1 = (128 / (2 * NN)) > 1 ? (128 / (2 * NN)) : 1;
  if (cap < 1) return 0;
  out[0] = Variant{"vjp", E1, 256, launch_vjp<N, E1, 256>};
  return 1;
}

constexpr size_t kSmemMax = 220 * 1024;

template <int N, int EPB, int NT>
void add_one(Variant *out, int cap, int &k) {
  if constexpr (sizeof(double) * 10 * EPB * N * N * N + 4096 <= kSmemMax && EPB <= 64) {
    if (k < cap) out[k++] = Variant{"eo", EPB, NT, launch_eo<N, EPB, NT>};
  }
}

template <int N, int EPB, int NT, int MINB>
void add_one_f(Variant *out, int cap, int &k) {
  if constexpr (sizeof(double) * 11 * EPB * N * N * N + 4096 <= kSmemMax && EPB <= 64) {
    if (k < cap)
      out[k++] = Variant{MINB > 1 ? "eof" : "eofu", EPB, NT, launch_eof<N, EPB, NT, MINB>};
  }
}

template <int N>
int add_eo(Variant *out, int cap) {
  constexpr int NN = N * N;
  constexpr int E1 = (128 / (2 * NN)) > 1 ? (128 / (2 * NN)) : 1;
  int k = 0;
  add_one<N, E1, 128>(out, cap, k);
  add_one<N, E1, 256>(out, cap, k);
  add_one<N, 2 * E1, 128>(out, cap, k);
  add_one<N, 2 * E1, 256>(out, cap, k);
  add_one_f<N, E1, 128, 6>(out, cap, k);
  add_one_f<N, E1, 256, 3>(out, cap, k);
  add_one_f<N, E1, 128, 1>(out, cap, k);
  add_one_f<N, E1, 256, 1>(out, cap, k);
  return k;
}

}  // namespace

int eo_variants(int n, Variant *out, int cap) {
  switch (n) {
    case 2: return add_eo<2>(out, cap);
    case 3: return add_eo<3>(out, cap);
    case 4: return add_eo<4>(out, cap);
    case 5: return add_eo<5>(out, cap);
    case 6: return add_eo<6>(out, cap);
    case 7: return add_eo<7>(out, cap);
    case 8: return add_eo<8>(out, cap);
    case 9: return add_eo<9>(out, cap);
    case 10: return add_eo<10>(out, cap);
    case 11: return add_eo<11>(out, cap);
    case 12: return add_eo<12>(out, cap);
    default: return 0;
  }
}

int batch_epb(int n) { return (n >= 2 && n <= kBatchMaxN) ? bEPB(n) : 0; }

size_t batch_smem(int n) {
  return (n >= 2 && n <= kBatchMaxN) ? sizeof(double) * 10 * bEPB(n) * n * n * n : 0;
}

// the kernel's shared-memory limit is one setting per function for every
// batch alive: set it to the largest tile of any order, so that creating a
// batch of small orders never lowers it under a live batch of larger ones
cudaError_t batch_prepare(size_t smem) {
  size_t most = smem;
  for (int n = 2; n <= kBatchMaxN; n++) most = std::max(most, batch_smem(n));
  return cudaFuncSetAttribute(batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)most);
}

cudaError_t batch_launch(const StageParams *d_params, const int *d_gn, const int *d_gblk0,
                         int ngroup, int ntile, int grid, size_t smem, cudaStream_t st) {
  batch_kernel<<<grid, kBatchNT, smem, st>>>(d_params, d_gn, d_gblk0, ngroup, ntile);
  return cudaGetLastError();
}

int vjp_variants(int n, Variant *out, int cap) {
  switch (n) {
    case 2: return add_vjp<2>(out, cap);
    case 3: return add_vjp<3>(out, cap);
    case 4: return add_vjp<4>(out, cap);
    case 5: return add_vjp<5>(out, cap);
    case 6: return add_vjp<6>(out, cap);
    case 7: return add_vjp<7>(out, cap);
    case 8: return add_vjp<8>(out, cap);
    case 9: return add_vjp<9>(out, cap);
    case 10: return add_vjp<10>(out, cap);
    case 11: return add_vjp<11>(out, cap);
    case 12: return add_vjp<12>(out, cap);
    default: return 0;
  }
}

cudaError_t eo_upload(int n, const double *D) {
  if (n < 2 || n > NMAX) return cudaErrorInvalidValue;
  const int m = n / 2, odd = n & 1, c = n / 2;
  double Dt[NMAX * NMAX];
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) Dt[i * n + j] = D[j * n + i];
  for (int tr = 0; tr < 2; tr++) {
    const double *X = tr ? Dt : D;
    double A[MMAX][MMAX + 1] = {}, B[MMAX][MMAX] = {}, C[MMAX] = {};
    for (int i = 0; i < m; i++) {
      for (int j = 0; j < m; j++) {
        A[i][j] = 0.5 * (X[i * n + j] + X[i * n + (n - 1 - j)]);
        B[i][j] = 0.5 * (X[i * n + j] - X[i * n + (n - 1 - j)]);
      }
      if (odd) A[i][m] = X[i * n + c];
    }
    if (odd)
      for (int j = 0; j < m; j++) C[j] = 0.5 * (X[c * n + j] - X[c * n + (n - 1 - j)]);
    const size_t slot = (size_t)tr * (NMAX + 1) + n;
    cudaError_t e;
    if ((e = cudaMemcpyToSymbol(cEA, A, sizeof(A), sizeof(A) * slot)) != cudaSuccess) return e;
    if ((e = cudaMemcpyToSymbol(cEB, B, sizeof(B), sizeof(B) * slot)) != cudaSuccess) return e;
    if ((e = cudaMemcpyToSymbol(cEC, C, sizeof(C), sizeof(C) * slot)) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace nmgk
