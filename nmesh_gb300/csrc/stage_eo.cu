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
#include <cstdio>

#include "stage.cuh"

namespace nmgk {
namespace {

constexpr int MMAX = NMAX / 2;
__constant__ double cEA[NMAX + 1][MMAX][MMAX + 1];  // A_ij, j < m; A_im = D_ic (odd n)
__constant__ double cEB[NMAX + 1][MMAX][MMAX];      // B_ij
__constant__ double cEC[NMAX + 1][MMAX];            // middle row (odd n): B_cj

template <int N>
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
    double S = ODD ? cEA[N][i][M] * uc : cEA[N][i][0] * e[0];
    double T = cEB[N][i][0] * o[0];
#pragma unroll
    for (int j = ODD ? 0 : 1; j < M; j++) S = fma(cEA[N][i][j], e[j], S);
#pragma unroll
    for (int j = 1; j < M; j++) T = fma(cEB[N][i][j], o[j], T);
    out[i] = S + T;
    out[N - 1 - i] = T - S;
  }
  if (ODD) {
    double c = cEC[N][0] * o[0];
#pragma unroll
    for (int j = 1; j < M; j++) c = fma(cEC[N][j], o[j], c);
    out[M] = c;
  }
}

template <int N, int EPB, int NT>
__global__ void __launch_bounds__(NT) eo_kernel(StageParams P) {
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
      line_deriv<N>(sW + (fld * EPB + le) * NP + base, st, out);
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
cudaError_t launch_eo(const StageParams &P, cudaStream_t st) {
  constexpr int NP = N * N * N;
  const size_t shmem = sizeof(double) * 10 * EPB * NP;
  if (P.nelem <= 0)
    return cudaFuncSetAttribute(eo_kernel<N, EPB, NT>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shmem);
  eo_kernel<N, EPB, NT><<<(P.nelem + EPB - 1) / EPB, NT, shmem, st>>>(P);
  return cudaGetLastError();
}

constexpr size_t kSmemMax = 220 * 1024;

template <int N, int EPB, int NT>
void add_one(Variant *out, int cap, int &k) {
  if constexpr (sizeof(double) * 10 * EPB * N * N * N + 4096 <= kSmemMax && EPB <= 64) {
    if (k < cap) out[k++] = Variant{"eo", EPB, NT, launch_eo<N, EPB, NT>};
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

cudaError_t eo_upload(int n, const double *D) {
  if (n < 2 || n > NMAX) return cudaErrorInvalidValue;
  const int m = n / 2, odd = n & 1, c = n / 2;
  double A[MMAX][MMAX + 1] = {}, B[MMAX][MMAX] = {}, C[MMAX] = {};
  for (int i = 0; i < m; i++) {
    for (int j = 0; j < m; j++) {
      A[i][j] = 0.5 * (D[i * n + j] + D[i * n + (n - 1 - j)]);
      B[i][j] = 0.5 * (D[i * n + j] - D[i * n + (n - 1 - j)]);
    }
    if (odd) A[i][m] = D[i * n + c];
  }
  if (odd)
    for (int j = 0; j < m; j++) C[j] = 0.5 * (D[c * n + j] - D[c * n + (n - 1 - j)]);
  cudaError_t e;
  if ((e = cudaMemcpyToSymbol(cEA, A, sizeof(A), sizeof(A) * n)) != cudaSuccess) return e;
  if ((e = cudaMemcpyToSymbol(cEB, B, sizeof(B), sizeof(B) * n)) != cudaSuccess) return e;
  return cudaMemcpyToSymbol(cEC, C, sizeof(C), sizeof(C) * n);
}

}  // namespace nmgk
