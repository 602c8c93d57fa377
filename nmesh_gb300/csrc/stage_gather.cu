// stage_gather.cu -- "gather" variant of the fused stage kernel: one thread
// per node computes all directional derivatives of its node with full
// n-point dot products (12 on curvilinear, 6 on Cartesian elements), then
// applies the chain rule.  Simple and balanced; the "eo" variant issues
// fewer FP64 instructions.
#include "stage.cuh"

namespace nmgk {
namespace {

template <int N, int EPB, int NT>
__global__ void __launch_bounds__(NT) gather_kernel(StageParams P) {
  constexpr int NP = N * N * N, NN = N * N;
  extern __shared__ double smem[];
  double *sW = smem;                 // [4][EPB][NP]
  double *sR = smem + 4 * EPB * NP;  // [4][EPB][NP]
  __shared__ double sD[N * N];
  __shared__ int sCs[EPB];
  __shared__ double sScale[EPB][3];
  __shared__ double sG[EPB][3];

  const int e0 = P.ebase + blockIdx.x * EPB;
  const int tid = threadIdx.x;
  for (int q = tid; q < N * N; q += NT) sD[q] = P.D[q];
  for (int q = tid; q < EPB; q += NT) {
    const int e = elem_at(P, e0 + q);
    sCs[q] = (e < P.nelem) ? P.cslot[e] : -1;
    for (int d = 0; d < 3; d++) sScale[q][d] = (e < P.nelem) ? P.scale[e * 3 + d] : 0.;
    for (int d = 0; d < 3; d++) sG[q][d] = (e < P.nelem) ? P.gcart[e * 3 + d] : 0.;
  }
  const double t = stage_time(P);
  stage_in<N, EPB, NT>(P, sW, e0);
  __syncthreads();

  for (int q = tid; q < EPB * NP; q += NT) {
    const int le = q / NP, node = q - le * NP;
    const int i = node % N, j = (node / N) % N, k = node / NN;
    const double *pi = sW + (0 * EPB + le) * NP;
    const double *cx = sW + (1 * EPB + le) * NP;
    const double *cy = sW + (2 * EPB + le) * NP;
    const double *cz = sW + (3 * EPB + le) * NP;
    double rpi, rcx, rcy, rcz;
    const int cs = sCs[le];
    if (cs < 0) {
      double dpx = 0, dpy = 0, dpz = 0, dcx = 0, dcy = 0, dcz = 0;
#pragma unroll
      for (int l = 0; l < N; l++) {
        const double Dx = sD[i * N + l], Dy = sD[j * N + l], Dz = sD[k * N + l];
        const int ix = l + N * (j + N * k), iy = i + N * (l + N * k), iz = i + N * (j + N * l);
        dpx = fma(Dx, pi[ix], dpx);
        dpy = fma(Dy, pi[iy], dpy);
        dpz = fma(Dz, pi[iz], dpz);
        dcx = fma(Dx, cx[ix], dcx);
        dcy = fma(Dy, cy[iy], dcy);
        dcz = fma(Dz, cz[iz], dcz);
      }
      const double s0 = sScale[le][0], s1 = sScale[le][1], s2 = sScale[le][2];
      rpi = fma(s0, dcx, fma(s1, dcy, s2 * dcz));
      rcx = s0 * dpx;
      rcy = s1 * dpy;
      rcz = s2 * dpz;
    } else {
      double dp[3] = {0, 0, 0}, dcxa[3] = {0, 0, 0}, dcya[3] = {0, 0, 0}, dcza[3] = {0, 0, 0};
#pragma unroll
      for (int l = 0; l < N; l++) {
        const double Dx = sD[i * N + l], Dy = sD[j * N + l], Dz = sD[k * N + l];
        const int ix = l + N * (j + N * k), iy = i + N * (l + N * k), iz = i + N * (j + N * l);
        dp[0] = fma(Dx, pi[ix], dp[0]);
        dp[1] = fma(Dy, pi[iy], dp[1]);
        dp[2] = fma(Dz, pi[iz], dp[2]);
        dcxa[0] = fma(Dx, cx[ix], dcxa[0]);
        dcxa[1] = fma(Dy, cx[iy], dcxa[1]);
        dcxa[2] = fma(Dz, cx[iz], dcxa[2]);
        dcya[0] = fma(Dx, cy[ix], dcya[0]);
        dcya[1] = fma(Dy, cy[iy], dcya[1]);
        dcya[2] = fma(Dz, cy[iz], dcya[2]);
        dcza[0] = fma(Dx, cz[ix], dcza[0]);
        dcza[1] = fma(Dy, cz[iy], dcza[1]);
        dcza[2] = fma(Dz, cz[iz], dcza[2]);
      }
      const double *M = P.metric + (size_t)cs * 9 * NP + node;
      double m[9];
#pragma unroll
      for (int q2 = 0; q2 < 9; q2++) m[q2] = __ldg(M + q2 * NP);
      rpi = 0.;
      rcx = 0.;
      rcy = 0.;
      rcz = 0.;
#pragma unroll
      for (int a = 0; a < 3; a++) {
        rpi = fma(m[a * 3 + 0], dcxa[a], rpi);
        rpi = fma(m[a * 3 + 1], dcya[a], rpi);
        rpi = fma(m[a * 3 + 2], dcza[a], rpi);
        rcx = fma(m[a * 3 + 0], dp[a], rcx);
        rcy = fma(m[a * 3 + 1], dp[a], rcy);
        rcz = fma(m[a * 3 + 2], dp[a], rcz);
      }
    }
    sR[(0 * EPB + le) * NP + node] = rpi;
    sR[(1 * EPB + le) * NP + node] = rcx;
    sR[(2 * EPB + le) * NP + node] = rcy;
    sR[(3 * EPB + le) * NP + node] = rcz;
  }
  __syncthreads();
  face_terms<N, EPB, NT>(P, sW, sR, sCs, sG, e0, t);
  epilogue<N, EPB, NT, false>(P, sW, sR, sCs, e0);
}

template <int N, int EPB, int NT>
cudaError_t launch_gather(const StageParams &P, cudaStream_t st) {
  constexpr int NP = N * N * N;
  const size_t shmem = sizeof(double) * 8 * EPB * NP;
  if (P.nelem <= 0)
    return cudaFuncSetAttribute(gather_kernel<N, EPB, NT>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shmem);
  const int ne = P.ecount > 0 ? P.ecount : P.nelem;
  gather_kernel<N, EPB, NT><<<(ne + EPB - 1) / EPB, NT, shmem, st>>>(P);
  return cudaGetLastError();
}

constexpr int epb_for(int np) { return np >= 343 ? 1 : (512 / np > 64 ? 64 : 512 / np); }

template <int N>
int add_gather(Variant *out, int cap) {
  constexpr int E = epb_for(N * N * N);
  int k = 0;
  if (k < cap) out[k++] = Variant{"gather", E, 256, launch_gather<N, E, 256>};
  return k;
}

}  // namespace

int gather_variants(int n, Variant *out, int cap) {
  switch (n) {
    case 2: return add_gather<2>(out, cap);
    case 3: return add_gather<3>(out, cap);
    case 4: return add_gather<4>(out, cap);
    case 5: return add_gather<5>(out, cap);
    case 6: return add_gather<6>(out, cap);
    case 7: return add_gather<7>(out, cap);
    case 8: return add_gather<8>(out, cap);
    case 9: return add_gather<9>(out, cap);
    case 10: return add_gather<10>(out, cap);
    case 11: return add_gather<11>(out, cap);
    case 12: return add_gather<12>(out, cap);
    default: return 0;
  }
}

}  // namespace nmgk
