// nmg.cu -- device context, FP64 DG right-hand side + RK4 stage kernels and
// the C ABI of include/nmg.h.
//
// One fused kernel per RK4 stage evaluates r = RHS(w) for the first-order
// scalar wave (reference: src/tests/scalarwave1/scalarwave1.c:242-321 with
// src/main/dg/dg.c:30-151, numflux1d.c:85-112) and applies the stage update
// of evolve_RK4_mesh (src/main/evolve/RungeKutta.c:19-82) in its epilogue, so
// that the stage's state is read once and written once.  On GB300 the FP64
// FMA pipe (measured 1.18 TFLOP/s, DMMA 1.05 TFLOP/s) and not HBM bounds this
// work, so the kernels are organised to issue as few FP64 instructions as
// possible: the lift factors of curvilinear faces and the chain-rule metric
// are precomputed on the host, the LLF flux is specialised to the wave
// system's constant speed 1, and Cartesian elements use 6 directional
// derivatives per node instead of 12.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/nmg.h"
#include "mesh.h"

#define NF 5
#define NMAX 12

namespace {

// per-launch parameters
struct StageParams {
  int nelem;
  const double *win;    // w read by the RHS (neighbour traces too)
  const double *u0;     // u at the start of the step
  double *acc;          // u accumulator
  double *wout;         // next stage's w
  double *rout;         // RHS output (mode 0)
  int mode;             // 0: r only; 1..4: RK4 stage
  double t;             // time of this RHS evaluation
  double cacc, cw;      // stage coefficients: acc += cacc*r, wout = u0 + cw*r
  const double *tdev;   // if non-null: step time read from tdev[*stepdev]
  const int *stepdev;
  double tofs_dt;       // stage time = step time + tofs_dt
  // mesh
  const int *nb;        // [E][6]
  const int *code;      // [E][6]
  const int *cslot;     // [E] curvilinear slot or -1
  const int *bslot;     // [E][6] outer-face slot or -1
  const double *scale;  // [E][3] dXb/dx of Cartesian elements
  const double *gcart;  // [E][3] dXb/dx / (2 w_end): lift factor of Cartesian faces
  const double *metric; // [C][9][np] M[a][i] = dXb^a/dx^i
  const double *fac;    // [C][6][nn][4] (g*n0, g*n1, g*n2, g), g = sqrtgdiag/(2w)
  const double *bxyz;   // [B][3][nn] coordinates of outer-face nodes
  const double *bnrm;   // [B][3][nn] outward unit normals there
  int bc;               // NMG_BC_*
  double k0, k1, k2, om;
  const double *D;      // [n][n] D[i*n+j] = l_j'(x_i)
  double w_end;         // LGL weight of the end points
};

constexpr int NT = 256;
template <int N>
struct Cfg {
  static constexpr int NP = N * N * N;
  static constexpr int NN = N * N;
  static constexpr int EPB = (NP >= 343) ? 1 : (512 / NP > 64 ? 64 : 512 / NP);
};

template <int N>
__device__ __forceinline__ int face_node_d(int f, int a, int b) {
  const int d = f >> 1, p = (f & 1) * (N - 1);
  return d == 0 ? p + N * (a + N * b) : d == 1 ? a + N * (p + N * b) : a + N * (b + N * p);
}

template <int N>
__global__ void __launch_bounds__(NT) dg_stage_kernel(StageParams P) {
  constexpr int NP = Cfg<N>::NP, NN = Cfg<N>::NN, EPB = Cfg<N>::EPB;
  extern __shared__ double smem[];
  double *sW = smem;                 // [4][EPB][NP]
  double *sR = smem + 4 * EPB * NP;  // [4][EPB][NP]
  __shared__ double sD[N * N];
  __shared__ int sCs[EPB];
  __shared__ double sScale[EPB][3];
  __shared__ double sG[EPB][3];

  const int e0 = blockIdx.x * EPB;
  const int tid = threadIdx.x;
  for (int q = tid; q < N * N; q += NT) sD[q] = P.D[q];
  for (int q = tid; q < EPB; q += NT) {
    int e = e0 + q;
    sCs[q] = (e < P.nelem) ? P.cslot[e] : -1;
    for (int d = 0; d < 3; d++) sScale[q][d] = (e < P.nelem) ? P.scale[e * 3 + d] : 0.;
    for (int d = 0; d < 3; d++) sG[q][d] = (e < P.nelem) ? P.gcart[e * 3 + d] : 0.;
  }
  double t = P.t;
  if (P.tdev) t = P.tdev[*P.stepdev] + P.tofs_dt;

  // stage pi, cx, cy, cz of w
  for (int q = tid; q < EPB * 4 * NP; q += NT) {
    int le = q / (4 * NP), rem = q - le * 4 * NP, f = rem / NP, node = rem - f * NP;
    int e = e0 + le;
    double v = 0.;
    if (e < P.nelem) v = P.win[((size_t)e * NF + f) * NP + node];
    sW[(f * EPB + le) * NP + node] = v;
  }
  __syncthreads();

  // ---- volume terms: r_pi = div c, r_c = grad pi ----
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
      for (int q2 = 0; q2 < 9; q2++) m[q2] = M[q2 * NP];
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

  // ---- surface terms, one direction at a time (faces 2d, 2d+1 disjoint) ----
#pragma unroll 1
  for (int d = 0; d < 3; d++) {
    for (int q = tid; q < EPB * 2 * NN; q += NT) {
      const int le = q / (2 * NN), rem = q - le * 2 * NN, s = rem / NN, ab = rem - s * NN;
      const int e = e0 + le;
      if (e >= P.nelem) continue;
      const int a = ab % N, b = ab / N, f = 2 * d + s;
      const int node = face_node_d<N>(f, a, b);
      const double ui0 = sW[(0 * EPB + le) * NP + node];
      const double ui1 = sW[(1 * EPB + le) * NP + node];
      const double ui2 = sW[(2 * EPB + le) * NP + node];
      const double ui3 = sW[(3 * EPB + le) * NP + node];
      // face factors g*n and g with g = sqrtgdiag/(2 w_end)
      double gn0, gn1, gn2, g;
      const int cs = sCs[le];
      if (cs < 0) {
        g = sG[le][d];
        const double sg = (f & 1) ? g : -g;
        gn0 = d == 0 ? sg : 0.;
        gn1 = d == 1 ? sg : 0.;
        gn2 = d == 2 ? sg : 0.;
      } else {
        const double *F4 = P.fac + (((size_t)cs * 6 + f) * NN + ab) * 4;
        gn0 = F4[0]; gn1 = F4[1]; gn2 = F4[2]; g = F4[3];
      }
      double ua0, ua1, ua2, ua3;
      const int nbe = P.nb[e * 6 + f];
      if (nbe >= 0) {
        const int cd = P.code[e * 6 + f], f2 = cd & 7, o = cd >> 3;
        const int sw = o & 1, fa = (o >> 1) & 1, fb = (o >> 2) & 1;
        int aa = sw ? b : a, bb = sw ? a : b;
        aa = fa ? N - 1 - aa : aa;
        bb = fb ? N - 1 - bb : bb;
        const double *W2 = P.win + (size_t)nbe * NF * NP + face_node_d<N>(f2, aa, bb);
        ua0 = W2[0];
        ua1 = W2[NP];
        ua2 = W2[2 * NP];
        ua3 = W2[3 * NP];
      } else {
        const int bs = P.bslot[e * 6 + f];
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
          const double *Nr = P.bnrm + (size_t)bs * 3 * NN + ab;
          const double n0 = Nr[0], n1 = Nr[NN], n2 = Nr[2 * NN];
          const double cnv = ui1 * n0 + ui2 * n1 + ui3 * n2;
          const double wout = ui0 - cnv;
          const double dcn = -0.5 * wout - cnv;  // exterior c.n minus interior c.n
          ua0 = 0.5 * wout;
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
      *r1 = fma(dpi, gn0, fma(g, dcx, *r1));
      *r2 = fma(dpi, gn1, fma(g, dcy, *r2));
      *r3 = fma(dpi, gn2, fma(g, dcz, *r3));
    }
    __syncthreads();
  }

  // ---- epilogue: r out or RK4 stage update ----
  for (int q = tid; q < EPB * NF * NP; q += NT) {
    const int le = q / (NF * NP), rem = q - le * NF * NP, f = rem / NP, node = rem - f * NP;
    const int e = e0 + le;
    if (e >= P.nelem) continue;
    const size_t idx = ((size_t)e * NF + f) * NP + node;
    const double r = (f < 4) ? sR[(f * EPB + le) * NP + node] : sW[(0 * EPB + le) * NP + node];
    if (P.mode == 0) {
      P.rout[idx] = r;
    } else if (P.mode == 1) {
      const double u = P.u0[idx];
      P.acc[idx] = fma(P.cacc, r, u);
      P.wout[idx] = fma(P.cw, r, u);
    } else if (P.mode == 4) {
      P.acc[idx] = fma(P.cacc, r, P.acc[idx]);
    } else {
      P.acc[idx] = fma(P.cacc, r, P.acc[idx]);
      P.wout[idx] = fma(P.cw, r, P.u0[idx]);
    }
  }
}

__global__ void advance_step_kernel(int *step) { *step += 1; }

// FP64 FMA throughput probe: 8 independent FMA chains per thread
__global__ void __launch_bounds__(256) fp64_peak_kernel(double *out, int iters, double a, double b) {
  double x[8];
#pragma unroll
  for (int c = 0; c < 8; c++) x[c] = threadIdx.x * 1e-3 + c;
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int c = 0; c < 8; c++) x[c] = fma(x[c], a, b);
  }
  double s = 0;
#pragma unroll
  for (int c = 0; c < 8; c++) s += x[c];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <int N>
cudaError_t launch_stage(const StageParams &P, cudaStream_t st) {
  constexpr int NP = Cfg<N>::NP, EPB = Cfg<N>::EPB;
  const size_t shmem = sizeof(double) * 8 * EPB * NP;
  if (P.nelem <= 0) {  // used once per context before any capture: set the
                       // dynamic shared memory limit of this instantiation
    return cudaFuncSetAttribute(dg_stage_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)shmem);
  }
  const int grid = (P.nelem + EPB - 1) / EPB;
  dg_stage_kernel<N><<<grid, NT, shmem, st>>>(P);
  return cudaGetLastError();
}

typedef cudaError_t (*LaunchFn)(const StageParams &, cudaStream_t);
LaunchFn launcher_for(int n) {
  switch (n) {
    case 2: return launch_stage<2>;
    case 3: return launch_stage<3>;
    case 4: return launch_stage<4>;
    case 5: return launch_stage<5>;
    case 6: return launch_stage<6>;
    case 7: return launch_stage<7>;
    case 8: return launch_stage<8>;
    case 9: return launch_stage<9>;
    case 10: return launch_stage<10>;
    case 11: return launch_stage<11>;
    case 12: return launch_stage<12>;
    default: return nullptr;
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------
struct nmg_ctx {
  std::string err;
  int n = 0, np = 0, nn = 0;
  int64_t nelem = 0, ncurvi = 0, nbface = 0;
  size_t state_len = 0;
  int bc = 0;
  double k[3] = {0, 0, 0};
  cudaStream_t stream = nullptr;
  LaunchFn launch = nullptr;
  // device arrays
  int *d_nb = nullptr, *d_code = nullptr, *d_cslot = nullptr, *d_bslot = nullptr;
  double *d_gcart = nullptr;
  double *d_scale = nullptr, *d_metric = nullptr, *d_fac = nullptr, *d_bxyz = nullptr,
         *d_bnrm = nullptr;
  double *d_D = nullptr, w_end = 0;
  double *d_buf[4] = {nullptr, nullptr, nullptr, nullptr};  // two states + two stage buffers
  int cur = 0;  // d_buf[cur] holds u
  double *d_times = nullptr;
  int *d_step = nullptr;
  int times_cap = 0;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};  // one RK4 step, u in d_buf[0] / d_buf[1]
  double graph_dt = 0;
  int64_t launches = 0;
};

static int set_err(nmg_ctx *c, int code, const std::string &msg) {
  if (c) c->err = msg;
  return code;
}

#define CK(call)                                                                   \
  do {                                                                             \
    cudaError_t e_ = (call);                                                       \
    if (e_ != cudaSuccess)                                                         \
      return set_err(c, NMG_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

static StageParams base_params(nmg_ctx *c) {
  StageParams P;
  std::memset(&P, 0, sizeof(P));
  P.nelem = (int)c->nelem;
  P.nb = c->d_nb;
  P.code = c->d_code;
  P.cslot = c->d_cslot;
  P.bslot = c->d_bslot;
  P.scale = c->d_scale;
  P.gcart = c->d_gcart;
  P.metric = c->d_metric;
  P.fac = c->d_fac;
  P.bxyz = c->d_bxyz;
  P.bnrm = c->d_bnrm;
  P.D = c->d_D;
  P.w_end = c->w_end;
  P.bc = c->bc;
  P.k0 = c->k[0];
  P.k1 = c->k[1];
  P.k2 = c->k[2];
  P.om = sqrt(c->k[0] * c->k[0] + c->k[1] * c->k[1] + c->k[2] * c->k[2]);
  return P;
}

// enqueue the 4 stage launches of one RK4 step with u in d_buf[cur]
static int enqueue_step(nmg_ctx *c, int cur, double t, double dt, bool devtime) {
  double *U = c->d_buf[cur], *ACC = c->d_buf[1 - cur], *WA = c->d_buf[2], *WB = c->d_buf[3];
  const double cacc[4] = {dt / 6., dt / 3., dt / 3., dt / 6.};
  const double cw[4] = {dt / 2., dt / 2., dt, 0.};
  const double tofs[4] = {0., 0.5 * dt, 0.5 * dt, dt};
  const double *win[4] = {U, WA, WB, WA};
  double *wout[4] = {WA, WB, WA, nullptr};
  for (int s = 0; s < 4; s++) {
    StageParams P = base_params(c);
    P.win = win[s];
    P.u0 = U;
    P.acc = ACC;
    P.wout = wout[s];
    P.mode = s + 1;
    P.cacc = cacc[s];
    P.cw = cw[s];
    if (devtime) {
      P.tdev = c->d_times;
      P.stepdev = c->d_step;
      P.tofs_dt = tofs[s];
    } else {
      // reference: mesh->time = t, t+0.5*dt, t+0.5*dt, t+dt
      P.t = (s == 0) ? t : (s == 3) ? t + dt : t + 0.5 * dt;
    }
    CK(c->launch(P, c->stream));
    c->launches++;
  }
  return NMG_OK;
}

extern "C" {

int nmg_create(const nmg_mesh *m, int32_t bc_kind, const double k[3], nmg_ctx **out) {
  if (!out) return NMG_EINVAL;
  *out = nullptr;
  nmg_ctx *c = new (std::nothrow) nmg_ctx;
  if (!c) return NMG_ENOMEM;
  *out = c;
  if (!m) return set_err(c, NMG_EINVAL, "nmg_create: null mesh");
  if (bc_kind != NMG_BC_EXACT_PLANEWAVE && bc_kind != NMG_BC_OUTGOING)
    return set_err(c, NMG_EINVAL, "nmg_create: unknown bc kind");
  c->launch = launcher_for(m->n);
  if (!c->launch) return set_err(c, NMG_EUNSUP, "nmg_create: n must be in [2,12]");
  int dev = 0;
  CK(cudaGetDevice(&dev));
  const int n = m->n, np = n * n * n, nn = n * n;
  const int64_t E = m->nelem;
  if (E <= 0 || E > (int64_t)1 << 30) return set_err(c, NMG_EINVAL, "nmg_create: bad element count");
  c->n = n; c->np = np; c->nn = nn; c->nelem = E;
  c->bc = bc_kind;
  if (k) for (int d = 0; d < 3; d++) c->k[d] = k[d];
  c->state_len = (size_t)E * NF * np;

  // host-side packing of per-element data
  std::vector<int> cslot(E, -1), bslot(E * 6, -1);
  std::vector<double> scale(E * 3, 0.), gcart(E * 3, 0.);
  int64_t C = 0, B = 0;
  for (int64_t e = 0; e < E; e++) {
    if (m->curvi[e]) cslot[e] = (int)C++;
    for (int f = 0; f < 6; f++)
      if (m->nb[e * 6 + f] < 0) bslot[e * 6 + f] = (int)B++;
    for (int d = 0; d < 3; d++)
      scale[e * 3 + d] = 2. / (m->bbox[e * 6 + 2 * d + 1] - m->bbox[e * 6 + 2 * d]);
    for (int d = 0; d < 3; d++) gcart[e * 3 + d] = 0.5 * scale[e * 3 + d] / m->w[0];
  }
  c->ncurvi = C;
  c->nbface = B;
  std::vector<double> metric((size_t)std::max<int64_t>(C, 1) * 9 * np, 0.);
  std::vector<double> fac((size_t)std::max<int64_t>(C, 1) * 6 * nn * 4, 0.);
  std::vector<double> bxyz((size_t)std::max<int64_t>(B, 1) * 3 * nn, 0.);
  std::vector<double> bnrm((size_t)std::max<int64_t>(B, 1) * 3 * nn, 0.);
  for (int64_t e = 0; e < E; e++) {
    const double *X9 = &m->dXdx[(size_t)e * 9 * np];
    const double *sc = &scale[e * 3];
    if (cslot[e] >= 0) {
      double *Mt = &metric[(size_t)cslot[e] * 9 * np];
      for (int a = 0; a < 3; a++)
        for (int i = 0; i < 3; i++)
          for (int q = 0; q < np; q++) Mt[(a * 3 + i) * np + q] = sc[a] * X9[(a * 3 + i) * np + q];
      for (int f = 0; f < 6; f++) {
        const int d = f >> 1, p = (f & 1) * (n - 1);
        const double sig = (f & 1) ? 1. : -1.;
        for (int b = 0; b < n; b++)
          for (int a = 0; a < n; a++) {
            const int node = nmg::face_node(n, f, a, b);
            const double v0 = X9[(d * 3 + 0) * np + node], v1 = X9[(d * 3 + 1) * np + node],
                         v2 = X9[(d * 3 + 2) * np + node];
            const double mag = sqrt(v0 * v0 + v1 * v1 + v2 * v2);
            const double g = 0.5 * sc[d] * mag / m->w[p];  // sqrtgdiag / (2 w_end)
            double *F4 = &fac[(((size_t)cslot[e] * 6 + f) * nn + a + n * b) * 4];
            F4[0] = g * sig * v0 / mag;
            F4[1] = g * sig * v1 / mag;
            F4[2] = g * sig * v2 / mag;
            F4[3] = g;
          }
      }
    }
    for (int f = 0; f < 6; f++) {
      const int bs = bslot[e * 6 + f];
      if (bs < 0) continue;
      const int d = f >> 1;
      const double sig = (f & 1) ? 1. : -1.;
      for (int b = 0; b < n; b++)
        for (int a = 0; a < n; a++) {
          const int node = nmg::face_node(n, f, a, b), ab = a + n * b;
          for (int q = 0; q < 3; q++)
            bxyz[((size_t)bs * 3 + q) * nn + ab] = m->xyz[((size_t)e * 3 + q) * np + node];
          const double v0 = X9[(d * 3 + 0) * np + node], v1 = X9[(d * 3 + 1) * np + node],
                       v2 = X9[(d * 3 + 2) * np + node];
          const double mag = sqrt(v0 * v0 + v1 * v1 + v2 * v2);
          bnrm[((size_t)bs * 3 + 0) * nn + ab] = sig * v0 / mag;
          bnrm[((size_t)bs * 3 + 1) * nn + ab] = sig * v1 / mag;
          bnrm[((size_t)bs * 3 + 2) * nn + ab] = sig * v2 / mag;
        }
    }
  }
  std::vector<int> code(m->code.begin(), m->code.end());
  CK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  auto up = [&](auto **dst, const auto &vec) -> cudaError_t {
    size_t bytes = vec.size() * sizeof(vec[0]);
    cudaError_t e2 = cudaMalloc((void **)dst, bytes);
    if (e2 != cudaSuccess) return e2;
    return cudaMemcpy(*dst, vec.data(), bytes, cudaMemcpyHostToDevice);
  };
  CK(up(&c->d_nb, m->nb));
  CK(up(&c->d_code, code));
  CK(up(&c->d_cslot, cslot));
  CK(up(&c->d_bslot, bslot));
  CK(up(&c->d_scale, scale));
  CK(up(&c->d_gcart, gcart));
  CK(up(&c->d_metric, metric));
  CK(up(&c->d_fac, fac));
  CK(up(&c->d_bxyz, bxyz));
  CK(up(&c->d_bnrm, bnrm));
  for (int b = 0; b < 4; b++) {
    CK(cudaMalloc((void **)&c->d_buf[b], c->state_len * sizeof(double)));
    CK(cudaMemset(c->d_buf[b], 0, c->state_len * sizeof(double)));
  }
  CK(cudaMalloc((void **)&c->d_step, sizeof(int)));
  {
    StageParams P0;
    std::memset(&P0, 0, sizeof(P0));
    CK(c->launch(P0, c->stream));  // nelem == 0: only sets the smem limit
  }
  // basis (same D for every element)
  CK(up(&c->d_D, m->D));
  c->w_end = m->w[0];
  CK(cudaDeviceSynchronize());
  return NMG_OK;
}

void nmg_destroy(nmg_ctx *c) {
  if (!c) return;
  for (int g = 0; g < 2; g++)
    if (c->graph[g]) cudaGraphExecDestroy(c->graph[g]);
  cudaFree(c->d_nb); cudaFree(c->d_code); cudaFree(c->d_cslot); cudaFree(c->d_bslot);
  cudaFree(c->d_scale); cudaFree(c->d_gcart); cudaFree(c->d_metric); cudaFree(c->d_fac); cudaFree(c->d_bxyz);
  cudaFree(c->d_bnrm); cudaFree(c->d_D);
  for (int b = 0; b < 4; b++) cudaFree(c->d_buf[b]);
  cudaFree(c->d_times); cudaFree(c->d_step);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

const char *nmg_last_error(const nmg_ctx *c) { return c ? c->err.c_str() : "null context"; }
int64_t nmg_state_size(const nmg_ctx *c) { return c ? (int64_t)c->state_len : -1; }
int64_t nmg_kernel_launches(const nmg_ctx *c) { return c ? c->launches : -1; }
void *nmg_stream(nmg_ctx *c) { return c ? (void *)c->stream : nullptr; }
double *nmg_state_device_ptr(nmg_ctx *c) { return c ? c->d_buf[c->cur] : nullptr; }

int nmg_set_state(nmg_ctx *c, const double *host_u) {
  if (!c || !host_u) return set_err(c, NMG_EINVAL, "nmg_set_state: null argument");
  CK(cudaMemcpyAsync(c->d_buf[c->cur], host_u, c->state_len * sizeof(double),
                     cudaMemcpyHostToDevice, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return NMG_OK;
}

int nmg_get_state(nmg_ctx *c, double *host_u) {
  if (!c || !host_u) return set_err(c, NMG_EINVAL, "nmg_get_state: null argument");
  CK(cudaMemcpyAsync(host_u, c->d_buf[c->cur], c->state_len * sizeof(double),
                     cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return NMG_OK;
}

int nmg_rhs(nmg_ctx *c, double t, const double *w_dev, double *r_dev) {
  if (!c || !w_dev || !r_dev) return set_err(c, NMG_EINVAL, "nmg_rhs: null argument");
  StageParams P = base_params(c);
  P.win = w_dev;
  P.rout = r_dev;
  P.mode = 0;
  P.t = t;
  CK(c->launch(P, c->stream));
  c->launches++;
  return NMG_OK;
}

int nmg_rhs_host(nmg_ctx *c, double t, const double *w_host, double *r_host) {
  if (!c || !w_host || !r_host) return set_err(c, NMG_EINVAL, "nmg_rhs_host: null argument");
  const size_t bytes = c->state_len * sizeof(double);
  CK(cudaMemcpyAsync(c->d_buf[2], w_host, bytes, cudaMemcpyHostToDevice, c->stream));
  int rc = nmg_rhs(c, t, c->d_buf[2], c->d_buf[3]);
  if (rc) return rc;
  CK(cudaMemcpyAsync(r_host, c->d_buf[3], bytes, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return NMG_OK;
}

int nmg_rk4_step(nmg_ctx *c, double t, double dt) {
  if (!c) return NMG_EINVAL;
  int rc = enqueue_step(c, c->cur, t, dt, false);
  if (rc) return rc;
  c->cur = 1 - c->cur;
  CK(cudaStreamSynchronize(c->stream));
  return NMG_OK;
}

// capture one RK4 step (u in d_buf[cur]) reading its time from the device
static int capture_step_graph(nmg_ctx *c, int cur, double dt) {
  cudaGraph_t g;
  CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  int64_t l0 = c->launches;
  int rc = enqueue_step(c, cur, 0., dt, true);
  advance_step_kernel<<<1, 1, 0, c->stream>>>(c->d_step);
  cudaError_t e1 = cudaGetLastError();
  cudaError_t e2 = cudaStreamEndCapture(c->stream, &g);
  c->launches = l0;  // captured, not launched
  if (rc) return rc;
  CK(e1);
  CK(e2);
  if (c->graph[cur]) cudaGraphExecDestroy(c->graph[cur]);
  cudaError_t e3 = cudaGraphInstantiate(&c->graph[cur], g, 0);
  cudaGraphDestroy(g);
  CK(e3);
  return NMG_OK;
}

int nmg_rk4_steps(nmg_ctx *c, double t, double dt, int32_t nsteps) {
  if (!c || nsteps < 0) return set_err(c, NMG_EINVAL, "nmg_rk4_steps: bad argument");
  if (nsteps == 0) return NMG_OK;
  // step times as evolve_mesh accumulates them (long double), main.c:610-626
  std::vector<double> times(nsteps);
  long double Te = t, te = 0.;
  for (int s = 0; s < nsteps; s++) {
    times[s] = (double)(Te + te);
    te += dt;
  }
  if (nsteps > c->times_cap) {
    cudaFree(c->d_times);
    c->d_times = nullptr;
    CK(cudaMalloc((void **)&c->d_times, sizeof(double) * nsteps));
    c->times_cap = nsteps;
    for (int g = 0; g < 2; g++)
      if (c->graph[g]) { cudaGraphExecDestroy(c->graph[g]); c->graph[g] = nullptr; }
  }
  if (dt != c->graph_dt) {
    for (int g = 0; g < 2; g++)
      if (c->graph[g]) { cudaGraphExecDestroy(c->graph[g]); c->graph[g] = nullptr; }
    c->graph_dt = dt;
  }
  for (int g = 0; g < 2; g++)
    if (!c->graph[g]) {
      int rc = capture_step_graph(c, g, dt);
      if (rc) return rc;
    }
  CK(cudaMemcpyAsync(c->d_times, times.data(), sizeof(double) * nsteps, cudaMemcpyHostToDevice,
                     c->stream));
  CK(cudaMemsetAsync(c->d_step, 0, sizeof(int), c->stream));
  for (int s = 0; s < nsteps; s++) {
    CK(cudaGraphLaunch(c->graph[c->cur], c->stream));
    c->launches += 5;
    c->cur = 1 - c->cur;
  }
  CK(cudaStreamSynchronize(c->stream));
  return NMG_OK;
}

int nmg_fp64_peak(double *gflops) {
  nmg_ctx *c = nullptr;  // for CK: errors are returned without a context
  if (!gflops) return NMG_EINVAL;
  int dev = 0, sms = 0;
  CK(cudaGetDevice(&dev));
  CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int blocks = sms * 4, threads = 256, iters = 512;
  double *out = nullptr;
  CK(cudaMalloc((void **)&out, sizeof(double) * blocks * threads));
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  fp64_peak_kernel<<<blocks, threads>>>(out, 64, 1.0000001, 1e-9);
  CK(cudaGetLastError());
  float best = 1e30f;
  for (int r = 0; r < 5; r++) {
    CK(cudaEventRecord(e0));
    fp64_peak_kernel<<<blocks, threads>>>(out, iters, 1.0000001, 1e-9);
    CK(cudaEventRecord(e1));
    CK(cudaEventSynchronize(e1));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    best = std::min(best, ms);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  *gflops = 2.0 * 8 * iters * (double)blocks * threads / (best * 1e6);
  return NMG_OK;
}

int nmg_rk4_steps_host(nmg_ctx *c, double t, double dt, int32_t nsteps, double *host_u) {
  if (!c || !host_u) return set_err(c, NMG_EINVAL, "nmg_rk4_steps_host: null argument");
  const size_t bytes = c->state_len * sizeof(double);
  CK(cudaMemcpyAsync(c->d_buf[c->cur], host_u, bytes, cudaMemcpyHostToDevice, c->stream));
  int rc = nmg_rk4_steps(c, t, dt, nsteps);
  if (rc) return rc;
  CK(cudaMemcpyAsync(host_u, c->d_buf[c->cur], bytes, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return NMG_OK;
}

}  // extern "C"
