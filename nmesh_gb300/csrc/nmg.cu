// nmg.cu -- device context and C ABI (include/nmg.h) of the GB300-native
// nmesh evolution path.
//
// One fused kernel per RK4 stage evaluates r = RHS(w) for the first-order
// scalar wave and applies the stage update of evolve_RK4_mesh
// (src/main/evolve/RungeKutta.c:19-82) in its epilogue (stage.cuh).  On
// GB300 the FP64 FMA pipe (measured 1.18 TFLOP/s; DMMA 1.05 TFLOP/s) and
// not HBM bounds this work, so the kernels minimise FP64 instructions, and
// the per-context autotuner picks the kernel variant and tile shape
// (elements and threads per CTA) by timing each candidate on this mesh.
//
// Device buffers of a context: the mesh data (face table, Cartesian scale
// factors, curvilinear metric in two layouts, curvilinear lift factors,
// outer-face coordinates and normals) and four state buffers: u and the u
// accumulator (swapped after every step) and two stage buffers w.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/nmg.h"
#include "ctx.h"
#include "mesh.h"
#include "stage.cuh"

using nmgk::StageParams;
using nmgk::Variant;

namespace {

__global__ void advance_step_kernel(int *step) { *step += 1; }

// FP64 FMA throughput probe: 8 independent FMA chains per thread
__global__ void __launch_bounds__(256) fp64_peak_kernel(double *out, int iters, double a,
                                                        double b) {
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

// FP64 tensor-core (DMMA, mma.sync m8n8k4 f64) throughput probe: 4
// independent accumulator chains per warp; one mma is 8 x 8 x 4 FMA
__global__ void __launch_bounds__(256) dmma_peak_kernel(double *out, int iters, double a,
                                                        double b) {
  const double av = a + threadIdx.x * 1e-9, bv = b;
  double c[4][2];
#pragma unroll
  for (int k = 0; k < 4; k++) c[k][0] = c[k][1] = k * 1e-3;
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int k = 0; k < 4; k++)
      asm volatile(
          "mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};"
          : "+d"(c[k][0]), "+d"(c[k][1])
          : "d"(av), "d"(bv));
  }
  double s = 0;
#pragma unroll
  for (int k = 0; k < 4; k++) s += c[k][0] + c[k][1];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// Traces of faces joined across the parts of a batched problem: per link
// (target group, ghost slot, source group, element, face, orientation),
// field (pi, c) and target face node, the source face plane interpolated at
// the node's position, sum_b l_b(t) sum_a l_a(s) W[a, b] with the source's
// LGL Lagrange basis in barycentric form (weights btab).
__global__ void plink_kernel(const int *links, int nlink, const int *gn, double *const *ghost,
                             const double *const *wsrc, const double *xtab, const double *btab) {
  constexpr int M = nmgk::kBatchMaxN;
  const int64_t tot = (int64_t)nlink * 4 * M * M;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < tot;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int l = (int)(i / (4 * M * M)), rem = (int)(i % (4 * M * M));
    const int fld = rem / (M * M), ab = rem % (M * M);
    const int *L = links + 6 * l;
    const int tg = L[0], ts = L[1], sg = L[2], se = L[3], sf = L[4], o = L[5];
    const int nt = gn[tg], ns = gn[sg];
    const int a = ab % M, b = ab / M;
    if (a >= nt || b >= nt) continue;
    const double *xt = xtab + nt * M, *xs = xtab + ns * M, *bs = btab + ns * M;
    double u = (o & 1) ? xt[b] : xt[a], v = (o & 1) ? xt[a] : xt[b];
    if (o & 2) u = -u;
    if (o & 4) v = -v;
    double la[M], lb[M];
    for (int k = 0; k < ns; k++) {
      double pa = bs[k], pb = bs[k];
      for (int j = 0; j < ns; j++)
        if (j != k) {
          pa *= u - xs[j];
          pb *= v - xs[j];
        }
      la[k] = pa;
      lb[k] = pb;
    }
    const int nps = ns * ns * ns;
    const double *W = wsrc[sg] + ((size_t)se * NF + fld) * nps;
    const int d = sf >> 1, pq = (sf & 1) * (ns - 1);
    double val = 0.;
    for (int kb = 0; kb < ns; kb++) {
      double row = 0.;
      for (int ka = 0; ka < ns; ka++) {
        const int node = d == 0 ? pq + ns * (ka + ns * kb)
                                : (d == 1 ? ka + ns * (pq + ns * kb) : ka + ns * (kb + ns * pq));
        row = fma(la[ka], W[node], row);
      }
      val = fma(lb[kb], row, val);
    }
    ghost[tg][((size_t)ts * 4 + fld) * nt * nt + a + nt * b] = val;
  }
}

constexpr int kMaxVariants = 24;

// Objective J = dt sum_nodes W phi^2 of one state, in two deterministic
// passes: per-block partial sums (fixed-order tree), then one thread adds
// the partials in order and accumulates dt * sum into *out.
constexpr int kObjThreads = 256;
__global__ void __launch_bounds__(kObjThreads)
    obj_partial_kernel(const double *u, const double *W, int nelem, int np, double *partial) {
  __shared__ double sh[kObjThreads];
  double s = 0.;
  const int64_t nn = (int64_t)nelem * np;
  const int64_t per = (nn + gridDim.x - 1) / gridDim.x;
  const int64_t b0 = per * blockIdx.x, b1 = min(nn, b0 + per);
  for (int64_t q = b0 + threadIdx.x; q < b1; q += kObjThreads) {
    const int64_t e = q / np, node = q - e * np;
    const double phi = u[(e * NF + 4) * np + node];
    s = fma(W[q] * phi, phi, s);
  }
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = kObjThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

__global__ void obj_final_kernel(const double *partial, int nblk, double dt, double *out) {
  double s = 0.;
  for (int b = 0; b < nblk; b++) s += partial[b];
  *out += dt * s;
}

// 0d norms: per element and field the quadrature sums of v and v^2 with the
// weights w_i w_j w_k / |det(dXb/dx)| (NodeVolumeIntegral,
// src/main/coordinates/integrals.c:12-60), min and max; then one thread per
// field adds the element partials in element order
constexpr int kNormThreads = 128;
__global__ void __launch_bounds__(kNormThreads)
    norms_elem_kernel(int n, int nelem, const double *u, const int *cslot, const double *scale,
                      const double *metric, const double *fvgeo, int allfv,
                      const unsigned char *isfv, const double *wl, const double *wu,
                      double *part) {
  __shared__ double sh[4][kNormThreads];
  const int np = n * n * n, e = blockIdx.x;
  if (e >= nelem) return;
  const bool efv = allfv || (isfv && isfv[e]);
  const double *w = efv ? wu : wl;
  const int cs = cslot[e];
  const double s0 = scale[e * 3], s1 = scale[e * 3 + 1], s2 = scale[e * 3 + 2];
  for (int l = -1; l < NF; l++) {   // l = -1: the volume (v = 1)
    double a1 = 0., a2 = 0., lo = 1e300, hi = -1e300;
    for (int q = threadIdx.x; q < np; q += kNormThreads) {
      const int i = q % n, j = (q / n) % n, k = q / (n * n);
      double det;
      if (cs < 0) {
        det = s0 * s1 * s2;
      } else if (efv) {
        det = fvgeo[(size_t)cs * 13 * np + q];
      } else {
        const double *M = metric + (size_t)cs * 9 * np + q;
        const double m00 = M[0], m01 = M[np], m02 = M[2 * np], m10 = M[3 * np], m11 = M[4 * np],
                     m12 = M[5 * np], m20 = M[6 * np], m21 = M[7 * np], m22 = M[8 * np];
        det = m00 * (m11 * m22 - m12 * m21) - m01 * (m10 * m22 - m12 * m20) +
              m02 * (m10 * m21 - m11 * m20);
      }
      const double qw = det != 0. ? w[i] * w[j] * w[k] / fabs(det) : 0.;
      const double v = l < 0 ? 1. : u[((size_t)e * NF + l) * np + q];
      a1 += qw * v;
      a2 += qw * v * v;
      lo = fmin(lo, v);
      hi = fmax(hi, v);
    }
    sh[0][threadIdx.x] = a1;
    sh[1][threadIdx.x] = a2;
    sh[2][threadIdx.x] = lo;
    sh[3][threadIdx.x] = hi;
    __syncthreads();
    for (int s = kNormThreads / 2; s > 0; s >>= 1) {
      if (threadIdx.x < s) {
        sh[0][threadIdx.x] += sh[0][threadIdx.x + s];
        sh[1][threadIdx.x] += sh[1][threadIdx.x + s];
        sh[2][threadIdx.x] = fmin(sh[2][threadIdx.x], sh[2][threadIdx.x + s]);
        sh[3][threadIdx.x] = fmax(sh[3][threadIdx.x], sh[3][threadIdx.x + s]);
      }
      __syncthreads();
    }
    if (threadIdx.x == 0)
      for (int c = 0; c < 4; c++) part[((size_t)e * (NF + 1) + (l + 1)) * 4 + c] = sh[c][0];
    __syncthreads();
  }
}

__global__ void norms_final_kernel(int nelem, const double *part, double *out) {
  const int l = threadIdx.x;  // 0: volume, 1..5: fields
  if (l > NF) return;
  double a1 = 0., a2 = 0., lo = 1e300, hi = -1e300;
  for (int e = 0; e < nelem; e++) {
    const double *p = part + ((size_t)e * (NF + 1) + l) * 4;
    a1 += p[0];
    a2 += p[1];
    lo = fmin(lo, p[2]);
    hi = fmax(hi, p[3]);
  }
  out[l * 4] = a1;
  out[l * 4 + 1] = a2;
  out[l * 4 + 2] = lo;
  out[l * 4 + 3] = hi;
}

// adjoint source of J at one step: lambda_phi += coef W phi
__global__ void adj_source_kernel(double *lambda, const double *u, const double *W, int nelem,
                                  int np, double coef) {
  const int64_t nn = (int64_t)nelem * np;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < nn;
       q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = q / np, node = q - e * np;
    const int64_t idx = (e * NF + 4) * np + node;
    lambda[idx] = fma(coef * W[q], u[idx], lambda[idx]);
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------
struct nmg_ctx {
  std::string err;
  const char *err_static = nullptr;  // set instead of err by allocation-free paths
  int n = 0, np = 0, nn = 0;
  int device = -1;   // CUDA device the context's memory lives on
  int64_t nelem = 0, ncurvi = 0, nbface = 0;
  size_t state_len = 0;
  int bc = 0;
  double k[3] = {0, 0, 0};
  cudaStream_t stream = nullptr;
  Variant variants[kMaxVariants];
  Variant vjp;  // transposed stage kernel (the tensor-core one where compiled)
  Variant vjp_alt[2];  // the FP64 and the tensor-core transposed kernels
  int nvjp_alt = 0;
  int nvariants = 0;
  int sel = -1;      // selected variant, -1: autotune on first use
  bool tuned = false;
  std::string tune_log;
  // device arrays
  int *d_nb = nullptr, *d_code = nullptr, *d_cslot = nullptr, *d_bslot = nullptr,
      *d_cmask = nullptr;
  double *d_scale = nullptr, *d_gcart = nullptr, *d_metric = nullptr, *d_metricp = nullptr,
         *d_fac = nullptr, *d_bxyz = nullptr, *d_bnrm = nullptr, *d_D = nullptr;
  double *d_buf[4] = {nullptr, nullptr, nullptr, nullptr};
  int cur = 0;  // d_buf[cur] holds u
  double *d_times = nullptr;
  int *d_step = nullptr;
  int times_cap = 0;
  // finite-volume mesh: options and geometry (stage_fv.cu)
  int numflux = NMG_NUMFLUX_LLF;
  bool fv = false;     // some elements are finite-volume
  bool mixed = false;  // ... and some DG: variants[0, ndg) DG, [ndg, n) FV
  int ndg = 0, fsel = -1;
  bool ftuned = false;
  int nfvel = 0, nghost = 0;
  int *d_fvlist = nullptr, *d_gtab = nullptr;
  unsigned char *d_isfv = nullptr;
  double *d_ghost = nullptr, *d_gM = nullptr;
  double *d_fvbxyz = nullptr, *d_fvbnrm = nullptr;  // outer faces on equally spaced points
  int ghost_cap = 0;
  // non-conforming faces: their traces (slots of d_ghost) are interpolated
  // from the neighbour faces each stage (stage_fv.cu: hang_kernel)
  int nhang = 0;
  int *d_hoff = nullptr;    // [H*nn + 1] contribution offsets per face node
  int *d_hsrc = nullptr;    // [C][2] source element, source face
  double *d_hw = nullptr;   // [C][2][n] Lagrange weights at the node's position
  // the transposed lists (adjoint): per slot and source-face node, the
  // (slot * nn + node) pairs that read it and their weights; slot owners
  int *d_toff = nullptr, *d_tsrc = nullptr, *d_hface = nullptr;
  double *d_tw = nullptr;
  std::vector<int32_t> h_hoff, h_hsrc, h_hface;
  std::vector<double> h_hw;
  // switchable contexts: element types can change (nmg_set_element_types)
  bool switchable = false;
  std::vector<int32_t> h_nb, h_code0, h_bslot0, h_fv;  // face table without the mixed bit,
                                                       // outer-face slots, current types
  double *d_PR = nullptr;      // [3][n][n] LGL -> uniform (P), uniform -> LGL (R), and
                               // the modal analysis matrix of the LGL points (A)
  std::vector<int32_t> h_score;  // trouble score of each element
  int *d_conv = nullptr;       // [E] element list of a conversion
  double *d_mm = nullptr;      // [E][5][2] min/max of u_p per element and field
  int *d_trb = nullptr;        // [E] trouble flag of the last check
  int *d_score = nullptr;      // [E] trouble score (node->dat->info->trbl_score)
  double *d_up = nullptr;      // u_p: state at the start of a checked step
  // substep redo (evolve_redo_troubled = substep): the stage's r, the stage
  // input with the troubled elements converted, and the face tables of the
  // troubled elements as finite-volume elements among old-type neighbours
  double *d_r = nullptr, *d_w2 = nullptr, *d_ghost2 = nullptr;
  int *d_tlist = nullptr, *d_code2 = nullptr, *d_bslot2 = nullptr, *d_gtab2 = nullptr;
  int ghost2_cap = 0;
  double *d_pers = nullptr;    // [E][5] Persson indicators of the last check
  double *d_wq = nullptr;      // [2][n] LGL and trapezoid (equally spaced) weights
  double *d_npart = nullptr;   // [E][6][4] partial norms
  int fv_rec = NMG_FV_REC_WENOM3_2, fv_extrap = NMG_FV_EXTRAP_DNFN1;
  int fv_surf = NMG_FV_SURF_LINEAR;   // traces from FV neighbours (fv_surface_interp)
  // coordinates_midpoint_data = yes: midpoint factors of curvilinear elements
  bool fv_mid = false;
  // exponential filter after each step (evolve_filter_all = yes)
  bool filter_on = false;
  // limiter (scalarwave1_limiter = MRS or minmodB): per element and field
  // the MRS node average / extrema or the minmodB coefficients c000, c100,
  // c010, c001 (d_lim, [E][NF][4]), the face neighbours of every element
  // face (CSR [E*6+1]), alpha h^1.5 (MRS) or alpha h (minmodB) per element;
  // d_mmb: [2 analysis rows; 2 synthesis columns][typ][n] for minmodB
  bool lim_on = false;
  int lim_kind = NMG_LIMITER_NONE, lim_scale_bound = 0;
  double lim_bos3 = 0.;
  double *d_lim = nullptr, *d_alpha_h = nullptr, *d_wl = nullptr, *d_wu = nullptr;
  double *d_mmb = nullptr;
  int *d_lnboff = nullptr, *d_lnb = nullptr, *d_limited = nullptr;
  int filter_jpow = 1, filter_fv = 1;
  double *d_filt = nullptr;   // [2][nn] F of LGL and of equally spaced points
  double *d_fooj = nullptr;   // [cslot][np] det(dXb/dx) on the LGL points
  double *d_fvmid = nullptr;          // [cslot][3][5][np]
  nmg_mesh geom;                      // element bboxes, patches and point sets
  std::vector<int> h_cslot;
  std::vector<double> h_xl, h_xu;     // LGL and equally spaced points
  double fv_w3ratio = 2.;
  double *d_fvgeo = nullptr, *d_fvdist = nullptr, *d_fvdxb = nullptr;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};  // one RK4 step, u in d_buf[0] / d_buf[1]
  // host round trips: the last stage runs in element chunks whose results are
  // copied back on a second stream while later chunks compute
  static constexpr int kChunks = 32;   // capacity; nchunks are used
  int nchunks = 16;                    // NMG_COPY_CHUNKS overrides (1..32)
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t chunk_ev[kChunks] = {}, h2d_ev[kChunks] = {};
  // second compute stream of the streamed step: element groups / chunks of
  // one stage alternate between the two so that one launch's tail overlaps
  // the next one's start (they touch disjoint elements)
  cudaStream_t stream2 = nullptr;
  cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
  // first-stage element groups of a chunked host->device copy: group k holds
  // the elements whose face neighbourhood lies in the copy chunks 0..k
  int *d_elist = nullptr;
  std::vector<int> h2d_off;   // [kChunks + 1] group offsets into d_elist
  int64_t h2d_chunk = 0;      // elements per copy chunk
  double graph_dt = 0;
  int graph_sel = -1;
  int method = NMG_EVOLVE_RK4;   // time integrator of nmg_evolve_steps
  int graph_method = -1;         // the one the step graphs were captured with
  int64_t graph_launches = 5;
  int64_t launches = 0;
};

static int set_err(nmg_ctx *c, int code, const std::string &msg) {
  if (c) {
    c->err = msg;
    c->err_static = nullptr;
  }
  return code;
}

static StageParams base_params(nmg_ctx *c);
extern "C" {
static int rk4_step_plain(nmg_ctx *c, double t, double dt);
}

size_t nmg_ctx_state_len(const nmg_ctx *c) { return c->state_len; }
int nmg_ctx_device(const nmg_ctx *c) { return c->device; }

int nmg_ctx_fail_static(nmg_ctx *c, int code, const char *msg) {
  c->err_static = msg;
  return code;
}

// One stage with variant v.  On a mixed DG / finite-volume mesh a stage is
// three launches: the interpolated interface traces of the stage input, the
// DG kernel over all elements (writing only the DG ones) and the
// finite-volume kernel over the finite-volume elements.
static cudaError_t run_stage(nmg_ctx *c, int v, StageParams P, bool traces = true) {
  cudaError_t e;
  if (c->nhang > 0 && traces) {
    e = nmgk::hang_launch(c->nhang, c->n, c->d_hoff, c->d_hsrc, c->d_hw, P.win, c->d_ghost,
                          c->stream);
    if (e != cudaSuccess) return e;
    c->launches++;
  }
  if (c->mixed) {
    e = nmgk::ghost_launch(c->nghost, c->n, c->d_gtab, c->d_isfv, c->d_gM, P.win, c->d_ghost,
                           c->stream);
    if (e != cudaSuccess) return e;
    c->launches++;
    P.skip = c->d_isfv;
    if ((e = c->variants[v].launch(P, c->stream)) != cudaSuccess) return e;
    c->launches++;
    P.skip = nullptr;
    P.fvlist = c->d_fvlist;
    P.nfvel = c->nfvel;
    if ((e = c->variants[c->fsel].launch(P, c->stream)) != cudaSuccess) return e;
    c->launches++;
    return cudaSuccess;
  }
  e = c->variants[v].launch(P, c->stream);
  if (e == cudaSuccess) c->launches++;
  return e;
}

// one RK4 step u_in -> u_out with explicit stage buffers s1, s2, forward
// (the selected variants) or transposed (vjp), enqueued on the context stream
// one transposed stage: the non-conforming faces' adjoint slots from rbar,
// then the transposed stage kernel
static cudaError_t vjp_stage(nmg_ctx *c, const StageParams &P) {
  cudaError_t e;
  if (c->nhang > 0) {
    e = nmgk::hang_adj_launch(c->nhang, c->n, c->d_toff, c->d_tsrc, c->d_tw, c->d_hface,
                              c->d_cslot, c->d_fac, c->d_gcart, P.win, c->d_ghost, c->stream);
    if (e != cudaSuccess) return e;
    c->launches++;
  }
  e = c->vjp.launch(P, c->stream);
  if (e == cudaSuccess) c->launches++;
  return e;
}

static cudaError_t apply_filter(nmg_ctx *c, double *buf);
static cudaError_t apply_limiter(nmg_ctx *c, double *buf);

// limiter (bool lim): the context's MRS limiter on every stage output and on
// u_out, as enqueue_step applies it (the adjoint paths never set it)
static int step_buffers(nmg_ctx *c, bool vjp, double t, double dt, const double *u_in,
                        double *u_out, double *s1, double *s2, bool lim = false) {
  const double cacc[4] = {dt / 6., dt / 3., dt / 3., dt / 6.};
  const double cw[4] = {dt / 2., dt / 2., dt, 0.};
  const double ts[4] = {t, t + 0.5 * dt, t + 0.5 * dt, t + dt};
  const double *win[4] = {u_in, s1, s2, s1};
  double *wout[4] = {s1, s2, s1, nullptr};
  for (int s = 0; s < 4; s++) {
    StageParams P = base_params(c);
    P.win = win[s];
    P.u0 = u_in;
    P.acc = u_out;
    P.wout = wout[s];
    P.mode = s + 1;
    P.cacc = cacc[s];
    P.cw = cw[s];
    P.t = ts[s];
    cudaError_t e;
    if (vjp) {
      e = vjp_stage(c, P);
    } else {
      e = run_stage(c, c->sel >= 0 ? c->sel : 0, P);
      if (e == cudaSuccess && lim && P.wout) e = apply_limiter(c, P.wout);
    }
    if (e != cudaSuccess) return nmg_ctx_fail_static(c, NMG_ECUDA, cudaGetErrorString(e));
  }
  if (lim) {
    cudaError_t e = apply_limiter(c, u_out);
    if (e != cudaSuccess) return nmg_ctx_fail_static(c, NMG_ECUDA, cudaGetErrorString(e));
  }
  return NMG_OK;
}

int nmg_ctx_rk4_step_buffers(nmg_ctx *c, double t, double dt, const double *u_in,
                             double *u_out, double *s1, double *s2) {
  if (c->mixed && c->fsel < 0) c->fsel = c->ndg;
  // the same step as nmg_rk4_step: limiter inside the step, filter after it
  // (both use buffers the context allocated when they were switched on)
  int rc = step_buffers(c, false, t, dt, u_in, u_out, s1, s2, true);
  if (rc) return rc;
  cudaError_t e = apply_filter(c, u_out);
  if (e != cudaSuccess) return nmg_ctx_fail_static(c, NMG_ECUDA, cudaGetErrorString(e));
  e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return nmg_ctx_fail_static(c, NMG_ECUDA, cudaGetErrorString(e));
  return NMG_OK;
}

#define CK(call)                                                                        \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess)                                                              \
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
  P.cmask = c->d_cmask;
  P.scale = c->d_scale;
  P.gcart = c->d_gcart;
  P.metric = c->d_metric;
  P.metricp = c->d_metricp;
  P.fac = c->d_fac;
  P.bxyz = c->d_bxyz;
  P.bnrm = c->d_bnrm;
  P.D = c->d_D;
  P.n = c->n;
  P.fv_rec = c->fv_rec;
  P.fv_extrap = c->fv_extrap;
  P.fv_w3ratio = c->fv_w3ratio;
  P.fvgeo = c->d_fvgeo;
  P.fvdist = c->d_fvdist;
  P.fvdxb = c->d_fvdxb;
  P.ghost = c->d_ghost;
  P.fvmid = c->fv_mid ? c->d_fvmid : nullptr;
  P.numflux = c->numflux;
  P.fvbxyz = c->d_fvbxyz;
  P.fvbnrm = c->d_fvbnrm;
  P.bc = c->bc;
  P.k0 = c->k[0];
  P.k1 = c->k[1];
  P.k2 = c->k[2];
  P.om = sqrt(c->k[0] * c->k[0] + c->k[1] * c->k[1] + c->k[2] * c->k[2]);
  return P;
}

// Autotuner: time the compiled variants on an RHS of the current state and
// keep the fastest (on a mixed mesh the DG and the finite-volume variants
// separately).  Runs once per context, before any graph capture.
static int tune_range(nmg_ctx *c, int v0, int v1, bool fvpart, int *best_out) {
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  float best = 1e30f;
  int bestv = v0;
  for (int v = v0; v < v1; v++) {
    StageParams P = base_params(c);
    P.win = c->d_buf[c->cur];
    P.rout = c->d_buf[3];
    P.mode = 0;
    if (c->mixed) {
      if (fvpart) {
        P.fvlist = c->d_fvlist;
        P.nfvel = c->nfvel;
      } else {
        P.skip = c->d_isfv;
      }
    }
    CK(c->variants[v].launch(P, c->stream));  // warm-up
    float tot = 0;
    const int reps = 3;
    CK(cudaEventRecord(e0, c->stream));
    for (int r = 0; r < reps; r++) CK(c->variants[v].launch(P, c->stream));
    CK(cudaEventRecord(e1, c->stream));
    CK(cudaEventSynchronize(e1));
    CK(cudaEventElapsedTime(&tot, e0, e1));
    tot /= reps;
    char buf[96];
    snprintf(buf, sizeof buf, "%s:%d:%d=%.4fms ", c->variants[v].name, c->variants[v].epb,
             c->variants[v].nt, tot);
    c->tune_log += buf;
    if (tot < best) { best = tot; bestv = v; }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *best_out = bestv;
  return NMG_OK;
}

static int autotune(nmg_ctx *c) {
  if (c->tuned && (!c->mixed || c->ftuned || (c->nfvel == 0 && c->fsel >= 0))) return NMG_OK;
  const char *force = getenv("NMG_KERNEL");  // e.g. "eo", "gather", "eo:1:128"
  const int ndg = c->mixed ? c->ndg : c->nvariants;
  if (force && *force) {
    for (int v = 0; v < c->nvariants; v++) {
      char buf[64];
      snprintf(buf, sizeof buf, "%s:%d:%d", c->variants[v].name, c->variants[v].epb,
               c->variants[v].nt);
      if (!strcmp(force, c->variants[v].name) || !strcmp(force, buf)) {
        if (v < ndg && c->sel < 0) c->sel = v;
        if (v >= ndg && c->mixed && c->fsel < 0) c->fsel = v;
        break;
      }
    }
  }
  if (c->sel >= 0) c->tuned = true;
  if (c->fsel >= 0) c->ftuned = true;
  if (!c->tuned || (c->mixed && !c->ftuned)) c->tune_log.clear();
  if (!c->tuned) {
    int rc = tune_range(c, 0, ndg, false, &c->sel);
    if (rc) return rc;
    c->tuned = true;
  }
  if (c->mixed && !c->ftuned) {
    if (c->nfvel == 0) {  // nothing to time yet (a switchable context without FV elements)
      if (c->fsel < 0) c->fsel = c->ndg;
    } else {
      int rc = tune_range(c, c->ndg, c->nvariants, true, &c->fsel);
      if (rc) return rc;
      c->ftuned = true;
    }
  }
  return NMG_OK;
}

// the exponential filter of the state in buf (after a step)
static cudaError_t apply_filter(nmg_ctx *c, double *buf) {
  if (!c->filter_on) return cudaSuccess;
  cudaError_t e = nmgk::filter_launch(c->n, (int)c->nelem, buf, c->mixed ? c->d_isfv : nullptr,
                                      c->d_filt, c->d_cslot, c->d_fooj, c->d_fvgeo,
                                      c->d_scale, c->filter_jpow, c->filter_fv,
                                      (c->fv && !c->mixed) ? 1 : 0, c->stream);
  if (e == cudaSuccess) c->launches++;
  return e;
}

// evolve_limiter_mesh with the MRS or minmodB limiter on buf (all elements)
static cudaError_t apply_limiter(nmg_ctx *c, double *buf) {
  if (!c->lim_on) return cudaSuccess;
  const unsigned char *isfv = c->mixed ? c->d_isfv : nullptr;
  const int allfv = (c->fv && !c->mixed) ? 1 : 0, n = c->n;
  cudaError_t e =
      c->lim_kind == NMG_LIMITER_MINMODB
          ? nmgk::mmb_limiter_launch(n, (int)c->nelem, buf, isfv, allfv, c->d_mmb,
                                     c->d_mmb + 4 * n, c->d_lim, c->d_lnboff, c->d_lnb,
                                     c->d_alpha_h, c->lim_bos3, c->lim_scale_bound,
                                     c->d_limited, c->stream)
          : nmgk::limiter_launch(n, (int)c->nelem, buf, isfv, allfv, c->d_wl, c->d_wu, c->d_lim,
                                 c->d_lnboff, c->d_lnb, c->d_alpha_h, c->d_limited, c->stream);
  if (e == cudaSuccess) c->launches += 2;
  return e;
}

static int launch_stage(nmg_ctx *c, const StageParams &P) {
  int rc = autotune(c);
  if (rc) return rc;
  CK(run_stage(c, c->sel, P));
  return NMG_OK;
}

// Stages of Euler and sspRK3 (evolve_Euler_mesh, evolve_sspRK3_mesh,
// src/main/evolve/RungeKutta.c:84-200): Euler u = u_p + dt r(u_p, t);
// sspRK3 u += dt/6 r1 with w = u_p + dt r1; u += dt/6 r2 with
// w = 0.75 u_p + 0.25 (w + dt r2) at t + dt; u += (dt 2/3) r3 at t + dt/2.
static int enqueue_step_other(nmg_ctx *c, int cur, double t, double dt, bool devtime,
                              int method) {
  double *U = c->d_buf[cur], *ACC = c->d_buf[1 - cur], *WA = c->d_buf[2], *WB = c->d_buf[3];
  const int ns = method == NMG_EVOLVE_EULER ? 1 : 3;
  const int mode[3] = {method == NMG_EVOLVE_EULER ? 5 : 1, 6, 4};
  const double cacc[3] = {method == NMG_EVOLVE_EULER ? dt : dt / 6., dt / 6., dt * 2. / 3.};
  const double cw[3] = {dt, dt, 0.};
  const double tofs[3] = {0., dt, 0.5 * dt};
  const double *win[3] = {U, WA, WB};
  double *wout[3] = {method == NMG_EVOLVE_EULER ? nullptr : WA, WB, nullptr};
  for (int s = 0; s < ns; s++) {
    StageParams P = base_params(c);
    P.win = win[s];
    P.u0 = U;
    P.acc = ACC;
    P.wout = wout[s];
    P.mode = mode[s];
    P.cacc = cacc[s];
    P.cw = cw[s];
    if (devtime) {
      P.tdev = c->d_times;
      P.stepdev = c->d_step;
      P.tofs_dt = tofs[s];
    } else {
      P.t = (s == 0) ? t : (s == 1) ? t + dt : t + 0.5 * dt;
    }
    int rc = launch_stage(c, P);
    if (rc) return rc;
    if (P.wout) CK(apply_limiter(c, P.wout));  // RungeKutta.c:161,173
  }
  CK(apply_limiter(c, ACC));
  return NMG_OK;
}

// enqueue the 4 stage launches of one RK4 step with u in d_buf[cur] (or the
// stages of another time integrator)
static int enqueue_step(nmg_ctx *c, int cur, double t, double dt, bool devtime,
                        int method = NMG_EVOLVE_RK4) {
  if (method != NMG_EVOLVE_RK4) return enqueue_step_other(c, cur, t, dt, devtime, method);
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
    int rc = launch_stage(c, P);
    if (rc) return rc;
    // the reference limits w before each later stage (RungeKutta.c:45-67)
    if (P.wout) CK(apply_limiter(c, P.wout));
  }
  CK(apply_limiter(c, ACC));  // and the new u after the step (evolve.c:143-144)
  return NMG_OK;
}

// Finite-volume geometry of element e (coordinates_midpoint_data = no: the
// midpoint factors are those of the grid points): distance of each face to
// its nearest midpoint (set_nodemidpoints_to_face_distXb,
// src/main/coordinates/get_coords.c:1807-1836) and, on curvilinear elements,
// per node 1/J = det(dXb/dx) (coordinates.c:174-223, utilities.c:199-211),
// sqrtgdiag (coordinates.c:728-800) and the unit normals of the faces 2d+1
// (utilities.c:48-88), in the reference's operation order.
static void fv_pack_element(const nmg_mesh &m, int64_t e, int cs, const double *X9,
                            std::vector<double> *geo, std::vector<double> *dist) {
  const int n = m.n, np = n * n * n;
  const double *bb = &m.bbox[e * 6];
  for (int f = 0; f < 6; f++) {
    const int d = f / 2, right = f % 2, id = (n - 2) * right;
    const double Xbm = 0.5 * (m.xu[id] + m.xu[id + 1]);
    const double Xbf = (2. * bb[f] - (bb[2 * d + 1] + bb[2 * d])) / (bb[2 * d + 1] - bb[2 * d]);
    (*dist)[e * 6 + f] = std::fabs(Xbm - Xbf);
  }
  if (cs < 0) return;
  double *G = &(*geo)[(size_t)cs * 13 * np];
  const double d0 = 2. / (bb[1] - bb[0]), d1 = 2. / (bb[3] - bb[2]), d2 = 2. / (bb[5] - bb[4]);
  const double dXbdX[3] = {d0, d1, d2};
  for (int q = 0; q < np; q++) {
    double M[3][3];
    for (int a = 0; a < 3; a++)
      for (int b = 0; b < 3; b++) M[a][b] = X9[(a * 3 + b) * np + q];
    const double det = M[0][0] * M[1][1] * M[2][2] - M[0][2] * M[1][1] * M[2][0] +
                       M[0][1] * M[1][2] * M[2][0] + M[0][2] * M[1][0] * M[2][1] -
                       M[0][0] * M[1][2] * M[2][1] - M[0][1] * M[1][0] * M[2][2];
    G[q] = d0 * d1 * d2 * det;
    for (int d = 0; d < 3; d++) {
      double g = 0.0;
      for (int l = 0; l < 3; l++) g += M[d][l] * M[d][l];
      G[(1 + d) * np + q] = dXbdX[d] * sqrt(g);
      double smag = sqrt(M[d][0] * M[d][0] + M[d][1] * M[d][1] + M[d][2] * M[d][2]);
      if (smag == 0.0) smag = 1.;
      for (int l = 0; l < 3; l++) G[(4 + 3 * d + l) * np + q] = M[d][l] / smag;
    }
  }
}

/* piecewise-linear basis function k of the points xp at x
   (basis_pw_linear, src/main/basis/interpolate.c:53-100) */
static double pw_linear_basis(int k, double x, int n, const double *xu) {
  if (n <= 1) return 1.;
  if (x < xu[1]) {
    if (k == 0) return (x - xu[1]) / (xu[0] - xu[1]);
    if (k == 1) return (x - xu[0]) / (xu[1] - xu[0]);
    return 0.;
  }
  if (x >= xu[n - 2]) {
    const int n0 = n - 2, n1 = n - 1, l = k - n0;
    if (l == 0) return (x - xu[n1]) / (xu[n0] - xu[n1]);
    if (l == 1) return (x - xu[n0]) / (xu[n1] - xu[n0]);
    return 0.;
  }
  if (k < n - 1 && x >= xu[k] && x < xu[k + 1]) return (x - xu[k + 1]) / (xu[k] - xu[k + 1]);
  if (k > 0 && x >= xu[k - 1] && x < xu[k]) return (x - xu[k - 1]) / (xu[k] - xu[k - 1]);
  return 0.;
}

/* piecewise-parabolic basis function k of the points xp at x
   (basis_pw_parab, src/main/basis/interpolate.c:106-224) */
static double pw_parab_basis(int k, double x, int np, const double *xp)
{
  int m, m1, m2;
  double xml, xmr, xmll, xmrr;
  if (np < 3) return pw_linear_basis(k, x, np, xp);
  if (np == 3) {
    if (k == 0) return (x - xp[1]) * (x - xp[2]) / ((xp[0] - xp[1]) * (xp[0] - xp[2]));
    if (k == 1) return (x - xp[0]) * (x - xp[2]) / ((xp[1] - xp[0]) * (xp[1] - xp[2]));
    if (k == 2) return (x - xp[0]) * (x - xp[1]) / ((xp[2] - xp[0]) * (xp[2] - xp[1]));
    return 0.;
  }
  xmr = 0.5 * (xp[0] + xp[1]);
  if (x < xmr) {
    if (k == 0) return (x - xp[1]) * (x - xp[2]) / ((xp[0] - xp[1]) * (xp[0] - xp[2]));
    if (k == 1) return (x - xp[0]) * (x - xp[2]) / ((xp[1] - xp[0]) * (xp[1] - xp[2]));
    if (k == 2) return (x - xp[0]) * (x - xp[1]) / ((xp[2] - xp[0]) * (xp[2] - xp[1]));
    return 0.;
  }
  xml = 0.5 * (xp[np - 2] + xp[np - 1]);
  if (x >= xml) {
    int n0 = np - 3, n1 = np - 2, n2 = np - 1, l = k - n0;
    if (l == 0) return (x - xp[n1]) * (x - xp[n2]) / ((xp[n0] - xp[n1]) * (xp[n0] - xp[n2]));
    if (l == 1) return (x - xp[n0]) * (x - xp[n2]) / ((xp[n1] - xp[n0]) * (xp[n1] - xp[n2]));
    if (l == 2) return (x - xp[n0]) * (x - xp[n1]) / ((xp[n2] - xp[n0]) * (xp[n2] - xp[n1]));
    return 0.;
  }
  if (k <= 0) {
    m = 0;
    xmr = 0.5 * (xp[m] + xp[m + 1]);
    xml = xp[m] - (xmr - xp[m]);
    xmll = xml - (xmr - xml);
    xmrr = 0.5 * (xp[m + 1] + xp[m + 2]);
    m1 = 1;
    m2 = 2;
  } else if (k < np - 1) {
    m = k;
    xml = 0.5 * (xp[m] + xp[m - 1]);
    xmr = 0.5 * (xp[m] + xp[m + 1]);
    if (k < np - 2) xmrr = 0.5 * (xp[m + 1] + xp[m + 2]);
    else xmrr = xmr + (xmr - xml);
    if (k >= 2) xmll = 0.5 * (xp[m - 1] + xp[m - 2]);
    else xmll = xml - (xmr - xml);
    m1 = k - 1;
    m2 = k + 1;
  } else {
    m = np - 1;
    xml = 0.5 * (xp[m - 1] + xp[m]);
    xmr = xp[m] + (xp[m] - xml);
    xmll = 0.5 * (xp[m - 2] + xp[m - 1]);
    xmrr = xmr + (xmr - xml);
    m1 = m - 2;
    m2 = m - 1;
  }
  if (x >= xml && x < xmr)
    return (x - xp[m1]) * (x - xp[m2]) / ((xp[m] - xp[m1]) * (xp[m] - xp[m2]));
  if (x >= xmll && x < xml)
    return (x - xp[m - 2]) * (x - xp[m - 1]) / ((xp[m] - xp[m - 2]) * (xp[m] - xp[m - 1]));
  if (x >= xmr && x < xmrr)
    return (x - xp[m + 1]) * (x - xp[m + 2]) / ((xp[m] - xp[m + 1]) * (xp[m] - xp[m + 2]));
  return 0.;
}

// Legendre polynomial P_i(x) by the recurrence of LegendreP
// (src/main/basis/Legendre.c:14-38)
static double legendre_p(int i, double x) {
  double Pk = 0., P0 = 1., P1 = x;
  if (i == 0) return P0;
  if (i == 1) return P1;
  for (int kk = 2; kk <= i; kk++) {
    Pk = (x * (2 * kk - 1) * P1 - (kk - 1) * P0) / kk;
    P0 = P1;
    P1 = Pk;
  }
  return Pk;
}

static void drop_graphs(nmg_ctx *c) {
  for (int g = 0; g < 2; g++)
    if (c->graph[g]) {
      cudaGraphExecDestroy(c->graph[g]);
      c->graph[g] = nullptr;
    }
}

extern "C" {

// Type-dependent tables of a context with finite-volume elements: element
// flags and list, face codes with the mixed bit, interface-trace slots.
// Rebuilt and uploaded whenever element types change.
static int upload_type_tables(nmg_ctx *c) {
  const int64_t E = c->nelem;
  const int nn = c->nn;
  std::vector<unsigned char> isfv(E, 0);
  std::vector<int> fvlist, gtab;
  std::vector<int32_t> code(c->h_code0), bslot(c->h_bslot0);
  for (int64_t e = 0; e < E; e++) {
    if (c->h_fv[e]) {
      isfv[e] = 1;
      fvlist.push_back((int)e);
    }
    for (int f = 0; f < 6; f++) {
      const int nbe = c->h_nb[e * 6 + f];
      if (nbe >= 0 && (c->h_fv[e] != 0) != (c->h_fv[nbe] != 0)) {
        code[e * 6 + f] |= NMG_CODE_MIXED;
        bslot[e * 6 + f] = (int)(gtab.size() / 4);
        gtab.insert(gtab.end(), {(int)e, f, nbe, code[e * 6 + f]});
      }
    }
  }
  c->nfvel = (int)fvlist.size();
  c->nghost = (int)(gtab.size() / 4);
  if (c->nghost > c->ghost_cap) {
    cudaFree(c->d_ghost);
    c->d_ghost = nullptr;
    CK(cudaMalloc((void **)&c->d_ghost, sizeof(double) * 4 * nn * c->nghost));
    CK(cudaMemset(c->d_ghost, 0, sizeof(double) * 4 * nn * c->nghost));
    c->ghost_cap = c->nghost;
  }
  CK(cudaMemcpy(c->d_code, code.data(), sizeof(int32_t) * E * 6, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(c->d_bslot, bslot.data(), sizeof(int32_t) * E * 6, cudaMemcpyHostToDevice));
  if (c->mixed) {
    CK(cudaMemcpy(c->d_isfv, isfv.data(), E, cudaMemcpyHostToDevice));
    if (!fvlist.empty())
      CK(cudaMemcpy(c->d_fvlist, fvlist.data(), sizeof(int) * fvlist.size(),
                    cudaMemcpyHostToDevice));
    if (!gtab.empty())
      CK(cudaMemcpy(c->d_gtab, gtab.data(), sizeof(int) * gtab.size(), cudaMemcpyHostToDevice));
  }
  drop_graphs(c);
  return NMG_OK;
}

static int create_impl(const nmg_mesh *m, int32_t bc_kind, const double k[3], bool switchable,
                       nmg_ctx **out) {
  if (!out) return NMG_EINVAL;
  *out = nullptr;
  nmg_ctx *c = new (std::nothrow) nmg_ctx;
  if (!c) return NMG_ENOMEM;
  *out = c;
  if (!m) return set_err(c, NMG_EINVAL, "nmg_create: null mesh");
  if (bc_kind != NMG_BC_EXACT_PLANEWAVE && bc_kind != NMG_BC_OUTGOING)
    return set_err(c, NMG_EINVAL, "nmg_create: unknown bc kind");
  int64_t nfv = 0;
  for (size_t e = 0; e < m->fv.size(); e++) nfv += m->fv[e] ? 1 : 0;
  c->switchable = switchable;
  const int64_t H = (int64_t)m->hface.size() / 2;
  if (H > 0 && (nfv > 0 || switchable))
    return set_err(c, NMG_EUNSUP,
                   "nmg_create: non-conforming faces are supported on DG meshes only");
  if (const char *nc = getenv("NMG_COPY_CHUNKS")) {
    const int v = atoi(nc);
    if (v >= 1 && v <= nmg_ctx::kChunks) c->nchunks = v;
  }
  c->fv = nfv > 0 || switchable;
  c->mixed = (nfv > 0 && nfv < m->nelem) || switchable;
  if (c->mixed) {
    c->ndg = nmgk::eo_variants(m->n, c->variants, kMaxVariants);
    c->ndg += nmgk::gather_variants(m->n, c->variants + c->ndg, kMaxVariants - c->ndg);
    c->ndg += nmgk::tc_variants(m->n, c->variants + c->ndg, kMaxVariants - c->ndg);
    const int nf = nmgk::fv_variants(m->n, c->variants + c->ndg, kMaxVariants - c->ndg);
    if (c->ndg == 0 || nf == 0)
      return set_err(c, NMG_EUNSUP, "nmg_create: mixed DG / finite-volume n must be in [2,12]");
    c->nvariants = c->ndg + nf;
  } else if (c->fv) {
    c->nvariants = nmgk::fv_variants(m->n, c->variants, kMaxVariants);
    if (c->nvariants == 0) return set_err(c, NMG_EUNSUP, "nmg_create: finite-volume n must be in [2,13]");
  } else {
    c->nvariants = nmgk::eo_variants(m->n, c->variants, kMaxVariants);
    c->nvariants += nmgk::gather_variants(m->n, c->variants + c->nvariants,
                                          kMaxVariants - c->nvariants);
    c->nvariants += nmgk::tc_variants(m->n, c->variants + c->nvariants,
                                      kMaxVariants - c->nvariants);
    if (c->nvariants == 0) return set_err(c, NMG_EUNSUP, "nmg_create: n must be in [2,12]");
    if (nmgk::vjp_variants(m->n, &c->vjp_alt[0], 1) != 1)
      return set_err(c, NMG_EUNSUP, "nmg_create: no transposed kernel for this n");
    c->nvjp_alt = 1 + nmgk::tcvjp_variants(m->n, &c->vjp_alt[1], 1);
    c->vjp = c->vjp_alt[c->nvjp_alt - 1];  // the tensor-core one where it exists
  }
  int dev = 0;
  CK(cudaGetDevice(&dev));
  c->device = dev;
  const int n = m->n, np = n * n * n, nn = n * n;
  const int64_t E = m->nelem;
  if (E <= 0 || E > (int64_t)1 << 30) return set_err(c, NMG_EINVAL, "nmg_create: bad element count");
  c->n = n; c->np = np; c->nn = nn; c->nelem = E;
  c->bc = bc_kind;
  if (k) for (int d = 0; d < 3; d++) c->k[d] = k[d];
  c->state_len = (size_t)E * NF * np;
  c->h_xl = m->x;
  c->h_xu = m->xu;

  // element types and the type-independent face table
  c->h_fv.assign(E, 0);
  for (int64_t e = 0; e < E && !m->fv.empty(); e++) c->h_fv[e] = m->fv[e] ? 1 : 0;
  c->h_nb.assign(m->nb.begin(), m->nb.end());
  c->h_code0.resize(E * 6);
  for (int64_t q = 0; q < E * 6; q++) c->h_code0[q] = m->code[q] & ~NMG_CODE_MIXED;

  // host-side packing of per-element data
  std::vector<int> cslot(E, -1);
  c->h_bslot0.assign(E * 6, -1);
  std::vector<double> scale(E * 3, 0.), gcart(E * 3, 0.);
  int64_t C = 0, B = 0;
  for (int64_t e = 0; e < E; e++) {
    if (m->curvi[e]) cslot[e] = (int)C++;
    for (int f = 0; f < 6; f++)
      if (m->nb[e * 6 + f] < 0) c->h_bslot0[e * 6 + f] = (int)B++;
    for (int d = 0; d < 3; d++)
      scale[e * 3 + d] = 2. / (m->bbox[e * 6 + 2 * d + 1] - m->bbox[e * 6 + 2 * d]);
    for (int d = 0; d < 3; d++) gcart[e * 3 + d] = 0.5 * scale[e * 3 + d] / m->w[0];
  }
  c->ncurvi = C;
  c->nbface = B;
  c->h_cslot = cslot;
  // what the midpoint factors and the filter's Jacobian need later: the
  // maps, not the node arrays
  c->geom.n = m->n;
  c->geom.nelem = m->nelem;
  c->geom.pat = m->pat;
  c->geom.bbox = m->bbox;
  c->geom.curvi = m->curvi;
  c->geom.x = m->x;
  c->geom.xu = m->xu;
  c->geom.patches = m->patches;
  // which geometries are needed: DG (LGL points) for DG elements, FV
  // (equally spaced points) for FV elements, both for every element of a
  // switchable context
  const bool anydg = nfv < E || switchable;
  std::vector<double> metric, metricp, fac, bxyz, bnrm, fvbxyz, fvbnrm, fvgeo, fvdist, fvdxb;
  std::vector<int> cmask((size_t)std::max<int64_t>(C, 1), 0);
  const int64_t Cdg = anydg ? C : 0;
  const int64_t Cfv = c->fv ? C : 0;
  try {
    metric.assign((size_t)std::max<int64_t>(Cdg, 1) * 9 * np, 0.);
    metricp.assign((size_t)std::max<int64_t>(Cdg, 1) * 9 * np, 0.);
    fac.assign((size_t)std::max<int64_t>(Cdg, 1) * 6 * nn * 4, 0.);
    fvgeo.assign((size_t)std::max<int64_t>(Cfv, 1) * 13 * np, 0.);
    fvdist.assign((size_t)(c->fv ? E : 1) * 6, 0.);
    fvdxb.assign((size_t)n, 0.);
    bxyz.assign((size_t)std::max<int64_t>(B, 1) * 3 * nn, 0.);
    bnrm.assign((size_t)std::max<int64_t>(B, 1) * 3 * nn, 0.);
    fvbxyz.assign((size_t)(c->fv ? std::max<int64_t>(B, 1) : 1) * 3 * nn, 0.);
    fvbnrm.assign((size_t)(c->fv ? std::max<int64_t>(B, 1) : 1) * 3 * nn, 0.);
  } catch (const std::bad_alloc &) {
    return set_err(c, NMG_ENOMEM, "nmg_create: host out of memory");
  }
  std::vector<double> gx(3 * np), gX(9 * np);  // geometry of the other point type
  for (int64_t e = 0; e < E; e++) {
    const double *sc = &scale[e * 3];
    const int cs = cslot[e];
    const bool efv = c->h_fv[e] != 0;
    for (int pass = 0; pass < 2; pass++) {
      const bool uni = pass == 1;   // pass 0: DG geometry, pass 1: FV geometry
      if (uni ? !(efv || switchable) : !(!efv || switchable)) continue;
      const double *X3 = &m->xyz[(size_t)e * 3 * np];
      const double *X9 = &m->dXdx[(size_t)e * 9 * np];
      if (uni != efv) {
        if (!nmg::element_geometry(*m, e, uni, gx.data(), gX.data()))
          return set_err(c, NMG_EUNSUP,
                         "nmg_create: switchable context needs the patch map of every "
                         "curvilinear element (a generated mesh)");
        X3 = gx.data();
        X9 = gX.data();
      }
      if (uni) {
        fv_pack_element(*m, e, cs, X9, &fvgeo, &fvdist);
      } else if (cs >= 0) {
        double *Mt = &metric[(size_t)cs * 9 * np];
        double *Mp = &metricp[(size_t)cs * 9 * np];
        int mask = 0;
        for (int a = 0; a < 3; a++)
          for (int i = 0; i < 3; i++) {
            for (int q = 0; q < np; q++) {
              const double v = sc[a] * X9[(a * 3 + i) * np + q];
              Mt[(a * 3 + i) * np + q] = v;
              if (v != 0.) mask |= 1 << (a * 3 + i);
            }
            // pass-major: [a][i][position q along the a-line][line L]
            for (int L = 0; L < nn; L++) {
              const int l0 = L % n, l1 = L / n;
              for (int q = 0; q < n; q++) {
                const int node = a == 0 ? q + n * (l0 + n * l1)
                               : a == 1 ? l0 + n * (q + n * l1)
                                        : l0 + n * (l1 + n * q);
                Mp[(a * 3 + i) * np + q * nn + L] = sc[a] * X9[(a * 3 + i) * np + node];
              }
            }
          }
        cmask[cs] = mask;
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
              double *F4 = &fac[(((size_t)cs * 6 + f) * nn + a + n * b) * 4];
              F4[0] = g * sig * v0 / mag;
              F4[1] = g * sig * v1 / mag;
              F4[2] = g * sig * v2 / mag;
              F4[3] = g;
            }
        }
      }
      // outer faces: coordinates and unit normals on this point type
      std::vector<double> &BX = uni ? fvbxyz : bxyz, &BN = uni ? fvbnrm : bnrm;
      for (int f = 0; f < 6; f++) {
        const int bs = c->h_bslot0[e * 6 + f];
        if (bs < 0 || m->nb[e * 6 + f] >= 0) continue;
        const int d = f >> 1;
        const double sig = (f & 1) ? 1. : -1.;
        for (int b = 0; b < n; b++)
          for (int a = 0; a < n; a++) {
            const int node = nmg::face_node(n, f, a, b), ab = a + n * b;
            for (int q = 0; q < 3; q++) BX[((size_t)bs * 3 + q) * nn + ab] = X3[q * np + node];
            const double v0 = X9[(d * 3 + 0) * np + node], v1 = X9[(d * 3 + 1) * np + node],
                         v2 = X9[(d * 3 + 2) * np + node];
            const double mag = sqrt(v0 * v0 + v1 * v1 + v2 * v2);
            BN[((size_t)bs * 3 + 0) * nn + ab] = sig * v0 / mag;
            BN[((size_t)bs * 3 + 1) * nn + ab] = sig * v1 / mag;
            BN[((size_t)bs * 3 + 2) * nn + ab] = sig * v2 / mag;
          }
      }
    }
  }
  // 1D transfer matrices between the two point sets
  std::vector<double> gM(2 * (size_t)nn, 0.), PR(3 * (size_t)nn, 0.);
  if (c->mixed) {
    // M[0][p][j]: Lagrange weight of LGL point j at the equally spaced point
    // p (Lagrange_of_x with the weights of Lagrange_winterp); M[1][p][j]:
    // piecewise-linear weight of equally spaced point j at LGL point p
    // (basis_pw_linear), src/main/basis/Lagrange.c:15-27,151-159 and
    // src/main/basis/interpolate.c:53-100
    const double *xl = m->x.data(), *xu = m->xu.data();
    std::vector<double> wl(n);
    for (int i = 0; i < n; i++) {
      double denom = 1.;
      for (int j = 0; j < n; j++)
        if (j != i) denom *= (xl[i] - xl[j]);
      wl[i] = 1. / denom;
    }
    for (int p = 0; p < n; p++)
      for (int j = 0; j < n; j++) {
        double prod = 1.;
        for (int q = 0; q < n; q++)
          if (q != j) prod *= (xu[p] - xl[q]);
        gM[p * n + j] = prod * wl[j];
        gM[nn + p * n + j] = pw_linear_basis(j, xl[p], n, xu);
      }
    // element switches: P = the same Lagrange matrix (LGL -> equally spaced,
    // gridpoints.c:158-178) and R = P^{-1} (uniform -> LGL; the reference's
    // default PseudoInv (P^T P)^{-1} P^T is the inverse of the square P),
    // inverted by Gauss-Jordan elimination with partial pivoting
    std::vector<long double> A(nn), I(nn, 0.L);
    for (int q = 0; q < nn; q++) A[q] = gM[q];
    for (int i = 0; i < n; i++) I[i * n + i] = 1.L;
    for (int col = 0; col < n; col++) {
      int piv = col;
      for (int r = col + 1; r < n; r++)
        if (fabsl(A[r * n + col]) > fabsl(A[piv * n + col])) piv = r;
      for (int q = 0; q < n; q++) {
        std::swap(A[col * n + q], A[piv * n + q]);
        std::swap(I[col * n + q], I[piv * n + q]);
      }
      const long double d = A[col * n + col];
      for (int q = 0; q < n; q++) {
        A[col * n + q] /= d;
        I[col * n + q] /= d;
      }
      for (int r = 0; r < n; r++)
        if (r != col) {
          const long double fct = A[r * n + col];
          for (int q = 0; q < n; q++) {
            A[r * n + q] -= fct * A[col * n + q];
            I[r * n + q] -= fct * I[col * n + q];
          }
        }
    }
    for (int q = 0; q < nn; q++) {
      PR[q] = gM[q];
      PR[nn + q] = (double)I[q];
    }
    // modal analysis matrix of the LGL points with normalised Legendre
    // polynomials (LGL_AT_ST_matrices, src/main/basis/Legendre.c:14-38,277-310):
    // A[i][j] = w_j P_i(x_j) / sqrt(c_i), 1/c_i = (2i+1)/2 (i/2 for i = N)
    const int N = n - 1;
    for (int i = 0; i < n; i++) {
      double ooci = 0.5 * (2 * i + 1);
      if (i == N && N != 0) ooci = 0.5 * i;
      const double oosci = sqrt(ooci);
      for (int j = 0; j < n; j++) {
        const double x = xl[j];
        double Pk = 0., P0 = 1., P1 = x, Pi;
        if (i == 0) {
          Pi = P0;
        } else if (i == 1) {
          Pi = P1;
        } else {
          for (int kk = 2; kk <= i; kk++) {
            Pk = (x * (2 * kk - 1) * P1 - (kk - 1) * P0) / kk;
            P0 = P1;
            P1 = Pk;
          }
          Pi = Pk;
        }
        PR[2 * nn + i * n + j] = m->w[j] * (Pi * oosci);
      }
    }
  }
  if (c->fv) {
    // midpoint spacings of the uniform points (set_nm_nodemidpoint_distsXb_dir)
    std::vector<double> Xb(n), Xbm(std::max(n - 1, 1));
    for (int i = 0; i < n; i++) Xb[i] = m->xu[i];
    for (int i = 0; i < n - 1; i++) Xbm[i] = 0.5 * (Xb[i] + Xb[i + 1]);
    for (int i = 1; i < n - 1; i++) fvdxb[i] = Xbm[i] - Xbm[i - 1];
  }
  CK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  auto up = [&](auto **dst, const auto &vec) -> cudaError_t {
    size_t bytes = vec.size() * sizeof(vec[0]);
    cudaError_t e2 = cudaMalloc((void **)dst, std::max<size_t>(bytes, 16));
    if (e2 != cudaSuccess || bytes == 0) return e2;
    return cudaMemcpy(*dst, vec.data(), bytes, cudaMemcpyHostToDevice);
  };
  // non-conforming faces take their trace from slot h of the interface-trace
  // buffer (the kernels' ghost-trace path); their bslot is that slot, not an
  // outer-face slot
  for (int64_t h = 0; h < H; h++) {
    const int64_t q = (int64_t)m->hface[2 * h] * 6 + m->hface[2 * h + 1];
    if (m->nb[q] < 0) return set_err(c, NMG_EMESH, "nmg_create: non-conforming face without neighbour");
    c->h_code0[q] |= NMG_CODE_MIXED;
    c->h_bslot0[q] = (int)h;
  }
  CK(up(&c->d_nb, m->nb));
  CK(up(&c->d_code, c->h_code0));
  CK(up(&c->d_cslot, cslot));
  CK(up(&c->d_bslot, c->h_bslot0));
  CK(up(&c->d_cmask, cmask));
  CK(up(&c->d_scale, scale));
  CK(up(&c->d_gcart, gcart));
  CK(up(&c->d_metric, metric));
  CK(up(&c->d_metricp, metricp));
  CK(up(&c->d_fac, fac));
  CK(up(&c->d_bxyz, bxyz));
  CK(up(&c->d_bnrm, bnrm));
  CK(up(&c->d_D, m->D));
  {
    std::vector<double> wq(2 * (size_t)n);
    for (int i = 0; i < n; i++) wq[i] = m->w[i];
    for (int i = 0; i < n; i++)  // uniform_x_wTrapez (Legendre.c:701-719)
      wq[n + i] = (n == 1) ? 2. : (i == 0 || i == n - 1) ? 1. / (n - 1) : 2. / (n - 1);
    CK(up(&c->d_wq, wq));
  }
  if (c->fv) {
    CK(up(&c->d_fvgeo, fvgeo));
    CK(up(&c->d_fvdist, fvdist));
    CK(up(&c->d_fvdxb, fvdxb));
    CK(up(&c->d_fvbxyz, fvbxyz));
    CK(up(&c->d_fvbnrm, fvbnrm));
  }
  if (anydg) CK(nmgk::eo_upload(n, m->D.data()));
  if (anydg) CK(nmgk::tc_upload(n, m->D.data()));
  if (c->mixed) {
    CK(cudaMalloc((void **)&c->d_isfv, E));
    CK(cudaMalloc((void **)&c->d_fvlist, sizeof(int) * E));
    CK(cudaMalloc((void **)&c->d_gtab, sizeof(int) * E * 6 * 4));
    CK(up(&c->d_gM, gM));
    CK(up(&c->d_PR, PR));
  }
  if (c->fv) {
    int rc = upload_type_tables(c);
    if (rc) return rc;
  }
  if (H > 0) {
    // per contribution the Lagrange weights of the source face's points at
    // the node's position in both in-plane directions (Lagrange_of_x,
    // src/main/basis/Lagrange.c:151-159, with the weights of :15-27)
    const double *xl = m->x.data();
    std::vector<double> wl(n);
    for (int i = 0; i < n; i++) {
      double denom = 1.;
      for (int j = 0; j < n; j++)
        if (j != i) denom *= (xl[i] - xl[j]);
      wl[i] = 1. / denom;
    }
    const size_t Cn = m->hsrc.size() / 2;
    std::vector<double> hw(Cn * 2 * n);
    for (size_t q = 0; q < Cn; q++)
      for (int dd = 0; dd < 2; dd++)
        for (int k2 = 0; k2 < n; k2++) {
          double prod = 1.;
          for (int j = 0; j < n; j++)
            if (j != k2) prod *= (m->hpos[2 * q + dd] - xl[j]);
          hw[(q * 2 + dd) * n + k2] = prod * wl[k2];
        }
    CK(up(&c->d_hoff, m->hoff));
    CK(up(&c->d_hsrc, m->hsrc));
    CK(up(&c->d_hw, hw));
    // host copies for the transposed lists, built on the first adjoint call
    c->h_hoff = m->hoff;
    c->h_hsrc = m->hsrc;
    c->h_hface = m->hface;
    c->h_hw = hw;
    CK(cudaMalloc((void **)&c->d_ghost, sizeof(double) * 4 * nn * H));
    CK(cudaMemset(c->d_ghost, 0, sizeof(double) * 4 * nn * H));
    c->ghost_cap = (int)H;
    c->nhang = (int)H;
  }
  for (int b = 0; b < 4; b++) {
    CK(cudaMalloc((void **)&c->d_buf[b], c->state_len * sizeof(double)));
    CK(cudaMemset(c->d_buf[b], 0, c->state_len * sizeof(double)));
  }
  CK(cudaMalloc((void **)&c->d_step, sizeof(int)));
  const int ndgv = c->mixed ? c->ndg : (c->fv ? 0 : c->nvariants);
  for (int v = 0; v < ndgv; v++) {
    StageParams P0;
    std::memset(&P0, 0, sizeof(P0));
    CK(c->variants[v].launch(P0, c->stream));  // nelem == 0: only sets the smem limit
  }
  if (!c->fv) {
    StageParams P0;
    std::memset(&P0, 0, sizeof(P0));
    for (int v = 0; v < c->nvjp_alt; v++) CK(c->vjp_alt[v].launch(P0, c->stream));
  } else {
    for (int v = c->mixed ? c->ndg : 0; v < c->nvariants; v++) {
      StageParams P0;
      std::memset(&P0, 0, sizeof(P0));
      P0.n = n;
      CK(c->variants[v].launch(P0, c->stream));  // smem limit of this n
    }
  }
  CK(cudaDeviceSynchronize());
  return NMG_OK;
}

int nmg_create(const nmg_mesh *m, int32_t bc_kind, const double k[3], nmg_ctx **out) {
  return create_impl(m, bc_kind, k, false, out);
}

int nmg_create_switchable(const nmg_mesh *m, int32_t bc_kind, const double k[3], nmg_ctx **out) {
  return create_impl(m, bc_kind, k, true, out);
}

// ---------------------------------------------------------------------------
// element switches between DG and finite volume, trouble indicators
// ---------------------------------------------------------------------------
// switch element types to fv[], converting the resident state of every
// element whose type changes (LGL -> uniform with P, uniform -> LGL with R)
static int switch_types(nmg_ctx *c, const int32_t *fv, int *nto_fv, int *nto_dg) {
  const int64_t E = c->nelem;
  std::vector<int> lst;
  int a = 0, b = 0;
  for (int64_t e = 0; e < E; e++)
    if (fv[e] && !c->h_fv[e]) { lst.push_back((int)e); a++; }
  for (int64_t e = 0; e < E; e++)
    if (!fv[e] && c->h_fv[e]) { lst.push_back((int)e); b++; }
  if (nto_fv) *nto_fv = a;
  if (nto_dg) *nto_dg = b;
  if (lst.empty()) return NMG_OK;
  if (!c->d_conv) CK(cudaMalloc((void **)&c->d_conv, sizeof(int) * E));
  CK(cudaMemcpyAsync(c->d_conv, lst.data(), sizeof(int) * lst.size(), cudaMemcpyHostToDevice,
                     c->stream));
  const int nn = c->nn;
  CK(nmgk::convert_launch(c->n, c->d_conv, a, c->d_PR, c->d_buf[c->cur], c->stream));
  CK(nmgk::convert_launch(c->n, c->d_conv + a, b, c->d_PR + nn, c->d_buf[c->cur], c->stream));
  c->launches += (a > 0) + (b > 0);
  CK(cudaStreamSynchronize(c->stream));
  for (int64_t e = 0; e < E; e++) c->h_fv[e] = fv[e] ? 1 : 0;
  return upload_type_tables(c);
}

static int ensure_trouble_buffers(nmg_ctx *c) {
  const int64_t E = c->nelem;
  if (!c->d_mm) CK(cudaMalloc((void **)&c->d_mm, sizeof(double) * E * NF * 2));
  if (!c->d_trb) CK(cudaMalloc((void **)&c->d_trb, sizeof(int) * E));
  if (!c->d_pers) CK(cudaMalloc((void **)&c->d_pers, sizeof(double) * E * NF));
  if (!c->d_up) CK(cudaMalloc((void **)&c->d_up, sizeof(double) * c->state_len));
  if ((int64_t)c->h_score.size() != E) c->h_score.assign(E, 0);
  return NMG_OK;
}

static int trouble_flags(nmg_ctx *c, const double *u, const double *u_p,
                         const nmg_trouble_params *tp, std::vector<int32_t> *flags) {
  CK(nmgk::trouble_launch(c->n, (int)c->nelem, u, u_p, c->d_mm, c->d_nb, c->d_isfv,
                          c->d_PR + 2 * c->nn, tp->rdmp_deltafac, tp->rdmp_delta0,
                          tp->rdmp_epsilon, tp->persson_max, tp->persson_uscale, c->d_trb,
                          c->d_pers, c->stream));
  c->launches += 2;
  flags->resize(c->nelem);
  CK(cudaMemcpyAsync(flags->data(), c->d_trb, sizeof(int32_t) * c->nelem,
                     cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return NMG_OK;
}

int nmg_set_element_types(nmg_ctx *c, const int32_t *fv) {
  if (!c || !fv) return set_err(c, NMG_EINVAL, "nmg_set_element_types: null argument");
  if (!c->switchable)
    return set_err(c, NMG_EUNSUP, "nmg_set_element_types: context is not switchable");
  return switch_types(c, fv, nullptr, nullptr);
}

int nmg_get_element_types(nmg_ctx *c, int32_t *fv) {
  if (!c || !fv) return set_err(c, NMG_EINVAL, "nmg_get_element_types: null argument");
  for (int64_t e = 0; e < c->nelem; e++) fv[e] = c->h_fv.empty() ? 0 : c->h_fv[e];
  return NMG_OK;
}

int nmg_trouble_check(nmg_ctx *c, const double *u_dev, const double *u_p_dev,
                      const nmg_trouble_params *tp, int32_t *flags, double *persson) {
  if (!c || !u_dev || !u_p_dev || !tp || !flags)
    return set_err(c, NMG_EINVAL, "nmg_trouble_check: null argument");
  if (!c->switchable)
    return set_err(c, NMG_EUNSUP, "nmg_trouble_check: context is not switchable");
  int rc = ensure_trouble_buffers(c);
  if (rc) return rc;
  std::vector<int32_t> fl;
  if ((rc = trouble_flags(c, u_dev, u_p_dev, tp, &fl))) return rc;
  std::memcpy(flags, fl.data(), sizeof(int32_t) * c->nelem);
  if (persson)
    CK(cudaMemcpy(persson, c->d_pers, sizeof(double) * c->nelem * NF, cudaMemcpyDeviceToHost));
  return NMG_OK;
}

int nmg_get_trouble_scores(nmg_ctx *c, int32_t *scores) {
  if (!c || !scores) return set_err(c, NMG_EINVAL, "nmg_get_trouble_scores: null argument");
  for (int64_t e = 0; e < c->nelem; e++)
    scores[e] = (int64_t)c->h_score.size() == c->nelem ? c->h_score[e] : 0;
  return NMG_OK;
}

// evolve_set_trouble_score (src/main/evolve/trouble.c:27-110) on every
// element from its flag, then the global score of
// evolve_read_trouble_score_mesh (trouble.c:132-160)
static int score_update(nmg_ctx *c, const std::vector<int32_t> &fl) {
  const int maxt = 1073741824;
  int smax = INT32_MIN, smin = INT32_MAX;
  for (int64_t e = 0; e < c->nelem; e++) {
    int32_t &sc = c->h_score[e];
    if (fl[e] > 0) sc = sc <= 0 ? 1 : sc + 1;
    else if (fl[e] == 0) sc = 0;
    else sc = sc >= 0 ? -1 : sc - 1;
    if (sc < -maxt) sc = -maxt;
    if (sc > maxt) sc = maxt;
    smax = std::max(smax, sc);
    smin = std::min(smin, sc);
  }
  return smax > 0 ? smax : smin;
}

// y = x + a z over whole elements: all elements (list null) or the listed
__global__ void elem_axpy_kernel(int64_t count, int per, const int *list, double *y,
                                 const double *x, double a, const double *z) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < count * per;
       q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k = q / per;
    const int64_t e = list ? list[k] : k;
    const size_t idx = (size_t)e * per + (size_t)(q - k * per);
    y[idx] = x[idx] + a * z[idx];
  }
}

static cudaError_t elem_axpy(nmg_ctx *c, int64_t count, const int *list, double *y,
                             const double *x, double a, const double *z) {
  if (count <= 0) return cudaSuccess;
  const int per = NF * c->np;
  const int64_t grid = std::min<int64_t>((count * per + 255) / 256, 152 * 32);
  elem_axpy_kernel<<<(unsigned)grid, 256, 0, c->stream>>>(count, per, list, y, x, a, z);
  c->launches++;
  return cudaGetLastError();
}

// r of the troubled elements T (T[0, ndg) were DG, now finite volume) with
// every neighbour in its old type and with its old data, as the reference's
// per-element redo does (each redone element is swapped back until all are
// done, RungeKutta.c:221-330): a face towards a neighbour of the old DG type
// takes its trace interpolated from that neighbour's old data w_old, the
// element's own data is the converted w_new.
static int redo_rhs(nmg_ctx *c, const std::vector<int> &T, const double *w_old,
                    const double *w_new, double *R, double t) {
  const int64_t E = c->nelem;
  const int nn = c->nn;
  std::vector<int32_t> code(c->h_code0), bslot(c->h_bslot0);
  std::vector<int> gtab;
  for (int e : T)
    for (int f = 0; f < 6; f++) {
      const int64_t q = (int64_t)e * 6 + f;
      const int nbe = c->h_nb[q];
      if (nbe < 0) continue;
      if (!c->h_fv[nbe]) {  // old type DG (h_fv still holds the old types)
        code[q] = c->h_code0[q] | NMG_CODE_MIXED;
        bslot[q] = (int)(gtab.size() / 4);
        gtab.insert(gtab.end(), {e, f, nbe, code[q]});
      }
    }
  const int ng = (int)(gtab.size() / 4);
  if (!c->d_code2) {
    CK(cudaMalloc((void **)&c->d_code2, sizeof(int) * E * 6));
    CK(cudaMalloc((void **)&c->d_bslot2, sizeof(int) * E * 6));
    CK(cudaMalloc((void **)&c->d_gtab2, sizeof(int) * E * 6 * 4));
  }
  if (ng > c->ghost2_cap) {
    CK(cudaStreamSynchronize(c->stream));
    cudaFree(c->d_ghost2);
    c->d_ghost2 = nullptr;
    CK(cudaMalloc((void **)&c->d_ghost2, sizeof(double) * 4 * nn * ng));
    c->ghost2_cap = ng;
  }
  CK(cudaMemcpyAsync(c->d_code2, code.data(), sizeof(int) * E * 6, cudaMemcpyHostToDevice,
                     c->stream));
  CK(cudaMemcpyAsync(c->d_bslot2, bslot.data(), sizeof(int) * E * 6, cudaMemcpyHostToDevice,
                     c->stream));
  if (ng > 0) {
    CK(cudaMemcpyAsync(c->d_gtab2, gtab.data(), sizeof(int) * gtab.size(),
                       cudaMemcpyHostToDevice, c->stream));
    CK(nmgk::ghost_launch(ng, c->n, c->d_gtab2, c->d_isfv, c->d_gM, w_old, c->d_ghost2,
                          c->stream));
    c->launches++;
  }
  StageParams Q = base_params(c);
  Q.win = w_new;
  Q.mode = 0;
  Q.rout = R;
  Q.t = t;
  Q.code = c->d_code2;
  Q.bslot = c->d_bslot2;
  Q.ghost = c->d_ghost2;
  Q.fvlist = c->d_tlist;
  Q.nfvel = (int)T.size();
  CK(c->variants[c->fsel >= 0 ? c->fsel : c->ndg].launch(Q, c->stream));
  c->launches++;
  // the host tables above must live until the copies are done
  CK(cudaStreamSynchronize(c->stream));
  return NMG_OK;
}

// One RK4 step with evolve_redo_troubled = substep (evolve_RK4_mesh,
// src/main/evolve/RungeKutta.c:19-80): after each substep u += c_s r the
// elements are scored; if the global score is positive, every element with
// a positive score takes the substep back (u -= c_s r), the DG ones are
// switched to finite volume (u, u_p and w converted), r is recomputed on
// them and the substep applied again (evolve_trouble_redo_u_step_mesh,
// RungeKutta.c:221-330).  At the end of the step finite-volume elements
// whose score reached -4 notroubles switch back to DG (evolve.c:98-140).
static int rk4_step_substep(nmg_ctx *c, double t, double dt, const nmg_trouble_params *tp,
                            int32_t *switched) {
  int rc = autotune(c);
  if (rc) return rc;
  if (c->fsel < 0) c->fsel = c->ndg;
  const int64_t E = c->nelem;
  const size_t bytes = c->state_len * sizeof(double);
  if (!c->d_r) CK(cudaMalloc((void **)&c->d_r, bytes));
  if (!c->d_w2) CK(cudaMalloc((void **)&c->d_w2, bytes));
  if (!c->d_tlist) CK(cudaMalloc((void **)&c->d_tlist, sizeof(int) * E));
  const int cur = c->cur;
  double *U = c->d_buf[cur], *ACC = c->d_buf[1 - cur], *W = c->d_buf[2], *R = c->d_r,
         *W2 = c->d_w2;
  const double cacc[4] = {dt / 6., dt / 3., dt / 3., dt / 6.};
  const double cw[3] = {dt / 2., dt / 2., dt};
  const double ts[4] = {t, t + 0.5 * dt, t + 0.5 * dt, t + dt};
  int nfv = 0;
  CK(cudaMemcpyAsync(W, U, bytes, cudaMemcpyDeviceToDevice, c->stream));  // w = u
  for (int s = 0; s < 4; s++) {
    StageParams P = base_params(c);
    P.win = W;
    P.mode = 0;
    P.rout = R;
    P.t = ts[s];
    CK(run_stage(c, c->sel, P));                                    // r = RHS(w)
    CK(elem_axpy(c, E, nullptr, ACC, s == 0 ? W : ACC, cacc[s], R));  // u += c_s r
    std::vector<int32_t> fl;
    if ((rc = trouble_flags(c, ACC, U, tp, &fl))) return rc;
    if (score_update(c, fl) > 0) {
      std::vector<int> T;
      for (int64_t e = 0; e < E; e++)
        if (c->h_score[e] > 0 && !c->h_fv[e]) T.push_back((int)e);
      const int ndgT = (int)T.size();
      for (int64_t e = 0; e < E; e++)
        if (c->h_score[e] > 0 && c->h_fv[e]) T.push_back((int)e);
      CK(cudaMemcpyAsync(c->d_tlist, T.data(), sizeof(int) * T.size(), cudaMemcpyHostToDevice,
                         c->stream));
      CK(elem_axpy(c, (int64_t)T.size(), c->d_tlist, ACC, ACC, -cacc[s], R));  // u -= c_s r
      CK(cudaMemcpyAsync(W2, W, bytes, cudaMemcpyDeviceToDevice, c->stream));
      for (double *buf : {W2, ACC, U}) {
        CK(nmgk::convert_launch(c->n, c->d_tlist, ndgT, c->d_PR, buf, c->stream));
        c->launches += ndgT > 0;
      }
      if ((rc = redo_rhs(c, T, W, W2, R, ts[s]))) return rc;
      CK(elem_axpy(c, (int64_t)T.size(), c->d_tlist, ACC, ACC, cacc[s], R));  // u += c_s r
      for (int i = 0; i < ndgT; i++) c->h_fv[T[i]] = 1;
      nfv += ndgT;
      CK(cudaStreamSynchronize(c->stream));
      if ((rc = upload_type_tables(c))) return rc;
    }
    if (s < 3) CK(elem_axpy(c, E, nullptr, W, U, cw[s], R));  // w = u_p + a r
  }
  c->cur = 1 - cur;
  int smax = INT32_MIN, smin = INT32_MAX;
  for (int64_t e = 0; e < E; e++) {
    smax = std::max(smax, c->h_score[e]);
    smin = std::min(smin, c->h_score[e]);
  }
  const int global = smax > 0 ? smax : smin;
  const int notr = tp->notroubles * 4;
  int ndg = 0;
  if (global > 0 || global <= -notr) {
    std::vector<int32_t> types(c->h_fv);
    for (int64_t e = 0; e < E; e++)
      if (c->h_fv[e] && c->h_score[e] <= -notr) types[e] = 0;
    if ((rc = switch_types(c, types.data(), nullptr, &ndg))) return rc;
  }
  if (switched) {
    switched[0] = nfv;
    switched[1] = ndg;
  }
  CK(apply_filter(c, c->d_buf[c->cur]));  // evolve_filter_evosys_mesh after the step
  CK(cudaStreamSynchronize(c->stream));
  return NMG_OK;
}

// One RK4 step with trouble detection, as evolve_mesh does with
// evolve_redo_troubled = step (src/main/evolve/evolve.c:74-140): step,
// score every element (evolve_set_trouble_score, trouble.c:27-110), and if
// the global score is positive go back to u_p, switch the troubled DG
// elements to finite volume (trouble.c:187-260) and redo the step; finally
// switch finite-volume elements whose score reached -notroubles back to DG
// (trouble.c:288-373).
int nmg_rk4_step_trouble(nmg_ctx *c, double t, double dt, const nmg_trouble_params *tp,
                         int32_t *switched) {
  if (!c || !tp) return set_err(c, NMG_EINVAL, "nmg_rk4_step_trouble: null argument");
  if (!c->switchable)
    return set_err(c, NMG_EUNSUP, "nmg_rk4_step_trouble: context is not switchable");
  if (c->lim_on)
    return set_err(c, NMG_EUNSUP, "nmg_rk4_step_trouble: the limiter is not built into the trouble flow");
  if (tp->redo != NMG_REDO_STEP && tp->redo != NMG_REDO_SUBSTEP)
    return set_err(c, NMG_EINVAL, "nmg_rk4_step_trouble: unknown redo mode");
  int rc = ensure_trouble_buffers(c);
  if (rc) return rc;
  if (tp->redo == NMG_REDO_SUBSTEP) return rk4_step_substep(c, t, dt, tp, switched);
  const int64_t E = c->nelem;
  const size_t bytes = c->state_len * sizeof(double);
  CK(cudaMemcpyAsync(c->d_up, c->d_buf[c->cur], bytes, cudaMemcpyDeviceToDevice, c->stream));
  if ((rc = rk4_step_plain(c, t, dt))) return rc;
  std::vector<int32_t> fl;
  if ((rc = trouble_flags(c, c->d_buf[c->cur], c->d_up, tp, &fl))) return rc;
  const int global = score_update(c, fl);
  int nfv = 0, ndg = 0;
  if (global > 0) {
    // go back to u_p, switch the troubled elements, redo the step
    CK(cudaMemcpyAsync(c->d_buf[c->cur], c->d_up, bytes, cudaMemcpyDeviceToDevice, c->stream));
    std::vector<int32_t> types(c->h_fv);
    for (int64_t e = 0; e < E; e++)
      if (c->h_score[e] > 0) types[e] = 1;
    if ((rc = switch_types(c, types.data(), &nfv, nullptr))) return rc;
    if ((rc = rk4_step_plain(c, t, dt))) return rc;
  }
  if (global > 0 || global <= -tp->notroubles) {
    std::vector<int32_t> types(c->h_fv);
    for (int64_t e = 0; e < E; e++)
      if (c->h_fv[e] && c->h_score[e] <= -tp->notroubles) types[e] = 0;
    if ((rc = switch_types(c, types.data(), nullptr, &ndg))) return rc;
  }
  if (switched) {
    switched[0] = nfv;
    switched[1] = ndg;
  }
  CK(apply_filter(c, c->d_buf[c->cur]));  // evolve_filter_evosys_mesh after the step
  CK(cudaStreamSynchronize(c->stream));
  return NMG_OK;
}

int nmg_norms(nmg_ctx *c, const double *u_dev, double *out) {
  if (!c || !out) return set_err(c, NMG_EINVAL, "nmg_norms: null argument");
  const int64_t E = c->nelem;
  if (!c->d_npart) CK(cudaMalloc((void **)&c->d_npart, sizeof(double) * E * (NF + 1) * 4 + 256));
  const double *u = u_dev ? u_dev : c->d_buf[c->cur];
  norms_elem_kernel<<<(unsigned)E, kNormThreads, 0, c->stream>>>(
      c->n, (int)E, u, c->d_cslot, c->d_scale, c->d_metric, c->d_fvgeo,
      (c->fv && !c->mixed) ? 1 : 0, c->mixed ? c->d_isfv : nullptr, c->d_wq, c->d_wq + c->n,
      c->d_npart);
  CK(cudaGetLastError());
  double *fin = c->d_npart + E * (NF + 1) * 4;  // the 256 spare bytes: 24 doubles
  norms_final_kernel<<<1, 32, 0, c->stream>>>((int)E, c->d_npart, fin);
  CK(cudaGetLastError());
  c->launches += 2;
  double h[(NF + 1) * 4];
  CK(cudaMemcpyAsync(h, fin, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  // out: Vol, then per field VolInt, mean, rms, min, max, maxAbs
  const double vol = h[0];
  out[0] = vol;
  for (int l = 0; l < NF; l++) {
    const double *q = h + (l + 1) * 4;
    double *o = out + 1 + l * 6;
    o[0] = q[0];
    o[1] = q[0] / vol;
    o[2] = sqrt(fabs(q[1] / vol));
    o[3] = q[2];
    o[4] = q[3];
    o[5] = fabs(q[3]) > fabs(q[2]) ? fabs(q[3]) : fabs(q[2]);
  }
  return NMG_OK;
}

int nmg_set_numflux(nmg_ctx *c, int32_t kind) {
  if (!c) return NMG_EINVAL;
  if (kind != NMG_NUMFLUX_LLF && kind != NMG_NUMFLUX_UPWIND)
    return set_err(c, NMG_EINVAL, "nmg_set_numflux: unknown numerical flux");
  c->numflux = kind;
  drop_graphs(c);
  return NMG_OK;
}

int nmg_set_fv_surface_interp(nmg_ctx *c, int32_t mode) {
  if (!c) return NMG_EINVAL;
  if (!c->mixed)
    return set_err(c, NMG_EUNSUP, "nmg_set_fv_surface_interp: no DG / finite-volume faces");
  if (mode != NMG_FV_SURF_LINEAR && mode != NMG_FV_SURF_PARABOLIC)
    return set_err(c, NMG_EINVAL, "nmg_set_fv_surface_interp: unknown mode");
  // M[1][p][j]: weight of equally spaced point j at LGL point p
  const int n = c->n, nn = c->nn;
  std::vector<double> M1(nn);
  for (int p = 0; p < n; p++)
    for (int j = 0; j < n; j++)
      M1[p * n + j] = mode == NMG_FV_SURF_PARABOLIC
                          ? pw_parab_basis(j, c->h_xl[p], n, c->h_xu.data())
                          : pw_linear_basis(j, c->h_xl[p], n, c->h_xu.data());
  CK(cudaStreamSynchronize(c->stream));
  CK(cudaMemcpy(c->d_gM + nn, M1.data(), sizeof(double) * nn, cudaMemcpyHostToDevice));
  c->fv_surf = mode;
  return NMG_OK;
}

// S_ij = P_j(x_i) / sqrt(c_j), 1/c_j = (2j+1)/2 (j/2 for j = N), and the
// analysis matrix A: w_j S_ji on LGL points (typ 0), S^-1 by Gauss-Jordan
// elimination with partial pivoting on equally spaced points (typ 1)
// (LGL_AT_ST_matrices, Legendre_AT_ST_matrices, src/main/basis/
// Legendre.c:277-310,723-729); plain double arithmetic, as the oracle's
static void legendre_sa(int n, int typ, const double *x, const double *w, double *S, double *A) {
  const int nn = n * n;
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      double ooc = 0.5 * (2 * j + 1);
      if (j == n - 1 && n - 1 != 0) ooc = 0.5 * j;
      S[i * n + j] = legendre_p(j, x[i]) * sqrt(ooc);
    }
  if (typ == 0) {
    for (int i = 0; i < n; i++)
      for (int j = 0; j < n; j++) A[i * n + j] = w[j] * S[j * n + i];
    return;
  }
  std::vector<double> M(S, S + nn), I(nn, 0.);
  for (int i = 0; i < n; i++) I[i * n + i] = 1.;
  for (int col = 0; col < n; col++) {
    int piv = col;
    for (int r = col + 1; r < n; r++)
      if (fabs(M[r * n + col]) > fabs(M[piv * n + col])) piv = r;
    for (int q = 0; q < n; q++) {
      std::swap(M[col * n + q], M[piv * n + q]);
      std::swap(I[col * n + q], I[piv * n + q]);
    }
    const double d = M[col * n + col];
    for (int q = 0; q < n; q++) {
      M[col * n + q] /= d;
      I[col * n + q] /= d;
    }
    for (int r = 0; r < n; r++)
      if (r != col) {
        const double fac = M[r * n + col];
        for (int q = 0; q < n; q++) {
          M[r * n + q] -= fac * M[col * n + q];
          I[r * n + q] -= fac * I[col * n + q];
        }
      }
  }
  std::copy(I.begin(), I.end(), A);
}

int nmg_set_limiter(nmg_ctx *c, int32_t kind, double alpha) {
  return nmg_set_limiter_ex(c, kind, alpha, 0.5, 0);
}

int nmg_set_limiter_ex(nmg_ctx *c, int32_t kind, double alpha, double beta, int32_t scale_bound) {
  if (!c) return NMG_EINVAL;
  if (kind != NMG_LIMITER_NONE && kind != NMG_LIMITER_MRS && kind != NMG_LIMITER_MINMODB)
    return set_err(c, NMG_EUNSUP, "nmg_set_limiter: kind must be none, MRS or minmodB");
  if (kind != NMG_LIMITER_NONE && !(alpha >= 0.))
    return set_err(c, NMG_EINVAL, "nmg_set_limiter: alpha must be >= 0");
  if (kind == NMG_LIMITER_MINMODB && !(beta >= 0.))
    return set_err(c, NMG_EINVAL, "nmg_set_limiter: beta must be >= 0");
  if (scale_bound != 0 && scale_bound != 1)
    return set_err(c, NMG_EINVAL, "nmg_set_limiter: scale_bound must be 0 or 1");
  drop_graphs(c);
  if (kind == NMG_LIMITER_NONE) {
    c->lim_on = false;
    c->lim_kind = NMG_LIMITER_NONE;
    return NMG_OK;
  }
  const int n = c->n;
  const int64_t E = c->nelem;
  if (!c->d_lnboff) {
    // face neighbours (nfnb / fnb): the neighbour element of a conforming
    // face, every distinct source element of a non-conforming one
    std::vector<std::vector<int>> extra(E * 6);
    const int nn = n * n;
    for (int64_t h = 0; h < c->nhang; h++) {
      const int64_t q = (int64_t)c->h_hface[2 * h] * 6 + c->h_hface[2 * h + 1];
      for (int cidx = c->h_hoff[h * nn]; cidx < c->h_hoff[(h + 1) * nn]; cidx++) {
        const int e2 = c->h_hsrc[2 * cidx];
        if (std::find(extra[q].begin(), extra[q].end(), e2) == extra[q].end())
          extra[q].push_back(e2);
      }
    }
    std::vector<int> off(1, 0), nbl;
    for (int64_t q = 0; q < E * 6; q++) {
      if (!extra[q].empty()) nbl.insert(nbl.end(), extra[q].begin(), extra[q].end());
      else if (c->h_nb[q] >= 0) nbl.push_back(c->h_nb[q]);
      off.push_back((int)nbl.size());
    }
    if (nbl.empty()) nbl.push_back(0);
    std::vector<double> x(n), wl(n), wu(n), xu(n), D((size_t)n * n);
    nmg::lgl_basis(n, x.data(), wl.data(), D.data());
    nmg::uniform_basis(n, xu.data(), wu.data(), D.data());
    // minmodB tables: analysis rows 0, 1 and synthesis columns 0, 1
    std::vector<double> mmb(8 * (size_t)n), S((size_t)n * n), A((size_t)n * n);
    for (int typ = 0; typ < 2; typ++) {
      legendre_sa(n, typ, typ ? xu.data() : x.data(), wl.data(), S.data(), A.data());
      for (int i = 0; i < n; i++) {
        mmb[(typ * 2 + 0) * n + i] = A[i];
        mmb[(typ * 2 + 1) * n + i] = A[n + i];
        mmb[4 * n + (typ * 2 + 0) * n + i] = S[i * n];
        mmb[4 * n + (typ * 2 + 1) * n + i] = S[i * n + 1];
      }
    }
    auto up = [&](auto **dst, const auto &vec) -> cudaError_t {
      const size_t bytes = vec.size() * sizeof(vec[0]);
      cudaError_t e2 = cudaMalloc((void **)dst, std::max<size_t>(bytes, 16));
      if (e2 != cudaSuccess || bytes == 0) return e2;
      return cudaMemcpy(*dst, vec.data(), bytes, cudaMemcpyHostToDevice);
    };
    CK(up(&c->d_lnb, nbl));
    CK(up(&c->d_wl, wl));
    CK(up(&c->d_wu, wu));
    CK(up(&c->d_mmb, mmb));
    CK(cudaMalloc((void **)&c->d_lim, sizeof(double) * E * NF * 4));
    CK(cudaMalloc((void **)&c->d_alpha_h, sizeof(double) * E));
    CK(cudaMalloc((void **)&c->d_limited, sizeof(int) * E));
    CK(up(&c->d_lnboff, off));  // last: marks the tables complete
  }
  // MRS: alpha h^1.5 (limiter.c:121-124); minmodB: alpha h
  // (limiter.c:292-302); h the largest bbox extent
  std::vector<double> ah(E);
  for (int64_t e = 0; e < E; e++) {
    const double *bb = &c->geom.bbox[e * 6];
    const double h = std::max(bb[1] - bb[0], std::max(bb[3] - bb[2], bb[5] - bb[4]));
    ah[e] = kind == NMG_LIMITER_MRS ? alpha * pow(h, 1.5) : alpha * h;
  }
  CK(cudaMemcpy(c->d_alpha_h, ah.data(), sizeof(double) * E, cudaMemcpyHostToDevice));
  c->lim_kind = kind;
  c->lim_bos3 = beta / sqrt(3.);
  c->lim_scale_bound = scale_bound;
  c->lim_on = true;
  return NMG_OK;
}

int nmg_get_limited(nmg_ctx *c, int32_t *limited) {
  if (!c || !limited) return set_err(c, NMG_EINVAL, "nmg_get_limited: null argument");
  if (!c->d_limited) return set_err(c, NMG_EUNSUP, "nmg_get_limited: no limiter set");
  CK(cudaMemcpy(limited, c->d_limited, sizeof(int) * c->nelem, cudaMemcpyDeviceToHost));
  return NMG_OK;
}

int nmg_set_filter(nmg_ctx *c, int32_t on, double alp, double s, int32_t dn, int32_t jpower,
                   int32_t filter_fv) {
  if (!c) return NMG_EINVAL;
  if (jpower != 0 && jpower != 1)
    return set_err(c, NMG_EINVAL, "nmg_set_filter: jpower must be 0 or 1");
  drop_graphs(c);
  if (!on) {
    c->filter_on = false;
    return NMG_OK;
  }
  const int n = c->n, np = c->np, nn = c->nn;
  // F = S diag(f) A per point type: S_ij = P_j(x_i)/sqrt(c_j) with
  // 1/c_j = (2j+1)/2 (j/2 for j = N); A = w_j S_ji on LGL points
  // (LGL_AT_ST_matrices) and A = S^-1 on equally spaced points
  // (Legendre_AT_ST_matrices, src/main/basis/Legendre.c:277-310,723-729);
  // f_k = exp(-alp (k/N')^s), N' = n - 1 - dn (1 if <= 0) (filter.c:19-56)
  double Nf = n - 1 - dn;
  if (Nf <= 0.) Nf = 1.;
  std::vector<double> F(2 * (size_t)nn), f(n);
  for (int k = 0; k < n; k++) f[k] = exp(-alp * pow(k / Nf, s));
  for (int typ = 0; typ < 2; typ++) {
    const double *x = typ == 0 ? c->h_xl.data() : c->h_xu.data();
    std::vector<long double> S(nn), A(nn);
    for (int i = 0; i < n; i++)
      for (int j = 0; j < n; j++) {
        double ooc = 0.5 * (2 * j + 1);
        if (j == n - 1 && n - 1 != 0) ooc = 0.5 * j;
        S[i * n + j] = legendre_p(j, x[i]) * sqrt(ooc);
      }
    if (typ == 0) {
      std::vector<double> w(n), D((size_t)nn), xx(n);
      nmg::lgl_basis(n, xx.data(), w.data(), D.data());
      for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) A[i * n + j] = w[j] * (double)S[j * n + i];
    } else {
      std::vector<long double> M(S), I(nn, 0.L);
      for (int i = 0; i < n; i++) I[i * n + i] = 1.L;
      for (int col = 0; col < n; col++) {
        int piv = col;
        for (int r = col + 1; r < n; r++)
          if (fabsl(M[r * n + col]) > fabsl(M[piv * n + col])) piv = r;
        for (int q = 0; q < n; q++) {
          std::swap(M[col * n + q], M[piv * n + q]);
          std::swap(I[col * n + q], I[piv * n + q]);
        }
        const long double d = M[col * n + col];
        for (int q = 0; q < n; q++) {
          M[col * n + q] /= d;
          I[col * n + q] /= d;
        }
        for (int r = 0; r < n; r++)
          if (r != col) {
            const long double fac = M[r * n + col];
            for (int q = 0; q < n; q++) {
              M[r * n + q] -= fac * M[col * n + q];
              I[r * n + q] -= fac * I[col * n + q];
            }
          }
      }
      A = I;
    }
    for (int p = 0; p < n; p++)
      for (int q = 0; q < n; q++) {
        long double sum = 0.L;
        for (int k = 0; k < n; k++) sum += S[p * n + k] * (long double)f[k] * A[k * n + q];
        F[typ * nn + p * n + q] = (double)sum;
      }
  }
  if (!c->d_filt) CK(cudaMalloc((void **)&c->d_filt, sizeof(double) * 2 * nn));
  CK(cudaMemcpy(c->d_filt, F.data(), sizeof(double) * 2 * nn, cudaMemcpyHostToDevice));
  if (jpower && !c->d_fooj && c->ncurvi > 0) {
    // det(dXb/dx) on the LGL points of the curvilinear elements
    std::vector<double> J((size_t)c->ncurvi * np), xyz(3 * (size_t)np), dX(9 * (size_t)np);
    for (int64_t e = 0; e < c->nelem; e++) {
      const int cs = c->h_cslot[e];
      if (cs < 0) continue;
      if (!nmg::element_geometry(c->geom, e, false, xyz.data(), dX.data()))
        return set_err(c, NMG_EUNSUP, "nmg_set_filter: needs the maps of a generated mesh");
      const double *bb = &c->geom.bbox[e * 6];
      const double d0 = 2. / (bb[1] - bb[0]), d1 = 2. / (bb[3] - bb[2]), d2 = 2. / (bb[5] - bb[4]);
      for (int q = 0; q < np; q++) {
        double M[3][3];
        for (int a = 0; a < 3; a++)
          for (int b = 0; b < 3; b++) M[a][b] = dX[(a * 3 + b) * np + q];
        const double det = M[0][0] * M[1][1] * M[2][2] - M[0][2] * M[1][1] * M[2][0] +
                           M[0][1] * M[1][2] * M[2][0] + M[0][2] * M[1][0] * M[2][1] -
                           M[0][0] * M[1][2] * M[2][1] - M[0][1] * M[1][0] * M[2][2];
        J[(size_t)cs * np + q] = d0 * d1 * d2 * det;
      }
    }
    CK(cudaMalloc((void **)&c->d_fooj, sizeof(double) * J.size()));
    CK(cudaMemcpy(c->d_fooj, J.data(), sizeof(double) * J.size(), cudaMemcpyHostToDevice));
  }
  CK(nmgk::filter_prepare(n));
  c->filter_jpow = jpower;
  c->filter_fv = filter_fv ? 1 : 0;
  c->filter_on = true;
  return NMG_OK;
}

int nmg_set_fv_midpoint_data(nmg_ctx *c, int32_t on) {
  if (!c) return NMG_EINVAL;
  if (!c->fv) return set_err(c, NMG_EUNSUP, "nmg_set_fv_midpoint_data: no finite-volume elements");
  if (on && !c->d_fvmid && c->ncurvi > 0) {
    // per curvilinear element and direction d, at the midpoint right of each
    // node: sqrtgdiag_d, det(dXb/dx) and the unit normal of direction d, in
    // the operation order of the grid-point values (coordinates.c:174-223,
    // 337-420, utilities.c:48-80)
    const int n = c->n, np = c->np;
    std::vector<double> mid((size_t)c->ncurvi * 15 * np, 0.), dX((size_t)27 * np);
    for (int64_t e = 0; e < c->nelem; e++) {
      const int cs = c->h_cslot[e];
      if (cs < 0) continue;
      if (!nmg::element_midpoint_dXdx(c->geom, e, dX.data()))
        return set_err(c, NMG_EUNSUP,
                       "nmg_set_fv_midpoint_data: needs the maps of a generated mesh");
      const double *bb = &c->geom.bbox[e * 6];
      const double d0 = 2. / (bb[1] - bb[0]), d1 = 2. / (bb[3] - bb[2]), d2 = 2. / (bb[5] - bb[4]);
      const double dXbdX[3] = {d0, d1, d2};
      double *Gm = &mid[(size_t)cs * 15 * np];
      for (int d = 0; d < 3; d++)
        for (int q = 0; q < np; q++) {
          const int id[3] = {q % n, (q / n) % n, q / (n * n)};
          if (id[d] >= n - 1) continue;
          double M[3][3];
          for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) M[a][b] = dX[((size_t)d * 9 + a * 3 + b) * np + q];
          const double det = M[0][0] * M[1][1] * M[2][2] - M[0][2] * M[1][1] * M[2][0] +
                             M[0][1] * M[1][2] * M[2][0] + M[0][2] * M[1][0] * M[2][1] -
                             M[0][0] * M[1][2] * M[2][1] - M[0][1] * M[1][0] * M[2][2];
          double g = 0.0;
          for (int l = 0; l < 3; l++) g += M[d][l] * M[d][l];
          double smag = sqrt(M[d][0] * M[d][0] + M[d][1] * M[d][1] + M[d][2] * M[d][2]);
          if (smag == 0.0) smag = 1.;
          Gm[(d * 5 + 0) * np + q] = dXbdX[d] * sqrt(g);
          Gm[(d * 5 + 1) * np + q] = d0 * d1 * d2 * det;
          for (int l = 0; l < 3; l++) Gm[(d * 5 + 2 + l) * np + q] = M[d][l] / smag;
        }
    }
    CK(cudaMalloc((void **)&c->d_fvmid, sizeof(double) * mid.size()));
    CK(cudaMemcpy(c->d_fvmid, mid.data(), sizeof(double) * mid.size(), cudaMemcpyHostToDevice));
  }
  c->fv_mid = on != 0;
  drop_graphs(c);
  return NMG_OK;
}

int nmg_set_fv(nmg_ctx *c, int32_t rec, int32_t extrap, double w3ratio) {
  if (!c) return NMG_EINVAL;
  if (!c->fv) return set_err(c, NMG_EUNSUP, "nmg_set_fv: the mesh has no finite-volume elements");
  if (rec < NMG_FV_REC_1 || rec > NMG_FV_REC_WENOMZ_2)
    return set_err(c, NMG_EINVAL, "nmg_set_fv: unknown reconstruction");
  if (extrap != NMG_FV_EXTRAP_NO && extrap != NMG_FV_EXTRAP_DNFN1)
    return set_err(c, NMG_EINVAL, "nmg_set_fv: unknown div(f) extrapolation");
  if (!(w3ratio > 0.)) return set_err(c, NMG_EINVAL, "nmg_set_fv: w3ratio must be > 0");
  c->fv_rec = rec;
  c->fv_extrap = extrap;
  c->fv_w3ratio = w3ratio;
  drop_graphs(c);
  return NMG_OK;
}

void nmg_destroy(nmg_ctx *c) {
  if (!c) return;
  drop_graphs(c);
  cudaFree(c->d_nb); cudaFree(c->d_code); cudaFree(c->d_cslot); cudaFree(c->d_bslot);
  cudaFree(c->d_cmask); cudaFree(c->d_scale); cudaFree(c->d_gcart); cudaFree(c->d_metric);
  cudaFree(c->d_metricp); cudaFree(c->d_fac); cudaFree(c->d_bxyz); cudaFree(c->d_bnrm);
  cudaFree(c->d_D);
  cudaFree(c->d_fvgeo); cudaFree(c->d_fvdist); cudaFree(c->d_fvdxb);
  cudaFree(c->d_fvlist); cudaFree(c->d_gtab); cudaFree(c->d_isfv); cudaFree(c->d_ghost);
  cudaFree(c->d_hoff); cudaFree(c->d_hsrc); cudaFree(c->d_hw);
  cudaFree(c->d_toff); cudaFree(c->d_tsrc); cudaFree(c->d_tw); cudaFree(c->d_hface); cudaFree(c->d_fvmid);
  cudaFree(c->d_filt); cudaFree(c->d_fooj);
  cudaFree(c->d_lim); cudaFree(c->d_alpha_h); cudaFree(c->d_wl); cudaFree(c->d_wu);
  cudaFree(c->d_lnboff); cudaFree(c->d_lnb); cudaFree(c->d_limited); cudaFree(c->d_mmb);
  cudaFree(c->d_gM); cudaFree(c->d_fvbxyz); cudaFree(c->d_fvbnrm); cudaFree(c->d_PR);
  cudaFree(c->d_conv); cudaFree(c->d_mm); cudaFree(c->d_trb); cudaFree(c->d_score);
  cudaFree(c->d_r); cudaFree(c->d_w2); cudaFree(c->d_ghost2); cudaFree(c->d_tlist);
  cudaFree(c->d_code2); cudaFree(c->d_bslot2); cudaFree(c->d_gtab2);
  cudaFree(c->d_up); cudaFree(c->d_pers); cudaFree(c->d_wq); cudaFree(c->d_npart);
  for (int b = 0; b < 4; b++) cudaFree(c->d_buf[b]);
  cudaFree(c->d_times); cudaFree(c->d_step);
  for (int k = 0; k < nmg_ctx::kChunks; k++) {
    if (c->chunk_ev[k]) cudaEventDestroy(c->chunk_ev[k]);
    if (c->h2d_ev[k]) cudaEventDestroy(c->h2d_ev[k]);
  }
  cudaFree(c->d_elist);
  if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
  if (c->stream2) cudaStreamDestroy(c->stream2);
  if (c->fork_ev) cudaEventDestroy(c->fork_ev);
  if (c->join_ev) cudaEventDestroy(c->join_ev);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

const char *nmg_last_error(const nmg_ctx *c) {
  if (!c) return "null context";
  return c->err_static ? c->err_static : c->err.c_str();
}
int64_t nmg_state_size(const nmg_ctx *c) { return c ? (int64_t)c->state_len : -1; }
int64_t nmg_kernel_launches(const nmg_ctx *c) { return c ? c->launches : -1; }
void *nmg_stream(nmg_ctx *c) { return c ? (void *)c->stream : nullptr; }
double *nmg_state_device_ptr(nmg_ctx *c) { return c ? c->d_buf[c->cur] : nullptr; }

int nmg_set_kernel(nmg_ctx *c, const char *spec) {
  if (!c) return NMG_EINVAL;
  if (!spec || !*spec || !strcmp(spec, "auto")) {
    c->sel = -1;
    c->tuned = false;
    c->fsel = -1;
    c->ftuned = false;
    drop_graphs(c);
    return NMG_OK;
  }
  for (int v = 0; v < c->nvjp_alt; v++) {  // the transposed kernel ("vjp" or "tcvjp")
    if (!strcmp(spec, c->vjp_alt[v].name)) {
      c->vjp = c->vjp_alt[v];
      return NMG_OK;
    }
  }
  for (int v = 0; v < c->nvariants; v++) {
    char buf[64];
    snprintf(buf, sizeof buf, "%s:%d:%d", c->variants[v].name, c->variants[v].epb,
             c->variants[v].nt);
    if (!strcmp(spec, c->variants[v].name) || !strcmp(spec, buf)) {
      if (c->mixed && v >= c->ndg) {  // the finite-volume part of a mixed mesh
        c->fsel = v;
        c->ftuned = true;
      } else {
        c->sel = v;
        c->tuned = true;
      }
      drop_graphs(c);
      return NMG_OK;
    }
  }
  return set_err(c, NMG_EINVAL, std::string("nmg_set_kernel: unknown variant ") + spec);
}

int nmg_kernel_info(nmg_ctx *c, char *buf, int32_t len) {
  if (!c || !buf || len <= 0) return NMG_EINVAL;
  std::string s;
  if (c->sel >= 0) {
    char b[64];
    snprintf(b, sizeof b, "%s:%d:%d", c->variants[c->sel].name, c->variants[c->sel].epb,
             c->variants[c->sel].nt);
    s = b;
  } else {
    s = "untuned";
  }
  if (c->mixed) {
    char b[64];
    if (c->fsel >= 0)
      snprintf(b, sizeof b, " + %s:%d:%d", c->variants[c->fsel].name, c->variants[c->fsel].epb,
               c->variants[c->fsel].nt);
    else
      snprintf(b, sizeof b, " + untuned");
    s += b;
  }
  s += " | candidates:";
  for (int v = 0; v < c->nvariants; v++) {
    char b[64];
    snprintf(b, sizeof b, " %s:%d:%d", c->variants[v].name, c->variants[v].epb,
             c->variants[v].nt);
    s += b;
  }
  if (!c->tune_log.empty()) s += " | timings: " + c->tune_log;
  snprintf(buf, (size_t)len, "%s", s.c_str());
  return NMG_OK;
}

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
  return launch_stage(c, P);
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

// one RK4 step of the resident state without the filter
static int rk4_step_plain(nmg_ctx *c, double t, double dt) {
  int rc = enqueue_step(c, c->cur, t, dt, false);
  if (rc) return rc;
  c->cur = 1 - c->cur;
  CK(cudaStreamSynchronize(c->stream));
  return NMG_OK;
}

int nmg_rk4_step(nmg_ctx *c, double t, double dt) {
  if (!c) return NMG_EINVAL;
  int rc = rk4_step_plain(c, t, dt);
  if (rc) return rc;
  CK(apply_filter(c, c->d_buf[c->cur]));
  CK(cudaStreamSynchronize(c->stream));
  return NMG_OK;
}

// capture one step (u in d_buf[cur]) reading its time from the device
static int capture_step_graph(nmg_ctx *c, int cur, double dt, int method) {
  int rc = autotune(c);  // never tune inside a capture
  if (rc) return rc;
  cudaGraph_t g;
  CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  int64_t l0 = c->launches;
  rc = enqueue_step(c, cur, 0., dt, true, method);
  if (!rc && apply_filter(c, c->d_buf[1 - cur]) != cudaSuccess) rc = NMG_ECUDA;
  advance_step_kernel<<<1, 1, 0, c->stream>>>(c->d_step);
  cudaError_t e1 = cudaGetLastError();
  cudaError_t e2 = cudaStreamEndCapture(c->stream, &g);
  c->graph_launches = c->launches - l0 + 1;  // stage launches + step counter
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

static int steps_impl(nmg_ctx *c, double t, double dt, int32_t nsteps, int method);

int nmg_rk4_steps(nmg_ctx *c, double t, double dt, int32_t nsteps) {
  if (!c || nsteps < 0) return set_err(c, NMG_EINVAL, "nmg_rk4_steps: bad argument");
  return steps_impl(c, t, dt, nsteps, NMG_EVOLVE_RK4);
}

int nmg_set_evolve_method(nmg_ctx *c, int32_t method) {
  if (!c) return NMG_EINVAL;
  if (method != NMG_EVOLVE_RK4 && method != NMG_EVOLVE_EULER && method != NMG_EVOLVE_SSPRK3)
    return set_err(c, NMG_EINVAL, "nmg_set_evolve_method: unknown method");
  c->method = method;
  return NMG_OK;
}

int nmg_evolve_steps(nmg_ctx *c, double t, double dt, int32_t nsteps) {
  if (!c || nsteps < 0) return set_err(c, NMG_EINVAL, "nmg_evolve_steps: bad argument");
  return steps_impl(c, t, dt, nsteps, c->method);
}

int nmg_evolve_steps_host(nmg_ctx *c, double t, double dt, int32_t nsteps, double *host_u) {
  if (!c || !host_u || nsteps < 0)
    return set_err(c, NMG_EINVAL, "nmg_evolve_steps_host: bad argument");
  const size_t bytes = c->state_len * sizeof(double);
  CK(cudaMemcpyAsync(c->d_buf[c->cur], host_u, bytes, cudaMemcpyHostToDevice, c->stream));
  int rc = steps_impl(c, t, dt, nsteps, c->method);
  if (rc) return rc;
  CK(cudaMemcpyAsync(host_u, c->d_buf[c->cur], bytes, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return NMG_OK;
}

static int steps_impl(nmg_ctx *c, double t, double dt, int32_t nsteps, int method) {
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
    drop_graphs(c);
  }
  if (dt != c->graph_dt || c->graph_sel != c->sel * 64 + c->fsel ||
      c->graph_method != method) {
    drop_graphs(c);
    c->graph_dt = dt;
    c->graph_method = method;
  }
  for (int g = 0; g < 2; g++)
    if (!c->graph[g]) {
      int rc = capture_step_graph(c, g, dt, method);
      if (rc) return rc;
    }
  c->graph_sel = c->sel * 64 + c->fsel;
  CK(cudaMemcpyAsync(c->d_times, times.data(), sizeof(double) * nsteps, cudaMemcpyHostToDevice,
                     c->stream));
  CK(cudaMemsetAsync(c->d_step, 0, sizeof(int), c->stream));
  for (int s = 0; s < nsteps; s++) {
    CK(cudaGraphLaunch(c->graph[c->cur], c->stream));
    c->launches += c->graph_launches;
    c->cur = 1 - c->cur;
  }
  CK(cudaStreamSynchronize(c->stream));
  return NMG_OK;
}

// One RK4 step of u = d_buf[cur] at time t whose final stage runs in element
// chunks; each chunk's new u is copied to host_u on the copy stream as soon
// as the chunk is done (the chunks start at multiples of the variant's
// elements per CTA, so every element is computed by the same tile as in an
// unchunked launch and the result is bitwise the same).
static int prepare_h2d_groups(nmg_ctx *c) {
  if (c->d_elist) return NMG_OK;
  const int64_t E = c->nelem;
  const int K = c->nchunks;
  const int64_t chunk = (E + K - 1) / K;
  std::vector<std::vector<int>> grp(K);
  for (int64_t e = 0; e < E; e++) {
    int64_t r = e / chunk;
    for (int f = 0; f < 6; f++) {
      const int nb = c->h_nb[e * 6 + f];
      if (nb >= 0) r = std::max<int64_t>(r, nb / chunk);
    }
    grp[r].push_back((int)e);
  }
  std::vector<int> lst;
  c->h2d_off.assign(nmg_ctx::kChunks + 1, (int)0);
  for (int k = 0; k < K; k++) {
    lst.insert(lst.end(), grp[k].begin(), grp[k].end());
    c->h2d_off[k + 1] = (int)lst.size();
  }
  c->h2d_chunk = chunk;
  CK(cudaMalloc((void **)&c->d_elist, sizeof(int) * std::max<size_t>(lst.size(), 1)));
  CK(cudaMemcpy(c->d_elist, lst.data(), sizeof(int) * lst.size(), cudaMemcpyHostToDevice));
  return NMG_OK;
}

static int last_step_streamed(nmg_ctx *c, double t, double dt, double *host_u,
                              const double *host_in) {
  int rc = autotune(c);
  if (rc) return rc;
  if (!c->copy_stream) {
    CK(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&c->stream2, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&c->fork_ev, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&c->join_ev, cudaEventDisableTiming));
    for (int k = 0; k < nmg_ctx::kChunks; k++) {
      CK(cudaEventCreateWithFlags(&c->chunk_ev[k], cudaEventDisableTiming));
      CK(cudaEventCreateWithFlags(&c->h2d_ev[k], cudaEventDisableTiming));
    }
  }
  if (host_in && (rc = prepare_h2d_groups(c))) return rc;
  const int cur = c->cur;
  double *U = c->d_buf[cur], *ACC = c->d_buf[1 - cur], *WA = c->d_buf[2], *WB = c->d_buf[3];
  const double cacc[4] = {dt / 6., dt / 3., dt / 3., dt / 6.};
  const double cw[4] = {dt / 2., dt / 2., dt, 0.};
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
    P.t = (s == 0) ? t : (s == 3) ? t + dt : t + 0.5 * dt;
    if (s == 0 && host_in) {
      // copy u in chunks; each element group runs as soon as its face
      // neighbourhood has arrived (per element the same arithmetic)
      const size_t per = (size_t)NF * c->np;
      for (int k = 0; k < c->nchunks; k++) {
        const int64_t ea = k * c->h2d_chunk, eb = std::min<int64_t>(c->nelem, ea + c->h2d_chunk);
        if (eb > ea)
          CK(cudaMemcpyAsync(U + ea * per, host_in + ea * per, (size_t)(eb - ea) * per * sizeof(double),
                             cudaMemcpyHostToDevice, c->copy_stream));
        CK(cudaEventRecord(c->h2d_ev[k], c->copy_stream));
      }
      CK(cudaEventRecord(c->fork_ev, c->stream));
      CK(cudaStreamWaitEvent(c->stream2, c->fork_ev, 0));
      for (int k = 0; k < c->nchunks; k++) {
        cudaStream_t sk = (k & 1) ? c->stream2 : c->stream;
        CK(cudaStreamWaitEvent(sk, c->h2d_ev[k], 0));
        const int n0 = c->h2d_off[k], n1 = c->h2d_off[k + 1];
        if (n1 == n0) continue;
        StageParams Q = P;
        Q.elist = c->d_elist;
        Q.ebase = n0;
        Q.ecount = n1 - n0;
        CK(c->variants[c->sel].launch(Q, sk));
        c->launches++;
      }
      CK(cudaEventRecord(c->join_ev, c->stream2));
      CK(cudaStreamWaitEvent(c->stream, c->join_ev, 0));
      continue;
    }
    if (s < 3) {
      CK(run_stage(c, c->sel, P));
      continue;
    }
    const int64_t E = c->nelem, epb = std::max(1, c->variants[c->sel].epb);
    int64_t chunk = (E + c->nchunks - 1) / c->nchunks;
    chunk = (chunk + epb - 1) / epb * epb;
    const size_t per = (size_t)NF * c->np;
    // the stage's face traces (non-conforming faces) once, before the chunks
    if (c->nhang > 0) {
      CK(nmgk::hang_launch(c->nhang, c->n, c->d_hoff, c->d_hsrc, c->d_hw, P.win, c->d_ghost,
                           c->stream));
      c->launches++;
    }
    CK(cudaEventRecord(c->fork_ev, c->stream));
    CK(cudaStreamWaitEvent(c->stream2, c->fork_ev, 0));
    int k = 0;
    for (int64_t ea = 0; ea < E; ea += chunk, k++) {
      const int64_t eb = std::min(E, ea + chunk);
      cudaStream_t sk = ((k & 1) && !c->mixed) ? c->stream2 : c->stream;
      P.ebase = (int)ea;
      P.ecount = (int)(eb - ea);
      if (c->mixed)
        CK(run_stage(c, c->sel, P, ea == 0));  // (not reached: mixed meshes step unstreamed)
      else
        CK(c->variants[c->sel].launch(P, sk));
      if (!c->mixed) c->launches++;
      CK(cudaEventRecord(c->chunk_ev[k], sk));
      CK(cudaStreamWaitEvent(c->copy_stream, c->chunk_ev[k], 0));
      CK(cudaMemcpyAsync(host_u + ea * per, ACC + ea * per, (size_t)(eb - ea) * per * sizeof(double),
                         cudaMemcpyDeviceToHost, c->copy_stream));
    }
  }
  CK(cudaStreamSynchronize(c->copy_stream));
  CK(cudaStreamSynchronize(c->stream2));
  CK(cudaStreamSynchronize(c->stream));
  c->cur = 1 - cur;
  return NMG_OK;
}

int nmg_rk4_steps_host(nmg_ctx *c, double t, double dt, int32_t nsteps, double *host_u) {
  if (!c || !host_u) return set_err(c, NMG_EINVAL, "nmg_rk4_steps_host: null argument");
  if (nsteps < 0) return set_err(c, NMG_EINVAL, "nmg_rk4_steps_host: bad argument");
  const size_t bytes = c->state_len * sizeof(double);
  int rc;
  if (!c->fv && !c->nhang && !c->filter_on && !c->lim_on && nsteps == 1)  // copy in, step, copy out overlapped
    return last_step_streamed(c, t, dt, host_u, host_u);
  CK(cudaMemcpyAsync(c->d_buf[c->cur], host_u, bytes, cudaMemcpyHostToDevice, c->stream));
  if (c->mixed || c->filter_on || c->lim_on || nsteps == 0) {
    rc = nmg_rk4_steps(c, t, dt, nsteps);
    if (rc) return rc;
    CK(cudaMemcpyAsync(host_u, c->d_buf[c->cur], bytes, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return NMG_OK;
  }
  // all steps but the last through the step graphs, the last one streamed
  // back; step times accumulated as evolve_mesh does (main.c:610-626)
  if (nsteps > 1 && (rc = nmg_rk4_steps(c, t, dt, nsteps - 1))) return rc;
  long double Te = t, te = 0.;
  for (int s = 0; s < nsteps - 1; s++) te += dt;
  return last_step_streamed(c, (double)(Te + te), dt, host_u, nullptr);
}

// ---------------------------------------------------------------------------
// adjoint (vector-Jacobian) entry points
// ---------------------------------------------------------------------------
// The transposed non-conforming lists (first adjoint call): contribution q
// of slot h, node t reads source node (j, k) of the source face, which is
// itself slot h2, with weight B1[j] B2[k] / (contributions of the node).
static int ensure_hang_transpose(nmg_ctx *c) {
  if (c->nhang <= 0 || c->d_toff) return NMG_OK;
  const int n = c->n, nn = n * n;
  const int64_t H = c->nhang;
  std::vector<int64_t> slot_of(c->nelem * 6, -1);
  for (int64_t h = 0; h < H; h++) slot_of[(int64_t)c->h_hface[2 * h] * 6 + c->h_hface[2 * h + 1]] = h;
  std::vector<int> cnt((size_t)H * nn + 1, 0);
  for (int pass = 0; pass < 2; pass++) {
    std::vector<int> toff, tsrc;
    std::vector<double> tw;
    if (pass == 1) {
      toff.assign((size_t)H * nn + 1, 0);
      for (size_t q = 0; q < (size_t)H * nn; q++) toff[q + 1] = toff[q] + cnt[q];
      tsrc.assign(std::max(toff.back(), 1), 0);
      tw.assign(tsrc.size(), 0.);
    }
    std::vector<int> fill(pass == 1 ? toff.begin() : toff.end(), toff.end());
    for (int64_t h = 0; h < H; h++)
      for (int t = 0; t < nn; t++) {
        const int c0 = c->h_hoff[h * nn + t], c1 = c->h_hoff[h * nn + t + 1];
        const double inv = c1 - c0 > 1 ? 1. / (c1 - c0) : 1.;
        for (int q = c0; q < c1; q++) {
          const int64_t h2 = slot_of[(int64_t)c->h_hsrc[2 * q] * 6 + c->h_hsrc[2 * q + 1]];
          if (h2 < 0) return set_err(c, NMG_EMESH, "non-conforming source face without a slot");
          for (int k = 0; k < n; k++)
            for (int j = 0; j < n; j++) {
              const size_t at = (size_t)h2 * nn + j + n * k;
              if (pass == 0) {
                cnt[at]++;
              } else {
                const int i = fill[at]++;
                tsrc[i] = (int)(h * nn + t);
                tw[i] = c->h_hw[(q * 2) * n + j] * c->h_hw[(q * 2 + 1) * n + k] * inv;
              }
            }
        }
      }
    if (pass == 1) {
      auto up = [&](auto **dst, const auto &vec) -> cudaError_t {
        const size_t bytes = vec.size() * sizeof(vec[0]);
        cudaError_t e2 = cudaMalloc((void **)dst, std::max<size_t>(bytes, 16));
        if (e2 != cudaSuccess || bytes == 0) return e2;
        return cudaMemcpy(*dst, vec.data(), bytes, cudaMemcpyHostToDevice);
      };
      CK(up(&c->d_tsrc, tsrc));
      CK(up(&c->d_tw, tw));
      CK(up(&c->d_hface, c->h_hface));
      CK(up(&c->d_toff, toff));  // last: marks the lists complete
    }
  }
  return NMG_OK;
}

int nmg_rhs_vjp(nmg_ctx *c, double t, const double *w_dev, const double *rbar_dev,
                double *wbar_dev) {
  (void)t;
  (void)w_dev;  // the RHS is linear in w: its Jacobian does not depend on w
  if (!c || !rbar_dev || !wbar_dev || rbar_dev == wbar_dev)
    return set_err(c, NMG_EINVAL, "nmg_rhs_vjp: need distinct rbar and wbar device buffers");
  if (c->fv) return set_err(c, NMG_EUNSUP, "nmg_rhs_vjp: finite-volume RHS is nonlinear");
  if (c->lim_on) return set_err(c, NMG_EUNSUP, "nmg_rhs_vjp: the limiter is nonlinear");
  if (c->numflux != NMG_NUMFLUX_LLF)
    return set_err(c, NMG_EUNSUP, "nmg_rhs_vjp: the transposed kernel implements LLF only");
  if (int rc = ensure_hang_transpose(c)) return rc;
  StageParams P = base_params(c);
  P.win = rbar_dev;
  P.rout = wbar_dev;
  P.mode = 0;
  CK(vjp_stage(c, P));
  CK(cudaStreamSynchronize(c->stream));
  return NMG_OK;
}

int nmg_rk4_step_vjp(nmg_ctx *c, double t, double dt, const double *u_n_dev, double *ubar_dev) {
  (void)u_n_dev;  // linear RHS: the step's Jacobian is P(dt L), independent of u_n
  if (!c || !ubar_dev) return set_err(c, NMG_EINVAL, "nmg_rk4_step_vjp: null argument");
  if (c->fv) return set_err(c, NMG_EUNSUP, "nmg_rk4_step_vjp: finite-volume RHS is nonlinear");
  if (c->lim_on) return set_err(c, NMG_EUNSUP, "nmg_rk4_step_vjp: the limiter is nonlinear");
  if (c->numflux != NMG_NUMFLUX_LLF)
    return set_err(c, NMG_EUNSUP, "nmg_rk4_step_vjp: the transposed kernel implements LLF only");
  int rc = ensure_hang_transpose(c);
  if (rc) return rc;
  double *acc = c->d_buf[1 - c->cur];  // free between steps
  rc = step_buffers(c, true, t, dt, ubar_dev, acc, c->d_buf[2], c->d_buf[3]);
  if (rc) return rc;
  CK(cudaMemcpyAsync(ubar_dev, acc, c->state_len * sizeof(double), cudaMemcpyDeviceToDevice,
                     c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return NMG_OK;
}

// J(u0) = sum_{s=1..nsteps} dt sum_nodes W phi(t_s)^2 and dJ/du0 by the
// discrete adjoint of the RK4 trajectory, with u checkpointed every
// ckpt_every steps and the states of each segment recomputed in reverse.
int nmg_adjoint_gradient(nmg_ctx *c, double t0, double dt, int32_t nsteps, int32_t ckpt_every,
                         const double *weight_dev, double *J, double *grad_dev) {
  if (c && c->fv) return set_err(c, NMG_EUNSUP, "nmg_adjoint_gradient: finite-volume RHS is nonlinear");
  if (c && c->lim_on) return set_err(c, NMG_EUNSUP, "nmg_adjoint_gradient: the limiter is nonlinear");
  if (c && c->numflux != NMG_NUMFLUX_LLF)
    return set_err(c, NMG_EUNSUP, "nmg_adjoint_gradient: the transposed kernel implements LLF only");
  if (!c || !weight_dev || !J || !grad_dev || nsteps <= 0 || ckpt_every <= 0)
    return set_err(c, NMG_EINVAL, "nmg_adjoint_gradient: bad argument");
  int rc = autotune(c);
  if (rc) return rc;
  if ((rc = ensure_hang_transpose(c))) return rc;
  const size_t L = c->state_len, bytes = L * sizeof(double);
  const int K = ckpt_every, nck = (nsteps + K - 1) / K;
  const int np = c->np, E = (int)c->nelem;
  const int nseg = std::max(K, 2);  // the forward sweep ping-pongs through them
  std::vector<double *> ck(nck, nullptr), seg(nseg, nullptr);
  double *lam[2] = {nullptr, nullptr}, *jdev = nullptr, *partial = nullptr;
  const int nblk = 4 * 152;
  // step times as evolve_mesh accumulates them (main.c:610-626)
  std::vector<double> ts(nsteps + 1);
  {
    long double Te = t0, te = 0.;
    for (int s = 0; s <= nsteps; s++) {
      ts[s] = (double)(Te + te);
      te += dt;
    }
  }
  auto cleanup = [&]() {
    for (auto p : ck) cudaFree(p);
    for (auto p : seg) cudaFree(p);
    cudaFree(lam[0]);
    cudaFree(lam[1]);
    cudaFree(jdev);
    cudaFree(partial);
  };
  auto fail = [&](cudaError_t e, const char *what) {
    cleanup();
    return set_err(c, NMG_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
  };
  cudaError_t e;
  for (int i = 0; i < nck; i++)
    if ((e = cudaMalloc((void **)&ck[i], bytes)) != cudaSuccess) return fail(e, "checkpoint");
  for (int i = 0; i < nseg; i++)
    if ((e = cudaMalloc((void **)&seg[i], bytes)) != cudaSuccess) return fail(e, "segment");
  for (int i = 0; i < 2; i++)
    if ((e = cudaMalloc((void **)&lam[i], bytes)) != cudaSuccess) return fail(e, "adjoint");
  if ((e = cudaMalloc((void **)&jdev, sizeof(double))) != cudaSuccess) return fail(e, "J");
  if ((e = cudaMalloc((void **)&partial, nblk * sizeof(double))) != cudaSuccess)
    return fail(e, "partials");
  cudaStream_t st = c->stream;
  double *WA = c->d_buf[2], *WB = c->d_buf[3];
  // forward sweep: J and the checkpoints
  cudaMemsetAsync(jdev, 0, sizeof(double), st);
  cudaMemcpyAsync(ck[0], c->d_buf[c->cur], bytes, cudaMemcpyDeviceToDevice, st);
  {
    const double *u = ck[0];
    for (int s = 1; s <= nsteps; s++) {
      double *out = seg[(s - 1) % nseg];
      if ((rc = step_buffers(c, false, ts[s - 1], dt, u, out, WA, WB))) { cleanup(); return rc; }
      obj_partial_kernel<<<nblk, kObjThreads, 0, st>>>(out, weight_dev, E, np, partial);
      obj_final_kernel<<<1, 1, 0, st>>>(partial, nblk, dt, jdev);
      c->launches += 2;
      if (s % K == 0 && s / K < nck)
        cudaMemcpyAsync(ck[s / K], out, bytes, cudaMemcpyDeviceToDevice, st);
      u = out;
    }
  }
  // reverse sweep
  cudaMemsetAsync(lam[0], 0, bytes, st);
  int li = 0;
  for (int cidx = nck - 1; cidx >= 0; cidx--) {
    const int s0 = cidx * K, s1 = std::min(nsteps, s0 + K);
    const double *u = ck[cidx];
    for (int s = s0 + 1; s <= s1; s++) {  // recompute u_{s0+1..s1}
      if ((rc = step_buffers(c, false, ts[s - 1], dt, u, seg[s - s0 - 1], WA, WB))) {
        cleanup();
        return rc;
      }
      u = seg[s - s0 - 1];
    }
    for (int s = s1; s > s0; s--) {
      adj_source_kernel<<<nblk, 256, 0, st>>>(lam[li], seg[s - s0 - 1], weight_dev, E, np,
                                              2.0 * dt);
      if ((rc = step_buffers(c, true, ts[s - 1], dt, lam[li], lam[1 - li], WA, WB))) {
        cleanup();
        return rc;
      }
      c->launches++;
      li = 1 - li;
    }
  }
  cudaMemcpyAsync(grad_dev, lam[li], bytes, cudaMemcpyDeviceToDevice, st);
  double Jh = 0.;
  cudaMemcpyAsync(&Jh, jdev, sizeof(double), cudaMemcpyDeviceToHost, st);
  e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return fail(e, "nmg_adjoint_gradient");
  if ((e = cudaGetLastError()) != cudaSuccess) return fail(e, "nmg_adjoint_gradient launch");
  *J = Jh;
  cleanup();
  return NMG_OK;
}

int nmg_fp64_dmma_peak(double *gflops) {
  nmg_ctx *c = nullptr;  // for CK: errors are returned without a context
  if (!gflops) return NMG_EINVAL;
  int dev = 0, sms = 0;
  CK(cudaGetDevice(&dev));
  CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int blocks = sms * 4, threads = 256, iters = 256;
  double *out = nullptr;
  CK(cudaMalloc((void **)&out, sizeof(double) * blocks * threads));
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  dmma_peak_kernel<<<blocks, threads>>>(out, 32, 1.0, 1e-9);
  CK(cudaGetLastError());
  float best = 1e30f;
  for (int r = 0; r < 5; r++) {
    CK(cudaEventRecord(e0));
    dmma_peak_kernel<<<blocks, threads>>>(out, iters, 1.0, 1e-9);
    CK(cudaEventRecord(e1));
    CK(cudaEventSynchronize(e1));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    best = std::min(best, ms);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  // per warp and iteration: 4 mma of 8 x 8 x 4 FMA (2 flops each)
  *gflops = 2.0 * 256 * 4 * iters * (double)blocks * (threads / 32) / (best * 1e6);
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

}  // extern "C"

// ---------------------------------------------------------------------------
// batched execution of many independent problems
// ---------------------------------------------------------------------------
struct nmg_batch {
  std::string err;
  int nprob = 0;
  std::vector<nmg_mesh *> gmesh;  // merged mesh of each order (owned)
  std::vector<nmg_ctx *> gctx;    // one context per order
  std::vector<int> gn, gblk0;     // per group, highest order first
  int ntile = 0;
  std::vector<int> pgroup;
  std::vector<int64_t> pelem0, pnelem;
  size_t smem = 0;
  int grid = 0;  // persistent CTAs, chosen by timing
  int grouped = 0;  // 1: one launch per order with that order's tuned variant
  int force_mode = 0;  // 0 autotune, 1 persistent only, 2 per-order launches only
  std::vector<StageParams> hparams;  // host copy of d_params
  std::string tune_log;
  cudaStream_t stream = nullptr;
  StageParams *d_params = nullptr;  // [parity][stage][group]
  int *d_gn = nullptr, *d_gblk0 = nullptr;
  double *d_times = nullptr;
  int *d_step = nullptr;
  int times_cap = 0;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  double graph_dt = 0;
  int cur = 0;
  int64_t launches = 0;
  // faces joined across the parts of one problem (p-nonconforming when the
  // parts' n differ): per face the target group and ghost slot, the source
  // group, element, face and orientation (nmg_batch_create_linked)
  int nlink = 0;
  int *d_links = nullptr;          // [nlink][6]
  double **d_ghostp = nullptr;     // [G] ghost arrays of the groups
  const double **d_wsrc = nullptr; // [2 parities][4 stages][G] stage inputs
  double *d_xtab = nullptr;        // [kBatchMaxN + 1][kBatchMaxN]: LGL points per n
  double *d_btab = nullptr;        // ... and their barycentric weights
};

static int batch_err(nmg_batch *b, int code, const std::string &msg) {
  if (b) b->err = msg;
  return code;
}

#define BK(call)                                                                          \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess)                                                                \
      return batch_err(b, NMG_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// per-group stage parameters of one RK4 step with u in buffer `parity`,
// stage times read from the batch's device time array
static void batch_params(nmg_batch *b, int parity, std::vector<StageParams> &out) {
  const int G = (int)b->gctx.size();
  out.assign(2 * 4 * G, StageParams());
  for (int par = 0; par < 2; par++)
    for (int s = 0; s < 4; s++)
      for (int g = 0; g < G; g++) {
        nmg_ctx *c = b->gctx[g];
        double *U = c->d_buf[par], *ACC = c->d_buf[1 - par], *WA = c->d_buf[2],
               *WB = c->d_buf[3];
        const double *win[4] = {U, WA, WB, WA};
        double *wout[4] = {WA, WB, WA, nullptr};
        StageParams P = base_params(c);
        P.win = win[s];
        P.u0 = U;
        P.acc = ACC;
        P.wout = wout[s];
        P.mode = s + 1;
        P.tdev = b->d_times;
        P.stepdev = b->d_step;
        out[(par * 4 + s) * G + g] = P;
      }
  (void)parity;
}

// stage coefficients depend on dt: fill them and upload all parameters
static int batch_upload_params(nmg_batch *b, double dt) {
  std::vector<StageParams> ps;
  batch_params(b, 0, ps);
  const int G = (int)b->gctx.size();
  const double cacc[4] = {dt / 6., dt / 3., dt / 3., dt / 6.};
  const double cw[4] = {dt / 2., dt / 2., dt, 0.};
  const double tofs[4] = {0., 0.5 * dt, 0.5 * dt, dt};
  for (int par = 0; par < 2; par++)
    for (int s = 0; s < 4; s++)
      for (int g = 0; g < G; g++) {
        StageParams &P = ps[(par * 4 + s) * G + g];
        P.cacc = cacc[s];
        P.cw = cw[s];
        P.tofs_dt = tofs[s];
      }
  BK(cudaMemcpy(b->d_params, ps.data(), ps.size() * sizeof(StageParams),
                cudaMemcpyHostToDevice));
  b->hparams = ps;
  if (b->nlink > 0) {
    std::vector<const double *> ws(8 * G);
    for (int q = 0; q < 8 * G; q++) ws[q] = ps[q].win;
    BK(cudaMemcpy(b->d_wsrc, ws.data(), sizeof(double *) * 8 * G, cudaMemcpyHostToDevice));
  }
  return NMG_OK;
}

static int batch_enqueue_stage(nmg_batch *b, int par, int s) {
  const int G = (int)b->gctx.size();
  for (int g = 0; g < G; g++) {  // traces of non-conforming faces first
    nmg_ctx *c = b->gctx[g];
    if (c->nhang <= 0) continue;
    BK(nmgk::hang_launch(c->nhang, c->n, c->d_hoff, c->d_hsrc, c->d_hw,
                         b->hparams[(par * 4 + s) * G + g].win, c->d_ghost, b->stream));
    b->launches++;
  }
  if (b->nlink > 0) {  // faces joined across parts
    const int64_t work = (int64_t)b->nlink * 4 * nmgk::kBatchMaxN * nmgk::kBatchMaxN;
    const int grid = (int)std::min<int64_t>((work + 255) / 256, 152 * 8);
    plink_kernel<<<grid, 256, 0, b->stream>>>(b->d_links, b->nlink, b->d_gn, b->d_ghostp,
                                              b->d_wsrc + (par * 4 + s) * G, b->d_xtab,
                                              b->d_btab);
    BK(cudaGetLastError());
    b->launches++;
  }
  if (b->grouped) {
    for (int g = 0; g < G; g++) {
      nmg_ctx *c = b->gctx[g];
      BK(c->variants[c->sel].launch(b->hparams[(par * 4 + s) * G + g], b->stream));
      b->launches++;
    }
  } else {
    BK(nmgk::batch_launch(b->d_params + (par * 4 + s) * G, b->d_gn, b->d_gblk0, G, b->ntile,
                          b->grid, b->smem, b->stream));
    b->launches++;
  }
  return NMG_OK;
}

static int batch_enqueue_step(nmg_batch *b, int par) {
  for (int s = 0; s < 4; s++) {
    int rc = batch_enqueue_stage(b, par, s);
    if (rc) return rc;
  }
  return NMG_OK;
}

static void batch_drop_graphs(nmg_batch *b) {
  for (int g = 0; g < 2; g++)
    if (b->graph[g]) {
      cudaGraphExecDestroy(b->graph[g]);
      b->graph[g] = nullptr;
    }
}

// autotuner of the batched launch: persistent grid size by timing stage 1
// (which reads u and writes only the accumulator and a stage buffer)
static int batch_autotune(nmg_batch *b, double dt) {
  if (b->grid > 0) return NMG_OK;
  int dev = 0, sms = 0;
  BK(cudaGetDevice(&dev));
  BK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  int rc = batch_upload_params(b, dt);
  if (rc) return rc;
  double t0 = 0.;
  BK(cudaMemcpyAsync(b->d_times, &t0, sizeof(double), cudaMemcpyHostToDevice, b->stream));
  BK(cudaMemsetAsync(b->d_step, 0, sizeof(int), b->stream));
  // each order's own variant first (the grouped mode launches those)
  for (auto c : b->gctx) {
    rc = autotune(c);
    if (rc) return batch_err(b, rc, std::string("batch autotune: ") + nmg_last_error(c));
  }
  // candidates: grid > 0 = one persistent launch with that many CTAs,
  // grid = 0 = one launch per order
  std::vector<int> cands;
  if (b->force_mode != 2) {
    cands.push_back(b->ntile);
    for (int k = 1; k <= 4; k++)
      if (sms * k < b->ntile) cands.push_back(sms * k);
  }
  if (b->force_mode != 1) cands.push_back(0);
  cudaEvent_t e0, e1;
  BK(cudaEventCreate(&e0));
  BK(cudaEventCreate(&e1));
  float best = 1e30f;
  int bestg = b->ntile;
  b->tune_log.clear();
  for (int grid : cands) {
    b->grouped = grid == 0;
    b->grid = grid == 0 ? b->ntile : grid;
    if ((rc = batch_enqueue_stage(b, 0, 0))) return rc;
    BK(cudaEventRecord(e0, b->stream));
    for (int r = 0; r < 3; r++)
      if ((rc = batch_enqueue_stage(b, 0, 0))) return rc;
    BK(cudaEventRecord(e1, b->stream));
    BK(cudaEventSynchronize(e1));
    float ms = 0;
    BK(cudaEventElapsedTime(&ms, e0, e1));
    ms /= 3;
    char buf[64];
    if (grid) snprintf(buf, sizeof buf, "persistent-grid%d=%.4fms ", grid, ms);
    else snprintf(buf, sizeof buf, "per-order-launches=%.4fms ", ms);
    b->tune_log += buf;
    if (ms < best) { best = ms; bestg = grid; }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  b->grouped = bestg == 0;
  b->grid = bestg == 0 ? b->ntile : bestg;
  return NMG_OK;
}

extern "C" {

static int batch_link_parts(nmg_batch *b, const nmg_mesh *const *meshes, int count,
                            const int32_t *problem);

static int batch_create_impl(const nmg_mesh *const *meshes, int32_t count, const int32_t *problem,
                             int32_t bc_kind, const double k[3], nmg_batch **out) {
  if (!out) return NMG_EINVAL;
  *out = nullptr;
  nmg_batch *b = new (std::nothrow) nmg_batch;
  if (!b) return NMG_ENOMEM;
  *out = b;
  if (!meshes || count <= 0) return batch_err(b, NMG_EINVAL, "nmg_batch_create: no meshes");
  b->nprob = count;
  std::vector<int> orders;
  for (int p = 0; p < count; p++) {
    if (!meshes[p]) return batch_err(b, NMG_EINVAL, "nmg_batch_create: null mesh");
    if (!meshes[p]->fv.empty())
      return batch_err(b, NMG_EUNSUP, "nmg_batch_create: finite-volume meshes are not batched");
    const int n = meshes[p]->n;
    if (nmgk::batch_epb(n) <= 0)
      return batch_err(b, NMG_EUNSUP, "nmg_batch_create: orders n in [2,10] only");
    if (std::find(orders.begin(), orders.end(), n) == orders.end()) orders.push_back(n);
  }
  std::sort(orders.begin(), orders.end(), [](int a, int c) { return a > c; });
  b->pgroup.assign(count, -1);
  b->pelem0.assign(count, 0);
  b->pnelem.assign(count, 0);
  int tile = 0;
  for (size_t g = 0; g < orders.size(); g++) {
    const int n = orders[g];
    std::vector<const nmg_mesh *> list;
    int64_t off = 0;
    for (int p = 0; p < count; p++)
      if (meshes[p]->n == n) {
        list.push_back(meshes[p]);
        b->pgroup[p] = (int)g;
        b->pelem0[p] = off;
        b->pnelem[p] = meshes[p]->nelem;
        off += meshes[p]->nelem;
      }
    nmg_mesh *mm = nullptr;
    if (nmg_mesh_concat(list.data(), (int)list.size(), &mm))
      return batch_err(b, NMG_EMESH, std::string("nmg_batch_create: ") + nmg_mesh_last_error());
    b->gmesh.push_back(mm);
    nmg_ctx *c = nullptr;
    int rc = nmg_create(mm, bc_kind, k, &c);
    b->gctx.push_back(c);
    if (rc) return batch_err(b, rc, std::string("nmg_batch_create: ") + nmg_last_error(c));
    b->gn.push_back(n);
    b->gblk0.push_back(tile);
    tile += (int)((mm->nelem + nmgk::batch_epb(n) - 1) / nmgk::batch_epb(n));
    b->smem = std::max(b->smem, nmgk::batch_smem(n));
  }
  b->ntile = tile;
  BK(nmgk::batch_prepare(b->smem));
  BK(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
  const int G = (int)b->gctx.size();
  BK(cudaMalloc((void **)&b->d_params, sizeof(StageParams) * 8 * G));
  BK(cudaMalloc((void **)&b->d_gn, sizeof(int) * G));
  BK(cudaMalloc((void **)&b->d_gblk0, sizeof(int) * G));
  BK(cudaMemcpy(b->d_gn, b->gn.data(), sizeof(int) * G, cudaMemcpyHostToDevice));
  BK(cudaMemcpy(b->d_gblk0, b->gblk0.data(), sizeof(int) * G, cudaMemcpyHostToDevice));
  BK(cudaMalloc((void **)&b->d_step, sizeof(int)));
  BK(cudaMalloc((void **)&b->d_times, sizeof(double)));
  b->times_cap = 1;
  if (problem) return batch_link_parts(b, meshes, count, problem);
  return NMG_OK;
}

int nmg_batch_create(const nmg_mesh *const *meshes, int32_t count, int32_t bc_kind,
                     const double k[3], nmg_batch **out) {
  return batch_create_impl(meshes, count, nullptr, bc_kind, k, out);
}

int nmg_batch_create_linked(const nmg_mesh *const *meshes, int32_t count, const int32_t *problem,
                            int32_t bc_kind, const double k[3], nmg_batch **out) {
  if (!problem) return NMG_EINVAL;
  return batch_create_impl(meshes, count, problem, bc_kind, k, out);
}

int64_t nmg_batch_linked_faces(const nmg_batch *b) { return b ? b->nlink : -1; }

}  // extern "C"

// Join the parts of each problem across their coinciding outer faces: each
// such face of part i becomes a face of its group's context whose exterior
// state is read from a ghost slot (the mixed-face path of the stage
// kernels), filled every stage by plink_kernel from part j's stage input.
static int batch_link_parts(nmg_batch *b, const nmg_mesh *const *meshes, int count,
                            const int32_t *problem) {
  struct OFace {
    int part;
    int64_t e;
    int f;
    double c[4][3];
  };
  auto corner = [&](const nmg_mesh *m, int64_t e, int f, int ca, int cb, double x[3]) {
    const int n = m->n, np = n * n * n;
    const int node = nmg::face_node(n, f, ca * (n - 1), cb * (n - 1));
    for (int d = 0; d < 3; d++) x[d] = m->xyz[((size_t)e * 3 + d) * np + node];
  };
  const double h = 1e-6, tol = 1e-9;
  auto key = [&](const double c[3]) {
    return std::to_string(std::llround(c[0] / h)) + "," + std::to_string(std::llround(c[1] / h)) +
           "," + std::to_string(std::llround(c[2] / h));
  };
  // outer faces of every part, hashed by their corner centroid
  std::vector<OFace> faces;
  std::unordered_map<std::string, std::vector<size_t>> where;
  for (int i = 0; i < count; i++) {
    const nmg_mesh *m = meshes[i];
    for (int64_t e = 0; e < m->nelem; e++)
      for (int f = 0; f < 6; f++) {
        if (m->nb[e * 6 + f] >= 0) continue;
        OFace F{i, e, f, {}};
        double cen[3] = {0, 0, 0};
        for (int t = 0; t < 4; t++) {
          corner(m, e, f, t & 1, t >> 1, F.c[t]);
          for (int d = 0; d < 3; d++) cen[d] += 0.25 * F.c[t][d];
        }
        where[key(cen)].push_back(faces.size());
        faces.push_back(F);
      }
  }
  const int G = (int)b->gctx.size();
  std::vector<std::vector<int64_t>> gfaces(G);  // per group: e * 6 + f of its joined faces
  std::vector<int> links;                       // [L][6] before slot numbers
  std::vector<int> link_group;
  for (const auto &kv : where) {
    const std::vector<size_t> &lst = kv.second;
    for (size_t x : lst)
      for (size_t y : lst) {
        if (x == y) continue;
        const OFace &A = faces[x], &B = faces[y];
        if (A.part == B.part || problem[A.part] != problem[B.part]) continue;
        int found = -1;
        for (int o = 0; o < 8 && found < 0; o++) {
          bool ok = true;
          for (int t = 0; t < 4 && ok; t++) {
            const int ca = t & 1, cb = t >> 1;
            int aa = (o & 1) ? cb : ca, bb = (o & 1) ? ca : cb;
            if (o & 2) aa = 1 - aa;
            if (o & 4) bb = 1 - bb;
            const double *p = B.c[aa + 2 * bb];
            double d2 = 0.;
            for (int d = 0; d < 3; d++) d2 += (A.c[t][d] - p[d]) * (A.c[t][d] - p[d]);
            ok = d2 <= tol * tol;
          }
          if (ok) found = o;
        }
        if (found < 0) continue;
        const int ga = b->pgroup[A.part], gb = b->pgroup[B.part];
        const int64_t ea = b->pelem0[A.part] + A.e, eb = b->pelem0[B.part] + B.e;
        gfaces[ga].push_back(ea * 6 + A.f);
        links.insert(links.end(), {ga, (int)(gfaces[ga].size() - 1), gb, (int)eb, B.f, found});
      }
  }
  b->nlink = (int)(links.size() / 6);
  if (b->nlink == 0) return NMG_OK;
  // the joined faces of each group read ghost slots after its hang slots
  std::vector<double *> ghostp(G, nullptr);
  for (int g = 0; g < G; g++) {
    nmg_ctx *c = b->gctx[g];
    const int64_t E = c->nelem;
    const int nh = c->nhang, nl = (int)gfaces[g].size();
    if (nl > 0) {
      std::vector<int> nb(E * 6), code(E * 6), bslot(E * 6);
      BK(cudaMemcpy(nb.data(), c->d_nb, sizeof(int) * E * 6, cudaMemcpyDeviceToHost));
      BK(cudaMemcpy(code.data(), c->d_code, sizeof(int) * E * 6, cudaMemcpyDeviceToHost));
      BK(cudaMemcpy(bslot.data(), c->d_bslot, sizeof(int) * E * 6, cudaMemcpyDeviceToHost));
      for (int q = 0; q < nl; q++) {
        const int64_t ef = gfaces[g][q];
        nb[ef] = (int)(ef / 6);  // any element: the ghost path reads the slot
        code[ef] = nmgk::kCodeMixed;
        bslot[ef] = nh + q;
      }
      BK(cudaMemcpy(c->d_nb, nb.data(), sizeof(int) * E * 6, cudaMemcpyHostToDevice));
      BK(cudaMemcpy(c->d_code, code.data(), sizeof(int) * E * 6, cudaMemcpyHostToDevice));
      BK(cudaMemcpy(c->d_bslot, bslot.data(), sizeof(int) * E * 6, cudaMemcpyHostToDevice));
      const size_t slots = (size_t)nh + nl;
      double *ng = nullptr;
      BK(cudaMalloc((void **)&ng, sizeof(double) * 4 * c->nn * slots));
      BK(cudaMemset(ng, 0, sizeof(double) * 4 * c->nn * slots));
      cudaFree(c->d_ghost);
      c->d_ghost = ng;
      c->ghost_cap = (int)slots;
      drop_graphs(c);
    }
    ghostp[g] = c->d_ghost;
  }
  for (int l = 0; l < b->nlink; l++) links[6 * l + 1] += b->gctx[links[6 * l]]->nhang;
  // LGL points and barycentric weights of every order (Lagrange.c:15-27)
  constexpr int M = nmgk::kBatchMaxN;
  std::vector<double> xt((M + 1) * M, 0.), bt((M + 1) * M, 0.);
  for (int n = 2; n <= M; n++) {
    std::vector<double> x(n), w(n), D(n * n);
    nmg::lgl_basis(n, x.data(), w.data(), D.data());
    for (int i = 0; i < n; i++) {
      double den = 1.;
      for (int j = 0; j < n; j++)
        if (j != i) den *= (x[i] - x[j]);
      xt[n * M + i] = x[i];
      bt[n * M + i] = 1. / den;
    }
  }
  BK(cudaMalloc((void **)&b->d_links, sizeof(int) * links.size()));
  BK(cudaMemcpy(b->d_links, links.data(), sizeof(int) * links.size(), cudaMemcpyHostToDevice));
  BK(cudaMalloc((void **)&b->d_ghostp, sizeof(double *) * G));
  BK(cudaMemcpy(b->d_ghostp, ghostp.data(), sizeof(double *) * G, cudaMemcpyHostToDevice));
  BK(cudaMalloc((void **)&b->d_wsrc, sizeof(double *) * 8 * G));
  BK(cudaMalloc((void **)&b->d_xtab, sizeof(double) * xt.size()));
  BK(cudaMalloc((void **)&b->d_btab, sizeof(double) * bt.size()));
  BK(cudaMemcpy(b->d_xtab, xt.data(), sizeof(double) * xt.size(), cudaMemcpyHostToDevice));
  BK(cudaMemcpy(b->d_btab, bt.data(), sizeof(double) * bt.size(), cudaMemcpyHostToDevice));
  return NMG_OK;
}

extern "C" {

void nmg_batch_destroy(nmg_batch *b) {
  if (!b) return;
  batch_drop_graphs(b);
  cudaFree(b->d_links);
  cudaFree(b->d_ghostp);
  cudaFree(b->d_wsrc);
  cudaFree(b->d_xtab);
  cudaFree(b->d_btab);
  for (auto c : b->gctx) nmg_destroy(c);
  for (auto m : b->gmesh) nmg_mesh_free(m);
  cudaFree(b->d_params);
  cudaFree(b->d_gn);
  cudaFree(b->d_gblk0);
  cudaFree(b->d_times);
  cudaFree(b->d_step);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

const char *nmg_batch_last_error(const nmg_batch *b) {
  return b ? b->err.c_str() : "null batch";
}

int64_t nmg_batch_problem_size(const nmg_batch *b, int32_t p) {
  if (!b || p < 0 || p >= b->nprob) return -1;
  const int n = b->gn[b->pgroup[p]];
  return b->pnelem[p] * NF * (int64_t)n * n * n;
}

static double *batch_problem_ptr(nmg_batch *b, int p) {
  const int g = b->pgroup[p];
  const int np = b->gctx[g]->np;
  return b->gctx[g]->d_buf[b->cur] + b->pelem0[p] * NF * (int64_t)np;
}

int nmg_batch_set_state(nmg_batch *b, int32_t p, const double *host_u) {
  if (!b || !host_u || p < 0 || p >= b->nprob)
    return batch_err(b, NMG_EINVAL, "nmg_batch_set_state: bad argument");
  BK(cudaMemcpy(batch_problem_ptr(b, p), host_u,
                nmg_batch_problem_size(b, p) * sizeof(double), cudaMemcpyHostToDevice));
  return NMG_OK;
}

int nmg_batch_get_state(nmg_batch *b, int32_t p, double *host_u) {
  if (!b || !host_u || p < 0 || p >= b->nprob)
    return batch_err(b, NMG_EINVAL, "nmg_batch_get_state: bad argument");
  BK(cudaMemcpy(host_u, batch_problem_ptr(b, p), nmg_batch_problem_size(b, p) * sizeof(double),
                cudaMemcpyDeviceToHost));
  return NMG_OK;
}

int nmg_rk4_steps_batched(nmg_batch *b, double t, double dt, int32_t nsteps) {
  if (!b || nsteps < 0) return batch_err(b, NMG_EINVAL, "nmg_rk4_steps_batched: bad argument");
  if (nsteps == 0) return NMG_OK;
  for (auto c : b->gctx) BK(cudaStreamSynchronize(c->stream));  // state copies are done
  std::vector<double> times(nsteps);
  long double Te = t, te = 0.;
  for (int s = 0; s < nsteps; s++) {
    times[s] = (double)(Te + te);
    te += dt;
  }
  if (nsteps > b->times_cap) {
    cudaFree(b->d_times);
    b->d_times = nullptr;
    BK(cudaMalloc((void **)&b->d_times, sizeof(double) * nsteps));
    b->times_cap = nsteps;
    batch_drop_graphs(b);
  }
  if (dt != b->graph_dt) {
    batch_drop_graphs(b);
    b->graph_dt = dt;
  }
  int rc = batch_autotune(b, dt);
  if (rc) return rc;
  if (!b->graph[0] || !b->graph[1]) {
    rc = batch_upload_params(b, dt);
    if (rc) return rc;
    for (int par = 0; par < 2; par++) {
      cudaGraph_t g;
      BK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
      int64_t l0 = b->launches;
      rc = batch_enqueue_step(b, par);
      advance_step_kernel<<<1, 1, 0, b->stream>>>(b->d_step);
      cudaError_t e1 = cudaGetLastError();
      cudaError_t e2 = cudaStreamEndCapture(b->stream, &g);
      b->launches = l0;
      if (rc) return rc;
      BK(e1);
      BK(e2);
      cudaError_t e3 = cudaGraphInstantiate(&b->graph[par], g, 0);
      cudaGraphDestroy(g);
      BK(e3);
    }
  }
  BK(cudaMemcpyAsync(b->d_times, times.data(), sizeof(double) * nsteps, cudaMemcpyHostToDevice,
                     b->stream));
  BK(cudaMemsetAsync(b->d_step, 0, sizeof(int), b->stream));
  for (int s = 0; s < nsteps; s++) {
    BK(cudaGraphLaunch(b->graph[b->cur], b->stream));
    b->launches += 5;
    b->cur = 1 - b->cur;
  }
  BK(cudaStreamSynchronize(b->stream));
  return NMG_OK;
}

int nmg_batch_info(nmg_batch *b, char *buf, int32_t len) {
  if (!b || !buf || len <= 0) return NMG_EINVAL;
  std::string s = "groups:";
  for (size_t g = 0; g < b->gn.size(); g++) {
    char t[96];
    snprintf(t, sizeof t, " n%d:%lld elems/%d per tile", b->gn[g],
             (long long)b->gctx[g]->nelem, nmgk::batch_epb(b->gn[g]));
    s += t;
  }
  char t[128];
  snprintf(t, sizeof t, " | mode %s | tiles %d | grid %d | launches %lld",
           b->grouped ? "per-order-launches" : "persistent", b->ntile, b->grid,
           (long long)b->launches);
  s += t;
  if (!b->tune_log.empty()) s += " | timings: " + b->tune_log;
  snprintf(buf, (size_t)len, "%s", s.c_str());
  return NMG_OK;
}

void *nmg_batch_stream(nmg_batch *b) { return b ? (void *)b->stream : nullptr; }

int nmg_batch_set_mode(nmg_batch *b, int32_t mode) {
  if (!b || mode < 0 || mode > 2) return batch_err(b, NMG_EINVAL, "nmg_batch_set_mode: 0, 1 or 2");
  b->force_mode = mode;
  b->grid = 0;  // re-tune on the next step
  batch_drop_graphs(b);
  return NMG_OK;
}

}  // extern "C"
