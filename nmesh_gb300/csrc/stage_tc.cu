// stage_tc.cu -- "tc" variant of the fused DG stage kernel (n = 7, 8, 9
// points per direction): the LGL directional derivatives on the tensor
// cores, exactly, by integer digits.
//
// GB300 issues about two FP64 FMAs per clock per SM, so the 10 directional
// line derivatives per node (two thirds of the FP64 work of the eo variant)
// are moved to the FP16 tensor pipe, which runs beside the FP64 pipe.  The
// arithmetic is an error-free splitting of the matrix products into digit
// products (the idea of Ozaki, Ogita, Oishi and Rump, "Error-free
// transformations of matrix multiplication by using fast routines of matrix
// multiplication and its applications", Numer. Algorithms 59, 2012), here
// with fixed-point digits:
//
// * each field of an element is put on one fixed-point grid: with Emax the
//   largest biased exponent of the field's values, u = X 2^(Emax-1086) with
//   X < 2^64 an integer (its top 56 bits are kept: 7 digits of 8 bits,
//   d_s = byte 7-s of X, carrying u's sign);
// * each row i of D is put on its own grid the same way (exponent FD_i, 7
//   digits delta_t, rounded to nearest at the 56th bit);
// * the tensor core forms, for every output i and digit group w = s + t
//   <= 6, acc_w = sum_p sum_{s+t=w} delta_t(D_ip) d_s(u_p): at most 9 points x
//   7 pairs of products below 2^16, so |acc_w| < 2^22 and every partial sum
//   is an integer that FP32 holds exactly (the accumulators start at
//   1.5 2^23, so their bit patterns are 0x4B400000 + acc_w: no conversion
//   instruction is needed to read them back);
// * T = sum_w acc_w 2^(40-8w) is formed in 64-bit integers and turned into
//   the FP64 value T 2^(Emax+FD_i-2100) (one conversion, rounded to
//   nearest, and an integer add to the exponent field).
//
// The dropped digit groups and digits leave an error of at most ~1.3 units of
// 2^-53 of max|u| x sum_p |D_ip| per output (checked against exact rationals),
// the size of the FP64 dot product's own rounding bound; the result is
// bitwise deterministic.  A field whose
// largest exponent is 2047 (inf or NaN) yields NaN derivatives; values below
// 2^-1022 (subnormals) count as zero, and derivatives below the normal range
// flush to zero.
//
// Layout: the digits of element-field values are stored once per node, 16 B
// each ([field][node][8 x fp16], slot 7 zero).  One MMA row is one line of
// nodes along the pass direction; ldmatrix gathers the 16-B rows of a line
// from that one layout for all three directions (bank-conflict free at n = 9:
// the node stride of a line is 1, 9 or 81).  K = (point, digit slot): n
// points rounded up to even x 8 (at n = 9, 10 x 8 = 80; an added point is a
// copy of the last with zero B rows); N =
// (output, group): 9 x 7 = 63 of 64 columns, arranged so that each thread of
// a quad holds all seven groups of the outputs it owns (t and t+4; output 8
// is summed over the quad; at n = 7, 8 the columns of outputs >= n are zero).
// A pass takes n^2 / 16 tiles of 16 lines, one warp each; the line left over
// at n = 7, 9 (49 = 3 x 16 + 1, 81 = 5 x 16 + 1) is an FP64 dot product in
// the next warp.  Everything after the derivatives
// (chain rule with the metric, LLF face lift, RK update) is the FP64 code of
// the other variants; the element's metric, lift factors and the u0 /
// accumulator blocks the stage reads are bulk-prefetched to L2 at the start.
//
// Reference semantics (paths within nmeshsource/nmesh): the derivative is
// src/main/coordinates/derivs.c:154-181 (D applied along each direction,
// then the chain rule of src/tests/scalarwave1/scalarwave1.c:242-284).
#include <cuda_fp16.h>

#include <cstdint>
#include <cstring>
#include <vector>

#include "stage.cuh"
#include "tc_device.cuh"

namespace nmgk {
namespace {

// r out (mode 0) or the RK stage update (modes of StageParams), with the
// loads of NB outputs per thread issued before their arithmetic
template <int N, int NT>
__device__ __forceinline__ void tc_epilogue(const StageParams &P, const double *Wg,
                                            const double *sR, int e) {
  constexpr int TNP = TcShape<N>::NP;
  constexpr int TOT = NF * TNP, NB = 4;
  if (P.skip && P.skip[e]) return;
  const size_t base = (size_t)e * NF * TNP;
  const int mode = P.mode;
  const bool need_u0 = mode == 1 || mode == 2 || mode == 3 || mode == 5 || mode == 6;
  const bool need_acc = mode == 2 || mode == 3 || mode == 4 || mode == 6;
  for (int q0 = threadIdx.x; q0 < TOT; q0 += NB * NT) {
    double r[NB], u[NB], ac[NB], wi[NB];
#pragma unroll
    for (int j = 0; j < NB; j++) {
      const int q = q0 + j * NT;
      r[j] = u[j] = ac[j] = wi[j] = 0.;
      if (q < TOT) {
        r[j] = q < 4 * TNP ? sR[q] : __ldg(Wg + (q - 4 * TNP));  // r_phi = pi
        if (need_u0) u[j] = __ldg(P.u0 + base + q);
        if (need_acc) ac[j] = P.acc[base + q];
        if (mode == 6) wi[j] = __ldg(P.win + base + q);
      }
    }
#pragma unroll
    for (int j = 0; j < NB; j++) {
      const int q = q0 + j * NT;
      if (q >= TOT) continue;
      const size_t idx = base + q;
      if (mode == 0) {
        P.rout[idx] = r[j];
      } else if (mode == 1) {
        P.acc[idx] = fma(P.cacc, r[j], u[j]);
        P.wout[idx] = fma(P.cw, r[j], u[j]);
      } else if (mode == 4) {
        P.acc[idx] = fma(P.cacc, r[j], ac[j]);
      } else if (mode == 5) {
        P.acc[idx] = fma(P.cacc, r[j], u[j]);
      } else if (mode == 6) {
        P.acc[idx] = fma(P.cacc, r[j], ac[j]);
        P.wout[idx] = fma(0.25, fma(P.cw, r[j], wi[j]), 0.75 * u[j]);
      } else {
        P.acc[idx] = fma(P.cacc, r[j], ac[j]);
        P.wout[idx] = fma(P.cw, r[j], u[j]);
      }
    }
  }
}

template <int N, int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB) tc_kernel(StageParams P) {
  using S = TcShape<N>;
  constexpr int TN = N, TNP = S::NP, TNN = S::NN, TTILES = S::TILES;
  constexpr int NWARP = NT / 32;
  constexpr int NLOAD = (4 * TNP + NT - 1) / NT;
  extern __shared__ __align__(16) unsigned char tsm[];
  double *sR = reinterpret_cast<double *>(tsm);           // [4][NP]: r_pi, r_c
  uint4 *sDig = reinterpret_cast<uint4 *>(sR + 4 * TNP);  // [4][NP] digits
  __shared__ int sCs[1];
  __shared__ int sMask;
  __shared__ int sEmax[4];
  __shared__ double sScale[3];
  __shared__ double sG[1][3];

  const int e0 = P.ebase + blockIdx.x;
  const int e = elem_at(P, e0);
  if (e >= P.nelem) return;  // whole CTA (one element per CTA)
  const int tid = threadIdx.x;
  const double *Wg = P.win + (size_t)e * NF * TNP;  // w of this element, [field][node]
  // all loads of w in flight at once
  double v[NLOAD];
#pragma unroll
  for (int k = 0; k < NLOAD; k++) {
    const int q = tid + k * NT;
    v[k] = q < 4 * TNP ? __ldg(Wg + q) : 0.;
  }
  if (tid == 0) {
    // the element's u0 / accumulator blocks and its metric go to L2 now, so
    // that the chain rule and the epilogue find them there
    // (only what the stage mode reads: the accumulator is write-only in
    // modes 1 and 5, and u0 is w itself in the first stage)
    const int md = P.mode;
    const size_t blk = (size_t)e * NF * TNP;
    if ((md == 1 || md == 2 || md == 3 || md == 5 || md == 6) && P.u0 && P.u0 != P.win)
      tc_prefetch_l2(P.u0 + blk, sizeof(double) * NF * TNP);
    if ((md == 2 || md == 3 || md == 4 || md == 6) && P.acc)
      tc_prefetch_l2(P.acc + blk, sizeof(double) * NF * TNP);
    const int cs = P.cslot[e];
    if (cs >= 0) {
      tc_prefetch_l2(P.metricp + (size_t)cs * 9 * TNP, sizeof(double) * 9 * TNP);
      tc_prefetch_l2(P.fac + (size_t)cs * 6 * TNN * 4, sizeof(double) * 6 * TNN * 4);
    }
    sCs[0] = cs;
    sMask = cs >= 0 ? P.cmask[cs] : (1 | (1 << 4) | (1 << 8));
    for (int d = 0; d < 3; d++) sScale[d] = P.scale[e * 3 + d];
    for (int d = 0; d < 3; d++) sG[0][d] = P.gcart[e * 3 + d];
  }
  if (tid < 4) sEmax[tid] = 0;
  for (int q = tid; q < 4 * TNP; q += NT) sR[q] = 0.;
  __syncthreads();
  {
    int em[4] = {0, 0, 0, 0};
#pragma unroll
    for (int k = 0; k < NLOAD; k++) {
      const int q = tid + k * NT, f = q / TNP;
      const int ex = (int)((unsigned long long)__double_as_longlong(v[k]) >> 52) & 0x7FF;
#pragma unroll
      for (int j = 0; j < 4; j++)
        if (f == j) em[j] = max(em[j], ex);
    }
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const unsigned m = __reduce_max_sync(0xffffffffu, (unsigned)em[j]);
      if ((tid & 31) == 0) atomicMax(&sEmax[j], (int)m);
    }
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < NLOAD; k++) {
    const int q = tid + k * NT;
    if (q < 4 * TNP) sDig[q] = tc_digits(v[k], sEmax[q / TNP]);
  }
  const double t = stage_time(P);
  // face terms first: their loads overlap the digit stores; face_terms ends with a barrier
  face_terms<N, 1, NT>(P, Wg, sR, sCs, sG, e0, t);

  const int warp = tid >> 5, lane = tid & 31, g = lane >> 2, tq = lane & 3;
  const int cs = sCs[0], mask = sMask;
  const uint32_t digbase = (uint32_t)__cvta_generic_to_shared(sDig);
  const int fd0 = cTcRowExp[N - 7][tq], fd1 = cTcRowExp[N - 7][min(tq + 4, 8)];
  const int fd8 = cTcRowExp[N - 7][8];
  const uint4 *gB = &gTcB[N - 7][0][0][0];
  const double *gD = gTcD[N - 7];

  // ---- volume terms, one direction per pass; warp w takes lines 16w..16w+15 ----
#pragma unroll 1
  for (int a = 0; a < 3; a++) {
    const int row = (mask >> (3 * a)) & 7;
#pragma unroll 1
    for (int tile = warp; tile < TTILES; tile += NWARP) {
      // ldmatrix row of this lane: line Lr, points 2kk + chunk (node nb + p ps)
      const int Lr = min(tile * 16 + (lane & 15), TNN - 1), chunk = lane >> 4;
      const int ps = a == 0 ? 1 : (a == 1 ? TN : TNN);
      const int nb = a == 0 ? TN * Lr : (a == 1 ? (Lr % TN) + TNN * (Lr / TN) : Lr);
      const uint32_t rowbase = digbase + (uint32_t)nb * 16u, pstep = (uint32_t)ps * 16u;
      // owned output slots: (g, t), (g, t+4), (g+8, t), (g+8, t+4), and output 8
      // of row g (t = 0) or g+8 (t = 1); their nodes and the chain-rule factors
      // M[a][i](node) of every i with M[a][i] != 0, all loaded before the MMAs
      int nodeS[5];
      bool okS[5];
      double m3[3][5];
#pragma unroll
      for (int sl = 0; sl < 5; sl++) {
        const int L = tile * 16 + g + (sl < 4 ? (sl >> 1) * 8 : tq * 8);
        const int i = sl < 4 ? tq + (sl & 1) * 4 : TN - 1;
        okS[sl] = L < TNN && i < TN && (sl < 4 ? true : (TN == 9 && tq < 2));
        nodeS[sl] = okS[sl] ? tc_node<N>(a, L, i) : 0;
#pragma unroll
        for (int i3 = 0; i3 < 3; i3++) {
          double m = 0.;
          if (okS[sl] && ((row >> i3) & 1))
            m = cs < 0 ? sScale[a]
                       : __ldg(P.metricp + (((size_t)cs * 3 + a) * 3 + i3) * TN * TNN + i * TNN + L);
          m3[i3][sl] = m;
        }
      }
      double rp[5] = {0., 0., 0., 0., 0.};
#pragma unroll 1
      for (int f = 0; f < 4; f++) {  // pi, then c_x, c_y, c_z
        if (f > 0 && !((row >> (f - 1)) & 1)) continue;
        double dv[5];
        tc_derivs<N>(gB, rowbase + (uint32_t)(f * TNP) * 16u, pstep, chunk, lane, tq, sEmax[f],
                     fd0, fd1, fd8, dv);
        // chain rule: r_c_i += M[a][i] d_a pi, r_pi += sum_i M[a][i] d_a c_i
#pragma unroll
        for (int sl = 0; sl < 5; sl++) {
          if (!okS[sl]) continue;
          if (f == 0) {
#pragma unroll
            for (int i3 = 0; i3 < 3; i3++) {
              if (!((row >> i3) & 1)) continue;
              double *r = sR + (1 + i3) * TNP + nodeS[sl];
              *r = fma(m3[i3][sl], dv[sl], *r);
            }
          } else {
            const double m = f == 1 ? m3[0][sl] : (f == 2 ? m3[1][sl] : m3[2][sl]);
            rp[sl] = fma(m, dv[sl], rp[sl]);
          }
        }
      }
#pragma unroll
      for (int sl = 0; sl < 5; sl++)
        if (okS[sl]) sR[nodeS[sl]] += rp[sl];
    }
    if (S::LAST && warp == TTILES % NWARP && lane < TN) {
      // the line left over (l0 = l1 = n - 1): output i of lane i as an FP64
      // dot product with D
      const int i = lane, L = TNN - 1, node = tc_node<N>(a, L, i);
      double d[4] = {0., 0., 0., 0.};
#pragma unroll
      for (int f = 0; f < 4; f++) {
        if (f > 0 && !((row >> (f - 1)) & 1)) continue;
#pragma unroll
        for (int p = 0; p < TN; p++)
          d[f] = fma(__ldg(gD + i * TN + p), __ldg(Wg + f * TNP + tc_node<N>(a, L, p)), d[f]);
      }
      double rpl = 0.;
#pragma unroll
      for (int i3 = 0; i3 < 3; i3++) {
        if (!((row >> i3) & 1)) continue;
        const double m = cs < 0 ? sScale[a]
                                : __ldg(P.metricp + (((size_t)cs * 3 + a) * 3 + i3) * TN * TNN +
                                        i * TNN + L);
        double *r = sR + (1 + i3) * TNP + node;
        *r = fma(m, d[0], *r);
        rpl = fma(m, d[1 + i3], rpl);
      }
      sR[node] += rpl;
    }
    __syncthreads();
  }
  // interior states of the faces and r_phi = pi come from w in global memory
  tc_epilogue<N, NT>(P, Wg, sR, e);
}

// Transposed stage (vector-Jacobian product, wbar = L^T rbar; the FP64
// form and the face terms are vjp_kernel's in stage_eo.cu): per direction a
// the fields y_pi = sum_i M[a][i] rbar_c_i and y_c_i = M[a][i] rbar_pi are
// formed in FP64 at every node, split into digits on their own grids, and
// D^T applied along a on the tensor cores adds into pibar, cbar_i.
template <int N, int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB) tcvjp_kernel(StageParams P) {
  using S = TcShape<N>;
  constexpr int TN = N, TNP = S::NP, TNN = S::NN, TTILES = S::TILES;
  constexpr int NWARP = NT / 32;
  extern __shared__ __align__(16) unsigned char tsm[];
  double *sR = reinterpret_cast<double *>(tsm);           // [4][NP]: pibar, cbar
  uint4 *sDig = reinterpret_cast<uint4 *>(sR + 4 * TNP);  // [4][NP] digits of y
  __shared__ int sCs[1];
  __shared__ int sMask;
  __shared__ int sEmax[3][4];
  __shared__ double sScale[3];
  __shared__ double sG[1][3];

  const int e = blockIdx.x;
  if (e >= P.nelem) return;
  const int tid = threadIdx.x;
  const double *Wg = P.win + (size_t)e * NF * TNP;  // rbar of this element
  if (tid == 0) {
    const int cs = P.cslot[e];
    if (cs >= 0) {
      tc_prefetch_l2(P.metric + (size_t)cs * 9 * TNP, sizeof(double) * 9 * TNP);
      tc_prefetch_l2(P.fac + (size_t)cs * 6 * TNN * 4, sizeof(double) * 6 * TNN * 4);
    }
    sCs[0] = cs;
    sMask = cs >= 0 ? P.cmask[cs] : (1 | (1 << 4) | (1 << 8));
    for (int d = 0; d < 3; d++) sScale[d] = P.scale[e * 3 + d];
    for (int d = 0; d < 3; d++) sG[0][d] = P.gcart[e * 3 + d];
  }
  if (tid < 12) sEmax[tid / 4][tid % 4] = 0;
  for (int q = tid; q < 4 * TNP; q += NT) sR[q] = 0.;
  __syncthreads();
  const int warp = tid >> 5, lane = tid & 31, g = lane >> 2, tq = lane & 3;
  const int cs = sCs[0], mask = sMask;
  const uint32_t digbase = (uint32_t)__cvta_generic_to_shared(sDig);
  const int fd0 = cTcRowExpT[N - 7][tq], fd1 = cTcRowExpT[N - 7][min(tq + 4, 8)];
  const int fd8 = cTcRowExpT[N - 7][8];
  const uint4 *gB = &gTcBT[N - 7][0][0][0];
  const double *gD = gTcDT[N - 7];
  const double *Mg = cs >= 0 ? P.metric + (size_t)cs * 9 * TNP : nullptr;  // [a*3+i][node]

#pragma unroll 1
  for (int a = 0; a < 3; a++) {
    const int row = (mask >> (3 * a)) & 7;
    // y at every node, in FP64 (one thread takes all four fields of its
    // nodes: rbar and the metric row read once), and each field's largest
    // exponent
    {
      constexpr int NNODE = (TNP + NT - 1) / NT;
      double y[4][NNODE];
      int em[4] = {0, 0, 0, 0};
#pragma unroll
      for (int k = 0; k < NNODE; k++) {
        const int node = tid + k * NT;
        double rp = 0., rc[3] = {0., 0., 0.}, m[3] = {0., 0., 0.};
        if (node < TNP) {
          rp = __ldg(Wg + node);
#pragma unroll
          for (int i3 = 0; i3 < 3; i3++)
            if ((row >> i3) & 1) {
              rc[i3] = __ldg(Wg + (1 + i3) * TNP + node);
              m[i3] = Mg ? __ldg(Mg + (a * 3 + i3) * TNP + node) : sScale[a];
            }
        }
        double y0 = 0.;
#pragma unroll
        for (int i3 = 0; i3 < 3; i3++) {
          y0 = fma(m[i3], rc[i3], y0);
          y[1 + i3][k] = m[i3] * rp;
        }
        y[0][k] = y0;
#pragma unroll
        for (int f = 0; f < 4; f++)
          em[f] = max(em[f], (int)((unsigned long long)__double_as_longlong(y[f][k]) >> 52) & 0x7FF);
      }
#pragma unroll
      for (int j = 0; j < 4; j++) {
        const unsigned mx = __reduce_max_sync(0xffffffffu, (unsigned)em[j]);
        if (lane == 0) atomicMax(&sEmax[a][j], (int)mx);
      }
      __syncthreads();
#pragma unroll
      for (int k = 0; k < NNODE; k++) {
        const int node = tid + k * NT;
        if (node < TNP)
#pragma unroll
          for (int f = 0; f < 4; f++) sDig[f * TNP + node] = tc_digits(y[f][k], sEmax[a][f]);
      }
      __syncthreads();
    }
#pragma unroll 1
    for (int tile = warp; tile < TTILES; tile += NWARP) {
      const int Lr = min(tile * 16 + (lane & 15), TNN - 1), chunk = lane >> 4;
      const int ps = a == 0 ? 1 : (a == 1 ? TN : TNN);
      const int nb = a == 0 ? TN * Lr : (a == 1 ? (Lr % TN) + TNN * (Lr / TN) : Lr);
      const uint32_t rowbase = digbase + (uint32_t)nb * 16u, pstep = (uint32_t)ps * 16u;
      int nodeS[5];
      bool okS[5];
#pragma unroll
      for (int sl = 0; sl < 5; sl++) {
        const int L = tile * 16 + g + (sl < 4 ? (sl >> 1) * 8 : tq * 8);
        const int i = sl < 4 ? tq + (sl & 1) * 4 : TN - 1;
        okS[sl] = L < TNN && i < TN && (sl < 4 ? true : (TN == 9 && tq < 2));
        nodeS[sl] = okS[sl] ? tc_node<N>(a, L, i) : 0;
      }
#pragma unroll 1
      for (int f = 0; f < 4; f++) {
        if (f == 0 ? row == 0 : !((row >> (f - 1)) & 1)) continue;
        double dv[5];
        tc_derivs<N>(gB, rowbase + (uint32_t)(f * TNP) * 16u, pstep, chunk, lane, tq,
                     sEmax[a][f], fd0, fd1, fd8, dv);
#pragma unroll
        for (int sl = 0; sl < 5; sl++)
          if (okS[sl]) sR[f * TNP + nodeS[sl]] += dv[sl];
      }
    }
    if (S::LAST && warp == TTILES % NWARP && lane < TN) {
      // the line left over: output i of lane i, FP64, y formed again
      const int i = lane, L = TNN - 1;
      double d[4] = {0., 0., 0., 0.};
#pragma unroll 1
      for (int p = 0; p < TN; p++) {
        const int nd = tc_node<N>(a, L, p);
        const double dt = __ldg(gD + i * TN + p), rp = __ldg(Wg + nd);
        double y0 = 0.;
#pragma unroll
        for (int i3 = 0; i3 < 3; i3++)
          if ((row >> i3) & 1) {
            const double m = Mg ? __ldg(Mg + (a * 3 + i3) * TNP + nd) : sScale[a];
            y0 = fma(m, __ldg(Wg + (1 + i3) * TNP + nd), y0);
            d[1 + i3] = fma(dt, m * rp, d[1 + i3]);
          }
        d[0] = fma(dt, y0, d[0]);
      }
      const int node = tc_node<N>(a, L, i);
#pragma unroll
      for (int f = 0; f < 4; f++) sR[f * TNP + node] += d[f];
    }
    __syncthreads();
  }
  vjp_faces_epilogue<N, 1, NT>(P, Wg, sR, sCs, sG, e);
}

template <int N, int NT, int MINB>
cudaError_t launch_tcvjp(const StageParams &P, cudaStream_t st) {
  constexpr size_t smem = TcShape<N>::SMEM;
  if (P.nelem <= 0) {
    cudaError_t e = cudaFuncSetAttribute(tcvjp_kernel<N, NT, MINB>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(tcvjp_kernel<N, NT, MINB>,
                                cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  }
  tcvjp_kernel<N, NT, MINB><<<P.nelem, NT, smem, st>>>(P);
  return cudaGetLastError();
}

template <int N, int NT, int MINB>
cudaError_t launch_tc(const StageParams &P, cudaStream_t st) {
  constexpr size_t smem = TcShape<N>::SMEM;
  if (P.nelem <= 0) {
    cudaError_t e = cudaFuncSetAttribute(tc_kernel<N, NT, MINB>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(tc_kernel<N, NT, MINB>,
                                cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  }
  const int ne = P.ecount > 0 ? P.ecount : P.nelem;
  tc_kernel<N, NT, MINB><<<ne, NT, smem, st>>>(P);
  return cudaGetLastError();
}

}  // namespace

int tc_variants(int n, Variant *out, int cap) {
  int k = 0;
  if (n == 9) {
    // three CTAs of 192 threads (96 registers: 5 warps of a sub-partition's
    // 16 K registers) or two of 256 per SM; three of 160 threads without
    // spills (128 registers) ran slower (3.51 vs 3.14 ms per stage)
    if (k < cap) out[k++] = Variant{"tc", 1, 192, launch_tc<9, 192, 3>};
    if (k < cap) out[k++] = Variant{"tc", 1, 256, launch_tc<9, 256, 2>};
  } else if (n == 8) {  // 4 tiles of 16 lines: one warp each
    if (k < cap) out[k++] = Variant{"tc", 1, 128, launch_tc<8, 128, 4>};
    if (k < cap) out[k++] = Variant{"tc", 1, 256, launch_tc<8, 256, 2>};
  } else if (n == 7) {  // 3 tiles and the line left over
    if (k < cap) out[k++] = Variant{"tc", 1, 128, launch_tc<7, 128, 4>};
    if (k < cap) out[k++] = Variant{"tc", 1, 256, launch_tc<7, 256, 2>};
  }
  return k;
}

int tcvjp_variants(int n, Variant *out, int cap) {
  if (cap < 1) return 0;
  if (n == 9) { out[0] = Variant{"tcvjp", 1, 192, launch_tcvjp<9, 192, 3>}; return 1; }
  if (n == 8) { out[0] = Variant{"tcvjp", 1, 128, launch_tcvjp<8, 128, 4>}; return 1; }
  if (n == 7) { out[0] = Variant{"tcvjp", 1, 128, launch_tcvjp<7, 128, 4>}; return 1; }
  return 0;
}

cudaError_t tc_upload(int n, const double *D) { return tc_upload_tables(n, D, true); }

}  // namespace nmgk
