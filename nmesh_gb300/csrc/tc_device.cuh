// tc_device.cuh -- device side of the tensor-core line derivatives (exact
// integer digit products on the FP16 tensor cores; the method is described
// in stage_tc.cu): the per-order shape, this translation unit's copies of
// the digit matrices (B fragments, row exponents, the matrix itself) of D
// and D^T, the digit split of FP64 values, the MMA loop over a 16-line tile
// and the recombination into FP64.  Every .cu file that includes it holds
// its own copies of the tables and fills them with tc_upload_tables().
#pragma once
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "tc_build.h"

namespace nmgk {
namespace {

constexpr int TNTILE = 8;        // n-tiles of 8 columns (9 outputs x 7 groups <= 64)
constexpr int TKSMAX = 5;        // k-steps of 16 at n = 9: 10 points x 8 digit slots
constexpr unsigned kMagic = 0x4B400000u;  // bit pattern of 1.5 * 2^23

// per order n (7, 8, 9): nodes, k-steps (points padded to an even count),
// full 16-line tiles per direction and whether one line is left over
template <int N>
struct TcShape {
  static constexpr int NP = N * N * N, NN = N * N;
  static constexpr int KS = (N + 1) / 2;
  static constexpr int TILES = NN / 16;
  static constexpr bool LAST = NN % 16 == 1;
  static_assert(NN % 16 == 0 || NN % 16 == 1, "lines per direction: 16 k or 16 k + 1");
  static constexpr size_t SMEM = sizeof(double) * 4 * NP + sizeof(uint4) * 4 * NP;
};

// B fragments per order, k-step, pair of n-tiles and lane: {b01, b23} of
// n-tile 2q, {b01, b23} of n-tile 2q+1 (mma.m16n8k16 B layout)
__device__ uint4 gTcB[3][TKSMAX][TNTILE / 2][32];
__constant__ int cTcRowExp[3][9];  // FD_i: biased exponent of max_p |D_ip|
__device__ double gTcD[3][81];     // D itself, for the line left over in a pass
// the same for D^T (the transposed, vector-Jacobian stage)
__device__ uint4 gTcBT[3][TKSMAX][TNTILE / 2][32];
__constant__ int cTcRowExpT[3][9];
__device__ double gTcDT[3][81];

__device__ __forceinline__ void mma16816(float *d, const uint32_t *a, uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ void ldsm_x4(uint32_t *r, uint32_t addr) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(addr));
}

// one bulk prefetch into L2 of the 16-byte-aligned part of [p, p + bytes)
// (the bulk copy wants a 16-byte-aligned start and a multiple of 16 bytes;
// trimming keeps it inside the range)
__device__ __forceinline__ void tc_prefetch_l2(const void *p, unsigned bytes) {
  const unsigned long long a = (unsigned long long)p;
  const unsigned long long lo = (a + 15ull) & ~15ull, hi = (a + bytes) & ~15ull;
  if (hi > lo)
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(lo),
                 "r"((unsigned)(hi - lo))
                 : "memory");
}

// 7 signed 8-bit digits of v on the grid of exponent Emax, as fp16 pairs
__device__ __forceinline__ uint4 tc_digits(double v, int emax) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  const int e = (int)(b >> 52) & 0x7FF;
  const unsigned long long m = e ? ((b & 0xFFFFFFFFFFFFFull) | (1ull << 52)) : 0ull;
  const int d = emax - e;  // >= 0
  const unsigned long long X = d < 64 ? (m << 11) >> d : 0ull;
  const unsigned hi = (unsigned)(X >> 32), lo = (unsigned)X;
  // 0x64dd = fp16 of 1024 + dd (exact); subtracting 1024 leaves the digit
  uint32_t h[4];
  h[0] = __byte_perm(hi, 0x64u, 0x4243);
  h[1] = __byte_perm(hi, 0x64u, 0x4041);
  h[2] = __byte_perm(lo, 0x64u, 0x4243);
  h[3] = __byte_perm(lo, 0x64u, 0x4541);  // digit 6, slot 7 = 1024 -> 0
  const bool neg = (b >> 63) != 0;
  const __half2 s2 = neg ? __floats2half2_rn(-1.f, -1.f) : __floats2half2_rn(1.f, 1.f);
  const __half2 o2 = neg ? __floats2half2_rn(1024.f, 1024.f) : __floats2half2_rn(-1024.f, -1024.f);
#pragma unroll
  for (int k = 0; k < 4; k++) {
    __half2 x = *reinterpret_cast<__half2 *>(&h[k]);
    x = __hfma2(x, s2, o2);
    h[k] = *reinterpret_cast<uint32_t *>(&x);
  }
  return make_uint4(h[0], h[1], h[2], h[3]);
}

// T 2^delta as FP64: T converted with one rounding to nearest, then its
// exponent field raised by delta (an integer add); a result outside the
// normal range flushes to zero or saturates to infinity
__device__ __forceinline__ double tc_to_double(long long T, int delta) {
  const double d = __ll2double_rn(T);
  const int hi = __double2hiint(d), ex = (hi >> 20) & 0x7FF, ne = ex + delta;
  if (ex != 0 && ne > 0 && ne < 2047) return __hiloint2double(hi + (delta << 20), __double2loint(d));
  if (ex == 0 || ne <= 0) return copysign(0., d);
  return copysign(__longlong_as_double(0x7FF0000000000000ll), d);
}

// node of point p of line L (L = l0 + n l1) along direction a
template <int N>
__device__ __forceinline__ int tc_node(int a, int L, int p) {
  return a == 0 ? p + N * L : (a == 1 ? (L % N) + N * p + N * N * (L / N) : L + N * N * p);
}

// derivatives along a of field f at this lane's owned output slots (see
// the kernel): the MMAs over the tile's 16 lines, then the digit groups
// combined into FP64 values.  Groups are paired in 32 bits first:
// p_k = acc_2k 2^8 + acc_2k+1 (|p_k| < 2^31), T = p_0 2^32 + p_1 2^16 + p_2 +
// floor(acc_6 / 2^8).
__device__ __forceinline__ int tc_pair(float hi, float lo) {
  return (int)(__float_as_uint(hi) * 256u + __float_as_uint(lo) - 257u * kMagic);
}

template <int N>
__device__ __forceinline__ void tc_derivs(const uint4 *__restrict__ gB, uint32_t rowaddr,
                                          uint32_t pstep, int chunk, int lane, int tq, int emax,
                                          int fd0, int fd1, int fd8, double *dv) {
  float acc[TNTILE][4];
#pragma unroll
  for (int i = 0; i < TNTILE; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) acc[i][j] = 12582912.f;
#pragma unroll 1
  for (int kk = 0; kk < TcShape<N>::KS; kk++) {
    const int p = min(2 * kk + chunk, N - 1);  // odd n: the padding point repeats the last
    uint32_t af[4];
    ldsm_x4(af, rowaddr + (uint32_t)p * pstep);
#pragma unroll
    for (int q = 0; q < TNTILE / 2; q++) {
      const uint4 bq = __ldg(gB + (kk * (TNTILE / 2) + q) * 32 + lane);
      mma16816(acc[2 * q], af, bq.x, bq.y);
      mma16816(acc[2 * q + 1], af, bq.z, bq.w);
    }
  }
  const bool bad = emax >= 2047;  // inf or NaN in the field
  // owned outputs t and t+4 of rows g (registers 0, 1) and g+8 (2, 3): slots
  // sb..sb+6 hold groups 0..6
#pragma unroll
  for (int o = 0; o < 4; o++) {
    const int rr = (o >> 1) * 2, sb = (o & 1) * 7;
#define TC_A(w) acc[(sb + (w)) >> 1][rr + ((sb + (w)) & 1)]
    const int p0 = tc_pair(TC_A(0), TC_A(1)), p1 = tc_pair(TC_A(2), TC_A(3));
    const int p2 = tc_pair(TC_A(4), TC_A(5));
    const int a6 = (int)(__float_as_uint(TC_A(6)) - kMagic);
#undef TC_A
    const long long T = ((long long)p0 << 32) + ((long long)p1 << 16) + (long long)p2 +
                        (long long)(a6 >> 8);
    dv[o] = bad ? __longlong_as_double(0x7FF8000000000000ll)
                : tc_to_double(T, emax + ((o & 1) ? fd1 : fd0) - 2100);
  }
  // output 8 (n = 9): groups 2t, 2t+1 here (t = 3: group 6 and an empty
  // column), summed over the quad
  if constexpr (N == 9) {
    long long P8[2];
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const int pp = tc_pair(acc[7][2 * h], acc[7][2 * h + 1]);
      P8[h] = tq < 3 ? ((long long)pp << (32 - 16 * tq)) : (long long)(pp >> 16);
      P8[h] += __shfl_xor_sync(0xffffffffu, P8[h], 1);
      P8[h] += __shfl_xor_sync(0xffffffffu, P8[h], 2);
    }
    dv[4] = bad ? __longlong_as_double(0x7FF8000000000000ll)
                : tc_to_double(tq == 0 ? P8[0] : P8[1], emax + fd8 - 2100);
  } else {
    dv[4] = 0.;
  }
}

// this translation unit's tables for the n x n matrix D (and D^T when
// transposed is set) of order n = 7, 8, 9
inline cudaError_t tc_upload_tables(int n, const double *D, bool transposed) {
  if (n < 7 || n > 9) return cudaSuccess;
  const size_t slot = (size_t)(n - 7);
  std::vector<tc::TcMatrix> Mv(1);  // per call: contexts may be created from several threads
  tc::TcMatrix &M = Mv[0];
  double Dt[81];
  for (int pass = 0; pass < (transposed ? 2 : 1); pass++) {
    if (pass == 1)
      for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) Dt[i * n + j] = D[j * n + i];
    tc::tc_build(n, pass ? Dt : D, M);
    cudaError_t err =
        cudaMemcpyToSymbol(pass ? gTcBT : gTcB, M.F, sizeof(M.F), sizeof(M.F) * slot);
    if (err != cudaSuccess) return err;
    if ((err = cudaMemcpyToSymbol(pass ? gTcDT : gTcD, M.X, sizeof(M.X), sizeof(M.X) * slot)) !=
        cudaSuccess)
      return err;
    if ((err = cudaMemcpyToSymbol(pass ? cTcRowExpT : cTcRowExp, M.fd, sizeof(M.fd),
                                  sizeof(M.fd) * slot)) != cudaSuccess)
      return err;
  }
  return cudaSuccess;
}

static_assert(sizeof(tc::Frag) == sizeof(uint4), "fragment layout");
static_assert(sizeof(tc::TcMatrix::F) == sizeof(gTcB[0]), "fragment array of one order");

}  // namespace
}  // namespace nmgk
