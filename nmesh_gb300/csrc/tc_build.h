// tc_build.h -- host-side digits of the matrices the tensor-core stage
// kernels multiply by (stage_tc.cu): for an n x n matrix X (row-major, rows =
// outputs; n = 7, 8, 9) the row exponents, and the mma.m16n8k16 B fragments
// of the digit matrix B[K = 8 p + s][column] that holds, in the column of
// output i and digit group w, the digit w - s of |X_ip| (with X_ip's sign) in
// row 8 p + s.  Plain C++ (no CUDA), so that a CPU test can build the same
// fragments and compare them with an independent restatement.
#pragma once
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <vector>

namespace nmgk {
namespace tc {

constexpr int kKStepsMax = 5;  // k-steps of 16 at n = 9 (10 points x 8 digit slots)
constexpr int kNTiles = 8;     // n-tiles of 8 columns
constexpr int kGroups = 7;     // digit groups kept

struct Frag {
  uint32_t x, y, z, w;  // {b01, b23} of n-tile 2q, {b01, b23} of n-tile 2q + 1
};

struct TcMatrix {
  Frag F[kKStepsMax][kNTiles / 2][32];  // [k-step][pair of n-tiles][lane]
  int fd[9];                            // biased exponent of max_p |X_ip|
  double X[81];                         // X itself
};

// 56-bit rounded fixed-point magnitude of x on the grid of exponent fd
// (the top 7 bytes of (m << 11) >> (fd - e), m the 53-bit significand,
// rounded at the dropped byte)
inline unsigned long long digits56(double x, int fd) {
  uint64_t b;
  std::memcpy(&b, &x, 8);
  const int e = (int)(b >> 52) & 0x7FF;
  if (!e) return 0;
  const uint64_t m = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
  const int d = fd - e;
  const uint64_t X = d < 64 ? (m << 11) >> d : 0;
  return (X + 0x80) >> 8;
}

// IEEE half of an integer, exact for |v| < 2048
inline uint16_t half_of_int(int v) {
  if (v == 0) return 0;
  const uint16_t s = v < 0 ? 0x8000 : 0;
  int a = v < 0 ? -v : v, ex = 0;
  while ((a >> ex) > 1) ex++;
  const int mant = (a << (10 - ex)) & 0x3FF;
  return (uint16_t)(s | ((ex + 15) << 10) | mant);
}

// column of B <-> (output, group): column 8 nt + 2 t + j is slot 2 nt + j of
// quad thread t; slots 0..6 hold groups 0..6 of output t, 7..13 those of
// output t + 4, 14..15 groups 2t, 2t + 1 of output 8
inline void column_slot(int col, int &i, int &w) {
  const int nt = col / 8, c8 = col % 8, t = c8 / 2, j = c8 % 2, sl = 2 * nt + j;
  if (sl < 7) { i = t; w = sl; }
  else if (sl < 14) { i = t + 4; w = sl - 7; }
  else { i = 8; w = 2 * t + (sl - 14); }
}

inline void tc_build(int n, const double *X, TcMatrix &out) {
  const int ks = (n + 1) / 2;
  unsigned long long Y[9][9] = {};
  int sg[9][9] = {};
  std::memset(&out, 0, sizeof(out));
  for (int i = 0; i < n; i++) {
    int mx = 0;
    for (int p = 0; p < n; p++) {
      uint64_t b;
      std::memcpy(&b, &X[i * n + p], 8);
      mx = std::max(mx, (int)(b >> 52) & 0x7FF);
    }
    out.fd[i] = mx;
    for (int p = 0; p < n; p++) {
      Y[i][p] = digits56(X[i * n + p], mx);
      sg[i][p] = X[i * n + p] < 0 ? -1 : 1;
    }
  }
  for (int q = 0; q < n * n; q++) out.X[q] = X[q];
  constexpr int NCOL = kNTiles * 8;
  std::vector<uint16_t> B(kKStepsMax * 16 * NCOL, 0);  // B[K][column]
  for (int col = 0; col < NCOL; col++) {
    int i, w;
    column_slot(col, i, w);
    if (i >= n || w >= kGroups) continue;
    for (int p = 0; p < n; p++)
      for (int s = 0; s < kGroups; s++) {
        const int tt = w - s;
        if (tt < 0 || tt >= kGroups) continue;
        const int dig = (int)((Y[i][p] >> (8 * (6 - tt))) & 0xFF);
        B[(8 * p + s) * NCOL + col] = half_of_int(sg[i][p] * dig);
      }
  }
  // fragment of lane (g, t) for (k-step kk, n-tile nt): B[16 kk + 2t (+1)]
  // and B[16 kk + 2t + 8 (+9)] of column 8 nt + g
  for (int kk = 0; kk < ks; kk++)
    for (int q = 0; q < kNTiles / 2; q++)
      for (int lane = 0; lane < 32; lane++) {
        const int g = lane >> 2, t = lane & 3;
        uint32_t r[4];
        for (int h = 0; h < 2; h++) {
          const int col = 8 * (2 * q + h) + g;
          const uint32_t b0 = B[(16 * kk + 2 * t) * NCOL + col];
          const uint32_t b1 = B[(16 * kk + 2 * t + 1) * NCOL + col];
          const uint32_t b2 = B[(16 * kk + 2 * t + 8) * NCOL + col];
          const uint32_t b3 = B[(16 * kk + 2 * t + 9) * NCOL + col];
          r[2 * h] = b0 | (b1 << 16);
          r[2 * h + 1] = b2 | (b3 << 16);
        }
        out.F[kk][q][lane] = Frag{r[0], r[1], r[2], r[3]};
      }
}

}  // namespace tc
}  // namespace nmgk
