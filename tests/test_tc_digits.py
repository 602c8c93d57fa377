"""The arithmetic of the tensor-core stage kernel (nmesh_gb300/csrc/stage_tc.cu),
restated in Python integers and checked against exact rational arithmetic on
the CPU, for the orders it is compiled for (7, 8, 9 points per line): the
8-bit digit split of the values and of D, the digit-group sums
the FP16 tensor cores form (they must stay below 2^22, where FP32 holds every
partial sum exactly, accumulators starting at 1.5 2^23), the 64-bit
recombination and the conversion to FP64.  The bound checked is the one
stated for the kernel: per output, a few units of 2^-53 of
max|u| x sum_p |D_ip| (the size of the FP64 dot product's own rounding
bound).  The GPU tests (tests/test_gpu_tc.py) check the kernel itself."""
import struct
from fractions import Fraction

import numpy as np
import pytest

TG = 7  # digit groups kept
ORDERS = [7, 8, 9]  # points per line with a tensor-core stage kernel


def _bits(v):
    return struct.unpack("<Q", struct.pack("<d", float(v)))[0]


def _from_bits(b):
    return struct.unpack("<d", struct.pack("<Q", b & (2 ** 64 - 1)))[0]


def _exp(v):
    return (_bits(v) >> 52) & 0x7FF


def _fixed(v, emax):
    """X = (m << 11) >> (emax - e) as in tc_digits (m the 53-bit significand)"""
    b = _bits(v)
    e = (b >> 52) & 0x7FF
    m = ((b & ((1 << 52) - 1)) | (1 << 52)) if e else 0
    d = emax - e
    return (((m << 11) & (2 ** 64 - 1)) >> d) if d < 64 else 0


def u_digits(v, emax):
    """7 signed digits of v (byte 7 - s of X), slot 7 zero"""
    X = _fixed(v, emax)
    sgn = -1 if _bits(v) >> 63 else 1
    return [sgn * ((X >> (8 * (7 - s))) & 0xFF) for s in range(7)] + [0]


def d_digits(x, fd):
    """7 digits of |D_ip| on the row grid fd, rounded at the dropped byte"""
    Y = (_fixed(x, fd) + 0x80) >> 8
    return [(Y >> (8 * (6 - t))) & 0xFF for t in range(7)]


def column(col):
    """(output i, group w) of B column col = 8 nt + 2 t + j (slot 2 nt + j of
    quad thread t), as tc_upload lays them out"""
    nt, c8 = col // 8, col % 8
    t, j = c8 // 2, c8 % 2
    sl = 2 * nt + j
    if sl < 7:
        return t, sl
    if sl < 14:
        return t + 4, sl - 7
    return 8, 2 * t + (sl - 14)


def b_matrix(D):
    N = D.shape[0]
    ks = (N + 1) // 2
    fd = [max(_exp(D[i, p]) for p in range(N)) for i in range(N)]
    B = np.zeros((16 * ks, 64), dtype=np.int64)
    for col in range(64):
        i, w = column(col)
        if i >= N or w >= TG:
            continue
        for p in range(N):
            dg = d_digits(D[i, p], fd[i])
            sg = -1 if D[i, p] < 0 else 1
            for s in range(TG):
                t = w - s
                if 0 <= t < TG:
                    B[8 * p + s, col] = sg * dg[t]
    return B, fd


def to_double(T, delta):
    """T 2^delta, rounded to nearest (cvt.rn.f64.s64 + exponent add)"""
    if T == 0:
        return 0.0
    d = float(T)  # Python rounds int -> float to nearest even
    return float(np.ldexp(d, delta))


def line_derivative(u, D, B, fd):
    N = D.shape[0]
    ks = (N + 1) // 2
    emax = max(_exp(v) for v in u)
    rows = [u_digits(v, emax) for v in u] + [u_digits(u[N - 1], emax)] * (2 * ks - N)
    C = np.array(rows, dtype=np.int64).reshape(-1) @ B
    assert np.abs(C).max() < 2 ** 22
    out = np.zeros(N)
    for t in range(4):
        for o in range(2):
            i = t + 4 * o
            if i >= N:
                continue
            acc = []
            for w in range(TG):
                sl = 7 * o + w
                acc.append(int(C[8 * (sl >> 1) + 2 * t + (sl & 1)]))
            p = [acc[2 * k] * 256 + acc[2 * k + 1] for k in range(3)]
            assert all(abs(x) < 2 ** 31 for x in p)
            T = (p[0] << 32) + (p[1] << 16) + p[2] + (acc[6] >> 8)
            assert abs(T) < 2 ** 63
            out[i] = to_double(T, emax + fd[i] - 2100)
    if N == 9:
        T8 = 0
        for t in range(4):
            a0, a1 = int(C[56 + 2 * t]), int(C[57 + 2 * t])
            pp = a0 * 256 + a1
            T8 += (pp << (32 - 16 * t)) if t < 3 else (pp >> 16)
        out[8] = to_double(T8, emax + fd[8] - 2100)
    return out


@pytest.fixture(scope="module", params=ORDERS)
def dmat(request):
    from oracle import nmo
    D = nmo.diffmat(request.param)
    B, fd = b_matrix(D)
    return D, B, fd


def test_columns_hold_every_output_group_once():
    seen = {}
    for col in range(64):
        i, w = column(col)
        if i < 9 and w < TG:
            assert (i, w) not in seen
            seen[(i, w)] = col
    assert len(seen) == 9 * TG


def test_digit_products_are_exact_and_within_fp64_rounding(dmat):
    D, B, fd = dmat
    N = D.shape[0]
    assert np.abs(B).max() <= 255
    rng = np.random.default_rng(2024 + N)
    worst = 0.0
    for trial in range(120):
        scale = 10.0 ** rng.uniform(-250, 250)
        u = rng.standard_normal(N) * scale
        if trial % 3 == 0:
            u *= 10.0 ** rng.uniform(-6, 6, N)
        if trial % 5 == 0:
            u[rng.integers(N)] = 0.0
        got = line_derivative(u, D, B, fd)
        bound = np.abs(u).max() * np.abs(D).sum(1)
        for i in range(N):
            exact = sum(Fraction(float(D[i, p])) * Fraction(float(u[p])) for p in range(N))
            worst = max(worst, abs(float(Fraction(got[i]) - exact)) / bound[i])
    assert worst <= 2.0 * 2.0 ** -53, worst / 2.0 ** -53


def test_zero_and_constant_lines(dmat):
    D, B, fd = dmat
    N = D.shape[0]
    assert np.array_equal(line_derivative(np.zeros(N), D, B, fd), np.zeros(N))
    # the derivative of a constant is zero up to the rounding bound
    c = np.full(N, 3.0)
    assert np.abs(line_derivative(c, D, B, fd)).max() <= 2.0 * 2.0 ** -53 * 3 * np.abs(D).sum(1).max()


HARNESS = r"""
#include <cstdio>
#include <cstring>
#include "tc_build.h"
int main() {
  int n;
  if (scanf("%d", &n) != 1) return 1;
  double X[81];
  for (int i = 0; i < n * n; i++) {
    unsigned long long b;
    if (scanf("%llx", &b) != 1) return 1;
    std::memcpy(&X[i], &b, 8);
  }
  static nmgk::tc::TcMatrix M;
  nmgk::tc::tc_build(n, X, M);
  for (int i = 0; i < 9; i++) printf("%d\n", M.fd[i]);
  for (int kk = 0; kk < nmgk::tc::kKStepsMax; kk++)
    for (int q = 0; q < nmgk::tc::kNTiles / 2; q++)
      for (int l = 0; l < 32; l++) {
        const nmgk::tc::Frag &f = M.F[kk][q][l];
        printf("%08x %08x %08x %08x\n", f.x, f.y, f.z, f.w);
      }
  return 0;
}
"""


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    import os
    import shutil
    import subprocess
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no C++ compiler")
    csrc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                        "nmesh_gb300", "csrc")
    d = tmp_path_factory.mktemp("tcb")
    src, exe = d / "h.cpp", d / "h"
    src.write_text(HARNESS)
    subprocess.run([cxx, "-O1", "-std=c++17", "-I", csrc, str(src), "-o", str(exe)], check=True)
    return str(exe)


def test_host_builder_matches_restatement(harness, dmat):
    """The library's host builder (nmesh_gb300/csrc/tc_build.h) gives, for D
    and D^T, the row exponents and the B fragments of the digit matrix
    restated here: FP16 bit patterns of the digits, laid out as
    mma.m16n8k16 wants its B operand (lane (g, t) holds rows 2t, 2t+1 and
    2t+8, 2t+9 of column g of each 16 x 8 block)."""
    import subprocess
    D = dmat[0]
    N = D.shape[0]
    for X in (D, np.ascontiguousarray(D.T)):
        B, fd = b_matrix(X)
        inp = f"{N}\n" + " ".join(f"{_bits(v):016x}" for v in X.ravel()) + "\n"
        out = subprocess.run([harness], input=inp, capture_output=True, text=True,
                             check=True).stdout.split("\n")
        assert [int(v) for v in out[:N]] == fd
        frags = [[int(w, 16) for w in line.split()] for line in out[9:] if line.strip()]
        h = np.zeros((80, 64), dtype=np.uint16)
        h[:B.shape[0]] = B.astype(np.float16).view(np.uint16)
        ks = (N + 1) // 2
        for kk in range(5):
            for q in range(4):
                for lane in range(32):
                    g, t = lane >> 2, lane & 3
                    want = []
                    for half in range(2):
                        col = 8 * (2 * q + half) + g
                        if kk < ks:
                            rows = [16 * kk + 2 * t, 16 * kk + 2 * t + 1,
                                    16 * kk + 2 * t + 8, 16 * kk + 2 * t + 9]
                            b = [int(h[r, col]) for r in rows]
                        else:
                            b = [0, 0, 0, 0]
                        want += [b[0] | (b[1] << 16), b[2] | (b[3] << 16)]
                    assert frags[(kk * 4 + q) * 32 + lane] == want, (kk, q, lane)


def _tc_node(N, a, L, p):
    """node of point p on line L along direction a (tc_node in tc_device.cuh)"""
    nn = N * N
    return p + N * L if a == 0 else ((L % N) + N * p + nn * (L // N) if a == 1 else L + nn * p)


@pytest.mark.parametrize("N", ORDERS)
def test_tile_slots_cover_every_node_once_and_rows_stay_aligned(N):
    """The work split of the tensor-core kernels (stage_tc.cu, and the GRHD
    DG kernel in grhd_evolve.cu), restated: per direction a, 16-line tiles
    whose lanes own outputs (g, t), (g, t+4), (g+8, t), (g+8, t+4) and, at
    n = 9, output 8 of row g or g+8, plus the line left over at odd n in
    FP64, write every node exactly once; and every ldmatrix row (16 bytes of
    digits, points clamped to n - 1) of the GRHD kernel's shared layout
    (digits of 5 fields first, then 15 n^3 doubles) lies inside the digit
    array on a 16-byte boundary."""
    NP, nn = N ** 3, N * N
    tiles, last = nn // 16, nn % 16 == 1
    ks = (N + 1) // 2
    for a in range(3):
        seen = np.zeros(NP, np.int64)
        for tile in range(tiles):
            for lane in range(32):
                g, tq = lane >> 2, lane & 3
                for sl in range(5):
                    L = tile * 16 + g + ((sl >> 1) * 8 if sl < 4 else tq * 8)
                    io = tq + (sl & 1) * 4 if sl < 4 else N - 1
                    ok = L < nn and io < N and (sl < 4 or (N == 9 and tq < 2))
                    if ok:
                        seen[_tc_node(N, a, L, io)] += 1
                # ldmatrix rows of this lane in the GRHD layout, field 4
                Lr, chunk = min(tile * 16 + (lane & 15), nn - 1), lane >> 4
                ps = 1 if a == 0 else (N if a == 1 else nn)
                nb = _tc_node(N, a, Lr, 0)
                for kk in range(ks):
                    p = min(2 * kk + chunk, N - 1)
                    addr = (4 * NP + nb + p * ps) * 16
                    assert addr % 16 == 0 and addr + 16 <= 5 * NP * 16
        if last:
            for io in range(N):
                seen[_tc_node(N, a, nn - 1, io)] += 1
        assert (seen == 1).all(), (a, np.nonzero(seen != 1)[0][:8])
