// weno.cuh -- midpoint reconstructions of a pencil of equally spaced
// values, the reference's rec1d routines (src/main/dg/rec1d.c:16-227,
// 880-1030 WENO3 / WENOm3_2, 1186-1368 WENO5 / WENOm5_2, 1627-1796 WENO-Z /
// WENOmZ_2) with u_scale = 1.  Included inside a namespace of each
// translation unit that uses them; with NMG_FV_FAST defined the nonlinear
// weights are normalised with one division instead of one per weight.
#pragma once

__device__ __forceinline__ double weno3_p(const double *q, double o0, double o1, double l00,
                                          double l01, double l10, double l11) {
  // q[0..2] = u[im-1], u[im], u[im+1]  (rec1d_p_WENO3, u_scale = 1)
  const double d1 = q[1] - q[0], d2 = q[2] - q[1];
  const double b1 = d1 * d1 + 1e-6 * 1.0, b2 = d2 * d2 + 1e-6 * 1.0;
  const double u1 = l00 * q[0] + l01 * q[1], u2 = l10 * q[1] + l11 * q[2];
#ifdef NMG_FV_FAST
  const double w1 = o0 * (b2 * b2), w2 = o1 * (b1 * b1);
  return (w1 * u1 + w2 * u2) / (w1 + w2);
#else
  const double ob1 = o0 / (b1 * b1), ob2 = o1 / (b2 * b2);
  const double sum = ob1 + ob2;
  const double w1 = ob1 / sum, w2 = ob2 / sum;
  return w1 * u1 + w2 * u2;
#endif
}

__device__ __forceinline__ double weno3_m(const double *q, double o0, double o1, double l00,
                                          double l01, double l10, double l11) {
  // q[0..2] = u[im], u[im+1], u[im+2]  (rec1d_m_WENO3)
  const double d1 = q[1] - q[0], d2 = q[2] - q[1];
  const double b1 = d1 * d1 + 1e-6 * 1.0, b2 = d2 * d2 + 1e-6 * 1.0;
  const double u1 = l00 * q[0] + l01 * q[1], u2 = l10 * q[1] + l11 * q[2];
#ifdef NMG_FV_FAST
  const double w1 = o0 * (b2 * b2), w2 = o1 * (b1 * b1);
  return (w1 * u1 + w2 * u2) / (w1 + w2);
#else
  const double ob1 = o0 / (b1 * b1), ob2 = o1 / (b2 * b2);
  const double sum = ob1 + ob2;
  const double w1 = ob1 / sum, w2 = ob2 / sum;
  return w1 * u1 + w2 * u2;
#endif
}

#define NMG_C1312 (1.083333333333333333333333)

// q[0..4] = u[im-2..im+2]  (rec1d_p_WENO5_uniform)
__device__ __forceinline__ double weno5_p(const double *q) {
  const double oo6 = 1 / 6.;
  const double b01 = q[0] - 2. * q[1] + q[2], b02 = q[0] - 4. * q[1] + 3. * q[2];
  const double b11 = q[1] - 2. * q[2] + q[3], b12 = q[1] - q[3];
  const double b21 = q[2] - 2. * q[3] + q[4], b22 = 3. * q[2] - 4. * q[3] + q[4];
  const double b0 = NMG_C1312 * b01 * b01 + 0.25 * b02 * b02;
  const double b1 = NMG_C1312 * b11 * b11 + 0.25 * b12 * b12;
  const double b2 = NMG_C1312 * b21 * b21 + 0.25 * b22 * b22;
  const double e0 = b0 + 1e-40 * 1.0, e1 = b1 + 1e-40 * 1.0, e2 = b2 + 1e-40 * 1.0;
  const double u0 = (2. * oo6) * q[0] + (-7. * oo6) * q[1] + (11. * oo6) * q[2];
  const double u1 = (-oo6) * q[1] + (5. * oo6) * q[2] + (2. * oo6) * q[3];
  const double u2 = (2. * oo6) * q[2] + (5. * oo6) * q[3] + (-oo6) * q[4];
#ifdef NMG_FV_FAST
  const double a0 = e0 * e0, a1 = e1 * e1, a2 = e2 * e2;
  const double w0 = 1. * (a1 * a2), w1 = 6. * (a0 * a2), w2 = 3. * (a0 * a1);
  return (w0 * u0 + w1 * u1 + w2 * u2) / (w0 + w1 + w2);
#else
  const double o0 = 1. / (e0 * e0), o1 = 6. / (e1 * e1), o2 = 3. / (e2 * e2);
  const double oos = 1. / (o0 + o1 + o2);
  const double w0 = o0 * oos, w1 = o1 * oos, w2 = o2 * oos;
  return w0 * u0 + w1 * u1 + w2 * u2;
#endif
}

// q[0..4] = u[im-1..im+3]  (rec1d_m_WENO5_uniform)
__device__ __forceinline__ double weno5_m(const double *q) {
  const double oo6 = 1 / 6.;
  const double b21 = q[2] - 2. * q[3] + q[4], b22 = 3. * q[2] - 4. * q[3] + q[4];
  const double b11 = q[1] - 2. * q[2] + q[3], b12 = q[1] - q[3];
  const double b01 = q[0] - 2. * q[1] + q[2], b02 = q[0] - 4. * q[1] + 3. * q[2];
  const double b2 = NMG_C1312 * b21 * b21 + 0.25 * b22 * b22;
  const double b1 = NMG_C1312 * b11 * b11 + 0.25 * b12 * b12;
  const double b0 = NMG_C1312 * b01 * b01 + 0.25 * b02 * b02;
  const double e2 = b2 + 1e-40 * 1.0, e1 = b1 + 1e-40 * 1.0, e0 = b0 + 1e-40 * 1.0;
  const double u2 = (11. * oo6) * q[2] + (-7. * oo6) * q[3] + (2. * oo6) * q[4];
  const double u1 = (2. * oo6) * q[1] + (5. * oo6) * q[2] + (-oo6) * q[3];
  const double u0 = (-oo6) * q[0] + (5. * oo6) * q[1] + (2. * oo6) * q[2];
#ifdef NMG_FV_FAST
  const double a0 = e0 * e0, a1 = e1 * e1, a2 = e2 * e2;
  const double w2 = 1. * (a0 * a1), w1 = 6. * (a0 * a2), w0 = 3. * (a1 * a2);
  return (w0 * u0 + w1 * u1 + w2 * u2) / (w0 + w1 + w2);
#else
  const double o2 = 1. / (e2 * e2), o1 = 6. / (e1 * e1), o0 = 3. / (e0 * e0);
  const double oos = 1. / (o0 + o1 + o2);
  const double w2 = o2 * oos, w1 = o1 * oos, w0 = o0 * oos;
  return w0 * u0 + w1 * u1 + w2 * u2;
#endif
}

// q[0..4] = u[im-2..im+2]  (rec1d_p_WENOZ_uniform: the WENO5 stencils with
// the WENO-Z weights optw_k (1 + tau5 / (b_k + eps)), tau5 = |b0 - b2|)
__device__ __forceinline__ double wenoz_p(const double *q) {
  const double oo6 = 1 / 6.;
  const double b01 = q[0] - 2. * q[1] + q[2], b02 = q[0] - 4. * q[1] + 3. * q[2];
  const double b11 = q[1] - 2. * q[2] + q[3], b12 = q[1] - q[3];
  const double b21 = q[2] - 2. * q[3] + q[4], b22 = 3. * q[2] - 4. * q[3] + q[4];
  const double b0 = NMG_C1312 * b01 * b01 + 0.25 * b02 * b02;
  const double b1 = NMG_C1312 * b11 * b11 + 0.25 * b12 * b12;
  const double b2 = NMG_C1312 * b21 * b21 + 0.25 * b22 * b22;
  const double e0 = b0 + 1e-40 * 1.0, e1 = b1 + 1e-40 * 1.0, e2 = b2 + 1e-40 * 1.0;
  const double tau5 = fabs(b0 - b2);
  const double u0 = (2. * oo6) * q[0] + (-7. * oo6) * q[1] + (11. * oo6) * q[2];
  const double u1 = (-oo6) * q[1] + (5. * oo6) * q[2] + (2. * oo6) * q[3];
  const double u2 = (2. * oo6) * q[2] + (5. * oo6) * q[3] + (-oo6) * q[4];
#ifdef NMG_FV_FAST
  // weights times e0 e1 e2: one division
  const double w0 = 1. * ((e0 + tau5) * (e1 * e2)), w1 = 6. * ((e1 + tau5) * (e0 * e2)),
               w2 = 3. * ((e2 + tau5) * (e0 * e1));
  return (w0 * u0 + w1 * u1 + w2 * u2) / (w0 + w1 + w2);
#else
  const double o0 = 1. * (1. + tau5 / e0), o1 = 6. * (1. + tau5 / e1), o2 = 3. * (1. + tau5 / e2);
  const double oos = 1. / (o0 + o1 + o2);
  const double w0 = o0 * oos, w1 = o1 * oos, w2 = o2 * oos;
  return w0 * u0 + w1 * u1 + w2 * u2;
#endif
}

// q[0..4] = u[im-1..im+3]  (rec1d_m_WENOZ_uniform)
__device__ __forceinline__ double wenoz_m(const double *q) {
  const double oo6 = 1 / 6.;
  const double b21 = q[2] - 2. * q[3] + q[4], b22 = 3. * q[2] - 4. * q[3] + q[4];
  const double b11 = q[1] - 2. * q[2] + q[3], b12 = q[1] - q[3];
  const double b01 = q[0] - 2. * q[1] + q[2], b02 = q[0] - 4. * q[1] + 3. * q[2];
  const double b2 = NMG_C1312 * b21 * b21 + 0.25 * b22 * b22;
  const double b1 = NMG_C1312 * b11 * b11 + 0.25 * b12 * b12;
  const double b0 = NMG_C1312 * b01 * b01 + 0.25 * b02 * b02;
  const double e2 = b2 + 1e-40 * 1.0, e1 = b1 + 1e-40 * 1.0, e0 = b0 + 1e-40 * 1.0;
  const double tau5 = fabs(b0 - b2);
  const double u2 = (11. * oo6) * q[2] + (-7. * oo6) * q[3] + (2. * oo6) * q[4];
  const double u1 = (2. * oo6) * q[1] + (5. * oo6) * q[2] + (-oo6) * q[3];
  const double u0 = (-oo6) * q[0] + (5. * oo6) * q[1] + (2. * oo6) * q[2];
#ifdef NMG_FV_FAST
  const double w2 = 1. * ((e2 + tau5) * (e0 * e1)), w1 = 6. * ((e1 + tau5) * (e0 * e2)),
               w0 = 3. * ((e0 + tau5) * (e1 * e2));
  return (w0 * u0 + w1 * u1 + w2 * u2) / (w0 + w1 + w2);
#else
  const double o2 = 1. * (1. + tau5 / e2), o1 = 6. * (1. + tau5 / e1), o0 = 3. * (1. + tau5 / e0);
  const double oos = 1. / (o0 + o1 + o2);
  const double w2 = o2 * oos, w1 = o1 * oos, w0 = o0 * oos;
  return w0 * u0 + w1 * u1 + w2 * u2;
#endif
}

// Left (p) and right (m) states at midpoint im of a pencil of n values;
// v[j] = u[im - 2 + j] for the indices inside the pencil.
__device__ __forceinline__ double rec_p(int mode, int n, const double *v, int im, double r3) {
  if (mode == NMG_FV_REC_1) return v[2];
  if (mode == NMG_FV_REC_WENOM5_2 && im >= 2 && im <= n - 3) return weno5_p(v);
  if (mode == NMG_FV_REC_WENOMZ_2 && im >= 2 && im <= n - 3) return wenoz_p(v);
  if (im >= 1 && im <= n - 2) return weno3_p(v + 1, 1., r3, -0.5, 1.5, 0.5, 0.5);
  if (n < 3) return v[2];
  return 0.5 * v[2] + 0.5 * v[3];  // im == 0
}

__device__ __forceinline__ double rec_m(int mode, int n, const double *v, int im, double r3) {
  if (mode == NMG_FV_REC_1) return v[3];
  if (mode == NMG_FV_REC_WENOM5_2 && im >= 1 && im <= n - 4) return weno5_m(v + 1);
  if (mode == NMG_FV_REC_WENOMZ_2 && im >= 1 && im <= n - 4) return wenoz_m(v + 1);
  if (im >= 0 && im <= n - 3) return weno3_m(v + 2, r3, 1., 0.5, 0.5, 1.5, -0.5);
  if (n < 3) return v[3];
  return 0.5 * v[2] + 0.5 * v[3];  // im == n-2
}


// Both face values of cell c of a pencil of n values, v[j] = u[c - 2 + j]
// for the indices inside the pencil: *lft = the right state of midpoint c-1
// (rec_m there; c >= 1), *rgt = the left state of midpoint c (rec_p there;
// c <= n - 2).  The same expressions as rec_p / rec_m on the same five
// values, so the smoothness indicators and weight products of the cell are
// computed once for both faces.
__device__ __forceinline__ void rec_cell(int mode, int n, const double *v, int c, double r3,
                                         double *lft, double *rgt) {
  if (mode == NMG_FV_REC_1) {
    *lft = v[2];
    *rgt = v[2];
    return;
  }
  if (mode == NMG_FV_REC_WENOM5_2 && c >= 2 && c <= n - 3) {
    *rgt = weno5_p(v);
    *lft = weno5_m(v);
    return;
  }
  if (mode == NMG_FV_REC_WENOMZ_2 && c >= 2 && c <= n - 3) {
    *rgt = wenoz_p(v);
    *lft = wenoz_m(v);
    return;
  }
  if (c >= 1 && c <= n - 2) {
    *rgt = weno3_p(v + 1, 1., r3, -0.5, 1.5, 0.5, 0.5);
    *lft = weno3_m(v + 1, r3, 1., 0.5, 0.5, 1.5, -0.5);
    return;
  }
  // end cells: one face each (c == 0: midpoint 0; c == n-1: midpoint n-2)
  if (n < 3) {
    *lft = v[2];
    *rgt = v[2];
  } else {
    *rgt = 0.5 * v[2] + 0.5 * v[3];
    *lft = 0.5 * v[1] + 0.5 * v[2];
  }
}
