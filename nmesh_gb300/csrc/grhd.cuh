// grhd.cuh -- device pieces of the GRHD conservative -> primitive recovery
// shared by the pointwise entry points (grhd.cu) and the evolution
// (grhd_evolve.cu): f(p) of the pressure root and the reference's root
// finder newton1d_brak (src/utility/numerics/newton1d_brak.c:20-121:
// Newton-Raphson with a bracket and bisection fallback), restated.
// Included inside an anonymous namespace of each translation unit.
#pragma once

struct C2P {
  double D, tau, S2, gm1, gam;
  __device__ void operator()(double p, double *f, double *df) const {
    const double E = tau + D + p;
    const double v2 = S2 / (E * E);
    const double W = 1. / sqrt(1. - v2);
    const double rho = D / W;
    const double eps = (tau + D * (1. - W) + p * (1. - W * W)) / (D * W);
    const double cs2 = gam * gm1 * eps / (1. + gam * eps);
    *f = gm1 * rho * eps - p;
    *df = v2 * cs2 - 1.;
  }
};

// newton1d_brak: iterations (>= 0) or a negative error code, root in *x0
template <class F>
__device__ int newton1d_brak(double *x0, const F &fdf, double x1, double x2, int maxits,
                             double xacc) {
  int j, bisect;
  double f, fh, fl, df, xh, xl, xrt, dx, dxold, tmp;
  if (!isfinite(x1) || !isfinite(x2)) return -2 * maxits - 2;
  if ((x1 <= *x0 && *x0 <= x2) || (x2 <= *x0 && *x0 <= x1)) xrt = *x0;
  else xrt = 0.5 * (x1 + x2);
  fdf(x1, &fl, &df);
  fdf(x2, &fh, &df);
  j = 0;
  if (fl <= 0.0 && fh >= 0.0) j = 1;
  if (fl >= 0.0 && fh <= 0.0) j = 1;
  if (!j) return -2 * maxits - 3;
  if (fl == 0.0) { *x0 = x1; return 0; }
  if (fh == 0.0) { *x0 = x2; return 0; }
  if (fl < 0.0) { xl = x1; xh = x2; }
  else { xh = x1; xl = x2; }
  dxold = fabs(x2 - x1);
  dx = dxold;
  for (j = 1; j <= maxits; j++) {
    fdf(xrt, &f, &df);
    if (!isfinite(f)) return -j;
    if (f == 0.0) { *x0 = xrt; return j; }
    if (f < 0.0) xl = xrt;
    else xh = xrt;
    if (!isfinite(df)) bisect = 1;
    else bisect = (fabs(2.0 * f) > fabs(dxold * df));
    if (bisect == 0) {
      dxold = dx;
      dx = f / df;
      tmp = xrt;
      xrt -= dx;
      if (((xrt - xh) * (xrt - xl) > 0.0) || (tmp == xrt)) {
        bisect = 1; xrt = tmp; dx = dxold;
      }
    }
    if (bisect) {
      dxold = dx;
      dx = 0.5 * (xh - xl);
      xrt = xl + dx;
      if (xl == xrt) { *x0 = xrt; return j; }
    }
    if (fabs(dx) < xacc) { *x0 = xrt; return j; }
  }
  *x0 = xrt;
  return j;
}


// U of the primitives P at conformal factor ps (D = psi^6 rho W,
// S_i = psi^6 rho h W^2 psi^4 v^i, tau = psi^6 (rho h W^2 - p) - D)
__device__ __forceinline__ void p2c_point(const nmg_grhd_params &g, double ps, const double P[5],
                                          double U[5]) {
  const double ps4 = ps * ps * ps * ps, ps6 = ps4 * ps * ps;
  const double rho = P[0], vx = P[1], vy = P[2], vz = P[3], p = P[4];
  const double v2 = ps4 * (vx * vx + vy * vy + vz * vz);
  const double W = 1. / sqrt(1. - v2);
  const double eps = p / ((g.gamma - 1.) * rho);
  const double h = 1. + eps + p / rho;
  const double rhW2 = rho * h * W * W;
  const double D = ps6 * rho * W;
  U[0] = D;
  U[1] = ps6 * rhW2 * ps4 * vx;
  U[2] = ps6 * rhW2 * ps4 * vy;
  U[3] = ps6 * rhW2 * ps4 * vz;
  U[4] = ps6 * (rhW2 - p) - D;
}

// con2prim of one point: the pressure root of f (C2P) by newton1d_brak
// between the physical lower bound and a doubled upper bracket, starting
// from P[4]; below rho_atm, or where the root finder fails, the atmosphere
// (rho_atm, v = 0, p_atm) with U reset to match.  Returns the iterations
// (>= 0) or < 0 where the atmosphere was set.  Every loop is bounded.
__device__ __forceinline__ int c2p_point(const nmg_grhd_params &g, double ps, double U[5],
                                         double P[5]) {
  const double ps4 = ps * ps * ps * ps, ps6 = ps4 * ps * ps;
  const double D = U[0] / ps6, Sx = U[1] / ps6, Sy = U[2] / ps6;
  const double Sz = U[3] / ps6, tau = U[4] / ps6;
  const double S2 = (Sx * Sx + Sy * Sy + Sz * Sz) / ps4;
  C2P q{D, tau, S2, g.gamma - 1., g.gamma};
  int rc = -1;
  if (D >= g.rho_atm && isfinite(D) && isfinite(tau) && isfinite(S2)) {
    const double S = sqrt(S2);
    double plo = S - tau - D;
    plo = plo > 0. ? plo * (1. + 1e-14) : 0.;
    double phi = q.gm1 * (tau + D);
    if (phi < plo) phi = 2. * plo;
    if (phi <= 0.) phi = 1e-300;
    for (int k = 0; k < 200; k++) {
      double f, df;
      q(phi, &f, &df);
      if (f < 0.) break;
      phi *= 2.;
    }
    double p = P[4];
    const double xacc = g.tol * phi;
    rc = newton1d_brak(&p, q, plo, phi, g.maxits, xacc);
    if (rc >= 0) {
      const double E = tau + D + p;
      const double v2 = S2 / (E * E);
      const double W = 1. / sqrt(1. - v2);
      const double rho = D / W;
      if (!(rho >= g.rho_atm) || !(p > 0.) || !isfinite(W)) {
        rc = -1;
      } else {
        const double fac = 1. / (E * ps4);
        P[0] = rho;
        P[1] = Sx * fac;
        P[2] = Sy * fac;
        P[3] = Sz * fac;
        P[4] = p;
      }
    }
  }
  if (rc < 0) {
    const double eps_atm = g.p_atm / ((g.gamma - 1.) * g.rho_atm);
    const double h = 1. + eps_atm + g.p_atm / g.rho_atm;
    P[0] = g.rho_atm;
    P[1] = P[2] = P[3] = 0.;
    P[4] = g.p_atm;
    const double Da = ps6 * g.rho_atm;
    U[0] = Da;
    U[1] = U[2] = U[3] = 0.;
    U[4] = ps6 * (g.rho_atm * h - g.p_atm) - Da;
  }
  return rc;
}
