// grhd.cu -- pointwise GRHD conservative <-> primitive conversion on the
// device (ideal gas, conformally flat 3-metric gamma_ij = psi^4 delta_ij).
//
// The reference has no GRHD (its GRHD lives in external repositories); the
// one piece it has is the root finder this conversion needs, newton1d_brak
// (src/utility/numerics/newton1d_brak.c:20-121, Newton-Raphson with a
// bracket and bisection fallback), restated here as a device template.
// The physics is restated (parity unpinned):
//   D = psi^6 rho W, S_i = psi^6 rho h W^2 v_i, tau = psi^6 (rho h W^2 - p) - D,
//   v_i = psi^4 v^i, W = 1/sqrt(1 - v_i v^i), h = 1 + eps + p/rho,
//   p = (gamma - 1) rho eps;
// con2prim solves f(p) = (gamma-1) rho(p) eps(p) - p = 0 for the pressure
// (f'(p) ~ v^2 c_s^2 - 1), with the previous pressure as the starting guess,
// and sets the atmosphere (rho_atm, v = 0, p_atm; conserved variables reset)
// where D/psi^6 < rho_atm or the root finder fails.  Every iteration loop
// is bounded (maxits, 200 bracket doublings).  With a lapse alpha (static
// background, zero shift) it also gives the Valencia fluxes, the
// characteristic speeds and the Cowling source terms.  This file is
// compiled with -fmad=false so that it rounds like the host restatement.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>

#include "../../include/nmg.h"

namespace {

#include "grhd.cuh"

__global__ void prim2con_kernel(nmg_grhd_params g, int64_t npts, const double *psi,
                                const double *prim, double *cons) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < npts;
       i += (int64_t)gridDim.x * blockDim.x) {
    double P[5], U[5];
    for (int f = 0; f < 5; f++) P[f] = prim[f * npts + i];
    p2c_point(g, psi ? psi[i] : 1., P, U);
    for (int f = 0; f < 5; f++) cons[f * npts + i] = U[f];
  }
}

__global__ void con2prim_kernel(nmg_grhd_params g, int64_t npts, const double *psi,
                                double *cons, double *prim, int32_t *status) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < npts;
       i += (int64_t)gridDim.x * blockDim.x) {
    double P[5], U[5];
    for (int f = 0; f < 5; f++) {
      U[f] = cons[f * npts + i];
      P[f] = prim[f * npts + i];
    }
    const int rc = c2p_point(g, psi ? psi[i] : 1., U, P);
    for (int f = 0; f < 5; f++) {
      cons[f * npts + i] = U[f];
      prim[f * npts + i] = P[f];
    }
    status[i] = rc;
  }
}

// Valencia fluxes along direction d and the characteristic speeds there
// (static conformally flat background, zero shift)
__global__ void fluxes_kernel(nmg_grhd_params g, int64_t npts, int d, const double *alpha,
                              const double *psi, const double *prim, double *flux, double *lam) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < npts;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double al = alpha ? alpha[i] : 1., ps = psi ? psi[i] : 1.;
    const double ps4 = ps * ps * ps * ps, ps6 = ps4 * ps * ps;
    const double rho = prim[i];
    const double v[3] = {prim[npts + i], prim[2 * npts + i], prim[3 * npts + i]};
    const double p = prim[4 * npts + i];
    const double v2 = ps4 * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    const double W = 1. / sqrt(1. - v2);
    const double eps = p / ((g.gamma - 1.) * rho);
    const double h = 1. + eps + p / rho;
    const double rhW2 = rho * h * W * W;
    const double D = ps6 * rho * W, tau = ps6 * (rhW2 - p) - D, avd = al * v[d];
    const double cs2 = g.gamma * p / (rho * h);
    double disc = (1. - v2) * (1. / ps4 * (1. - v2 * cs2) - v[d] * v[d] * (1. - cs2));
    const double fac = al / (1. - v2 * cs2);
    flux[i] = avd * D;
    for (int j = 0; j < 3; j++) {
      const double Sj = ps6 * rhW2 * ps4 * v[j];
      flux[(1 + j) * npts + i] = avd * Sj + (j == d ? al * ps6 * p : 0.);
    }
    flux[4 * npts + i] = avd * tau + al * ps6 * p * v[d];
    if (disc < 0.) disc = 0.;
    lam[i] = fac * (v[d] * (1. - cs2) - sqrt(cs2) * sqrt(disc));
    lam[npts + i] = fac * (v[d] * (1. - cs2) + sqrt(cs2) * sqrt(disc));
  }
}

// Cowling source terms of S_j and tau (D has none)
__global__ void sources_kernel(nmg_grhd_params g, int64_t npts, const double *alpha,
                               const double *psi, const double *dalpha, const double *dpsi,
                               const double *prim, double *src) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < npts;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double al = alpha[i], ps = psi[i];
    const double ps4 = ps * ps * ps * ps, ps6 = ps4 * ps * ps;
    const double rho = prim[i];
    const double v[3] = {prim[npts + i], prim[2 * npts + i], prim[3 * npts + i]};
    const double p = prim[4 * npts + i];
    const double v2 = ps4 * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    const double W = 1. / sqrt(1. - v2);
    const double eps = p / ((g.gamma - 1.) * rho);
    const double h = 1. + eps + p / rho;
    const double rhW2 = rho * h * W * W;
    const double E = rhW2 - p;
    double vda = 0.;
    src[i] = 0.;
    for (int j = 0; j < 3; j++) {
      const double da = dalpha[j * npts + i], dp = dpsi[j * npts + i];
      src[(1 + j) * npts + i] = ps6 * (2. * al * (dp / ps) * (rhW2 * v2 + 3. * p) - E * da);
      vda += v[j] * da;
    }
    src[4 * npts + i] = -ps6 * rhW2 * vda;
  }
}

bool bad_params(const nmg_grhd_params *g) {
  return !g || !(g->gamma > 1.) || !(g->rho_atm > 0.) || !(g->p_atm > 0.) || !(g->tol > 0.) ||
         g->maxits <= 0 || g->maxits > 100000;
}

}  // namespace

extern "C" {

int nmg_grhd_prim2con(const nmg_grhd_params *g, int64_t npts, const double *psi_dev,
                      const double *prim_dev, double *cons_dev, void *stream) {
  if (bad_params(g) || npts < 0 || (npts > 0 && (!prim_dev || !cons_dev))) return NMG_EINVAL;
  if (npts == 0) return NMG_OK;
  const int grid = (int)std::min<int64_t>((npts + 255) / 256, 152 * 32);
  prim2con_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(*g, npts, psi_dev, prim_dev, cons_dev);
  return cudaGetLastError() == cudaSuccess ? NMG_OK : NMG_ECUDA;
}

int nmg_grhd_con2prim(const nmg_grhd_params *g, int64_t npts, const double *psi_dev,
                      double *cons_dev, double *prim_dev, int32_t *status_dev, void *stream) {
  if (bad_params(g) || npts < 0 || (npts > 0 && (!prim_dev || !cons_dev || !status_dev)))
    return NMG_EINVAL;
  if (npts == 0) return NMG_OK;
  const int grid = (int)std::min<int64_t>((npts + 127) / 128, 152 * 32);
  con2prim_kernel<<<grid, 128, 0, (cudaStream_t)stream>>>(*g, npts, psi_dev, cons_dev, prim_dev,
                                                          status_dev);
  return cudaGetLastError() == cudaSuccess ? NMG_OK : NMG_ECUDA;
}

int nmg_grhd_fluxes(const nmg_grhd_params *g, int64_t npts, int32_t dir, const double *alpha_dev,
                    const double *psi_dev, const double *prim_dev, double *flux_dev,
                    double *lam_dev, void *stream) {
  if (bad_params(g) || npts < 0 || dir < 0 || dir > 2 ||
      (npts > 0 && (!prim_dev || !flux_dev || !lam_dev)))
    return NMG_EINVAL;
  if (npts == 0) return NMG_OK;
  const int grid = (int)std::min<int64_t>((npts + 255) / 256, 152 * 32);
  fluxes_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(*g, npts, dir, alpha_dev, psi_dev,
                                                        prim_dev, flux_dev, lam_dev);
  return cudaGetLastError() == cudaSuccess ? NMG_OK : NMG_ECUDA;
}

int nmg_grhd_sources(const nmg_grhd_params *g, int64_t npts, const double *alpha_dev,
                     const double *psi_dev, const double *dalpha_dev, const double *dpsi_dev,
                     const double *prim_dev, double *src_dev, void *stream) {
  if (bad_params(g) || npts < 0 ||
      (npts > 0 && (!alpha_dev || !psi_dev || !dalpha_dev || !dpsi_dev || !prim_dev || !src_dev)))
    return NMG_EINVAL;
  if (npts == 0) return NMG_OK;
  const int grid = (int)std::min<int64_t>((npts + 255) / 256, 152 * 32);
  sources_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(*g, npts, alpha_dev, psi_dev,
                                                         dalpha_dev, dpsi_dev, prim_dev, src_dev);
  return cudaGetLastError() == cudaSuccess ? NMG_OK : NMG_ECUDA;
}

}  // extern "C"
